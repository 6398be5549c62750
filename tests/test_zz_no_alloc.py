"""The allocation-free dot product against the allocating one, through the C ABI.

``topt_reduce_dot_noalloc`` serves callers that cannot call cudaMalloc: a host
whose device memory is owned by its own pool, or a loop that must not stall
on the device synchronisation that cudaMalloc/cudaFree imply.  Its scratch is
a fixed device array instead of an allocation, so it must give the same
result as ``topt_reduce_dot`` (up to summation order, 1e-12 relative) on two
calls in a row -- the second call reuses the scratch the first one left --
and must refuse inputs larger than that scratch supports.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dot(lib, fn, x, y):
    import torch
    out = C.c_double()
    rc = getattr(lib, fn)(x.numel(), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                          C.byref(out), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.topt_last_error()
    return out.value


def test_noalloc_dot_matches_allocating_dot_twice(native_lib):
    import torch
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cpu").manual_seed(11)
    for n in (3_000_017, 65_537):
        x = torch.randn(n, generator=g, dtype=torch.float64).to(dev)
        y = torch.randn(n, generator=g, dtype=torch.float64).to(dev)
        ref = _dot(native_lib, "topt_reduce_dot", x, y)
        scale = float(torch.sum(torch.abs(x * y)).item())
        for _ in range(2):
            got = _dot(native_lib, "topt_reduce_dot_noalloc", x, y)
            assert abs(got - ref) <= 1e-12 * scale
        assert abs(ref - float(torch.dot(x, y).item())) <= 1e-12 * scale


def test_noalloc_dot_at_the_scratch_boundaries(native_lib):
    """One full chunk (65,536 elements, one partial sum), one element past
    4,095 full chunks (the last partial-sum slot holds a single product) and
    the maximum size (every slot used, the last chunk full), twice each; with
    x = y = 1 every partial is an integer, so the sum is exact."""
    import torch
    for n in (65_536, 4095 * 65_536 + 1, 4096 * 65_536):
        x = torch.ones(n, dtype=torch.float64, device="cuda")
        for _ in range(2):
            assert _dot(native_lib, "topt_reduce_dot_noalloc", x, x) == float(n)
        del x
        torch.cuda.empty_cache()


def test_noalloc_dot_rejects_sizes_beyond_its_scratch(native_lib):
    import torch
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = C.c_double()
    # the size check happens on the host before anything is launched
    rc = native_lib.topt_reduce_dot_noalloc(268_435_457, C.c_void_p(x.data_ptr()),
                                            C.c_void_p(x.data_ptr()), C.byref(out), None)
    assert rc == 4  # TOPT_BAD_INPUT
    assert b"maximum" in native_lib.topt_last_error()
    out.value = -1.0
    rc = native_lib.topt_reduce_dot_noalloc(0, None, None, C.byref(out), None)
    assert rc == 0 and out.value == 0.0
    assert np.isfinite(out.value)
