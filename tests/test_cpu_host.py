"""CPU checks of the product's host side: the C-ABI library loads and exports
every symbol declared in include/topt.h, the native pattern builder matches
the oracle's SciPy CSR bit for bit, and the set-up code (meshes, tasks,
element matrices, schedules) agrees with the oracle."""
import os
import re

import numpy as np
import pytest

from oracle import fem as ofem
from oracle import mesh as omesh
from oracle import problems
from oracle import schedule as osch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "topt.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(topt_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(native_lib):
    syms = _declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(native_lib, s)]
    assert not missing, missing
    from sktopt_gb300 import _native
    assert set(syms) == set(_native.SIGNATURES), set(syms) ^ set(_native.SIGNATURES)
    assert native_lib.topt_version().startswith(b"topt-gb300")


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_native_pattern_matches_scipy_csr(native_lib, kind):
    from sktopt_gb300.fea.engine import block_to_scalar_csr, pattern
    from sktopt_gb300.mesh import grid
    if kind == "hex":
        m, om = grid.create_box_hex(7, 3, 4), omesh.create_box_hex(7, 3, 4)
        Kl = ofem.hex_element_matrices(om.p[:, om.t[:, 0]], 0.3)[0]
    else:
        m = grid.create_box_tet(4, 3, 2, 2.0, 1.0, 1.0, jitter=0.2, seed=3)
        om = omesh.create_box_tet(4, 3, 2, 2.0, 1.0, 1.0, jitter=0.2, seed=3)
        Kl = ofem.element_matrices(om, 0.3)[0]
    assert np.array_equal(m.t, om.t) and np.allclose(m.p, om.p, rtol=0, atol=0)
    rp, ci, cp, co = pattern(m)
    K = ofem.assemble(om.t, Kl, np.ones(om.nelements), om.nnodes, 3)
    # contributions summed on the host in the pattern's order reproduce K
    nloc = m.t.shape[0]
    vals = np.zeros((ci.size, 3, 3))
    e, r = np.divmod(co, nloc * nloc)
    la, lb = np.divmod(r, nloc)
    blk = np.repeat(np.arange(ci.size), np.diff(cp))
    KK = Kl if Kl.ndim == 3 else np.broadcast_to(Kl, (om.nelements,) + Kl.shape)
    for c in range(3):
        for d in range(3):
            np.add.at(vals[:, c, d], blk, KK[e, 3 * la + c, 3 * lb + d])
    ip, idx, dat = block_to_scalar_csr(rp, ci, vals, 3)
    assert np.array_equal(ip, K.indptr) and np.array_equal(idx, K.indices)
    np.testing.assert_allclose(dat, K.data, rtol=0, atol=1e-14 * np.abs(K.data).max())
    # contributions of a block are listed in ascending element order
    for k in range(0, ci.size, max(1, ci.size // 50)):
        ek = e[cp[k]:cp[k + 1]]
        assert np.all(np.diff(ek) >= 0)


def test_pattern_rejects_bad_connectivity(native_lib):
    import ctypes as C
    t = np.array([[0], [1], [2], [9]], dtype=np.int32)   # node 9 out of range
    h = C.c_void_p()
    rc = native_lib.topt_pattern_build(4, 1, 4, t.ctypes.data_as(C.c_void_p), C.byref(h))
    assert rc == 4 and b"out of range" in native_lib.topt_last_error()


def test_cantilever_sets_match_oracle():
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(9, 5, 4)
    tsk.exlude_dirichlet_from_design()
    m, pb, design, fixed, vol = problems.cantilever(9, 5, 4)
    assert np.array_equal(tsk.design_elements, design)
    assert np.array_equal(np.sort(tsk.dirichlet_dofs), np.sort(pb.dirichlet_dofs))
    assert np.allclose(tsk.neumann_linear[0], pb.forces[0])
    assert np.allclose(tsk.elements_volume, vol)


def test_composer_matches_oracle_element_matrices():
    from sktopt_gb300.fea import composer
    from sktopt_gb300.mesh import grid
    m = grid.create_box_tet(2, 2, 2, 1.0, 1.0, 1.0, jitter=0.2, seed=9)
    om = omesh.create_box_tet(2, 2, 2, 1.0, 1.0, 1.0, jitter=0.2, seed=9)
    a = composer.element_matrices(m, 0.3)
    b = ofem.element_matrices(om, 0.3)
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=0, atol=1e-13 * np.abs(y).max())
    f = composer.source_vector(m, 1.0)
    assert np.isclose(f.sum(), 1.0)
    np.testing.assert_allclose(f, ofem.source_vector(om, 1.0), rtol=1e-13)


@pytest.mark.parametrize("kind,init,target,steps,curv", [
    ("Step", 1.0, 3.0, 3, None), ("StepAccelerating", 1.0, 2.0, 3, 2.0),
    ("StepDecelerating", 0.2, 0.9, 4, 3.0), ("SawtoothDecay", 0.3, 0.1, 3, None),
    ("Constant", 0.4, 0.4, None, None), ("StepToOne", None, 1.0, 4, None)])
def test_product_schedules_match_oracle(kind, init, target, steps, curv):
    from sktopt_gb300 import tools
    cfg = tools.SchedulerConfig.from_defaults("x", init, target, steps, None, curv, kind)
    s = tools.Scheduler.from_config(cfg)
    s.iters_max = 30
    for it in range(1, 33):
        assert s.value(it) == osch.value(kind, it, 30, init, target, steps, curv)


def test_product_rejects_bad_schedules():
    from sktopt_gb300 import tools
    with pytest.raises(ValueError):
        tools.SchedulerConfig.from_defaults(name="x", num_steps=3, target_value=0.5,
                                            scheduler_type="StepToOne")
