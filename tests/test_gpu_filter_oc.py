"""GPU parity of the Gaussian filter, projection and the OC loop against the oracle.

Filter matrix and applications: 1e-14 relative.  Projection: 1e-14.
OC loop (12x6x6 cantilever, spsolve-equivalent FP64 solves): per-iteration
compliance 1e-9 relative and densities 1e-7 absolute over 8 iterations.
"""
import numpy as np
import pytest

from oracle import filters as ofilt
from oracle import optim as oopt
from oracle import problems

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


@pytest.mark.parametrize("radius", [1.5, 2.2])
def test_gauss_filter_matrix_and_apply(native_lib, radius):
    import torch
    from sktopt_gb300.filters import SpacialFilter
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(9, 5, 4)
    tsk.exlude_dirichlet_from_design()
    m, pb, design, fixed, vol = problems.cantilever(9, 5, 4)
    mask = np.zeros(m.nelements, bool)
    mask[design] = True
    assert np.array_equal(mask, tsk.design_mask)
    f = SpacialFilter.from_defaults(tsk.mesh, tsk.elements_volume, radius, tsk.design_mask,
                                    device=_dev())
    of = ofilt.SpacialFilter(m, radius, mask)
    rp, ci, va = f.export_matrix()
    assert np.array_equal(rp, of.W.indptr) and np.array_equal(ci, of.W.indices)
    np.testing.assert_allclose(va, of.W.data, rtol=1e-14, atol=0)
    x = np.random.default_rng(0).uniform(0, 1, m.nelements)
    y = f.forward(torch.from_numpy(x).to(_dev())).cpu().numpy()
    np.testing.assert_allclose(y, of.forward(x), rtol=1e-14, atol=1e-15)
    g = f.gradient(torch.from_numpy(x).to(_dev())).cpu().numpy()
    np.testing.assert_allclose(g, of.gradient(x), rtol=1e-14, atol=1e-15)


def test_projection(native_lib):
    import torch
    from sktopt_gb300.core.projection import heaviside_projection_device
    x = np.random.default_rng(1).uniform(0, 1, 10007)
    xt = torch.from_numpy(x).to(_dev())
    h, dh = torch.empty_like(xt), torch.empty_like(xt)
    for beta in (1.0, 1.25, 8.0):
        heaviside_projection_device(xt, beta, 0.5, out=h, dout=dh)
        np.testing.assert_allclose(h.cpu().numpy(), ofilt.heaviside_projection(x, beta, 0.5),
                                   rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(dh.cpu().numpy(),
                                   ofilt.heaviside_projection_derivative(x, beta, 0.5),
                                   rtol=1e-13, atol=1e-15)


def _oc_cfg(n_iter):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config
    return OC_Config(max_iters=n_iter, filter_type="spacial",
                     filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                     p=tools.SchedulerConfig.constant(target_value=3.0),
                     vol_frac=tools.SchedulerConfig.constant(target_value=0.3),
                     move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                     E_min_coeff=1e-9, solver_option="spsolve")


def _oracle_opt(nx, ny, nz, n_iter):
    m, pb, design, fixed, vol = problems.cantilever(nx, ny, nz)
    filt = problems.gaussian_filter_for(m, design, 1.5)
    cfg = oopt.OracleConfig(max_iters=n_iter, p=oopt.Sched("Constant", 3.0, 3.0),
                            vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                            move_limit=oopt.Sched("Constant", 0.2, 0.2),
                            filter_radius=oopt.Sched("Constant", 1.5, 1.5), E_min_coeff=1e-9)
    return oopt.OracleOptimizer(cfg, pb, filt, design, fixed, vol), design


def test_oc_loop_matches_oracle(native_lib):
    from sktopt_gb300.core import OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    n_iter = 8
    opt = OC_Optimizer(_oc_cfg(n_iter), toy_problem.cantilever(12, 6, 6), device=_dev())
    opt.parameterize()
    ref, design = _oracle_opt(12, 6, 6, n_iter)
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories["compliance"][-1]
        assert abs(c - c_ref) <= 1e-9 * abs(c_ref), (k, c, c_ref)
        assert opt.recorder.histories["lmid"][-1] == pytest.approx(ref.hist["lmid"][-1],
                                                                   rel=1e-9)
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=1e-7)
        assert opt.kkt_residual == pytest.approx(ref.hist["kkt_residual"][-1], rel=1e-6)


def test_oc_fp32_bracketed_bisection_equals_fp64(native_lib):
    """FP32-bracketed bisection (its FP32 steps on the stencil form of W)
    takes the FP64 bisection's path: identical lmid, volume error, step count
    and density at every iteration."""
    import dataclasses
    from sktopt_gb300.core import OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    runs = []
    for bracket in (True, False):
        cfg = dataclasses.replace(_oc_cfg(6), bisection_fp32_bracket=bracket)
        opt = OC_Optimizer(cfg, toy_problem.cantilever(24, 12, 12), device=_dev())
        opt.parameterize()
        # the FP32 steps apply W as a 19-point stencil on this grid (r = 1.5)
        assert opt.filter.stencil_size == 19
        steps, rhos = [], []
        for _ in range(6):
            opt.optimize_steps(1)
            steps.append(opt.last_bisection_steps)
            rhos.append(opt._state.rho.cpu().numpy().copy())
        runs.append((opt.recorder.histories["lmid"], opt.recorder.histories["vol_error"],
                     steps, rhos))
    (l_a, v_a, s_a, r_a), (l_b, v_b, s_b, r_b) = runs
    assert list(l_a) == list(l_b)
    assert list(v_a) == list(v_b)
    assert s_a == s_b
    for a, b in zip(r_a, r_b):
        assert np.array_equal(a, b)


def test_oc_steps_equal_full_run_bitwise(native_lib):
    """The reference's determinism property (test_optimize_steps_equivalence.py:49)."""
    from sktopt_gb300.core import OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    a = OC_Optimizer(_oc_cfg(5), toy_problem.cantilever(10, 5, 5), device=_dev())
    a.parameterize()
    a.optimize()
    b = OC_Optimizer(_oc_cfg(5), toy_problem.cantilever(10, 5, 5), device=_dev())
    b.parameterize()
    for _ in range(5):
        b.optimize_steps(1)
    assert np.array_equal(a._state.rho.cpu().numpy(), b._state.rho.cpu().numpy())
    assert a.recorder.histories["compliance"] == b.recorder.histories["compliance"]
