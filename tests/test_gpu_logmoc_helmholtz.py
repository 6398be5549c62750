"""GPU parity of the percentile, the Helmholtz nodal filter and the LogMOC
loop against the oracle.

Percentile: bit-exact selection, lerp as numpy (1e-15 relative).
Helmholtz forward/gradient: 1e-10 relative (PCG to 1e-12 vs SuperLU).
LogMOC / OC-with-Helmholtz loops: per-iteration compliance 1e-8 relative,
densities 1e-6 absolute.
"""
import numpy as np
import pytest

from oracle import filters as ofilt
from oracle import mesh as omesh
from oracle import optim as oopt
from oracle import problems

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


@pytest.mark.parametrize("n,q", [(1, 95.0), (2, 50.0), (1000, 95.0), (100003, 95.0),
                                 (4097, 0.0), (4097, 100.0), (12345, 37.5)])
def test_percentile_matches_numpy(native_lib, n, q):
    import torch
    from sktopt_gb300.filters.base import DesignOps
    x = np.random.default_rng(n).standard_normal(n) * 10.0 ** np.random.default_rng(1).uniform(
        -8, 3, n)
    x[:: max(1, n // 7)] = 0.0
    xt = torch.from_numpy(x).to(_dev())
    ops = DesignOps()
    ops.lib = native_lib
    got = ops.percentile_abs(xt, q)
    ref = np.percentile(np.abs(x), q)
    assert got == pytest.approx(ref, rel=1e-15, abs=0.0)


@pytest.mark.parametrize("kind", ["hex", "tet", "tet_no_grid"])
def test_helmholtz_filter_matches_oracle(native_lib, kind):
    """tet_no_grid: the jittered tets with the logical grid dropped, as a
    mesh read from a file -- the nodal Helmholtz solves then run on the
    scalar (bs = 1) smoothed-aggregation hierarchy built on the GPU."""
    import torch
    from sktopt_gb300.filters import HelmholtzFilterNodal
    from sktopt_gb300.mesh import grid
    if kind == "hex":
        m, om = grid.create_box_hex(8, 5, 4, 0.25, 0.25, 0.25), \
            omesh.create_box_hex(8, 5, 4, 0.25, 0.25, 0.25)
        r = 0.3
    else:
        m = grid.create_box_tet(6, 4, 3, 1.5, 1.0, 0.75, jitter=0.2, seed=4)
        om = omesh.create_box_tet(6, 4, 3, 1.5, 1.0, 0.75, jitter=0.2, seed=4)
        r = 0.2
        if kind == "tet_no_grid":
            m = grid.GridMesh(m.p, m.t, "tet")
            assert not m.has_grid
    vol = omesh.elements_volume(om)
    mask = np.ones(m.nelements, bool)
    mask[:: 9] = False
    f = HelmholtzFilterNodal.from_defaults(m, vol, r, mask, device=_dev())
    of = ofilt.HelmholtzFilterNodal(om, vol, r, mask)
    x = np.random.default_rng(2).uniform(0.0, 1.0, m.nelements)
    y = f.forward(torch.from_numpy(x).to(_dev())).cpu().numpy()
    np.testing.assert_allclose(y, of.forward(x), rtol=1e-10, atol=1e-12)
    v = -np.random.default_rng(3).uniform(0.0, 1.0, m.nelements)
    g = f.gradient(torch.from_numpy(v).to(_dev())).cpu().numpy()
    np.testing.assert_allclose(g, of.gradient(v), rtol=1e-10, atol=1e-12)


def _cfgs(method, n_iter, filter_type, radius):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import LogMOC_Config, OC_Config
    kw = dict(max_iters=n_iter, filter_type=filter_type,
              filter_radius=tools.SchedulerConfig.constant(target_value=radius),
              p=tools.SchedulerConfig.constant(target_value=3.0),
              vol_frac=tools.SchedulerConfig.constant(target_value=0.3),
              move_limit=tools.SchedulerConfig.constant(target_value=0.2),
              E_min_coeff=1e-9, solver_option="spsolve")
    cfg = (LogMOC_Config if method == "logmoc" else OC_Config)(**kw)
    ocfg = oopt.OracleConfig(method=method, max_iters=n_iter, p=oopt.Sched("Constant", 3.0, 3.0),
                             vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                             move_limit=oopt.Sched("Constant", 0.2, 0.2),
                             filter_radius=oopt.Sched("Constant", radius, radius),
                             E_min_coeff=1e-9)
    if method == "logmoc":
        # LogMOC_Config keeps DensityMethodConfig's eta = 0.6 (OC_Config: 0.5)
        ocfg.lambda_lower, ocfg.lambda_upper = -1e7, 1e7
        ocfg.eta = oopt.Sched("Constant", 0.6, 0.6)
    return cfg, ocfg


@pytest.mark.parametrize("method,filter_type,radius", [
    ("logmoc", "spacial", 1.5), ("logmoc", "helmholtz", 0.6), ("oc", "helmholtz", 0.6)])
def test_loop_matches_oracle(native_lib, method, filter_type, radius):
    from sktopt_gb300.core import LogMOC_Optimizer, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    n_iter = 5
    cfg, ocfg = _cfgs(method, n_iter, filter_type, radius)
    Opt = LogMOC_Optimizer if method == "logmoc" else OC_Optimizer
    opt = Opt(cfg, toy_problem.cantilever(10, 5, 4), device=_dev())
    opt.parameterize()
    m, pb, design, fixed, vol = problems.cantilever(10, 5, 4)
    mask = np.zeros(m.nelements, bool)
    mask[design] = True
    filt = problems.gaussian_filter_for(m, design, radius) if filter_type == "spacial" else \
        ofilt.HelmholtzFilterNodal(m, vol, radius, mask)
    ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories["compliance"][-1]
        assert abs(c - c_ref) <= 1e-8 * abs(c_ref), (k, c, c_ref)
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=1e-6)
        assert opt.kkt_residual == pytest.approx(ref.hist["kkt_residual"][-1], rel=1e-5,
                                                 abs=1e-12)


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_helmholtz_vjp_is_the_exact_transpose(native_lib, kind):
    """<w, F(x + d) - F(x - d)> / 2 = <F^T w, d> for the filter's affine map F
    (forward) and its transpose vjp, with non-design elements present; the
    clamped reference ``gradient`` is not this transpose."""
    import torch
    from sktopt_gb300.filters import HelmholtzFilterNodal
    from sktopt_gb300.mesh import create_box_hex, create_box_tet
    m = create_box_hex(8, 5, 4) if kind == "hex" else \
        create_box_tet(6, 4, 3, 1.5, 1.0, 0.75, jitter=0.15, seed=2)
    rng = np.random.default_rng(17)
    mask = rng.random(m.nelements) > 0.2
    vol = omesh.elements_volume(omesh.GridMesh(m.p, m.t, kind, None, None, None))
    flt = HelmholtzFilterNodal(m, vol, 0.6 if kind == "hex" else 0.2, mask, device=_dev())
    x = torch.from_numpy(rng.uniform(0.1, 1.0, m.nelements)).to(_dev())
    d = torch.from_numpy(rng.standard_normal(m.nelements) * mask).to(_dev())
    w = torch.from_numpy(rng.standard_normal(m.nelements)).to(_dev())
    lhs = float(torch.dot(w, flt.forward_device(x + d) - flt.forward_device(x - d))) / 2.0
    rhs = float(torch.dot(flt.vjp_device(w), d))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1e-30), (lhs, rhs)
    assert torch.count_nonzero(flt.vjp_device(w)[torch.from_numpy(~mask).to(_dev())]) == 0


def test_helmholtz_filtered_compliance_gradient_matches_finite_differences(native_lib):
    """Compliance of H(F rho) with the Helmholtz filter through autograd (the
    exact transpose in backward) against FP64 central differences, step 1e-6,
    on the 12x6x6 cantilever."""
    import torch
    from sktopt_gb300.core.autograd import filtered_compliance
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.filters import HelmholtzFilterNodal
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(12, 6, 6)
    tsk.exlude_dirichlet_from_design()
    fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=LinearSolverConfig(
        solver="spsolve", rtol=1e-12), device=_dev())
    flt = HelmholtzFilterNodal(tsk.mesh, tsk.elements_volume, 0.8, tsk.design_mask,
                               device=_dev())
    g = torch.Generator(device="cpu").manual_seed(23)
    rho = (0.1 + 0.9 * torch.rand(tsk.mesh.nelements, generator=g, dtype=torch.float64)).to(_dev())
    x = rho.clone().requires_grad_(True)
    filtered_compliance(x, fem, flt, 3.0, 1.5, 0.5).backward()
    mask = torch.from_numpy(np.asarray(tsk.design_mask, bool)).to(_dev())
    h = 1e-6
    for k in range(3):
        d = torch.randn(rho.numel(), generator=g, dtype=torch.float64).to(_dev()) * mask
        with torch.no_grad():
            cp = float(filtered_compliance(rho + h * d, fem, flt, 3.0, 1.5, 0.5))
            cm = float(filtered_compliance(rho - h * d, fem, flt, 3.0, 1.5, 0.5))
        fd = (cp - cm) / (2 * h)
        ad = float(torch.dot(x.grad, d))
        assert abs(fd - ad) <= 1e-5 * abs(ad), (k, fd, ad)
