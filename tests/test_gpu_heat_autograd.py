"""Heat conduction against the oracle, and the autograd compliance against
central finite differences (FP64, step 1e-6, 1e-5 relative) and the oracle's
sensitivity chain."""
import numpy as np
import pytest

from oracle import fem as ofem
from oracle import filters as ofilt
from oracle import problems

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _fd_check(fn, rho, grad, dirs, h=1e-6, tol=1e-5):
    for d in dirs:
        fp = float(fn(rho + h * d))
        fm = float(fn(rho - h * d))
        fd = (fp - fm) / (2 * h)
        an = float((grad * d).sum())
        assert abs(fd - an) <= tol * max(abs(an), 1e-300), (fd, an)


def test_heat_matches_oracle(native_lib):
    import torch
    from sktopt_gb300.fea.solver_elastic import LinearSolverConfig
    from sktopt_gb300.fea.solver_heat import FEM_SimpLinearHeatConduction
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.heat_box(12, 6, 6, patch=4)
    m, pb, design, fixed, vol = problems.heat_box(12, 6, 6, patch=4)
    assert np.allclose(tsk.emit, pb.emit, rtol=1e-13)
    rho = np.random.default_rng(3).uniform(0.05, 1.0, m.nelements)
    J_ref, T_ref = pb.objectives(rho, 3.0, 1e-3)
    en_ref = pb.energy(rho, 3.0, 1e-3, T_ref)[:, 0]
    dc_ref = ofem.dC_drho_simp(rho, en_ref, 1.0, 1e-3, 3.0)
    for precision in ("fp64", "mixed"):
        fem = FEM_SimpLinearHeatConduction(tsk, 1e-3, solver_config=LinearSolverConfig(
            solver="spsolve", precision=precision, rtol=1e-12), device=_dev())
        u = np.zeros((tsk.n_dof, 1))
        J = fem.objectives_multi_load(rho, 3.0, u)
        tol = 1e-10 if precision == "fp64" else 1e-6
        assert abs(J[0] - J_ref[0]) <= tol * abs(J_ref[0])
        np.testing.assert_allclose(u, T_ref, rtol=0, atol=1e-8 * np.abs(T_ref).max())
        en = fem.energy_multi_load(rho, 3.0, u)[:, 0]
        assert np.linalg.norm(en - en_ref) <= 1e-8 * np.linalg.norm(en_ref)
        dc = fem.compliance_sensitivity_multi_load(rho, 3.0, u)[:, 0]
        assert np.linalg.norm(dc - dc_ref) <= 1e-8 * np.linalg.norm(dc_ref)


def _elastic_fem(tsk):
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    return FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=LinearSolverConfig(
        solver="spsolve", rtol=1e-12), device=_dev())


def test_autograd_compliance_matches_finite_differences(native_lib):
    import torch
    from sktopt_gb300.core.autograd import compliance
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(12, 6, 6)
    fem = _elastic_fem(tsk)
    g = torch.Generator(device="cpu").manual_seed(5)
    rho = (0.1 + 0.9 * torch.rand(tsk.mesh.nelements, generator=g, dtype=torch.float64)).to(_dev())
    x = rho.clone().requires_grad_(True)
    C = compliance(x, fem, 3.0)
    C.backward()
    dirs = [torch.randn(rho.numel(), generator=g, dtype=torch.float64).to(_dev())
            for _ in range(3)]
    # single components where the central difference resolves them: the three
    # largest |dC/drho_e| (a component far below max|grad| drowns in the
    # rounding of C itself, eps*C/h ~ 1e-7 here)
    for i in torch.topk(x.grad.abs(), 3).indices.tolist():
        e = torch.zeros_like(rho)
        e[i] = 1.0
        dirs.append(e)
    with torch.no_grad():
        _fd_check(lambda r: compliance(r, fem, 3.0), rho, x.grad, dirs)


def test_autograd_thermal_compliance_matches_finite_differences(native_lib):
    import torch
    from sktopt_gb300.core.autograd import compliance
    from sktopt_gb300.fea.solver_elastic import LinearSolverConfig
    from sktopt_gb300.fea.solver_heat import FEM_SimpLinearHeatConduction
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.heat_box(12, 6, 6, patch=4)
    fem = FEM_SimpLinearHeatConduction(tsk, 1e-3, solver_config=LinearSolverConfig(
        solver="spsolve", rtol=1e-12), device=_dev())
    g = torch.Generator(device="cpu").manual_seed(6)
    rho = (0.1 + 0.9 * torch.rand(tsk.mesh.nelements, generator=g, dtype=torch.float64)).to(_dev())
    x = rho.clone().requires_grad_(True)
    compliance(x, fem, 3.0).backward()
    dirs = [torch.randn(rho.numel(), generator=g, dtype=torch.float64).to(_dev())
            for _ in range(3)]
    with torch.no_grad():
        _fd_check(lambda r: compliance(r, fem, 3.0), rho, x.grad, dirs)


def test_filtered_compliance_gradient_matches_oracle_chain(native_lib):
    import torch
    from sktopt_gb300.core.autograd import filtered_compliance
    from sktopt_gb300.filters import SpacialFilter
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(12, 6, 6)
    tsk.exlude_dirichlet_from_design()
    fem = _elastic_fem(tsk)
    flt = SpacialFilter.from_defaults(tsk.mesh, tsk.elements_volume, 1.5, tsk.design_mask,
                                      device=_dev())
    rho = np.random.default_rng(9).uniform(0.1, 1.0, tsk.mesh.nelements)
    beta = 1.25
    x = torch.from_numpy(rho).to(_dev()).requires_grad_(True)
    C = filtered_compliance(x, fem, flt, 3.0, beta, 0.5)
    C.backward()
    # oracle chain: filter -> projection -> solve -> energy -> dC -> dH -> W^T
    m, pb, design, fixed, vol = problems.cantilever(12, 6, 6)
    f = problems.gaussian_filter_for(m, design, 1.5)
    rf = f.forward(rho)
    rp = ofilt.heaviside_projection(rf, beta, 0.5)
    comp, U = pb.objectives(rp, 3.0, 1e-9, "spsolve")
    en = pb.energy(rp, 3.0, 1e-9, U)[:, 0]
    dc = ofem.dC_drho_simp(rp, en, 1.0, 1e-9, 3.0)
    ref = f.gradient(dc * ofilt.heaviside_projection_derivative(rf, beta, 0.5))
    assert abs(float(C.detach()) - comp[0]) <= 1e-10 * abs(comp[0])
    gr = x.grad.cpu().numpy()
    assert np.linalg.norm(gr - ref) <= 1e-8 * np.linalg.norm(ref)


def test_ramp_interpolation_matches_oracle(native_lib):
    """RAMP (composer.py:25-39, derivatives.py:56-72): assembled operator,
    compliance, energies and sensitivities against the oracle, and a short
    OC loop with interpolation="RAMP" against the oracle loop."""
    import torch
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.mesh import toy_problem
    from oracle import optim as oopt
    dev = torch.device("cuda", 0)
    nx, ny, nz = 10, 5, 4
    tsk = toy_problem.cantilever(nx, ny, nz)
    m, pb, design, fixed, vol = problems.cantilever(nx, ny, nz)
    pb.interp = "RAMP"
    rho = np.random.default_rng(21).uniform(0.05, 1.0, tsk.mesh.nelements)
    q = 3.0
    comp_ref, U_ref = pb.objectives(rho, q, 1e-9, "spsolve")
    en_ref = pb.energy(rho, q, 1e-9, U_ref)
    dc_ref = ofem.dC_drho_ramp(rho, en_ref[:, 0], 1.0, 1e-9, q)
    fem = FEM_SimpLinearElasticity(tsk, 1e-9, density_interpolation=composer.ramp_interpolation,
                                   solver_config=LinearSolverConfig(solver="cg_pyamg", rtol=1e-12),
                                   device=dev)
    U = torch.zeros((3 * tsk.mesh.nnodes, 1), dtype=torch.float64, device=dev)
    rt = torch.from_numpy(rho).to(dev)
    comp = fem.solve_device(rt, q, U)
    assert abs(comp[0] - comp_ref[0]) <= 1e-10 * abs(comp_ref[0])
    en, dc = fem.engine.energy(U, rt, 1.0, 1e-9, q, want_dc=True)
    assert np.linalg.norm(en.cpu().numpy() - en_ref) <= 1e-9 * np.linalg.norm(en_ref)
    assert np.linalg.norm(dc.cpu().numpy()[:, 0] - dc_ref) <= 1e-9 * np.linalg.norm(dc_ref)
    # short OC loop
    n_iter = 4
    cfg = OC_Config(max_iters=n_iter, filter_type="spacial", interpolation="RAMP",
                    filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                    p=tools.SchedulerConfig.constant(target_value=q),
                    vol_frac=tools.SchedulerConfig.constant(target_value=0.3),
                    move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                    E_min_coeff=1e-9, solver_option="spsolve")
    opt = OC_Optimizer(cfg, toy_problem.cantilever(nx, ny, nz), device=dev)
    opt.parameterize()
    ocfg = oopt.OracleConfig(method="oc", max_iters=n_iter, p=oopt.Sched("Constant", q, q),
                             vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                             move_limit=oopt.Sched("Constant", 0.2, 0.2),
                             filter_radius=oopt.Sched("Constant", 1.5, 1.5),
                             E_min_coeff=1e-9, interpolation="RAMP")
    filt = problems.gaussian_filter_for(m, design, 1.5)
    ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories["compliance"][-1]
        assert abs(c - c_ref) <= 1e-9 * abs(c_ref), (k, c, c_ref)
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=1e-7)
