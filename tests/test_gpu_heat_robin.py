"""GPU parity of the heat plugin's Robin terms and objectives against the
oracle (oracle/heat_robin.py) on the plate of the reference's heat flow test
(8 x 8 x 1, Robin on two sides, T = 600 on a corner patch, k = 10).

Tolerances: FP64 objectives 1e-10 relative (heat exchange 1e-9: its
numerator cancels T - T_env), mixed 1e-6, each plus the rounding floor of the
objective, 4 eps |T|^T |K| |T| / |J|: with T = 600 on the Dirichlet nodes the
compliance T^T K T cancels by a factor of ~1e7, so two correct evaluations
differ by ~1e-9; temperatures 1e-8 of max |T|; adjoints, energies and
sensitivities 1e-8 relative L2 (mixed 1e-5).
The nodal density average is bit-identical (same summation order).
"""
import numpy as np
import pytest

from oracle import heat_robin as hr
from oracle import optim as oopt
from oracle import problems

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _fem(tsk, precision, pairing="reference"):
    from sktopt_gb300.fea.solver_elastic import LinearSolverConfig
    from sktopt_gb300.fea.solver_heat import FEM_SimpLinearHeatConduction
    return FEM_SimpLinearHeatConduction(
        tsk, 1e-3, solver_config=LinearSolverConfig(solver="cg_pyamg", precision=precision,
                                                    rtol=1e-12),
        device=_dev(), nodal_pairing=pairing)


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("pairing", ["reference", "element"])
def test_nodal_average_bitwise(native_lib, pairing):
    import torch
    from sktopt_gb300.fea.solver_heat import HeatRobinOps
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.heat_plate(12, 10, 3)
    m, *_ = problems.heat_plate(12, 10, 3)
    rho = np.random.default_rng(4).uniform(0, 1, m.nelements)
    ops = HeatRobinOps(tsk.mesh, pairing, device=_dev())
    out = torch.empty(m.nnodes, dtype=torch.float64, device=_dev())
    ops.nodal_average(torch.from_numpy(rho).to(_dev()), out)
    want, _ = hr.nodal_average(m, rho, pairing)
    assert np.array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("objective,avg_w", [("compliance", 0.0), ("heat_exchange", 0.0),
                                             ("heat_exchange", 0.5), ("averaged_temp", 0.0)])
def test_heat_robin_objectives_match_oracle(native_lib, objective, avg_w, precision):
    import torch
    from sktopt_gb300.mesh import toy_problem
    n = (12, 12, 3)
    tsk = toy_problem.heat_plate(*n, objective=objective, avg_temp_weight=avg_w)
    m, pb, *_ = problems.heat_plate(*n, objective=objective, avg_temp_weight=avg_w)
    assert pb.D.size > 0
    rho = np.random.default_rng(11).uniform(0.1, 1.0, m.nelements)
    p, kmin = 3.0, 10.0 * 1e-3
    J_ref, T_ref = pb.objectives(rho, p, kmin)
    en_ref = pb.energy(rho, p, kmin, T_ref)
    dc_ref = pb.custom_sensitivity(rho, p, kmin, T_ref)
    fem = _fem(tsk, precision)
    u = np.zeros((tsk.n_dof, 1))
    J = fem.objectives_multi_load(rho, p, u)
    K, _, _ = pb.operator(rho, p, kmin)
    aT = np.abs(T_ref[:, 0])
    floor = 4 * np.finfo(float).eps * (aT @ (abs(K) @ aT))
    tol = (1e-9 if objective == "heat_exchange" else 1e-10) if precision == "fp64" else 1e-6
    assert abs(J[0] - J_ref[0]) <= tol * abs(J_ref[0]) + floor, (J, J_ref, floor)
    np.testing.assert_allclose(u, T_ref, rtol=0, atol=1e-8 * np.abs(T_ref).max())
    vtol = 1e-8 if precision == "fp64" else 1e-5
    if objective != "compliance":
        assert _rel(fem.lam.cpu().numpy(), pb.lam) <= vtol
    assert _rel(fem.energy_multi_load(rho, p, u), en_ref) <= vtol
    assert _rel(fem.compliance_sensitivity_multi_load(rho, p, u), dc_ref) <= vtol


def test_heat_robin_two_dirichlet_values(native_lib):
    """Two Dirichlet values = two load cases; heat exchange with the
    avg_temp_weight scaling of several loads (solver_heat.py:855-868): six
    right-hand sides in two block solves."""
    from sktopt_gb300.mesh import toy_problem
    vals = [600.0, 450.0]
    tsk = toy_problem.heat_plate(12, 12, 3, objective="heat_exchange", avg_temp_weight=0.3,
                                 dirichlet_values=vals)
    m, pb, *_ = problems.heat_plate(12, 12, 3, objective="heat_exchange",
                                    avg_temp_weight=0.3, dirichlet_values=vals)
    rho = np.random.default_rng(12).uniform(0.1, 1.0, m.nelements)
    J_ref, T_ref = pb.objectives(rho, 3.0, 1e-2)
    fem = _fem(tsk, "fp64")
    u = np.zeros((tsk.n_dof, 2))
    J = fem.objectives_multi_load(rho, 3.0, u)
    K, _, _ = pb.operator(rho, 3.0, 1e-2)
    floor = max(4 * np.finfo(float).eps * (np.abs(T_ref[:, i]) @ (abs(K) @ np.abs(T_ref[:, i])))
                for i in range(2))
    np.testing.assert_allclose(J, J_ref, rtol=1e-9, atol=floor)
    np.testing.assert_allclose(u, T_ref, rtol=0, atol=1e-8 * np.abs(T_ref).max())
    assert _rel(fem.lam.cpu().numpy(), pb.lam) <= 1e-8
    assert _rel(fem.compliance_sensitivity_multi_load(rho, 3.0, u),
                pb.custom_sensitivity(rho, 3.0, 1e-2, T_ref)) <= 1e-8


@pytest.mark.parametrize("objective", ["compliance", "heat_exchange"])
def test_heat_robin_five_dirichlet_values(native_lib, objective):
    """Five load cases: the block solves, the compliance products and the
    heat-exchange integrals run in chunks of at most four columns."""
    from sktopt_gb300.mesh import toy_problem
    vals = [600.0, 550.0, 500.0, 450.0, 400.0]
    tsk = toy_problem.heat_plate(12, 12, 3, objective=objective, dirichlet_values=vals)
    m, pb, *_ = problems.heat_plate(12, 12, 3, objective=objective, dirichlet_values=vals)
    rho = np.random.default_rng(15).uniform(0.1, 1.0, m.nelements)
    J_ref, T_ref = pb.objectives(rho, 3.0, 1e-2)
    fem = _fem(tsk, "fp64")
    u = np.zeros((tsk.n_dof, len(vals)))
    J = fem.objectives_multi_load(rho, 3.0, u)
    K, _, _ = pb.operator(rho, 3.0, 1e-2)
    floor = max(4 * np.finfo(float).eps * (np.abs(T_ref[:, i]) @ (abs(K) @ np.abs(T_ref[:, i])))
                for i in range(len(vals)))
    np.testing.assert_allclose(J, J_ref, rtol=1e-9, atol=floor)
    np.testing.assert_allclose(u, T_ref, rtol=0, atol=1e-8 * np.abs(T_ref).max())


@pytest.mark.parametrize("objective", ["compliance", "heat_exchange"])
def test_heat_robin_oc_loop_matches_oracle(native_lib, objective):
    """OC loop on the plate (compliance: the reference flow test's task) against
    the oracle loop: per-iteration objective 1e-8 (the compliance cancels,
    see the module docstring), densities 1e-7.  Compliance with Robin data
    adds the explicit Robin gradient, whose grad rho / max(|grad rho|, 1e-12)
    turns the rounding noise of a uniform nodal density (|grad rho| ~ 1e-16)
    into terms ~1e-10: two correct evaluations differ there by ~1e-6 of the
    element sensitivity (measured: 4e-6 at most, densities 5e-7 after one
    step), so that case compares densities to 5e-6."""
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    n, n_iter, radius = (12, 12, 3), 4, 1.0
    cfg = OC_Config(max_iters=n_iter, filter_type="spacial",
                    filter_radius=tools.SchedulerConfig.constant(target_value=radius),
                    p=tools.SchedulerConfig.constant(target_value=3.0),
                    vol_frac=tools.SchedulerConfig.constant(target_value=0.4),
                    move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                    E_min_coeff=1e-3, solver_option="spsolve")
    opt = OC_Optimizer(cfg, toy_problem.heat_plate(*n, objective=objective), device=_dev())
    opt.parameterize()
    m, pb, design, fixed, vol = problems.heat_plate(*n, objective=objective)
    filt = problems.gaussian_filter_for(m, design, radius)
    ocfg = oopt.OracleConfig(max_iters=n_iter, p=oopt.Sched("Constant", 3.0, 3.0),
                             vol_frac=oopt.Sched("Constant", 0.4, 0.4),
                             move_limit=oopt.Sched("Constant", 0.2, 0.2),
                             filter_radius=oopt.Sched("Constant", radius, radius),
                             E_min_coeff=1e-3)
    ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories[objective][-1]
        assert abs(c - c_ref) <= 1e-8 * abs(c_ref), (k, c, c_ref)
        atol = 5e-6 if objective == "compliance" else 1e-7
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=atol)


def _tet_pair(n, objective, avg_w):
    from oracle import mesh as omesh
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.heat_plate_tet(*n, objective=objective, avg_temp_weight=avg_w)
    m = omesh.GridMesh(tsk.mesh.p, tsk.mesh.t, "tet", None, None, None)
    pb = hr.HeatRobinProblem(m, np.unique(np.asarray(tsk.dirichlet_nodes)), 600.0, k0=10.0,
                             robin_faces=[np.asarray(g) for g in tsk.robin_groups],
                             robin_coefficient=4.0e-5, robin_bc_value=300.0,
                             objective=objective, avg_temp_weight=avg_w)
    return tsk, m, pb


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("objective,avg_w", [("compliance", 0.0), ("heat_exchange", 0.5),
                                             ("averaged_temp", 0.0)])
def test_heat_robin_tetrahedra_match_oracle(native_lib, objective, avg_w, precision):
    """The plate meshed with jittered P1 tetrahedra: surface Robin terms on
    triangles, virtual Robin and heat-exchange forms with the 4-point rule,
    against the oracle's tetrahedral restatement (same tolerances as the
    hexahedral plate)."""
    import torch
    from sktopt_gb300.fea.solver_heat import HeatRobinOps
    tsk, m, pb = _tet_pair((10, 10, 2), objective, avg_w)
    assert not tsk.mesh.has_grid or tsk.mesh.kind == "tet"
    rho = np.random.default_rng(21).uniform(0.1, 1.0, m.nelements)
    # nodal average: same summation order, bitwise
    ops = HeatRobinOps(tsk.mesh, "reference", device=_dev())
    out = torch.empty(m.nnodes, dtype=torch.float64, device=_dev())
    ops.nodal_average(torch.from_numpy(rho).to(_dev()), out)
    assert np.array_equal(out.cpu().numpy(), hr.nodal_average(m, rho, "reference")[0])
    p, kmin = 3.0, 10.0 * 1e-3
    J_ref, T_ref = pb.objectives(rho, p, kmin)
    en_ref = pb.energy(rho, p, kmin, T_ref)
    dc_ref = pb.custom_sensitivity(rho, p, kmin, T_ref)
    fem = _fem(tsk, precision)
    u = np.zeros((tsk.n_dof, 1))
    J = fem.objectives_multi_load(rho, p, u)
    K, _, _ = pb.operator(rho, p, kmin)
    aT = np.abs(T_ref[:, 0])
    floor = 4 * np.finfo(float).eps * (aT @ (abs(K) @ aT))
    tol = (1e-9 if objective == "heat_exchange" else 1e-10) if precision == "fp64" else 1e-6
    assert abs(J[0] - J_ref[0]) <= tol * abs(J_ref[0]) + floor, (J, J_ref, floor)
    np.testing.assert_allclose(u, T_ref, rtol=0, atol=1e-8 * np.abs(T_ref).max())
    vtol = 1e-8 if precision == "fp64" else 1e-5
    if objective != "compliance":
        assert _rel(fem.lam.cpu().numpy(), pb.lam) <= vtol
    assert _rel(fem.energy_multi_load(rho, p, u), en_ref) <= vtol
    assert _rel(fem.compliance_sensitivity_multi_load(rho, p, u), dc_ref) <= vtol


def _jit_pair(n, objective, avg_w, drop_grid=False):
    import dataclasses
    from oracle import mesh as omesh
    from sktopt_gb300.mesh import toy_problem
    from sktopt_gb300.mesh.grid import GridMesh
    tsk = toy_problem.heat_plate(*n, objective=objective, avg_temp_weight=avg_w, jitter=0.2,
                                 seed=5)
    if drop_grid:
        tsk = dataclasses.replace(tsk, mesh=GridMesh(tsk.mesh.p, tsk.mesh.t, "hex"))
        assert not tsk.mesh.has_grid
    m = omesh.GridMesh(tsk.mesh.p, tsk.mesh.t, "hex", None, None, None)
    pb = hr.HeatRobinProblem(m, np.unique(np.asarray(tsk.dirichlet_nodes)), 600.0, k0=10.0,
                             robin_faces=[np.asarray(g) for g in tsk.robin_groups],
                             robin_coefficient=4.0e-5, robin_bc_value=300.0,
                             objective=objective, avg_temp_weight=avg_w)
    return tsk, m, pb


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("objective,avg_w,drop_grid", [("compliance", 0.0, False),
                                                       ("heat_exchange", 0.5, False),
                                                       ("averaged_temp", 0.0, False),
                                                       ("heat_exchange", 0.5, True)])
def test_heat_robin_general_hexahedra_match_oracle(native_lib, objective, avg_w, drop_grid,
                                                   precision):
    """The plate with its interior nodes jittered (general trilinear
    hexahedra, planar boundary faces): virtual Robin, heat-exchange and
    gradient forms with the Jacobian at every Gauss point, surface Robin
    terms on the faces' bilinear maps, against the oracle (same tolerances
    as the box plate).  drop_grid: the same mesh without its logical grid,
    as read from a file, solved on the scalar smoothed-aggregation
    hierarchy."""
    tsk, m, pb = _jit_pair((10, 10, 2), objective, avg_w, drop_grid)
    rho = np.random.default_rng(23).uniform(0.1, 1.0, m.nelements)
    p, kmin = 3.0, 10.0 * 1e-3
    J_ref, T_ref = pb.objectives(rho, p, kmin)
    en_ref = pb.energy(rho, p, kmin, T_ref)
    dc_ref = pb.custom_sensitivity(rho, p, kmin, T_ref)
    fem = _fem(tsk, precision)
    u = np.zeros((tsk.n_dof, 1))
    J = fem.objectives_multi_load(rho, p, u)
    K, _, _ = pb.operator(rho, p, kmin)
    aT = np.abs(T_ref[:, 0])
    floor = 4 * np.finfo(float).eps * (aT @ (abs(K) @ aT))
    tol = (1e-9 if objective == "heat_exchange" else 1e-10) if precision == "fp64" else 1e-6
    assert abs(J[0] - J_ref[0]) <= tol * abs(J_ref[0]) + floor, (J, J_ref, floor)
    np.testing.assert_allclose(u, T_ref, rtol=0, atol=1e-8 * np.abs(T_ref).max())
    vtol = 1e-8 if precision == "fp64" else 1e-5
    if objective != "compliance":
        assert _rel(fem.lam.cpu().numpy(), pb.lam) <= vtol
    assert _rel(fem.energy_multi_load(rho, p, u), en_ref) <= vtol
    assert _rel(fem.compliance_sensitivity_multi_load(rho, p, u), dc_ref) <= vtol
