"""GPU smoothed-aggregation multigrid for meshes without a logical grid.

* The aggregates are a partition into connected aggregates.
* P and the Galerkin coarse operator, from the GPU's own aggregates and
  lambda_max, equal their CPU restatement (``oracle.amg.
  sa_transfer_from_aggregates``) on the oracle's enforced matrix: 1e-10
  relative in FP64, 1e-5 in FP32.
* The AMG-preconditioned solves (FP64 PCG, mixed flexible CG, a 2-column
  block) reach 1e-8 and match SuperLU; they take far fewer iterations than
  block-Jacobi CG on the same system (the reference's cg_pyamg /
  cg_jacobi pair, solver_elastic.py:84-103).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import amg as oamg
from oracle import fem as ofem
from oracle import mesh as omesh

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _tet_problem(nx, ny, nz, seed=0):
    """Jittered 6-tet box 2 x 1 x 1 with the logical grid dropped, x = 0
    clamped, two load cases at the x = 2 bottom edge."""
    from sktopt_gb300.mesh import LinearElasticity, create_box_tet
    from sktopt_gb300.mesh.grid import GridMesh
    m = create_box_tet(nx, ny, nz, 2.0, 1.0, 1.0, jitter=0.2, seed=seed)
    mesh = GridMesh(m.p, m.t, "tet")
    assert not mesh.has_grid
    dn = np.nonzero(np.isclose(mesh.p[0], 0.0))[0]
    tip = np.nonzero(np.isclose(mesh.p[0], 2.0) & np.isclose(mesh.p[2], 0.0))[0]
    f1 = np.zeros(3 * mesh.nnodes)
    f1[3 * tip + 2] = -1.0 / tip.size
    f2 = np.zeros(3 * mesh.nnodes)
    f2[3 * tip + 1] = 1.0 / tip.size
    tsk = LinearElasticity.from_nodes(mesh, dn, "all", [tip, tip], [f1, f2],
                                      np.arange(mesh.nelements), 1.0, 0.3)
    om = omesh.GridMesh(mesh.p, mesh.t, "tet", None, None, None)
    pb = ofem.ElasticProblem(om, dn, [f1, f2])
    return mesh, tsk, pb


def _engine(mesh, tsk, mixed, **kw):
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.engine import FemEngine
    Ke, _, _ = composer.element_matrices(mesh, 0.3)
    return FemEngine(mesh, 3, Ke, tsk.dirichlet_mask, mixed=mixed, multigrid=True,
                     mg_coarse_max=200, device=_dev(), **kw)


def _rho(n, seed=1):
    g = np.random.default_rng(seed)
    return 0.01 + 0.99 * g.random(n)


def _p_matrix(X, n_fine, bs=3):
    rows = np.repeat(np.arange(n_fine), np.diff(X["p_ptr"]))
    nc = X["n_coarse"]
    Pb = sp.bsr_matrix((X["p_vals"], X["p_col"], X["p_ptr"]), shape=(n_fine * bs, nc * bs))
    assert rows.size == X["p_col"].size
    return Pb.tocsr()


@pytest.mark.parametrize("mixed", [False, True])
def test_transfer_matches_restatement(native_lib, mixed):
    import torch
    mesh, tsk, pb = _tet_problem(10, 5, 5)
    eng = _engine(mesh, tsk, mixed)
    assert eng.amg and eng.multigrid and eng.n_levels >= 2
    rho = _rho(mesh.nelements)
    eng.update(torch.from_numpy(rho).to(_dev()), 1.0, 1e-9, 3.0)
    X = eng.amg_export(0, 0 if mixed else 1)
    agg, nc = X["agg"], X["n_coarse"]
    n = mesh.nnodes
    # a partition of the nodes into connected aggregates
    assert agg.min() >= 0 and agg.max() == nc - 1 and np.unique(agg).size == nc
    K = pb.stiffness(rho, 3.0, 1e-9)
    A, _ = ofem.enforce(K, pb.forces[0], pb.dirichlet_dofs)
    G = sp.csr_matrix((np.ones(K.nnz), K.indices, K.indptr), shape=K.shape)
    node_graph = (sp.kron(sp.eye(n), np.ones((1, 3))) @ G @ sp.kron(sp.eye(n), np.ones((3, 1))))
    node_graph = sp.csr_matrix(node_graph)
    for a in np.unique(agg)[:: max(1, nc // 40)]:
        members = np.flatnonzero(agg == a)
        ncomp, _ = sp.csgraph.connected_components(node_graph[members][:, members],
                                                   directed=False)
        assert ncomp == 1
    # P and the coarse operator against the restatement on the same aggregates
    mask = np.zeros(3 * n, np.int64)
    mask[pb.dirichlet_dofs] = 1
    P_ref, Ac_ref, _ = oamg.sa_transfer_from_aggregates(A, agg.astype(np.int64), 1 - mask, 3,
                                                        X["lmax"])
    P = _p_matrix(X, n)
    tol = 1e-5 if mixed else 1e-10
    dP = abs(P - P_ref).max()
    assert dP <= tol * abs(P_ref).max(), dP
    dA = np.abs(X["coarse"] - Ac_ref).max()
    assert dA <= tol * np.abs(Ac_ref).max(), dA


@pytest.mark.parametrize("mixed", [False, True])
def test_amg_solve_matches_direct(native_lib, mixed):
    import torch
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    mesh, tsk, pb = _tet_problem(16, 8, 8, seed=2)
    cfg = LinearSolverConfig(solver="cg_pyamg", rtol=1e-8,
                             precision="mixed" if mixed else "fp64", warm_start=False)
    fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=cfg, device=_dev())
    assert fem.engine.amg and fem.engine.n_levels >= 3
    rho = _rho(mesh.nelements, 3)
    U = torch.zeros((3 * mesh.nnodes, 2), dtype=torch.float64, device=_dev())
    comp = fem.solve_device(torch.from_numpy(rho).to(_dev()), 3.0, U)
    st = fem.last_stats
    assert st.status == 0 and st.relres <= 1e-8
    K = pb.stiffness(rho, 3.0, 1e-9)
    F = np.column_stack(pb.forces)
    Ke, Fe = ofem.enforce(K, F, pb.dirichlet_dofs)
    u0 = ofem.solve(Ke, Fe, "spsolve")
    u = U.cpu().numpy()
    for j in range(2):
        assert np.linalg.norm(u[:, j] - u0[:, j]) <= 1e-6 * np.linalg.norm(u0[:, j])
        c0 = Fe[:, j] @ u0[:, j]
        assert abs(comp[j] - c0) <= 1e-8 * abs(c0)


def test_amg_far_fewer_iterations_than_block_jacobi(native_lib):
    import torch
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    mesh, tsk, pb = _tet_problem(16, 8, 8, seed=4)
    rho = torch.from_numpy(_rho(mesh.nelements, 5)).to(_dev())
    its = {}
    for name, pre in (("amg", "mg"), ("jacobi", "jacobi")):
        cfg = LinearSolverConfig(solver="cg_pyamg", rtol=1e-8, precision="fp64", precond=pre,
                                 warm_start=False)
        fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=cfg, device=_dev())
        U = torch.zeros((3 * mesh.nnodes, 2), dtype=torch.float64, device=_dev())
        fem.solve_device(rho, 3.0, U)
        assert fem.last_stats.status == 0
        its[name] = fem.last_stats.iters
    assert its["amg"] * 4 <= its["jacobi"], its


def test_amg_deterministic(native_lib):
    import torch
    mesh, tsk, pb = _tet_problem(10, 5, 5, seed=6)
    out = []
    for _ in range(2):
        eng = _engine(mesh, tsk, False)
        eng.update(torch.from_numpy(_rho(mesh.nelements, 7)).to(_dev()), 1.0, 1e-9, 3.0)
        out.append(eng.amg_export(0, 1))
    for k in ("agg", "p_ptr", "p_col", "p_vals", "coarse"):
        np.testing.assert_array_equal(out[0][k], out[1][k])
