"""V-cycle replay as a CUDA graph against kernel-by-kernel launches.

The graph holds the same kernels with the same arguments as the direct
V-cycle, so every solve must give bitwise the same displacements, the same
iteration counts and the same compliance with replay on and off: on the
matrix-free FP32 hierarchy of a hex cantilever (mixed solvers 3 and 4), on
the FP64 hierarchy (PCG), on the smoothed-aggregation hierarchy of a
tetrahedral mesh with two load cases, across operator updates (each one
re-records the graph), Chebyshev degree and interval changes (each a new
graph) and launch-shape changes (the graph is marked stale).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _engine(tsk, mixed, graphs, **kw):
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.engine import FemEngine
    Ke, _, _ = composer.element_matrices(tsk.mesh, 0.3)
    eng = FemEngine(tsk.mesh, 3, Ke, tsk.dirichlet_mask, mixed=mixed, multigrid=True,
                    device=_dev(), **kw)
    eng.set_vcycle_graphs(graphs)
    return eng


def _solves(eng, tsk, method, rtol, seeds, variants):
    import torch
    F = torch.from_numpy(np.ascontiguousarray(np.column_stack(tsk.neumann_linear))).to(_dev())
    out = []
    for seed in seeds:
        rho = np.random.default_rng(seed).uniform(0.05, 1.0, tsk.mesh.nelements)
        eng.update(torch.from_numpy(rho).to(_dev()), 1.0, 1e-9, 3.0)
        for kw in variants:
            U = torch.zeros_like(F)
            comp, st = eng.solve(F, U, method, 1, rtol, 2000, **kw)
            assert st.status == 0, (seed, kw, st)
            out.append((U.cpu().numpy(), comp, st.iters, st.outer))
    return out


def _same(a, b):
    assert len(a) == len(b)
    for (Ua, ca, ia, oa), (Ub, cb, ib, ob) in zip(a, b):
        assert ia == ib and oa == ob
        np.testing.assert_array_equal(ca, cb)
        np.testing.assert_array_equal(Ua, Ub)


@pytest.mark.parametrize("mixed,method", [(True, 4), (True, 3), (False, 0)])
def test_hex_replay_bitwise(native_lib, mixed, method):
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(24, 12, 12)
    variants = [{}, {"cheb_degree": 3}, {"cheb_ratio": 20.0}, {}]
    res = []
    for graphs in (False, True):
        eng = _engine(tsk, mixed, graphs)
        res.append(_solves(eng, tsk, method, 1e-8, (1, 2), variants))
    _same(*res)


def _tet_two_loads(nx, ny, nz, seed):
    """Jittered 6-tet box with the logical grid dropped (smoothed-aggregation
    hierarchy), x = 0 clamped, two load cases at the x = 2 bottom edge."""
    from sktopt_gb300.mesh import LinearElasticity, create_box_tet
    from sktopt_gb300.mesh.grid import GridMesh
    m = create_box_tet(nx, ny, nz, 2.0, 1.0, 1.0, jitter=0.2, seed=seed)
    mesh = GridMesh(m.p, m.t, "tet")
    dn = np.nonzero(np.isclose(mesh.p[0], 0.0))[0]
    tip = np.nonzero(np.isclose(mesh.p[0], 2.0) & np.isclose(mesh.p[2], 0.0))[0]
    f1 = np.zeros(3 * mesh.nnodes)
    f1[3 * tip + 2] = -1.0 / tip.size
    f2 = np.zeros(3 * mesh.nnodes)
    f2[3 * tip + 1] = 1.0 / tip.size
    return LinearElasticity.from_nodes(mesh, dn, "all", [tip, tip], [f1, f2],
                                       np.arange(mesh.nelements), 1.0, 0.3)


def test_tet_amg_two_loads_replay_bitwise(native_lib):
    tsk = _tet_two_loads(12, 6, 6, 3)
    res = []
    for graphs in (False, True):
        eng = _engine(tsk, True, graphs, mg_coarse_max=200)
        assert eng.amg
        res.append(_solves(eng, tsk, 4, 1e-8, (4, 5), [{}, {}]))
    _same(*res)


def test_stale_after_launch_shape_change(native_lib):
    """A row-mapping or tile change between two solves of the same operator
    must not replay the graph recorded with the old launch shapes."""
    import torch
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(20, 10, 10)
    F = torch.from_numpy(np.ascontiguousarray(np.column_stack(tsk.neumann_linear))).to(_dev())
    rho = torch.from_numpy(np.random.default_rng(7).uniform(1e-3, 1.0,
                                                            tsk.mesh.nelements)).to(_dev())
    res = []
    for graphs in (False, True):
        eng = _engine(tsk, True, graphs)
        eng.update(rho, 1.0, 1e-9, 3.0)
        one = []
        for mapping in (1, 3, 2):
            for lvl in range(1, eng.n_levels):
                eng.set_row_mapping(lvl, mapping)
            eng.set_mf_tile({1: 16, 3: 32, 2: 0}[mapping])
            U = torch.zeros_like(F)
            comp, st = eng.solve(F, U, 4, 1, 1e-8, 2000)
            assert st.status == 0
            one.append((U.cpu().numpy(), comp, st.iters, st.outer))
        res.append(one)
    _same(*res)
