"""The oracle's smoothed-aggregation AMG (the reference's ``cg_pyamg``
preconditioner, restated from PyAMG 5.x): aggregation known answers,
tentative-prolongator orthonormality, the V-cycle's symmetry, and the
preconditioned CG solution against the direct solve."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import amg, fem, problems


def _graph(edges, n):
    r = [i for i in range(n)] + [a for a, b in edges] + [b for a, b in edges]
    c = [i for i in range(n)] + [b for a, b in edges] + [a for a, b in edges]
    return sp.csr_matrix((np.ones(len(r)), (r, c)), shape=(n, n))


def test_standard_aggregation_path():
    S = _graph([(i, i + 1) for i in range(6)], 7)
    agg, na = amg.standard_aggregation(S)
    assert na == 3
    np.testing.assert_array_equal(agg, [0, 0, 1, 1, 1, 2, 2])


def test_standard_aggregation_grid_and_isolated():
    # 3x3 five-point grid (nodes 0..8) plus an isolated node 9
    e = []
    for y in range(3):
        for x in range(3):
            i = 3 * y + x
            if x < 2:
                e.append((i, i + 1))
            if y < 2:
                e.append((i, i + 3))
    S = _graph(e, 10)
    agg, na = amg.standard_aggregation(S)
    # pass 1: roots 0 ({0,1,3}) and 5 ({2,4,5,8}); pass 2: 6 -> via 3, 7 -> via 4
    assert na == 2
    np.testing.assert_array_equal(agg, [0, 0, 1, 0, 1, 1, 0, 1, 1, -1])


def test_pass3_aggregates_leftovers():
    # star 0-{1,2}, and a chain 3-4 whose nodes only touch each other after
    # pass 1 took 0's neighbourhood: 3 and 4 form a pass-1 aggregate too;
    # a triangle hanging off a pass-2 node exercises pass 3
    S = _graph([(0, 1), (0, 2), (2, 3), (3, 4), (4, 5), (5, 6), (4, 6)], 7)
    agg, na = amg.standard_aggregation(S)
    assert (agg >= 0).all()
    assert na == len(np.unique(agg))
    for a in range(na):              # every aggregate is connected
        members = np.flatnonzero(agg == a)
        sub = S[members][:, members]
        ncomp, _ = sp.csgraph.connected_components(sub, directed=False)
        assert ncomp == 1


def _system(size=(12, 6, 6), seed=0):
    m, pb, design, fixed, vol = problems.cantilever(*size)
    g = np.random.default_rng(seed)
    rho = 0.01 + 0.99 * g.random(m.nelements)
    K = pb.stiffness(rho, 3.0, 1e-9)
    return fem.enforce(K, pb.forces[0], pb.dirichlet_dofs)


def test_tentative_prolongator_orthonormal():
    Ke, _ = _system()
    agg, na = amg.standard_aggregation(amg.symmetric_strength(Ke))
    B = np.random.default_rng(1).random(Ke.shape[0]) + 0.5
    T, Bc = amg.fit_candidates(agg, na, B)
    np.testing.assert_allclose((T.T @ T).toarray(), np.eye(na), atol=1e-13)
    np.testing.assert_allclose(T @ Bc, B, rtol=1e-13)


def test_vcycle_is_symmetric_and_positive():
    Ke, _ = _system()
    ml = amg.SmoothedAggregationSolver(Ke)
    assert len(ml.levels) >= 2 and ml.shapes()[-1] <= 10 or len(ml.levels) == 10
    g = np.random.default_rng(2)
    x, y = g.standard_normal(Ke.shape[0]), g.standard_normal(Ke.shape[0])
    a, b = y @ ml.vcycle(x), x @ ml.vcycle(y)
    assert abs(a - b) <= 1e-9 * max(abs(a), abs(b))
    assert x @ ml.vcycle(x) > 0


@pytest.mark.parametrize("size", [(12, 6, 6), (20, 8, 8)])
def test_cg_pyamg_matches_direct(size):
    Ke, Fe = _system(size)
    st = {}
    u = amg.cg_pyamg(Ke, Fe, 1e-8, fem.default_maxiter(Ke.shape[0]), st)
    u0 = fem.solve(Ke, Fe, "spsolve")
    assert st["info"] == 0
    assert np.linalg.norm(Fe - Ke @ u) <= 1e-8 * np.linalg.norm(Fe) * 1.0001
    np.testing.assert_allclose(u, u0, rtol=0, atol=1e-6 * np.abs(u0).max())
    # the oracle FEM plugin's solver option routes here
    u2 = fem.solve(Ke, Fe, "cg_pyamg")
    np.testing.assert_array_equal(u, u2)
