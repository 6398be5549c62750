"""The reference's toy problems (sktopt/mesh/toy_problem.py:51-144) as set
up here: facet and element selection by midpoint (scikit-fem semantics,
interior facets included unless boundaries only) against a brute-force
restatement, and the supports, loads and design sets they produce."""
import numpy as np

from sktopt_gb300.mesh import (create_box_hex_len, elements_satisfying, facet_nodes_of,
                               facets_satisfying, get_points_in_range, toy_problem)


def _brute(mesh, pred, boundary_only):
    from sktopt_gb300.mesh.grid import element_faces
    faces = element_faces(mesh.kind)
    first, count = {}, {}
    for e in range(mesh.nelements):
        for f, loc in enumerate(faces):
            key = tuple(sorted(mesh.t[list(loc), e]))
            count[key] = count.get(key, 0) + 1
            first.setdefault(key, (e, f))
    out = []
    for key, ef in first.items():
        if boundary_only and count[key] != 1:
            continue
        if pred(mesh.p[:, list(key)].mean(axis=1)[:, None])[0]:
            out.append(ef)
    return sorted(out)


def test_facets_and_elements_satisfying_match_brute_force():
    mesh = create_box_hex_len(3.0, 2.0, 2.0, 1.0)
    pred = get_points_in_range((1.2, 3.1), (0.4, 1.6), (0.8, 2.0))
    for bo in (False, True):
        got = [tuple(r) for r in facets_satisfying(mesh, pred, boundaries_only=bo)]
        assert sorted(got) == _brute(mesh, pred, bo)
    # all facets of a 3 x 2 x 2 grid: 4*2*2 + 3*3*2 + 3*2*3 x/y/z faces
    assert len(facets_satisfying(mesh, lambda x: np.ones(x.shape[1], bool))) == 16 + 18 + 18
    c = np.mean(mesh.p[:, mesh.t], axis=1)
    el = elements_satisfying(mesh, get_points_in_range((0.0, 1.5), (0.0, 2.0), (0.0, 2.0)))
    np.testing.assert_array_equal(el, np.nonzero(c[0] <= 1.5)[0])


def test_toy_test_setup():
    tsk = toy_problem.toy_test()
    m = tsk.mesh
    assert (m.nelements, m.nnodes) == (192, 315)
    # supports: every DOF of the 7 x 5 nodes on x = 0
    fixed_nodes = np.unique(np.nonzero(tsk.dirichlet_mask)[0] // 3)
    np.testing.assert_array_equal(fixed_nodes, np.nonzero(np.isclose(m.p[0], 0.0))[0])
    # load: -100 along u^3 over 9 unit facets (4 of them interior)
    F = tsk.neumann_linear[0]
    assert np.isclose(F.sum(), -100.0) and np.all(F[0::3] == 0) and np.all(F[1::3] == 0)
    ff = facets_satisfying(m, get_points_in_range((6.8, 8.1), (2.4, 3.6), (2.8, 4.0)))
    assert len(ff) == 9
    loaded = np.unique(facet_nodes_of(m, ff))
    np.testing.assert_array_equal(np.nonzero(F)[0] // 3, loaded)


def test_toy2_setup():
    tsk = toy_problem.toy2()
    m = tsk.mesh
    assert m.nelements == 27 * 27 * 4 and tsk.n_tasks == 2
    F0, F1 = tsk.neumann_linear
    assert np.isclose(F0.sum(), -1.0) and np.isclose(F1.sum(), 1.0)
    assert np.all(F0[0::3] == 0) and np.all(F0[2::3] == 0)
    y0 = m.p[1, np.nonzero(F0)[0] // 3]
    y1 = m.p[1, np.nonzero(F1)[0] // 3]
    assert y0.min() >= 8.0 - 0.3 - 8.0 / 27 - 1e-12 and y1.max() <= 0.3 + 8.0 / 27 + 1e-12
    assert set(m.boundaries) == {"dirichlet", "neumann_0", "neumann_1"}
