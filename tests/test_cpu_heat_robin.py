"""CPU checks of the oracle's heat Robin / heat-exchange restatement
(oracle/heat_robin.py) against analytic identities, and of the task set-up.

* the 2x2x2 rule integrates |grad rho| of a linear nodal field exactly
  (|a| x volume) and the virtual Robin terms vanish (to rounding) for a
  uniform density;
* surface Robin matrices sum to h x area and their loads to h T_env x area;
* the explicit Robin gradient is the derivative, at fixed T, of
  G(rho) = int h rho^p (1 - rho)^q |grad rho| (2 T_env T - T^2)
  (central differences, 1e-6 relative);
* the reference's nodal-average pairing differs from the element pairing
  and both reproduce a uniform density;
* without Robin data and with T = 0 Dirichlet values the compliance
  objective equals the plain conduction problem's;
* the plate task's Dirichlet nodes and Robin facets match the oracle's;
* the oracle reproduces its committed golden fixtures (heat plate objectives,
  adjoints, energies, sensitivities; tet traction loads, also against the
  product's host-side traction assembly);
* on P1 tetrahedra and on general (jittered) hexahedra: the quadrature's
  volume and linear-field identities, surface sums and the product's surface
  matrices, the explicit gradient by central differences, and (hexahedra)
  the per-element conduction matrices of the oracle against the product's.
"""
import numpy as np
import pytest

from oracle import fem as ofem
from oracle import heat_robin as hr
from oracle import problems


def _plate(n=(6, 6, 2)):
    return problems.heat_plate(*n)


def test_linear_field_interface_integral_exact():
    m, pb, *_ = _plate()
    a = np.array([0.3, -0.2, 0.5])
    rho_n = 0.1 + a @ m.p * 0.01
    vol = 8.0 * 8.0 * 1.0
    den = hr.hx_den(m, pb.Q, rho_n)
    assert abs(den - 0.01 * np.linalg.norm(a) * vol) <= 1e-13 * den


def test_virtual_robin_vanishes_for_uniform_density():
    m, pb, *_ = _plate()
    Me, fe = hr.virtual_robin(m, pb.Q, np.full(m.nnodes, 0.4), 4e-5, 300.0, 3.0, 4.0)
    # |grad rho| of a constant field is rounding noise (~1e-17), not zero
    assert np.abs(Me).max() <= 1e-20 and np.abs(fe).max() <= 1e-17


def test_surface_robin_sums():
    m, pb, *_ = _plate((5, 4, 3))
    faces = problems.boundary_faces(m, problems.in_range((0, 0), (0, 8), (0, 1)))
    Me, load = hr.surface_robin(m, faces, 2.0, 300.0)
    area = 8.0 * 1.0
    assert abs(Me.sum() - 2.0 * area) <= 1e-12 * area
    assert abs(load.sum() - 2.0 * 300.0 * area) <= 1e-10 * area
    for M in Me:
        assert np.allclose(M, M.T, rtol=0, atol=1e-15)


def test_explicit_robin_gradient_finite_differences():
    m, pb, *_ = _plate((4, 4, 2))
    rng = np.random.default_rng(7)
    rho_n = rng.uniform(0.2, 0.8, m.nnodes)
    T = rng.uniform(250.0, 650.0, m.nnodes)
    h, te, p, q = 4e-5, 300.0, 3.0, 4.0
    N, dN, wd = pb.Q

    def G(r):
        rq, g = hr._at_qp(N, dN, m, r)
        tq, _ = hr._at_qp(N, dN, m, T)
        iface = np.sqrt(np.sum(g ** 2, axis=2))
        return float(np.sum(wd * h * rq ** p * (1 - rq) ** q * iface * (2 * te * tq - tq * tq)))

    grad = hr.robin_explicit_grad(m, pb.Q, rho_n, T, h, te, p, q)
    for n in rng.choice(m.nnodes, 6, replace=False):
        e = np.zeros(m.nnodes)
        e[n] = 1e-6
        fd = (G(rho_n + e) - G(rho_n - e)) / 2e-6
        assert abs(fd - grad[n]) <= 1e-6 * max(abs(grad).max(), 1e-300), (n, fd, grad[n])


def test_nodal_average_pairings():
    m, *_ = _plate((4, 3, 2))
    rng = np.random.default_rng(3)
    rho = rng.uniform(0, 1, m.nelements)
    ref, cnt = hr.nodal_average(m, rho, "reference")
    ele, cnt2 = hr.nodal_average(m, rho, "element")
    assert np.array_equal(cnt, cnt2)
    assert not np.allclose(ref, ele)
    # element pairing: the plain average over the node's elements
    want = np.zeros(m.nnodes)
    for e in range(m.nelements):
        want[m.t[:, e]] += rho[e]
    np.testing.assert_allclose(ele, want / cnt, rtol=1e-14)
    u = np.full(m.nelements, 0.37)
    np.testing.assert_allclose(hr.nodal_average(m, u, "reference")[0], 0.37, rtol=1e-15)


def test_no_robin_zero_dirichlet_matches_plain_conduction():
    m, pb, *_ = problems.heat_plate(10, 10, 2, dirichlet_values=0.0, robin=False)
    assert pb.D.size > 0
    emit = ofem.source_vector(m, 1.0)
    pb.emit = emit
    plain = ofem.HeatProblem(m, pb.D, k0=10.0, emit=emit)
    rho = np.random.default_rng(1).uniform(0.1, 1.0, m.nelements)
    J, T = pb.objectives(rho, 3.0, 1e-2)
    J0, T0 = plain.objectives(rho, 3.0, 1e-2)
    assert abs(J[0] - J0[0]) <= 1e-12 * abs(J0[0])
    np.testing.assert_allclose(T, T0, rtol=0, atol=1e-12 * np.abs(T0).max())


def test_plate_task_matches_oracle_sets():
    from sktopt_gb300.mesh import toy_problem
    t = toy_problem.heat_plate(10, 9, 3)
    m, pb, design, fixed, vol = problems.heat_plate(10, 9, 3)
    assert np.array_equal(t.mesh.t, m.t) and np.allclose(t.mesh.p, m.p, rtol=0, atol=1e-15)
    assert np.array_equal(np.sort(t.dirichlet_nodes), pb.D)
    got = [np.asarray(g) for g in t.robin_groups]
    want = [problems.boundary_faces(m, problems.in_range((0, 0), (0, 8), (0, 1))),
            problems.boundary_faces(m, problems.in_range((0, 8), (8, 8), (0, 1)))]
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    t.exlude_dirichlet_from_design()
    assert np.array_equal(np.sort(t.design_elements), np.sort(design))


def test_surface_matrices_match_oracle():
    from sktopt_gb300.fea.solver_heat import surface_robin_load, surface_robin_matrices
    from sktopt_gb300.mesh import toy_problem
    t = toy_problem.heat_plate(5, 4, 3)
    m, *_ = problems.heat_plate(5, 4, 3)
    for faces in t.robin_groups:
        Me, load = hr.surface_robin(m, faces, 4e-5, 300.0)
        np.testing.assert_allclose(surface_robin_matrices(t.mesh, faces, 4e-5).reshape(-1, 8, 8),
                                   Me, rtol=1e-13, atol=1e-20)
        np.testing.assert_allclose(surface_robin_load(t.mesh, faces, 4e-5, 300.0), load,
                                   rtol=1e-13, atol=1e-18)


@pytest.mark.parametrize("objective", ["compliance", "heat_exchange", "averaged_temp"])
def test_oracle_objectives_run(objective):
    m, pb, *_ = problems.heat_plate(10, 10, 2, objective=objective, avg_temp_weight=0.5)
    assert pb.D.size > 0
    rho = np.random.default_rng(2).uniform(0.1, 1.0, m.nelements)
    J, T = pb.objectives(rho, 3.0, 1e-2)
    assert np.all(np.isfinite(J)) and np.all(np.isfinite(T))
    assert np.abs(T[pb.D] - 600.0).max() == 0.0
    g = pb.custom_sensitivity(rho, 3.0, 1e-2, T)
    assert g.shape == (m.nelements, 1) and np.all(np.isfinite(g))


# --- golden fixtures (tests/golden/make_golden.py) ----------------------------
def test_heat_oracle_matches_golden():
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "heat_plate_12x12x3.npz"))
    nx, ny, nz = (int(v) for v in g["shape"])
    rho = g["rho"]
    for obj, w in (("compliance", 0.0), ("heat_exchange", 0.5), ("averaged_temp", 0.0)):
        m, pb, *_ = problems.heat_plate(nx, ny, nz, objective=obj, avg_temp_weight=w)
        if obj == "compliance":
            assert np.array_equal(hr.nodal_average(m, rho, "reference")[0], g["rho_nodal"])
        J, T = pb.objectives(rho, 3.0, 1e-2)
        np.testing.assert_allclose(J, g[f"{obj}_J"], rtol=1e-11)
        np.testing.assert_allclose(T, g[f"{obj}_T"], rtol=0, atol=1e-10)
        if f"{obj}_lam" in g:
            assert np.linalg.norm(pb.lam - g[f"{obj}_lam"]) <= \
                1e-10 * np.linalg.norm(g[f"{obj}_lam"])
        for key, val in (("energy", pb.energy(rho, 3.0, 1e-2, T)),
                         ("dc", pb.custom_sensitivity(rho, 3.0, 1e-2, T))):
            ref = g[f"{obj}_{key}"]
            assert np.linalg.norm(val - ref) <= 1e-9 * np.linalg.norm(ref), (obj, key)


def test_tractions_match_golden():
    import os
    from oracle import mesh as omesh
    from oracle import surface as osurf
    from sktopt_gb300.mesh import GridMesh, assemble_surface_forces, boundary_facets
    from sktopt_gb300.mesh import get_points_in_range as rng
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "tet_tractions.npz"))
    m = GridMesh(g["p"], g["t"], "tet")
    f1 = boundary_facets(m, rng((2.0, 2.0), (0, 9), (0, 9)))
    f2 = boundary_facets(m, rng((0, 2.0), (1.0, 1.0), (0, 9)))
    assert np.array_equal(f1, g["facets1"]) and np.array_equal(f2, g["facets2"])
    F = assemble_surface_forces(m, [f1, f2], ["u^3", "u^1"], [-2.0, 0.5])
    np.testing.assert_allclose(F[0], g["F1"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(F[1], g["F2"], rtol=1e-13, atol=1e-15)
    om = omesh.GridMesh(g["p"], g["t"], "tet", None, None, None)
    R = osurf.surface_forces(om, [f1, f2], ["u^3", "u^1"], [-2.0, 0.5])
    np.testing.assert_array_equal(R[0], g["F1"])
    np.testing.assert_array_equal(R[1], g["F2"])


def test_heat_plugin_argument_checks():
    """Host-side validation of the heat plugin (no GPU work): unknown
    objectives, per-group coefficients for the density-dependent Robin terms,
    Robin facets on tetrahedra, the nodal pairing name."""
    import dataclasses
    from sktopt_gb300.fea.solver_heat import FEM_SimpLinearHeatConduction
    from sktopt_gb300.mesh import LinearHeatConduction, create_box_tet, toy_problem
    tsk = toy_problem.heat_plate(10, 10, 2)
    with pytest.raises(ValueError):
        FEM_SimpLinearHeatConduction(dataclasses.replace(tsk, objective="flux"), 1e-3)
    with pytest.raises(ValueError):
        FEM_SimpLinearHeatConduction(dataclasses.replace(tsk, robin_coefficient=[4e-5, 4e-5]),
                                     1e-3)
    with pytest.raises(ValueError):
        FEM_SimpLinearHeatConduction(tsk, 1e-3, nodal_pairing="rows")
    with pytest.raises(ValueError, match="robin_coefficient"):
        FEM_SimpLinearHeatConduction(dataclasses.replace(tsk, robin_coefficient=None), 1e-3)
    with pytest.raises(ValueError):
        LinearHeatConduction.from_nodes(tsk.mesh, tsk.dirichlet_nodes, None,
                                        np.arange(tsk.mesh.nelements), objective="flux")
    m = create_box_tet(3, 2, 2, 1.0, 1.0, 1.0)
    from sktopt_gb300.mesh import boundary_facets
    f = boundary_facets(m)[:2]
    # tetrahedra: Robin facets stay rows (element, local face)
    tt = LinearHeatConduction.from_facets(m, f, 1.0, f, 1e-3, 300.0, True,
                                          np.arange(m.nelements), 1.0)
    assert [g.shape for g in tt.robin_groups] == [(2, 2)]
    np.testing.assert_array_equal(tt.robin_groups[0], f)


# --- P1 tetrahedra --------------------------------------------------------------
def _tet_plate(n=(6, 6, 2)):
    from oracle import mesh as omesh
    from sktopt_gb300.mesh import toy_problem
    t = toy_problem.heat_plate_tet(*n)
    m = omesh.GridMesh(t.mesh.p, t.mesh.t, "tet", None, None, None)
    return t, m


def test_tet_quadrature_linear_field_exact():
    t, m = _tet_plate()
    Q = hr.tet_quadrature(m)
    assert abs(Q[2].sum() - 64.0) <= 1e-12 * 64.0           # the plate's volume
    a = np.array([0.3, -0.2, 0.5])
    rho_n = 0.1 + a @ m.p * 0.01
    den = hr.hx_den(m, Q, rho_n)
    assert abs(den - 0.01 * np.linalg.norm(a) * 64.0) <= 1e-12 * den
    # the rule integrates quadratics exactly: int N_a N_b = V / 20 (1 + delta)
    N, dN, wd = Q
    M = np.einsum("eq,qa,qb->eab", wd, N, N)
    V = wd.sum(axis=1)
    want = V[:, None, None] / 20.0 * (np.ones((4, 4)) + np.eye(4))
    np.testing.assert_allclose(M, want, rtol=1e-13)


def test_tet_surface_robin_sums_and_product_match():
    from sktopt_gb300.fea.solver_heat import surface_robin_load, surface_robin_matrices
    t, m = _tet_plate((5, 4, 3))
    for faces, area in zip(t.robin_groups, (8.0 * 1.0, 8.0 * 1.0)):
        Me, load = hr.surface_robin(m, faces, 2.0, 300.0)
        assert abs(Me.sum() - 2.0 * area) <= 1e-12 * area
        assert abs(load.sum() - 2.0 * 300.0 * area) <= 1e-10 * area
        np.testing.assert_allclose(surface_robin_matrices(t.mesh, faces, 2.0).reshape(-1, 4, 4),
                                   Me, rtol=1e-13, atol=1e-20)
        np.testing.assert_allclose(surface_robin_load(t.mesh, faces, 2.0, 300.0), load,
                                   rtol=1e-13, atol=1e-18)


def test_tet_explicit_robin_gradient_finite_differences():
    t, m = _tet_plate((4, 4, 2))
    Q = hr.tet_quadrature(m)
    rng = np.random.default_rng(8)
    rho_n = rng.uniform(0.2, 0.8, m.nnodes)
    T = rng.uniform(250.0, 650.0, m.nnodes)
    h, te, p, q = 4e-5, 300.0, 3.0, 4.0
    N, dN, wd = Q

    def G(r):
        rq, g = hr._at_qp(N, dN, m, r)
        tq, _ = hr._at_qp(N, dN, m, T)
        iface = np.sqrt(np.sum(g ** 2, axis=2))
        return float(np.sum(wd * h * rq ** p * (1 - rq) ** q * iface * (2 * te * tq - tq * tq)))

    grad = hr.robin_explicit_grad(m, Q, rho_n, T, h, te, p, q)
    for n in rng.choice(m.nnodes, 6, replace=False):
        e = np.zeros(m.nnodes)
        e[n] = 1e-6
        fd = (G(rho_n + e) - G(rho_n - e)) / 2e-6
        assert abs(fd - grad[n]) <= 1e-6 * max(abs(grad).max(), 1e-300), (n, fd, grad[n])


# --- general (non-box) hexahedra ---------------------------------------------
def _jit_plate(n=(6, 6, 2), objective="compliance", avg_w=0.0):
    from oracle import mesh as omesh
    from sktopt_gb300.mesh import toy_problem
    t = toy_problem.heat_plate(*n, objective=objective, avg_temp_weight=avg_w, jitter=0.2,
                               seed=3)
    m = omesh.GridMesh(t.mesh.p, t.mesh.t, "hex", None, None, None)
    return t, m


def test_general_hex_mesh_is_not_boxes_and_keeps_the_boundary():
    from sktopt_gb300.mesh import toy_problem
    t, m = _jit_plate()
    assert not ofem._is_uniform_box(m)
    box = toy_problem.heat_plate(6, 6, 2).mesh.p
    # interior nodes moved by up to 0.2 h per axis, boundary coordinates kept
    assert 0.1 < np.abs(m.p - box).max() <= 0.2 * 8.0 / 6.0 + 1e-12
    for d, top in enumerate((8.0, 8.0, 1.0)):
        on = np.isclose(box[d], 0.0) | np.isclose(box[d], top)
        np.testing.assert_array_equal(m.p[d, on], box[d, on])


def test_general_hex_quadrature_exact_on_linear_fields():
    """2x2x2 Gauss on the trilinear map: detJ is of degree <= 2 per
    direction, so the weights sum to the plate's volume and |grad rho| of a
    linear nodal field (reproduced exactly by the trilinear element)
    integrates to |a| x volume; the per-element conduction matrices of the
    oracle and of the product's host code agree."""
    from sktopt_gb300.fea import composer
    t, m = _jit_plate()
    Q = hr.hex_quadrature(m)
    assert abs(Q[2].sum() - 64.0) <= 1e-12 * 64.0
    a = np.array([0.3, -0.2, 0.5])
    rho_n = 0.1 + a @ m.p * 0.01
    den = hr.hx_den(m, Q, rho_n)
    assert abs(den - 0.01 * np.linalg.norm(a) * 64.0) <= 1e-12 * den
    _, Kh_o, _ = ofem.element_matrices(m, 0.3)
    _, Kh_p, _ = composer.element_matrices(t.mesh, 0.3)
    assert Kh_p.ndim == 3
    np.testing.assert_allclose(Kh_p, Kh_o, rtol=0, atol=1e-12 * np.abs(Kh_o).max())


def test_general_hex_surface_robin_sums_and_product_match():
    from sktopt_gb300.fea.solver_heat import surface_robin_load, surface_robin_matrices
    t, m = _jit_plate((5, 4, 3))
    for faces, area in zip(t.robin_groups, (8.0 * 1.0, 8.0 * 1.0)):
        faces = np.asarray(faces)
        Me, load = hr.surface_robin(m, faces, 2.0, 300.0)
        assert abs(Me.sum() - 2.0 * area) <= 1e-12 * area
        assert abs(load.sum() - 2.0 * 300.0 * area) <= 1e-10 * area
        np.testing.assert_allclose(surface_robin_matrices(t.mesh, faces, 2.0).reshape(-1, 8, 8),
                                   Me, rtol=1e-13, atol=1e-20)
        np.testing.assert_allclose(surface_robin_load(t.mesh, faces, 2.0, 300.0), load,
                                   rtol=1e-13, atol=1e-18)


def test_general_hex_explicit_robin_gradient_finite_differences():
    t, m = _jit_plate((4, 4, 2))
    Q = hr.hex_quadrature(m)
    rng = np.random.default_rng(8)
    rho_n = rng.uniform(0.2, 0.8, m.nnodes)
    T = rng.uniform(250.0, 650.0, m.nnodes)
    h, te, p, q = 4e-5, 300.0, 3.0, 4.0
    N, dN, wd = Q

    def G(r):
        rq, g = hr._at_qp(N, dN, m, r)
        tq, _ = hr._at_qp(N, dN, m, T)
        iface = np.sqrt(np.sum(g ** 2, axis=2))
        return float(np.sum(wd * h * rq ** p * (1 - rq) ** q * iface * (2 * te * tq - tq * tq)))

    grad = hr.robin_explicit_grad(m, Q, rho_n, T, h, te, p, q)
    for n in rng.choice(m.nnodes, 6, replace=False):
        e = np.zeros(m.nnodes)
        e[n] = 1e-6
        fd = (G(rho_n + e) - G(rho_n - e)) / 2e-6
        assert abs(fd - grad[n]) <= 1e-6 * max(abs(grad).max(), 1e-300), (n, fd, grad[n])
