"""CPU checks of the oracle: known answers of the reference's own scheduler
tests, analytic properties of the element matrices, and the golden fixtures
(tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from oracle import fem as ofem
from oracle import filters as ofilt
from oracle import mesh as omesh
from oracle import optim as oopt
from oracle import problems
from oracle import schedule as osch

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# --- scheduler known answers (scikit-topt/tests/test_scheduler.py) ----------
def test_step_decelerating_endpoints_and_monotone():
    vals = [osch.schedule_step_decelerating(it=i, total=10, initial_value=1.0,
                                            target_value=5.0, num_steps=5, curvature=2.0)
            for i in (1, 3, 5, 7, 9)]
    assert np.isclose(vals[0], 1.0) and np.isclose(vals[-1], 5.0)
    assert all(a <= b for a, b in zip(vals, vals[1:]))


def test_decelerating_faster_early_slower_late():
    kw = dict(total=10, initial_value=1.0, target_value=5.0, num_steps=5, curvature=2.0)
    for it in (3, 7):
        acc = osch.schedule_step_accelerating(it=it, **kw)
        lin = osch.schedule_step(it=it, **kw)
        dec = osch.schedule_step_decelerating(it=it, **kw)
        assert acc < lin < dec


def test_curvature_one_matches_linear():
    kw = dict(total=10, initial_value=0.5, target_value=1.5, num_steps=4, curvature=1.0)
    for it in (1, 4, 7, 9):
        lin = osch.schedule_step(it=it, **kw)
        assert np.isclose(lin, osch.schedule_step_decelerating(it=it, **kw))
        assert np.isclose(lin, osch.schedule_step_accelerating(it=it, **kw))


def test_step_to_one_values():
    assert np.isclose(osch.value("StepToOne", 1, 8, num_steps=4), 0.25)
    assert np.isclose(osch.value("StepToOne", 8, 8, num_steps=4), 1.0)
    assert np.isclose(osch.value("StepAcceleratingToOne", 1, 10, num_steps=5, curvature=2.0),
                      0.2)


def test_default_beta_schedule_values():
    # DensityMethodConfig.beta default: step_accelerating 1 -> 2, 3 steps, curvature 2
    b = [osch.value("StepAccelerating", it, 30, 1.0, 2.0, 3, 2.0) for it in (1, 9, 10, 19, 20, 30)]
    assert b == [1.0, 1.0, 1.25, 1.25, 2.0, 2.0]


# --- element matrices ----------------------------------------------------------
def _rigid_modes(x):
    n = x.shape[1]
    R = np.zeros((3 * n, 6))
    for c in range(3):
        R[c::3, c] = 1.0
    R[0::3, 3], R[1::3, 3] = -x[1], x[0]
    R[1::3, 4], R[2::3, 4] = -x[2], x[1]
    R[0::3, 5], R[2::3, 5] = x[2], -x[0]
    return R


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_element_matrix_properties(kind):
    if kind == "hex":
        m = omesh.create_box_hex(1, 1, 1, 0.7, 1.1, 0.9)
        x = m.p[:, m.t[:, 0]]
        Ke, Kh = ofem.hex_element_matrices(x, 0.3)
        M = ofem.hex_mass_matrix(x)
        vol = 0.7 * 1.1 * 0.9
    else:
        m = omesh.create_box_tet(1, 1, 1, 1.0, 1.0, 1.0, jitter=0.0)
        x = m.p[:, m.t[:, 2]]
        Ke, Kh, M = ofem.tet_element_matrices(x, 0.3)
        vol = 1.0 / 6.0
    assert np.allclose(Ke, Ke.T, atol=1e-14)
    assert np.abs(Ke @ _rigid_modes(x)).max() < 1e-13
    w = np.linalg.eigvalsh(Ke)
    assert np.sum(w > 1e-10) == Ke.shape[0] - 6
    assert np.abs(Kh @ np.ones(Kh.shape[0])).max() < 1e-14
    assert np.isclose(M.sum(), vol)
    # uniform strain e_xx = 1: energy = 1/2 (lambda + 2 mu) V
    u = np.zeros(Ke.shape[0])
    u[0::3] = x[0]
    lam, mu = ofem.lame(1.0, 0.3)
    assert np.isclose(0.5 * u @ Ke @ u, 0.5 * (lam + 2 * mu) * vol)


def test_hex_volume_pattern_of_reference():
    # composer.py:191-248 sums six |tet| volumes in a fixed node pattern; with
    # MeshHex's local order that gives 5/6 of a unit cube (it cancels in
    # volume fractions on uniform grids).
    m = omesh.create_box_hex(2, 1, 1)
    assert np.allclose(omesh.elements_volume(m), 5.0 / 6.0)


def test_enforce_is_symmetric_with_unit_diagonal():
    m, pb, *_ = problems.cantilever(4, 2, 2)
    K = pb.stiffness(np.full(m.nelements, 0.5), 3.0, 1e-9)
    Ke, fe = ofem.enforce(K, np.ones(K.shape[0]), pb.dirichlet_dofs)
    assert abs(Ke - Ke.T).max() <= 1e-15 * abs(Ke).max()
    D = pb.dirichlet_dofs
    assert np.all(Ke.diagonal()[D] == 1.0) and np.all(fe[D] == 0.0)


# --- golden fixtures ----------------------------------------------------------
def test_oracle_state_matches_golden():
    g = np.load(os.path.join(GOLDEN, "cantilever_10x5x4_state.npz"))
    nx, ny, nz = g["shape"]
    m, pb, design, fixed, vol = problems.cantilever(int(nx), int(ny), int(nz))
    rho = g["rho"]
    K = pb.stiffness(rho, 3.0, 1e-9)
    Ke, Fe = ofem.enforce(K, np.column_stack(pb.forces), pb.dirichlet_dofs)
    assert np.array_equal(Ke.indptr, g["K_indptr"]) and np.array_equal(Ke.indices,
                                                                         g["K_indices"])
    np.testing.assert_allclose(Ke.data, g["K_data"], rtol=0, atol=1e-15)
    comp, U = pb.objectives(rho, 3.0, 1e-9, "spsolve")
    assert abs(comp[0] - g["compliance"]) <= 1e-12 * abs(g["compliance"])
    en = pb.energy(rho, 3.0, 1e-9, U)[:, 0]
    assert np.linalg.norm(en - g["energy"]) <= 1e-10 * np.linalg.norm(g["energy"])
    mask = np.zeros(m.nelements, bool)
    mask[design] = True
    f = ofilt.SpacialFilter(m, 1.5, mask)
    assert np.array_equal(f.W.indices, g["W_indices"])
    np.testing.assert_allclose(f.W.data, g["W_data"], rtol=1e-15)
    np.testing.assert_allclose(f.forward(g["filt_x"]), g["filt_fwd"], rtol=1e-14)
    np.testing.assert_allclose(f.gradient(g["filt_x"]), g["filt_grad"], rtol=1e-14)
    np.testing.assert_allclose(ofilt.heaviside_projection(g["filt_x"], 1.25), g["proj_b125"],
                               rtol=1e-15)


def test_oracle_oc_trajectory_matches_golden():
    g = np.load(os.path.join(GOLDEN, "cantilever_12x6x6_oc5.npz"))
    nx, ny, nz = (int(v) for v in g["shape"])
    m, pb, design, fixed, vol = problems.cantilever(nx, ny, nz)
    filt = problems.gaussian_filter_for(m, design, 1.5)
    cfg = oopt.OracleConfig(max_iters=len(g["compliance"]), p=oopt.Sched("Constant", 3.0, 3.0),
                            vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                            move_limit=oopt.Sched("Constant", 0.2, 0.2),
                            filter_radius=oopt.Sched("Constant", 1.5, 1.5), E_min_coeff=1e-9)
    opt = oopt.OracleOptimizer(cfg, pb, filt, design, fixed, vol)
    for k in range(len(g["compliance"])):
        c = opt.step()
        assert abs(c - g["compliance"][k]) <= 1e-11 * abs(g["compliance"][k])
        np.testing.assert_allclose(opt.rho, g["rho"][k], rtol=0, atol=1e-10)
    assert list(opt.hist["bisection_steps"]) == list(g["steps"])
