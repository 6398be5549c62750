"""The oracle (and the host-side schedules) against fixtures written by the
reference's own code (tests/golden/make_ref_fixtures.py runs the unmodified
scikit-topt 0.3.9 sources).  These pin every part of the restatement that
the reference computes with NumPy/SciPy itself; the scikit-fem arithmetic
(element matrices, assembly, enforce) stays the restatement's own."""
import os
import tempfile

import numpy as np
import pytest

from oracle import fem as ofem
from oracle import filters as ofilt
from oracle import mesh as omesh
from oracle import optim as oopt
from oracle import problems
from oracle import schedule as osched

G = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(G, name))


@pytest.fixture(scope="module")
def U():
    return _load("ref_units.npz")


def test_projection_matches_reference(U):
    x = U["proj_x"]
    for i in range(4):
        beta, eta = U[f"proj_param_{i}"]
        np.testing.assert_allclose(ofilt.heaviside_projection(x, beta, eta), U[f"proj_{i}"],
                                   rtol=1e-15, atol=1e-16)
        np.testing.assert_allclose(ofilt.heaviside_projection_derivative(x, beta, eta),
                                   U[f"dproj_{i}"], rtol=1e-15, atol=1e-16)


def test_interpolation_and_sensitivity_match_reference(U):
    rho, en = U["deriv_rho"], U["deriv_energy"]
    for p in (1.0, 3.0, 4.5):
        k = f"{p:g}".replace(".", "_")
        np.testing.assert_array_equal(ofem.E_simp(rho, 1.0, 1e-9, p), U[f"E_simp_p{k}"])
        np.testing.assert_array_equal(ofem.dE_drho_simp(rho, 1.0, 1e-9, p), U[f"dE_simp_p{k}"])
        np.testing.assert_array_equal(ofem.dC_drho_simp(rho, en, 1.0, 1e-9, p),
                                      U[f"dC_simp_p{k}"])
        np.testing.assert_array_equal(ofem.dC_drho_ramp(rho, en, 1.0, 1e-9, p),
                                      U[f"dC_ramp_p{k}"])
        np.testing.assert_array_equal(ofem.simp_interpolation(rho, 210e3, 210.0, p),
                                      U[f"simp_p{k}"])
        np.testing.assert_array_equal(ofem.ramp_interpolation(rho, 210e3, 210.0, p),
                                      U[f"ramp_p{k}"])
    lam, mu = ofem.lame(U["lame_E"], 0.3)
    np.testing.assert_allclose(lam, U["lame_lam"], rtol=1e-15)
    np.testing.assert_allclose(mu, U["lame_mu"], rtol=1e-15)


def _grid(p, t, kind):
    return omesh.GridMesh(p, t, kind, None, None, None)


def test_element_volumes_match_reference(U):
    vh = omesh.elements_volume(_grid(U["vol_hex_p"], U["vol_hex_t"], "hex"))
    np.testing.assert_allclose(vh, U["vol_hex"], rtol=1e-14)
    vt = omesh.elements_volume(_grid(U["vol_tet_p"], U["vol_tet_t"], "tet"))
    np.testing.assert_allclose(vt, U["vol_tet"], rtol=1e-14)


def test_orientation_fixes_match_reference(U):
    p_h = omesh.create_box_hex(5, 4, 3).p
    np.testing.assert_array_equal(omesh.fix_hexahedron_orientation(U["orient_hex_in"], p_h),
                                  U["orient_hex_out"])
    np.testing.assert_array_equal(
        omesh.fix_tetrahedron_orientation(U["orient_tet_in"], U["vol_tet_p"]),
        U["orient_tet_out"])


def test_elements_by_nodes_match_reference(U):
    m = omesh.create_box_hex(5, 4, 3)
    np.testing.assert_array_equal(omesh.get_elements_by_nodes(m, [U["ebn_nodes_a"]]),
                                  U["ebn_a"])
    np.testing.assert_array_equal(
        omesh.get_elements_by_nodes(m, [U["ebn_nodes_a"], U["ebn_nodes_b"]]), U["ebn_ab"])


SCHED_CASES = [
    ("constant", "Constant", None, 0.3, None, None),
    ("step", "Step", 1.0, 3.0, 3, None),
    ("step_to_one", "StepToOne", None, 1.0, 4, None),
    ("step_accelerating", "StepAccelerating", 1.0, 2.0, 3, 2.0),
    ("step_accelerating_to_one", "StepAcceleratingToOne", None, 1.0, 5, 3.0),
    ("step_decelerating", "StepDecelerating", 0.5, 0.1, 4, 2.0),
    ("step_decelerating_to_one", "StepDeceleratingToOne", None, 1.0, 3, 1.5),
    ("sawtooth_decay", "SawtoothDecay", 0.3, 0.1, 6, None),
]


def test_schedules_match_reference(U):
    """Oracle schedule functions and the product's host Schedulers against
    the reference's Schedulers.values_as_list for iterations 0..T+1."""
    from sktopt_gb300 import tools
    names = list(U["sched_names"])
    T = int(U["sched_iters_max"])
    ref = U["sched_values"]
    S = tools.SchedulerConfig
    confs = {
        "constant": S.constant(target_value=0.3),
        "step": S.step(init_value=1.0, target_value=3.0, num_steps=3),
        "step_to_one": S.step_to_one(num_steps=4),
        "step_accelerating": S.step_accelerating(init_value=1.0, target_value=2.0,
                                                 num_steps=3, curvature=2.0),
        "step_accelerating_to_one": S.step_accelerating_to_one(num_steps=5, curvature=3.0),
        "step_decelerating": S.step_decelerating(init_value=0.5, target_value=0.1,
                                                 num_steps=4, curvature=2.0),
        "step_decelerating_to_one": S.step_decelerating_to_one(num_steps=3, curvature=1.5),
        "sawtooth_decay": S.sawtooth_decay("move_limit", 0.3, 0.1, 3),
    }
    with tempfile.TemporaryDirectory() as d:
        sch = tools.Schedulers(d)
        for n in names:
            sch.add_object_from_config(confs[n], n)
        sch.set_iters_max(T)
        mine = np.array([sch.values_as_list(it, names) for it in range(0, T + 2)], float)
    np.testing.assert_allclose(mine, ref, rtol=1e-15, atol=0)
    for j, (n, kind, init, target, steps, curv) in enumerate(SCHED_CASES):
        assert names[j] == n
        vals = [osched.value(kind, it, T, init, target, steps, curv) for it in range(0, T + 2)]
        np.testing.assert_allclose(np.array(vals, float), ref[:, j], rtol=1e-15, atol=0)


def _filter_grid(U):
    m = omesh.create_box_hex(10, 5, 4)
    return m, U["filt_design_mask"]


def test_gaussian_filter_matches_reference(U):
    m, mask = _filter_grid(U)
    x = U["filt_x"]
    for i in range(2):
        r = float(U[f"filt_r{i}"])
        f = ofilt.SpacialFilter(m, r, mask)
        np.testing.assert_array_equal(f.W.indptr, U[f"filt_W_indptr_{i}"])
        np.testing.assert_array_equal(f.W.indices, U[f"filt_W_indices_{i}"])
        np.testing.assert_allclose(f.W.data, U[f"filt_W_data_{i}"], rtol=1e-15)
        np.testing.assert_allclose(f.forward(x), U[f"filt_fwd_{i}"], rtol=1e-14)
        np.testing.assert_allclose(f.gradient(x), U[f"filt_grad_{i}"], rtol=1e-14,
                                   atol=1e-16)


def test_bisection_matches_reference(U):
    m, mask = _filter_grid(U)
    f = ofilt.SpacialFilter(m, 1.5, mask)
    (rmin, rmax, move, eta, eps, vf, beta, beta_eta, srmin, srmax, tol, l1,
     l2) = U["bis_params"]
    ev = U["bis_vol"]
    lmid, verr, rd, sr, steps = oopt.bisection_with_physical_volume(
        U["bis_dC"], U["bis_rho_full"][U["bis_design"]], U["bis_rho_full"], U["bis_design"],
        f, rmin, rmax, move, eta, eps, vf, beta, beta_eta, ev, float(np.sum(ev)), srmin, srmax,
        max_iter=1000, tolerance=tol, l1=l1, l2=l2)
    assert lmid == float(U["bis_lmid"])
    np.testing.assert_allclose(verr, float(U["bis_vol_error"]), rtol=1e-12, atol=1e-16)
    np.testing.assert_array_equal(rd, U["bis_rho_design"])
    np.testing.assert_array_equal(sr, U["bis_scaling_rate"])


def test_log_update_matches_reference(U):
    eta, move, rmin, rmax, clip = U["llu_params"]
    rd, sr, lo, up = oopt.lagrangian_log_update(U["llu_rho_in"], U["llu_dL"], eta, move,
                                                rmin, rmax, clip)
    np.testing.assert_array_equal(rd, U["llu_rho_out"])
    np.testing.assert_array_equal(sr, U["llu_scaling_rate"])
    np.testing.assert_array_equal(lo, U["llu_lower"])
    np.testing.assert_array_equal(up, U["llu_upper"])


def _oracle_for(method, size, iters, load_frac=None, defaults=False, vf=0.3, radius=1.5,
                sensfilter=False):
    m, pb, design, fixed, vol = problems.cantilever(*size, load_frac=load_frac)
    filt = problems.gaussian_filter_for(m, design, radius)
    if defaults:
        cfg = oopt.OracleConfig(method=method, max_iters=iters,
                                filter_radius=oopt.Sched("Constant", radius, radius))
    else:
        C = lambda v: oopt.Sched("Constant", v, v)  # noqa: E731
        cfg = oopt.OracleConfig(method=method, max_iters=iters, p=C(3.0), vol_frac=C(vf),
                                move_limit=C(0.2), filter_radius=C(radius), E_min_coeff=1e-9,
                                sensitivity_filter=sensfilter)
    return oopt.OracleOptimizer(cfg, pb, filt, design, fixed, vol), design


@pytest.mark.parametrize("name,method,size,kw", [
    ("ref_loop_oc_12x6x6", "oc", (12, 6, 6), {}),
    ("ref_loop_logmoc_12x6x6", "logmoc", (12, 6, 6), {"vf": 0.4}),
    ("ref_loop_oc_defaults_10x5x4", "oc", (10, 5, 4),
     {"defaults": True, "load_frac": 0.25, "radius": 1.2}),
    ("ref_loop_oc_sensfilter_12x6x6", "oc", (12, 6, 6), {"sensfilter": True}),
])
def test_oracle_loop_matches_reference_driver(name, method, size, kw):
    """The oracle loop against the reference's DensityMethod loop (OC / log-MOC,
    reference filter, projection, schedules, masks) run with the oracle's FEM
    plugin: compliance, lmid / lambda_v and the densities."""
    R = _load(f"{name}.npz")
    n = int(R["iters"])
    opt, design = _oracle_for(method, size, n, **kw)
    np.testing.assert_array_equal(np.sort(design), np.sort(R["design"]))
    for it in range(1, n + 1):
        opt.step()
        if f"rho_it{it}" in R.files:
            np.testing.assert_allclose(opt.rho, R[f"rho_it{it}"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(opt.hist["compliance"], R["compliance"], rtol=1e-11)
    np.testing.assert_allclose(opt.hist["vol_error"], R["vol_error"], rtol=1e-8, atol=1e-13)
    key = "lmid" if method == "oc" else "lambda_v"
    np.testing.assert_allclose(opt.hist["lmid"], R[key], rtol=1e-11)
    np.testing.assert_allclose(opt.rho, R["rho_final"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("method", ["oc", "logmoc"])
def test_oracle_rho_update_matches_reference_hook(method):
    """OracleOptimizer's update against the reference's rho_update hook called
    as the driver calls it (two calls: the first sets the running scale, the
    second takes the EMA branch and a percentile)."""
    R = _load("ref_rho_update.npz")
    opt, design = _oracle_for(method, (12, 6, 6), 10)
    np.testing.assert_array_equal(np.sort(design), np.sort(R["design"]))
    for call in range(2):
        k = f"{method}_{call}"
        it, move, eta, beta, vf, pct = R[f"{k}_params"]
        pct = None if pct < 0 else float(pct)
        opt.rho = R[f"{k}_in_rho"].copy()
        dC = R[f"{k}_in_dC"].copy()
        rho_d = R[f"{k}_in_rho_design"].copy()
        if method == "oc":
            out = opt._oc_update(int(it), rho_d, dC, move, eta, beta, pct, vf)
            assert opt.hist["lmid"][-1] == float(R[f"{k}_out_lmid"])
        else:
            out = opt._logmoc_update(int(it), rho_d, dC, R[f"{k}_in_rho_projected"],
                                     R[f"{k}_in_rho_filtered"], move, eta, beta, pct, vf)
            np.testing.assert_allclose(opt.lambda_v, float(R[f"{k}_out_lambda_v"]),
                                       rtol=1e-14)
        np.testing.assert_allclose(out, R[f"{k}_out_rho_design"], rtol=0, atol=1e-14)
        np.testing.assert_allclose(opt.running_scale, float(R[f"{k}_out_running_scale"]),
                                   rtol=1e-15)
        np.testing.assert_allclose(opt.hist["kkt_residual"][-1], float(R[f"{k}_out_kkt"]),
                                   rtol=1e-13)
        np.testing.assert_allclose(opt.hist["vol_error"][-1], float(R[f"{k}_out_vol_error"]),
                                   rtol=1e-10, atol=1e-15)


def test_config_defaults_match_reference():
    """Every field of the reference's OC_Config, LogMOC_Config and
    LinearSolverConfig exists on the product's classes with the same default
    (schedules compared field by field); the product's extra fields are GPU
    options."""
    import dataclasses
    import json
    from sktopt_gb300.core import LogMOC_Config, OC_Config
    from sktopt_gb300.fea.solver_elastic import LinearSolverConfig
    with open(os.path.join(G, "ref_config_defaults.json")) as f:
        ref = json.load(f)

    def enc(v):
        if dataclasses.is_dataclass(v):
            return {f.name: enc(getattr(v, f.name)) for f in dataclasses.fields(v)}
        return v
    for name, cls in (("OC_Config", OC_Config), ("LogMOC_Config", LogMOC_Config),
                      ("LinearSolverConfig", LinearSolverConfig)):
        mine = cls()
        for field, want in ref[name].items():
            assert hasattr(mine, field), (name, field)
            got = enc(getattr(mine, field))
            if isinstance(want, dict):
                for k, v in want.items():
                    assert got.get(k) == v, (name, field, k, got.get(k), v)
            else:
                assert got == want, (name, field, got, want)
