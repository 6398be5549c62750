"""The GPU path against fixtures written by the reference's own code
(tests/golden/make_ref_fixtures.py): the reference's update hook called as
its driver calls it, and whole loops of the reference's driver (OC and
log-MOC with its Gaussian filter, projection, schedules and masks; the FEM
arithmetic is the oracle's restatement of scikit-fem)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(G, name))


def _dev():
    return torch.device("cuda", 0)


def _bench_cfg(Cfg, n_iter, precision="fp64", **over):
    from sktopt_gb300 import tools
    S = tools.SchedulerConfig
    kw = dict(max_iters=n_iter, filter_type="spacial",
              filter_radius=S.constant(target_value=1.5), p=S.constant(target_value=3.0),
              vol_frac=S.constant(target_value=0.3), move_limit=S.constant(target_value=0.2),
              E_min_coeff=1e-9, solver_option="spsolve", precision=precision)
    kw.update(over)
    return Cfg(**kw)


@pytest.mark.parametrize("method", ["oc", "logmoc"])
def test_rho_update_hook_matches_reference(native_lib, method):
    """rho_update with the reference's 16-argument signature, on NumPy
    buffers, twice in a row (the second call takes the EMA branches and, for
    OC, a percentile scale): every buffer the reference mutates, and the
    recorded multiplier, volume error and KKT residual."""
    from sktopt_gb300 import tools
    from sktopt_gb300.core import LogMOC_Config, LogMOC_Optimizer, OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    R = _load("ref_rho_update.npz")
    r15 = tools.SchedulerConfig.constant(target_value=1.5)
    if method == "oc":
        opt = OC_Optimizer(OC_Config(filter_type="spacial", filter_radius=r15),
                           toy_problem.cantilever(12, 6, 6), device=_dev())
    else:
        opt = LogMOC_Optimizer(LogMOC_Config(filter_type="spacial", filter_radius=r15),
                               toy_problem.cantilever(12, 6, 6), device=_dev())
    opt.parameterize()
    design = opt.tsk.design_elements
    np.testing.assert_array_equal(np.sort(design), np.sort(R["design"]))
    opt._ensure_state_initialized()
    ev = np.asarray(opt.tsk.elements_volume)[design]
    for call in range(2):
        k = f"{method}_{call}"
        it, move, eta, beta, vf, pct = R[f"{k}_params"]
        pct = None if pct < 0 else float(pct)
        # the full density of the caller's state: the second call's is the
        # first call's update written back, fixed elements held at 1
        # (common_density.py:1130-1134)
        opt._state.rho.copy_(torch.from_numpy(R[f"{k}_in_rho"]))
        rde = R[f"{k}_in_rho_design"].copy()
        dC = R[f"{k}_in_dC"].copy()
        nd = rde.size
        sr, lo, up = np.zeros(nd), np.zeros(nd), np.zeros(nd)
        opt.rho_update(int(it), rde, R[f"{k}_in_rho_projected"].copy(), dC, None, None, sr,
                       float(move), float(eta), float(beta), lo, up, pct, ev,
                       float(np.sum(ev)), float(vf))
        np.testing.assert_allclose(rde, R[f"{k}_out_rho_design"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(lo, R[f"{k}_out_clip_lower"], rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(up, R[f"{k}_out_clip_upper"], rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(sr, R[f"{k}_out_scaling_rate"], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(dC, R[f"{k}_out_dC"], rtol=1e-13, atol=0)
        assert opt.running_scale == pytest.approx(float(R[f"{k}_out_running_scale"]),
                                                  rel=1e-13)
        assert opt.kkt_residual == pytest.approx(float(R[f"{k}_out_kkt"]), rel=1e-9)
        h = opt.recorder.histories
        assert h["vol_error"][-1] == pytest.approx(float(R[f"{k}_out_vol_error"]),
                                                   rel=1e-8, abs=1e-14)
        if method == "oc":
            assert h["lmid"][-1] == pytest.approx(float(R[f"{k}_out_lmid"]), rel=1e-12)
        else:
            assert opt.lambda_v == pytest.approx(float(R[f"{k}_out_lambda_v"]), rel=1e-12)


def _run_loop(method, size, n_iter, fixture, precision, load_frac=None, **cfg_over):
    from sktopt_gb300.core import LogMOC_Config, LogMOC_Optimizer, OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    R = _load(fixture)
    Cfg, Opt = (OC_Config, OC_Optimizer) if method == "oc" else (LogMOC_Config,
                                                                 LogMOC_Optimizer)
    cfg = _bench_cfg(Cfg, int(R["iters"]), precision, **cfg_over)
    opt = Opt(cfg, toy_problem.cantilever(*size, load_frac=load_frac), device=_dev())
    opt.parameterize()
    if "design" in R.files:
        np.testing.assert_array_equal(np.sort(opt.tsk.design_elements), np.sort(R["design"]))
    snaps = {}
    for it in range(1, n_iter + 1):
        opt.optimize_steps(1)
        if f"rho_it{it}" in R.files:
            snaps[it] = opt._state.rho.cpu().numpy().copy()
    return opt, R, snaps


@pytest.mark.parametrize("fixture,method,size,precision,kw", [
    ("ref_loop_oc_12x6x6.npz", "oc", (12, 6, 6), "fp64", {}),
    ("ref_loop_oc_12x6x6.npz", "oc", (12, 6, 6), "mixed", {}),
    ("ref_loop_logmoc_12x6x6.npz", "logmoc", (12, 6, 6), "fp64", {"vf": 0.4}),
    ("ref_loop_oc_defaults_10x5x4.npz", "oc", (10, 5, 4), "fp64", {"defaults": True}),
    ("ref_loop_oc_sensfilter_12x6x6.npz", "oc", (12, 6, 6), "fp64",
     {"sensitivity_filter": True}),
])
def test_loop_matches_reference_driver(native_lib, fixture, method, size, precision, kw):
    """Whole loops against the reference driver: compliance per iteration
    (1e-9 on the FP64 path, 1e-6 mixed), the multiplier, and the densities."""
    from sktopt_gb300 import tools
    S = tools.SchedulerConfig
    over = {}
    load_frac = None
    if kw.get("defaults"):
        # reference defaults (p and beta continuation, sawtooth move limit,
        # vf 0.8, Emin 1e-3) with a 1.2-element Gaussian filter, load at 0.25 ny
        from sktopt_gb300.core import OC_Config
        d = OC_Config()
        over = dict(p=d.p, vol_frac=d.vol_frac, move_limit=d.move_limit,
                    E_min_coeff=d.E_min_coeff, filter_radius=S.constant(target_value=1.2))
        load_frac = 0.25
    if "vf" in kw:
        over["vol_frac"] = S.constant(target_value=kw["vf"])
    if kw.get("sensitivity_filter"):
        over["sensitivity_filter"] = True
    R = _load(fixture)
    n = int(R["iters"])
    opt, R, snaps = _run_loop(method, size, n, fixture, precision, load_frac, **over)
    tol = 1e-9 if precision == "fp64" else 1e-6
    comp = np.array(opt.recorder.histories["compliance"])
    np.testing.assert_allclose(comp, R["compliance"], rtol=tol)
    rtol_rho = 1e-7 if precision == "fp64" else 1e-4
    for it, rho in snaps.items():
        np.testing.assert_allclose(rho, R[f"rho_it{it}"], rtol=0, atol=rtol_rho)
    np.testing.assert_allclose(opt._state.rho.cpu().numpy(), R["rho_final"], rtol=0,
                               atol=rtol_rho)
    if method == "oc":
        np.testing.assert_allclose(opt.recorder.histories["lmid"], R["lmid"],
                                   rtol=1e-9 if precision == "fp64" else 1e-5)
    else:
        np.testing.assert_allclose(opt.recorder.histories["lambda_v"], R["lambda_v"],
                                   rtol=1e-9)


def test_c1_cantilever_matches_reference_driver(native_lib):
    """The 60x20x20 cantilever (24,000 elements, FP64), 10 of its 30 OC
    iterations, against the reference driver's run: compliance per
    iteration within 1e-9 and the density after iteration 10."""
    opt, R, snaps = _run_loop("oc", (60, 20, 20), 10, "ref_loop_oc_60x20x20.npz", "fp64")
    comp = np.array(opt.recorder.histories["compliance"])
    np.testing.assert_allclose(comp, R["compliance"][:10], rtol=1e-9)
    np.testing.assert_allclose(opt.recorder.histories["lmid"], R["lmid"][:10], rtol=1e-9)
    np.testing.assert_allclose(snaps[10], R["rho_it10"], rtol=0, atol=1e-7)
