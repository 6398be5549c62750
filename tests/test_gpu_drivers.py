"""Driver-level GPU tests: the multi-load tet configuration (log-space MOC,
Helmholtz filter, mixed solver against the FP64 solver) and the checkpoint /
restart files of common_density.py:711-745, 1199-1233.

Tolerances: mixed against FP64 compliance 1e-6 relative per iteration (the
mixed solve reaches the same FP64 residual 1e-8); densities 1e-5.
"""
import dataclasses
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _logmoc_cfg(n_iter, precision, radius):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import LogMOC_Config
    return LogMOC_Config(max_iters=n_iter, filter_type="helmholtz",
                         filter_radius=tools.SchedulerConfig.constant(target_value=radius),
                         p=tools.SchedulerConfig.constant(target_value=3.0),
                         vol_frac=tools.SchedulerConfig.constant(target_value=0.25),
                         move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                         E_min_coeff=1e-9, solver_option="cg_pyamg", precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_load_tet_logmoc_helmholtz_matches_oracle(native_lib, precision):
    """The multi-load unstructured configuration at small size against the
    oracle loop (same mesh, Dirichlet nodes, 4 point-load cases and design
    sets; NumPy/SciPy direct solves, the restated nodal Helmholtz filter and
    log-MOC update): compliance per iteration 1e-8 (FP64 path) / 1e-6
    (mixed), densities 1e-6 / 1e-5."""
    from oracle import fem as ofem
    from oracle import filters as ofilt
    from oracle import mesh as omesh
    from oracle import optim as oopt
    from sktopt_gb300.core import LogMOC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    n_iter, radius = 5, 3.2 * 0.25
    tsk = toy_problem.multi_load_tet(8, 4, 4, 2.0, 1.0, 1.0, jitter=0.2, seed=3)
    opt = LogMOC_Optimizer(_logmoc_cfg(n_iter, precision, radius), tsk, device=_dev())
    opt.parameterize()
    mesh = tsk.mesh
    om = omesh.GridMesh(mesh.p, mesh.t, "tet", None, None, None)
    dn = np.unique(np.asarray(tsk.dirichlet_nodes))
    pb = ofem.ElasticProblem(om, dn, [np.asarray(f) for f in tsk.neumann_linear])
    design = np.asarray(tsk.design_elements, dtype=np.int64)
    fixed = np.setdiff1d(np.arange(mesh.nelements), design)
    mask = np.zeros(mesh.nelements, bool)
    mask[design] = True
    vol = omesh.elements_volume(om)
    np.testing.assert_allclose(vol, np.asarray(tsk.elements_volume), rtol=1e-14)
    filt = ofilt.HelmholtzFilterNodal(om, vol, radius, mask)
    C = lambda v: oopt.Sched("Constant", v, v)  # noqa: E731
    ocfg = oopt.OracleConfig(method="logmoc", max_iters=n_iter, p=C(3.0), vol_frac=C(0.25),
                             move_limit=C(0.2), filter_radius=C(radius), E_min_coeff=1e-9)
    ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
    ctol, rtol = (1e-8, 1e-6) if precision == "fp64" else (1e-6, 1e-5)
    for k in range(n_iter):
        opt.optimize_steps(1)
        c_ref = ref.step()
        c = opt.recorder.histories["compliance"][-1]
        assert abs(c - c_ref) <= ctol * abs(c_ref), (k, c, c_ref)
        np.testing.assert_allclose(opt._state.rho.cpu().numpy(), ref.rho, rtol=0, atol=rtol)
        assert opt.lambda_v == pytest.approx(ref.lambda_v, rel=1e-6, abs=1e-12)


def test_multi_load_tet_logmoc_helmholtz_mixed_vs_fp64(native_lib):
    """The multi-load unstructured configuration at small size: jittered P1
    tets on a 2x1x1 box, bottom clamped, 4 point-load cases solved as one
    4-column block RHS, log-MOC, Helmholtz filter (radius 3.2 cells, the
    configuration's r/h), mixed against FP64."""
    from sktopt_gb300.core import LogMOC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    n_iter = 5
    hist = {}
    for precision in ("fp64", "mixed"):
        tsk = toy_problem.multi_load_tet(8, 4, 4, 2.0, 1.0, 1.0, jitter=0.2, seed=3)
        assert len(tsk.neumann_linear) == 4
        opt = LogMOC_Optimizer(_logmoc_cfg(n_iter, precision, 3.2 * 0.25), tsk, device=_dev())
        opt.parameterize()
        comps, rhos = [], []
        for _ in range(n_iter):
            opt.optimize_steps(1)
            comps.append(opt.recorder.histories["compliance"][-1])
            rhos.append(opt._state.rho.cpu().numpy().copy())
        st = opt.fem.solve_history[-1]
        assert st.status == 0 and st.relres <= 1e-8, st
        hist[precision] = (comps, rhos)
    for k in range(n_iter):
        c64, c32 = hist["fp64"][0][k], hist["mixed"][0][k]
        assert abs(c32 - c64) <= 1e-6 * abs(c64), (k, c32, c64)
        np.testing.assert_allclose(hist["mixed"][1][k], hist["fp64"][1][k], rtol=0, atol=1e-5)


def test_restart_from_checkpoint(native_lib, tmp_path):
    """Export writes data/NNNNNN-rho.npz every iteration and histories.npz;
    a restart from iteration k loads exactly the saved design densities and
    continues at k + 1."""
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    n_iter = 6
    cfg = OC_Config(max_iters=n_iter, filter_type="spacial",
                    filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                    p=tools.SchedulerConfig.constant(target_value=3.0),
                    vol_frac=tools.SchedulerConfig.constant(target_value=0.3),
                    move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                    E_min_coeff=1e-9, solver_option="cg_pyamg", export=True,
                    dst_path=str(tmp_path), record_times=n_iter)
    a = OC_Optimizer(cfg, toy_problem.cantilever(12, 6, 6), device=_dev())
    a.parameterize()
    a.optimize()
    files = sorted(os.listdir(tmp_path / "data"))
    assert files == [f"{i:06d}-rho.npz" for i in range(1, n_iter + 1)], files
    h = np.load(tmp_path / "histories.npz")
    assert len(h["compliance"]) == n_iter
    np.testing.assert_array_equal(h["compliance"], a.recorder.histories["compliance"])
    saved3 = np.load(tmp_path / "data" / "000003-rho.npz")["rho_design_elements"]
    b = OC_Optimizer(dataclasses.replace(cfg, restart=True, restart_from=3),
                     toy_problem.cantilever(12, 6, 6), device=_dev())
    b.parameterize()
    rho0, it0, it_end = b.initialize_density()
    assert it0 == 4 and it_end == n_iter + 1
    np.testing.assert_array_equal(rho0[b.tsk.design_elements], saved3)
    b.optimize()
    last = np.load(tmp_path / "data" / f"{n_iter:06d}-rho.npz")["rho_design_elements"]
    assert np.all(np.isfinite(last)) and last.shape == saved3.shape
    # VTU of every saved iteration (rho_projected, energy) and the final
    # thresholded design (common_density.py:1199-1204, 960-962)
    from sktopt_gb300.core.visualization import read_vtu
    vtus = sorted(os.listdir(tmp_path / "mesh_rho"))
    assert vtus == [f"info_mesh-{i:08d}.vtu" for i in range(1, n_iter + 1)], vtus
    v = read_vtu(tmp_path / "mesh_rho" / vtus[-1])
    assert set(v["cell_data"]) == {"rho_projected", "energy"}
    assert v["cell_data"]["rho_projected"].shape == (b.tsk.mesh.nelements,)
    np.testing.assert_array_equal(v["cell_data"]["rho_projected"],
                                  b._state.rho_projected.cpu().numpy())
    top = read_vtu(tmp_path / "cubic_top.vtu")
    assert 0 < top["connectivity"].shape[1] <= b.tsk.mesh.nelements
