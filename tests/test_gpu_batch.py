"""Batched uneven designs: every design of a concurrent batch follows exactly
the trajectory it has alone (bitwise densities and compliances)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev():
    import torch
    return torch.device("cuda", 0)


def _make(spec, n_iter):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    nx, ny, nz, vf, lf = spec

    def make():
        cfg = OC_Config(max_iters=n_iter, filter_type="spacial",
                        filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                        p=tools.SchedulerConfig.constant(target_value=3.0),
                        vol_frac=tools.SchedulerConfig.constant(target_value=vf),
                        move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                        E_min_coeff=1e-9, solver_option="cg_pyamg", precision="mixed")
        return OC_Optimizer(cfg, toy_problem.cantilever(nx, ny, nz, load_frac=lf),
                            device=_dev())
    return make


def test_batched_designs_match_individual_runs(native_lib):
    from sktopt_gb300.core import BatchedDesigns
    specs = [(16, 8, 8, 0.3, 0.5), (21, 9, 10, 0.45, 0.2), (12, 10, 8, 0.25, 0.9),
             (18, 8, 12, 0.35, 0.0)]
    n_iter = 4
    batch = BatchedDesigns([_make(s, n_iter) for s in specs], n_workers=4, device=_dev())
    batch.step(n_iter)
    for spec, bo in zip(specs, batch.opts):
        solo = _make(spec, n_iter)()
        solo.parameterize()
        solo.optimize_steps(n_iter)
        assert np.array_equal(bo._state.rho.cpu().numpy(), solo._state.rho.cpu().numpy()), spec
        assert list(bo.recorder.histories["compliance"]) == \
            list(solo.recorder.histories["compliance"]), spec


def _stretched(n_iter, autotune=False):
    """A design with 2 x 1 x 1 cells: another element matrix than the cubes."""
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import task
    from sktopt_gb300.mesh.grid import create_box_hex

    def make():
        mesh = create_box_hex(8, 4, 4, hx=2.0)
        ijk = mesh.node_ijk
        dn = np.nonzero(ijk[0] == 0)[0]
        ln = np.nonzero((ijk[0] == 8) & (ijk[2] == 0))[0]
        f = np.zeros(3 * mesh.nnodes)
        f[3 * ln + 2] = -1.0 / ln.size
        tsk = task.LinearElasticity.from_nodes(mesh, dn, "all", ln, [f],
                                               np.arange(mesh.nelements), 1.0, 0.3)
        cfg = OC_Config(max_iters=n_iter, filter_type="spacial",
                        filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                        E_min_coeff=1e-9, solver_option="cg_pyamg", precision="mixed",
                        autotune=autotune)
        return OC_Optimizer(cfg, tsk, device=_dev())
    return make


def test_batched_designs_with_different_element_matrices(native_lib):
    """Each handle passes its own element matrix to the fine-level operator
    (a kernel parameter), so designs with different element matrices share a
    batch and still follow their solo trajectories bit for bit."""
    from sktopt_gb300.core import BatchedDesigns
    n_iter = 3
    makers = [_make((8, 4, 4, 0.3, 0.5), n_iter), _stretched(n_iter)]
    batch = BatchedDesigns(makers, n_workers=2, device=_dev())
    batch.step(n_iter)
    for make, bo in zip(makers, batch.opts):
        solo = make()
        solo.parameterize()
        solo.optimize_steps(n_iter)
        assert np.array_equal(bo._state.rho.cpu().numpy(), solo._state.rho.cpu().numpy())
        assert list(bo.recorder.histories["compliance"]) == \
            list(solo.recorder.histories["compliance"])


def test_run_sharded_matches_solo_runs(native_lib):
    """A rank's share of a sharded batch (partition by element count) gives
    the same histories as running each design alone; without a process
    group every rank returns its own share."""
    from sktopt_gb300.core import partition_designs, run_sharded
    specs = [(12, 6, 6, 0.3, 0.5), (16, 6, 6, 0.4, 0.1), (10, 5, 5, 0.3, 0.9),
             (14, 7, 7, 0.35, 0.3), (12, 8, 6, 0.25, 0.6)]
    makers = [_make(s, 2) for s in specs]
    costs = [a * b * c for a, b, c, _, _ in specs]
    solo = {}
    for i, mk in enumerate(makers):
        o = mk()
        o.parameterize()
        o.optimize_steps(2)
        solo[i] = list(o.recorder.histories["compliance"])
    for rank in range(2):
        got = run_sharded(makers, costs, 2, rank=rank, world_size=2, n_workers=4)
        assert sorted(got) == partition_designs(costs, 2)[rank]
        for i, h in got.items():
            assert h == solo[i], (i, h, solo[i])
