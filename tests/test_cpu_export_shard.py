"""CPU: VTU output (sktopt/core/visualization.py:22-84,
sktopt/mesh/visualization.py:11-37) and the sharding of batched designs
across ranks (partition balanced by cost, one gather on rank 0, two gloo
ranks)."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def test_vtu_round_trip_and_connectivity_orders(tmp_path):
    from sktopt_gb300.core.visualization import export_mesh_with_info, read_vtu, write_vtu
    from sktopt_gb300.mesh import create_box_hex
    m = create_box_hex(3, 2, 2, 0.5, 1.0, 2.0)
    rho = np.linspace(0, 1, m.nelements)
    en = np.arange(m.nelements, dtype=float) ** 2
    export_mesh_with_info(m, cell_data_names=["rho_projected", "energy"],
                          cell_data_values=[rho, en], filepath=tmp_path / "a.vtu")
    r = read_vtu(tmp_path / "a.vtu")
    assert np.array_equal(r["points"], m.p)
    # the reference hands mesh.t to the writer unchanged
    assert np.array_equal(r["connectivity"], m.t)
    assert np.all(r["types"] == 12)
    assert np.array_equal(r["cell_data"]["rho_projected"], rho)
    assert np.array_equal(r["cell_data"]["energy"], en)
    # VTK order: nodes 0-3 the bottom face counter-clockwise, then the top
    write_vtu(tmp_path / "b.vtu", m.p, m.t, "hex", vtk_order=True)
    c = read_vtu(tmp_path / "b.vtu")["connectivity"]
    for e in range(m.nelements):
        x = m.p[:, c[:, e]]
        rel = (x - x[:, :1]) / np.array([[0.5], [1.0], [2.0]])
        want = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1),
                (0, 1, 1)]
        assert np.allclose(rel.T, want)


def test_export_submesh_thresholds_design_elements(tmp_path):
    from sktopt_gb300.core.visualization import export_submesh, read_vtu
    from sktopt_gb300.mesh import toy_problem
    tsk = toy_problem.cantilever(6, 3, 3)
    rho = np.random.default_rng(0).uniform(0, 1, tsk.mesh.nelements)
    export_submesh(tsk, rho, 0.5, tmp_path / "top.vtu")
    r = read_vtu(tmp_path / "top.vtu")
    design = np.asarray(tsk.design_elements)
    keep = np.setdiff1d(np.arange(tsk.mesh.nelements), design[rho[design] <= 0.5])
    assert r["connectivity"].shape[1] == keep.size
    verts = np.unique(tsk.mesh.t[:, keep])
    assert np.array_equal(r["points"], tsk.mesh.p[:, verts])
    # the kept cells' vertex sets, renumbered
    got = {tuple(sorted(verts[c])) for c in r["connectivity"].T}
    assert got == {tuple(sorted(tsk.mesh.t[:, e])) for e in keep}


def test_partition_designs_balanced_and_complete():
    from sktopt_gb300.core import partition_designs
    from sktopt_gb300.mesh import toy_problem
    specs = toy_problem.batched_cantilever_specs(256, seed=0)
    costs = [nx * ny * nz for nx, ny, nz, _, _ in specs]
    for world in (1, 2, 3, 8):
        parts = partition_designs(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
        assert parts == partition_designs(costs, world)        # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from sktopt_gb300.core import gather_design_results, partition_designs
    costs = [5, 3, 8, 1, 7, 2]
    mine = partition_designs(costs, world)[rank]
    res = gather_design_results({i: [float(i), float(rank)] for i in mine})
    out[rank] = res
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_design_results():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[1] is None
    got = out[0]
    assert sorted(got) == list(range(6))
    from sktopt_gb300.core import partition_designs
    parts = partition_designs([5, 3, 8, 1, 7, 2], 2)
    for r, p in enumerate(parts):
        for i in p:
            assert got[i] == [float(i), float(r)]


def _rank_subgroup(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from sktopt_gb300.core import gather_design_results
    grp = dist.new_group([1, 2])          # every rank creates it; rank 0 is not in it
    if rank in (1, 2):
        out[rank] = gather_design_results({rank * 10: [float(rank)]}, group=grp)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_into_a_subgroup_without_global_rank_zero():
    """A group of global ranks {1, 2}: the results land on global rank 1 (the
    group's rank 0), not on global rank 0."""
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_subgroup, args=(r, 3, port, out)) for r in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[2] is None
    assert out[1] == {10: [1.0], 20: [2.0]}


def test_partition_more_ranks_than_designs():
    from sktopt_gb300.core import partition_designs
    parts = partition_designs([3.0, 1.0, 2.0], 5)
    assert sorted(i for p in parts for i in p) == [0, 1, 2]
    assert sum(1 for p in parts if not p) == 2


def test_vtu_tetrahedra_with_point_data(tmp_path):
    from sktopt_gb300.core.visualization import read_vtu, write_vtu
    from sktopt_gb300.mesh import create_box_tet
    m = create_box_tet(2, 2, 1, 1.0, 1.0, 0.5, jitter=0.1, seed=3)
    pd = np.arange(m.nnodes, dtype=float)
    cd = np.linspace(-1, 1, m.nelements)
    write_vtu(tmp_path / "t.vtu", m.p, m.t, "tet", cell_data={"c": cd}, point_data={"T": pd})
    r = read_vtu(tmp_path / "t.vtu")
    assert np.all(r["types"] == 10) and np.array_equal(r["connectivity"], m.t)
    assert np.array_equal(r["point_data"]["T"], pd) and np.array_equal(r["cell_data"]["c"], cd)
