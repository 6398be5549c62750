"""The replicas path of bench.py on CPU: two gloo ranks agree on the job's
time (the maximum over ranks) and the barrier returns on both."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.replica_barrier()
    out[rank] = bench.replica_max(1.0 + rank)
    bench.replica_barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_max_time():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_single_process_replica_helpers_are_identity():
    import bench
    bench.replica_barrier()
    assert bench.replica_max(3.5) == 3.5
