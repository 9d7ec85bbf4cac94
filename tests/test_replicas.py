"""The replica path of bench.py on CPU: two gloo ranks join, meet at the
barrier and agree on the slowest time (no data-path collective: each rank
solves its own pairs)."""
import os
import socket
import sys

import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    r, w, local = bench.replica_setup(backend="gloo")
    bench.replica_barrier()
    slowest = bench.replica_max(10.0 + rank)  # rank 1 is the slow replica
    out[rank] = (r, w, local, slowest)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_slowest_time():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == (0, 2, 0, 11.0)
    assert res[1] == (1, 2, 1, 11.0)


def test_single_process_is_a_replica_of_one(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.replica_setup() == (0, 1, 0)
    bench.replica_barrier()
    assert bench.replica_max(3.5) == 3.5
