"""bench.py's replica aggregation on two gloo ranks (CPU): barrier, max over ranks of the
timed milliseconds and sum over ranks of the link updates give the whole-job throughput."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    barrier, mx, sm = bench.rank_reducers(dist, torch.device("cpu"))
    barrier()
    ms = [100.0, 250.0][rank]
    units = [1_000_000, 3_000_000][rank]
    out[rank] = bench.replica_value(units, ms, mx, sm)
    dist.destroy_process_group()


def test_replica_value_over_two_gloo_ranks():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        vals = dict(out)
    # 4e6 link updates over the slowest rank's 0.25 s, identical on both ranks
    assert vals[0] == vals[1] == pytest.approx(4_000_000 / 0.25)


def test_single_process_needs_no_group():
    import bench

    barrier, mx, sm = bench.rank_reducers(None, None)
    barrier()
    assert bench.replica_value(10, 1000.0, mx, sm) == 10.0
