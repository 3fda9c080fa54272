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


def test_batch_counts_only_successful_trajectories():
    """the batch leg's throughput counts the links of ensemble trajectories whose projection
    succeeded and names the ensembles that failed"""
    import numpy as np

    import bench

    status = np.array([[0, 7, 0], [0, 7, 7], [0, 7, 0]])  # 3 trajectories x 3 ensembles
    counted, failed = bench.counted_batch_link_updates(status, [2, 3, 4], 4, 10)
    links = np.array([2, 3, 4]) ** 4 * 4
    assert counted == (3 * links[0] + 0 * links[1] + 2 * links[2]) * 10
    assert failed == {1: 3, 2: 1}
    counted, failed = bench.counted_batch_link_updates(np.zeros((2, 2), dtype=int), [3, 5], 3, 1)
    assert counted == 2 * (27 * 3 + 125 * 3) and failed == {}
