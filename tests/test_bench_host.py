"""Host logic of bench.py's multi-rank mode on the CPU: ranks join a gloo
group of two; each rank's timed figures are reduced to the slowest rank's and
the whole-job rate counts every rank's units (independent replicas, no
collective on the data path)."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    # rank r: a step total of 10 + r ms and an end-to-end total of 3 - r s
    got = bench.replica_max([10.0 + rank, 3.0 - rank], dist, "cpu")
    dist.barrier()
    rate = bench.whole_job_rate(world, 1000, got[0] / 1e3)
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"max": got, "rate": rate}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    for r in res:
        assert r["max"] == [11.0, 3.0]  # each figure's slowest rank
        assert r["rate"] == pytest.approx(2 * 1000 / 0.011)


def test_one_process_keeps_its_own_figures():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_max([2.5, 7], None, None) == [2.5, 7.0]
    assert bench.whole_job_rate(1, 500, 0.25) == 2000.0
