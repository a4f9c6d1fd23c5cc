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


_REFERENCE_ARM = r"""
import json, sys, types
sys.path.insert(0, %r)
import bench
bench.WORKLOAD_ARGS = dict(bench.WORKLOAD_ARGS, n=16)
bench.run_reference(types.SimpleNamespace(gpus=1, steps=1, warmup=0))
maps = open("/proc/self/maps").read()
print(json.dumps({"product_imported": "ouranos_gb300" in sys.modules,
                  "product_mapped": "libouranos_gb300" in maps,
                  "oracle_mapped": "liboracle" in maps}))
"""


def test_reference_arm_loads_nothing_of_the_product():
    """The CPU reference arm builds its inputs with the oracle's own generator:
    the product package is never imported and its library never mapped; its
    config object carries the same keys as the GPU arm's."""
    import subprocess
    r = subprocess.run([sys.executable, "-c", _REFERENCE_ARM % ROOT], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["value"] > 0
    assert not probe["product_imported"] and not probe["product_mapped"] and probe["oracle_mapped"]
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.workload_config(16 * 16, 144, 10, 9, 1)
