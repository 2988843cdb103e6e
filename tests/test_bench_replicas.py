"""The multi-GPU path of bench.py is N independent replicas (one per rank, no
data-path collective): per-rank workloads of the same shape with different
seeded inputs, timings combined by the slowest rank.  Checked here on CPU with
world_size-2 gloo process groups; the reference arm's non-zero ranks exit
without work."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import torch
        got = bench.max_over_ranks(10.0 * (rank + 1), dist, torch.device("cpu"))
        wl = bench.workload("pe", rank)
        dist.barrier()
        out.put((rank, got, int(sum(wl["counts"])), float(wl["energies"][0][:1000].sum())))
    finally:
        dist.destroy_process_group()


def test_replicas_combine_by_slowest_rank_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]        # max over ranks, seen by every rank
    assert res[0][2] == res[1][2] == 1 << 24           # same per-rank work (weak scaling)
    assert res[0][3] != res[1][3]                      # independent inputs per replica


def test_single_process_max_is_identity():
    assert bench.max_over_ranks(3.5, None, None) == 3.5


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_workload_shapes():
    for name in ("pe", "al2o3_large", "al_small"):
        a, b = bench.workload(name, 0), bench.workload(name, 1)
        assert a["counts"] == b["counts"] and a["io"] == b["io"]
        assert not np.array_equal(a["energies"][0][:100], b["energies"][0][:100])
    with pytest.raises(KeyError):
        bench.workload("nope", 0)
