"""The multi-process path of bench.py on the CPU (gloo, world size 2): ranks join, the timed
region's time is the maximum over ranks, the aggregate counts every replica's bytes, and the
reference arm runs on rank 0 alone while the other ranks exit 0 without output."""

import json
import multiprocessing
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    w, r, _ = bench.dist_setup()
    slowest = bench.reduce_max(10.0 + r, w)
    bench.barrier(w)
    q.put((r, w, slowest, bench.aggregate(100.0, 2, slowest, w)))
    dist.destroy_process_group()


def test_two_ranks_take_the_max_and_aggregate():
    pytest.importorskip("torch")
    ctx = multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for _, world, slowest, agg in got:
        assert world == 2 and slowest == 11.0
        # two replicas x 100 bytes x 2 steps in 11 ms
        assert agg == pytest.approx(2 * 100.0 * 2 / 0.011 / 1e9)


def test_reference_arm_runs_on_rank_zero_only():
    pytest.importorskip("torch")
    port = free_port()
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "3", "--cpu-sample", str(1 << 16), "--cpu-procs", "2"]
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen(cmd, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    assert [p.returncode for p in procs] == [0, 0], [o[1][-500:] for o in outs]
    lines = [ln for ln in outs[0][0].splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert not [ln for ln in outs[1][0].splitlines() if ln.strip()]
