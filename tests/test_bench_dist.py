"""bench.py's multi-process path on CPU: two ranks over gloo (127.0.0.1).

The path shards as independent replicas, so the only exchange is the
timing: a barrier and a max over ranks.  Under torchrun the reference arm
runs on rank 0 alone, and only rank 0 prints the JSON line.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_max(rank, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": "2", "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist, ws, r, _ = bench._dist()
    bench._barrier(dist)
    q.put((r, ws, bench._max_over_ranks(dist, 1.5 + rank)))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_max, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
           "--workload", "small_1k", "--cpu-sample-reads", "300"]
    r = subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")


def test_reference_arm_loads_no_product_library():
    """The reference arm runs oracle/ code only: after a run, the process has
    not mapped libcrispy_gb300.so, and its config equals the GPU arm's."""
    code = (
        "import sys, json, argparse; sys.path.insert(0, %r); import bench\n"
        "a = argparse.Namespace(workload='small_1k', cpu_sample_reads=200, warmup=0, steps=1)\n"
        "line = bench.run_reference(a, None, 1, 0)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'loaded': 'libcrispy_gb300' in maps, 'config': line['config']}))\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["loaded"] is False
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    n = d["config"]["n_reads"]
    want = bench._config("small_1k", n, 6, 10, oracle.default_threshold(n, -1.0, 2),
                         oracle.default_threshold(n, -1.0, 1), 1)
    assert d["config"] == want
