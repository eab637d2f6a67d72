"""genDist chunk order against the library the reference orders with.

The reference sorts each chunk with thrust::sort_by_key on the device, float
distance keys carrying the read pairs (genCUDA.cu:39-45); equal distances
keep their input order only if that sort is stable.  The engine orders its
chunks with its own stable radix sort.  Here a chunk with many equal
distances (genetic distances are ratios of small integers) is ordered by
both: oracle/thrust_order.cu (built here with nvcc against CUDA's Thrust)
and the engine; the orders must agree element for element.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "oracle", "thrust_order.cu")


@pytest.fixture(scope="module")
def thrust_order(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("thrust") / "thrust_order")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", SRC, "-o", exe],
                   check=True)
    return exe


def _thrust_sort(exe, tmp, dist, pairs):
    src, dst = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    with open(src, "wb") as f:
        f.write(np.int64(len(dist)).tobytes())
        f.write(np.ascontiguousarray(dist, np.float32).tobytes())
        f.write(np.ascontiguousarray(pairs, np.uint32).tobytes())
    subprocess.run([exe, src, dst], check=True)
    raw = open(dst, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    d = np.frombuffer(raw[8:8 + 4 * n], np.float32)
    p = np.frombuffer(raw[8 + 4 * n:], np.uint32).reshape(-1, 2)
    return d, p


def test_chunk_order_matches_thrust(engine, thrust_order, tmp_path):
    reads = synth.make_read_set(synth.ReadSetSpec(1500, 30, 260, "normal", 250, 15, 6, 41))
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    engine.kmer_prepare(buf, offs, lens, 6)
    cnt = engine.kmer_run(0.6, cg.MODE_BATCHED, False)
    pairs, _ = engine.kmer_fetch(cnt, False)
    assert cnt > 20000
    thr = 0.35
    engine.gen_prepare(buf, offs, lens)
    chunks = engine.gen_run(pairs, 10, thr, cg.MODE_BATCHED)
    assert len(chunks) == 1   # fewer than 589,824 pairs: one window, one chunk
    dist, _, _, _ = engine.gen_align(pairs, 10)
    t = np.float32(thr)
    keep = (dist < t) | (np.abs((dist - t).astype(np.float32)).astype(np.float64) < 1e-5)
    d_in, p_in = dist[keep], pairs[keep].astype(np.uint32)
    assert len(np.unique(d_in)) < len(d_in) // 4, "the chunk should hold many equal distances"
    td, tp = _thrust_sort(thrust_order, str(tmp_path), d_in, p_in)
    _, gp, gd = chunks[0]
    assert np.array_equal(gd.view(np.uint32), td.view(np.uint32))
    assert np.array_equal(gp.astype(np.uint32), tp)
    # and the distances themselves are the oracle's
    od, _, _, _ = oracle.gen_all(buf, offs, lens, p_in.astype(np.int32), 10)
    assert np.array_equal(od.view(np.uint32), d_in.view(np.uint32))
