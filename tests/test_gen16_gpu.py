"""The two-cells-per-register genDist kernel (gen16_kernel) against the oracle.

Every shape of the kernel is forced in turn (CRISPY_GEN_SHAPE) on pairs of
1..600 nt at bands 10, 5, 3 and 2, so each shape runs pairs from one band
slot up to its full width, odd and even kBand, short and long reads,
identical reads.  The edge of the kernel's 16-bit key range is tested with
reads of 1,799-1,801 nt: L1 + L2 = 3,600 still runs in the 16-bit kernel,
3,601 and above in the 32-bit kernel.  Per pair the score, ML, AL and the
distance must be bit-exact (genCPU.cpp:290-466).
"""
import os

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu

# shape indices of the 16-bit kernel in the engine's shape list (after the
# 17 shapes of the 32-bit kernel)
N32 = 17
SHAPES16 = list(range(N32, N32 + 14))


@pytest.fixture()
def forced_shape():
    old = os.environ.get("CRISPY_GEN_SHAPE")
    yield
    if old is None:
        os.environ.pop("CRISPY_GEN_SHAPE", None)
    else:
        os.environ["CRISPY_GEN_SHAPE"] = old


def _check(got, want, pairs):
    d, s, ml, al = got
    od, os_, oml, oal = want
    bad = np.nonzero((s != os_) | (ml != oml) | (al != oal) | (d.view(np.uint32) != od.view(np.uint32)))[0]
    assert len(bad) == 0, (f"{len(bad)} pairs differ, first {pairs[bad[:4]].tolist()}: "
                           f"gpu {s[bad[:4]]},{ml[bad[:4]]},{al[bad[:4]]} oracle {os_[bad[:4]]},{oml[bad[:4]]},{oal[bad[:4]]}")


def test_every_shape_vs_oracle(engine, forced_shape):
    rng = np.random.default_rng(160)
    reads = synth.make_read_set(synth.ReadSetSpec(260, 12, 620, "uniform", 1, 600, 6, 161))
    reads += [b"A", b"CA", b"ACGTA", reads[5], reads[5][:-1], b"T" * 9]
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    pairs = rng.integers(0, n, size=(1500, 2)).astype(np.int32)
    pairs[:40, 1] = pairs[:40, 0]                      # identical reads
    pairs[40:46] = [[n - 6 + i, n - 1 - i] for i in range(6)]
    engine.gen_prepare(buf, offs, lens)
    want = {band: oracle.gen_all(buf, offs, lens, pairs, band) for band in (10, 5, 3, 2)}
    for shape in SHAPES16:
        os.environ["CRISPY_GEN_SHAPE"] = str(shape)
        for band, w in want.items():
            _check(engine.gen_align(pairs, band, cg.MODE_BATCHED), w, pairs)


def test_key_range_edge(engine, forced_shape):
    """L1 + L2 = 3,600 in the 16-bit kernel, 3,601 and 3,602 in the 32-bit one."""
    os.environ.pop("CRISPY_GEN_SHAPE", None)
    rng = np.random.default_rng(3600)
    root = rng.integers(0, 4, 1801)
    reads = []
    for ln, sub in ((1799, 0.01), (1800, 0.0), (1800, 0.03), (1801, 0.02), (1801, 0.3), (1700, 0.05)):
        r = root[:ln].copy()
        hit = rng.random(ln) < sub
        r[hit] = (r[hit] + rng.integers(1, 4, hit.sum())) % 4
        reads.append(bytes(np.array(list(b"AGTC"), np.uint8)[r]))
    buf, offs, lens = synth.pack_reads(reads)
    pairs = np.array([[i, j] for i in range(len(reads)) for j in range(len(reads))], np.int32)
    engine.gen_prepare(buf, offs, lens)
    for band in (10, 20, 40):
        want = oracle.gen_all(buf, offs, lens, pairs, band)
        for mode in (cg.MODE_BATCHED, cg.MODE_STAGED):
            _check(engine.gen_align(pairs, band, mode), want, pairs)


def test_staged_uses_one_shape_per_window(engine, forced_shape):
    """The staged form (one launch per load window in the window's widest
    shape) on uneven lengths and the batched form agree with the oracle."""
    os.environ.pop("CRISPY_GEN_SHAPE", None)
    reads = synth.make_read_set(synth.ReadSetSpec(500, 20, 520, "uniform", 300, 500, 6, 162))
    buf, offs, lens = synth.pack_reads(reads)
    rng = np.random.default_rng(162)
    pairs = rng.integers(0, len(lens), size=(6000, 2)).astype(np.int32)
    engine.gen_prepare(buf, offs, lens)
    want = oracle.gen_all(buf, offs, lens, pairs, 10)
    for mode in (cg.MODE_STAGED, cg.MODE_BATCHED):
        _check(engine.gen_align(pairs, 10, mode), want, pairs)
