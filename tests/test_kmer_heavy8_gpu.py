"""K = 8: the count bound of pairs without [same], against the oracle.

A pair whose two reads have different H keys has m = minsum(H) <= min(|H_a|,
|H_b|); it can pass only if its shorter read is H-heavy (|H| >= mmin[T]).
Both K = 8 tile kernels skip the pairs of two reads that are not.  The cases
put the threshold where reads are heavy or not by a few entries (|H| is
about half of T on these reads), plant reads rich in T and C (heavy at any
threshold) among ordinary ones, and run every form.
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _check(engine, reads, thr, mode):
    buf, offs, lens = synth.pack_reads(reads)
    engine.kmer_prepare(buf, offs, lens, 8)
    cnt = engine.kmer_run(thr, mode, True)
    pairs, d = engine.kmer_fetch(cnt, True)
    op, od = oracle.kmer_all(buf, offs, lens, 8, thr)
    assert cnt == len(op)
    assert np.array_equal(pairs, op)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    return cnt


def _tc_rich(rng, n, length):
    # mostly T and C: nearly every 8-mer starts with T or C (H)
    out = []
    for _ in range(n):
        s = rng.choice(np.frombuffer(b"TCTCTCTCAG", np.uint8), size=length)
        out.append(s.tobytes())
    return out


@pytest.mark.parametrize("thr", [0.105, 0.3, 0.45, 0.5, 0.55])
def test_heavy_threshold_edge(engine, thr):
    reads = synth.make_read_set(synth.ReadSetSpec(1400, 20, 260, "normal", 250, 30, 8, 601))
    for mode in (cg.MODE_BATCHED, cg.MODE_STAGED):
        _check(engine, reads, thr, mode)


def test_heavy_planted_reads(engine):
    rng = np.random.default_rng(602)
    base = synth.make_read_set(synth.ReadSetSpec(1200, 15, 260, "normal", 250, 30, 8, 602))
    rich = _tc_rich(rng, 40, 250)
    # near copies of one rich read pass each other at the default threshold
    twin = bytearray(rich[0])
    twin[100] = ord("A")
    reads = synth.preprocess_order(base + rich + [bytes(twin)])
    t = cg.default_threshold(len(reads), -1.0, 0)
    counts = [_check(engine, reads, t, mode) for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN)]
    assert counts[0] == counts[1] == counts[2] > 0


@pytest.mark.parametrize("queue", ["0", "1"])
@pytest.mark.parametrize("thr", [0.105, 0.2, 0.6])
def test_same_key_queue(engine, monkeypatch, queue, thr):
    # few centroids: large groups of reads with the same H key, so the
    # same-key ranges span many column groups; both forms of the batched
    # same-key pass (L sums queued, or the two-phase kernel)
    monkeypatch.setenv("CRISPY_KMER_K8_QUEUE", queue)
    reads = synth.make_read_set(synth.ReadSetSpec(2600, 6, 260, "normal", 250, 30, 8, 603))
    assert _check(engine, reads, thr, cg.MODE_BATCHED) > 0
