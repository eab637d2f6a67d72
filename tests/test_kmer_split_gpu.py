"""The bound pass of the 128-row tile kernel (K <= 6) against the oracle.

Every read's dense level entries are split in two sections by a hash of the
plane word (CRISPY_KMER_SPLIT: section 0's share in 1/256, 0 turns the split
off).  The first pass over a column group counts section 0 only; a column
whose every row read is provably below the threshold (m <= m0 + Ta - a0) is
done, the others are counted in full later.  Survivors, their order and
their distances must not depend on the split, the threshold or the read
order (the bound assumes nothing about lengths: a column shorter than a row
of its quarter stays alive).
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _reads(n, seed, k=6):
    return synth.make_read_set(synth.ReadSetSpec(n, max(4, n // 60), 520, "uniform", 300, 500, k, seed))


def _check(engine, reads, k, thr, mode):
    buf, offs, lens = synth.pack_reads(reads)
    engine.kmer_prepare(buf, offs, lens, k)
    cnt = engine.kmer_run(thr, mode, True)
    pairs, d = engine.kmer_fetch(cnt, True)
    op, od = oracle.kmer_all(buf, offs, lens, k, thr)
    assert cnt == len(op)
    assert np.array_equal(pairs, op)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    return cnt


@pytest.mark.parametrize("split", [0, 1, 40, 112, 200, 255])
def test_split_fractions(engine, monkeypatch, split):
    monkeypatch.setenv("CRISPY_KMER_SPLIT", str(split))
    reads = _reads(1500, 501)
    t = cg.default_threshold(len(reads), -1.0, 0)
    a = _check(engine, reads, 6, t, cg.MODE_BATCHED)
    assert a > 0
    assert _check(engine, reads, 6, t, cg.MODE_STAGED) == a


@pytest.mark.parametrize("thr", [0.0, 0.02, 0.08, 0.3, 1.0])
def test_split_thresholds(engine, thr):
    # thr 0: only identical K-mer multisets pass (R at its largest); thr 1:
    # every pair passes (R = 0, every column stays alive)
    reads = _reads(900, 502)
    _check(engine, reads, 6, thr, cg.MODE_BATCHED)


@pytest.mark.parametrize("k", [4, 5, 6])
def test_split_unsorted_reads(engine, k):
    # reads in random order: columns shorter than rows take the fallback
    reads = _reads(1300, 503 + k, k=k)
    rng = np.random.default_rng(k)
    shuffled = [reads[i] for i in rng.permutation(len(reads))]
    t = cg.default_threshold(len(shuffled), -1.0, 0)
    a = _check(engine, shuffled, k, t, cg.MODE_BATCHED)
    assert _check(engine, shuffled, k, t, cg.MODE_STAGED) == a


def test_split_many_alive_columns(engine):
    # few centroids and near-identical reads: most columns survive the bound
    # pass, so the lanes' stacks fill and full-pass rounds run at every step
    reads = synth.make_read_set(synth.ReadSetSpec(2500, 3, 520, "uniform", 300, 500, 6, 504))
    t = cg.default_threshold(len(reads), -1.0, 0)
    assert _check(engine, reads, 6, t, cg.MODE_BATCHED) > 10000


@pytest.mark.parametrize("k", [3, 6, 8])
def test_prep_kernels_agree(engine, monkeypatch, k):
    # the warp-per-read prep kernel (K = 8 reads of at most 512 tuples, or
    # CRISPY_KMER_PREP_WARP=1) and the block-per-read kernel
    # (CRISPY_KMER_PREP_WARP=0) must give the same survivors
    reads = _reads(700, 510 + k, k=k)
    t = 0.5 if k < 8 else 0.7
    monkeypatch.setenv("CRISPY_KMER_PREP_WARP", "0")
    a = _check(engine, reads, k, t, cg.MODE_BATCHED)
    monkeypatch.setenv("CRISPY_KMER_PREP_WARP", "1")
    assert _check(engine, reads, k, t, cg.MODE_BATCHED) == a


def test_split_autotuned(engine, monkeypatch):
    # without CRISPY_KMER_SPLIT the second batched run of a read set of >=
    # 8,192 reads times each candidate split once and keeps the fastest;
    # later runs of the same read set reuse it
    monkeypatch.delenv("CRISPY_KMER_SPLIT", raising=False)
    monkeypatch.delenv("CRISPY_AUTOTUNE", raising=False)
    reads = _reads(9000, 520)
    assert len(reads) >= 8192
    t = cg.default_threshold(len(reads), -1.0, 0)

    def entries():
        return [e for e in cg.tune_report() if e.get("stage") == "kmer" and e["reads"] == len(reads)]

    a = _check(engine, reads, 6, t, cg.MODE_BATCHED)
    assert entries() == []
    assert _check(engine, reads, 6, t, cg.MODE_BATCHED) == a
    e = entries()
    assert len(e) == 1 and e[0]["split"] in (0, 96, 112, 128, 144, 160)
    assert _check(engine, reads, 6, t, cg.MODE_BATCHED) == a
    assert _check(engine, reads, 6, t, cg.MODE_STAGED) == a
    assert len(entries()) == 1
