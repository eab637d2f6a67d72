"""genDist on the GPU vs the oracle.

Per pair: selected score, ML (mismatches + gap columns), AL (alignment
length) bit-exact and the FP32 distance bit-exact.  Per run: threshold,
589,824-pair windows, chunk flushes and the stable sort by distance.
Bands 1 (unbanded), 2, 3, 5, 10; widths from one slot per lane to the
wide-band path; L1 > L2 and L1 < L2; identical reads; length-1 reads.
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _reads(n, seed, root=260, cents=20, dist="normal", a=250, b=15):
    return synth.make_read_set(synth.ReadSetSpec(n, cents, root, dist, a, b, 6, seed))


def _align_check(engine, reads, pairs, band, mode):
    buf, offs, lens = synth.pack_reads(reads)
    engine.gen_prepare(buf, offs, lens)
    d, s, ml, al = engine.gen_align(pairs, band, mode)
    od, os_, oml, oal = oracle.gen_all(buf, offs, lens, pairs, band)
    bad = np.nonzero((s != os_) | (ml != oml) | (al != oal))[0]
    assert len(bad) == 0, f"{len(bad)} pairs differ, first {pairs[bad[:5]]}: gpu {s[bad[:5]]},{ml[bad[:5]]},{al[bad[:5]]} oracle {os_[bad[:5]]},{oml[bad[:5]]},{oal[bad[:5]]}"
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))


def _random_pairs(n, m, seed):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, n, m)
    b = rng.integers(0, n, m)
    return np.stack([a, b], 1).astype(np.int32)


@pytest.mark.parametrize("band", [10, 5, 3, 2, 1])
@pytest.mark.parametrize("mode", [cg.MODE_PLAIN, cg.MODE_STAGED, cg.MODE_BATCHED])
def test_gen_bands(engine, band, mode):
    reads = _reads(300, 50 + band)
    pairs = _random_pairs(len(reads), 3000, band)
    _align_check(engine, reads, pairs, band, mode)


def test_gen_uneven_and_long(engine):
    reads = _reads(400, 61, root=520, dist="uniform", a=300, b=500, cents=30)
    pairs = _random_pairs(len(reads), 4000, 2)
    for band in (10, 4, 2):
        _align_check(engine, reads, pairs, band, cg.MODE_BATCHED)
    longr = _reads(60, 62, root=2100, dist="uniform", a=1200, b=2048, cents=4)
    _align_check(engine, longr, _random_pairs(len(longr), 300, 3), 10, cg.MODE_BATCHED)
    _align_check(engine, longr, _random_pairs(len(longr), 80, 4), 2, cg.MODE_BATCHED)


def test_gen_edge_reads(engine):
    reads = [b"A", b"C", b"AC", b"ACGT", b"TTTT", b"ACGTACGTAC", b"GATTACA" * 3] + _reads(30, 71)
    n = len(reads)
    pairs = np.array([(i, j) for i in range(n) for j in range(n)], np.int32)
    for band in (10, 2, 1):
        for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN):
            _align_check(engine, reads, pairs, band, mode)


def test_gen_run_chunks_small(engine):
    reads = _reads(500, 81)
    buf, offs, lens = synth.pack_reads(reads)
    t = cg.default_threshold(len(reads), 0.35, 0)
    engine.kmer_prepare(buf, offs, lens, 6)
    cnt = engine.kmer_run(t, cg.MODE_BATCHED, False)
    pairs, _ = engine.kmer_fetch(cnt, False)
    engine.gen_prepare(buf, offs, lens)
    tg = cg.default_threshold(len(reads), -1.0, 1)
    for mode in (cg.MODE_PLAIN, cg.MODE_STAGED, cg.MODE_BATCHED, cg.MODE_BATCHED):
        got = engine.gen_run(pairs, 10, tg, mode)
        od, _, _, _ = oracle.gen_all(buf, offs, lens, pairs, 10)
        want = oracle.gen_chunks(pairs, od, tg)
        assert len(got) == len(want)
        for (ci, p, d), (wi, wp, wd) in zip(got, want):
            assert ci == wi
            assert np.array_equal(p, wp)
            assert np.array_equal(d.view(np.uint32), wd.view(np.uint32))
    # the device-resident hand-off gives the same chunks
    engine.kmer_run(t, cg.MODE_BATCHED, False)
    got2 = engine.gen_run_from_kmer(10, tg, cg.MODE_BATCHED)
    assert len(got2) == len(want)
    for (ci, p, d), (wi, wp, wd) in zip(got2, want):
        assert np.array_equal(p, wp) and np.array_equal(d.view(np.uint32), wd.view(np.uint32))


def test_gen_run_many_windows(engine):
    # > 2 load windows with every pair surviving: chunk flushes at 589,824
    reads = _reads(400, 91)
    n = len(reads)
    pairs = _random_pairs(n, 2 * cg.GEN_WINDOW + 12345, 5)
    buf, offs, lens = synth.pack_reads(reads)
    engine.gen_prepare(buf, offs, lens)
    got = engine.gen_run(pairs, 10, 1.0, cg.MODE_BATCHED)
    d, _, _, _ = engine.gen_align(pairs, 10, cg.MODE_BATCHED)
    want = oracle.gen_chunks(pairs, d, 1.0)
    assert [len(c[2]) for c in got] == [len(c[2]) for c in want]
    for (ci, p, dd), (wi, wp, wd) in zip(got, want):
        assert np.array_equal(p, wp) and np.array_equal(dd.view(np.uint32), wd.view(np.uint32))
    # the per-pair distances themselves against the oracle on a sample
    idx = np.random.default_rng(1).integers(0, len(pairs), 5000)
    od, _, _, _ = oracle.gen_all(buf, offs, lens, pairs[idx], 10)
    assert np.array_equal(d[idx].view(np.uint32), od.view(np.uint32))


def test_gen_bad_index_rejected(engine):
    reads = _reads(50, 95)
    buf, offs, lens = synth.pack_reads(reads)
    engine.gen_prepare(buf, offs, lens)
    with pytest.raises(cg.CrispyError) as e:
        engine.gen_run(np.array([[0, len(reads)]], np.int32), 10, 0.5)
    assert e.value.code == cg.E_INPUT


@pytest.mark.parametrize("k", [6, 8])
def test_gen_prepare_from_kmer_matches_upload(engine, k):
    # packing the reads left on the device by kmer_prepare gives the same
    # chunks as a second upload through gen_prepare (K = 8 jobs hold their
    # reads in a read order of their own; genDist takes them by read ID)
    reads = _reads(700, 83, root=520, dist="uniform", a=300, b=500, cents=25)
    buf, offs, lens = synth.pack_reads(reads)
    t = cg.default_threshold(len(reads), -1.0, 0) if k == 6 else 0.7
    tg = cg.default_threshold(len(reads), -1.0, 1)
    engine.kmer_prepare(buf, offs, lens, k)
    engine.kmer_run(t, cg.MODE_BATCHED, False)
    engine.gen_prepare(buf, offs, lens)
    want = engine.gen_run_from_kmer(10, tg, cg.MODE_BATCHED)
    engine.kmer_prepare(buf, offs, lens, k)
    engine.kmer_run(t, cg.MODE_BATCHED, False)
    engine.gen_prepare_from_kmer()
    got = engine.gen_run_from_kmer(10, tg, cg.MODE_BATCHED)
    assert len(got) == len(want) and sum(len(c[2]) for c in got) > 0
    for (ci, p, d), (wi, wp, wd) in zip(got, want):
        assert ci == wi and np.array_equal(p, wp) and np.array_equal(d.view(np.uint32), wd.view(np.uint32))


def test_gen_prepare_from_kmer_needs_kmer_job():
    with cg.Engine(0) as fresh:
        with pytest.raises(cg.CrispyError) as e:
            fresh.gen_prepare_from_kmer()
        assert e.value.code == cg.E_STATE
