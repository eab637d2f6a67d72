"""Oracle parity on the benchmark read sets themselves, at their full sizes.

* small_1k (1,000 reads, k = 6, band 10) and plain_20k (20,000 reads): the
  whole survivor list of kmerDist (pairs in stage order, distances bit for
  bit) and every genDist chunk (pairs, distances, chunk boundaries) equal
  the oracle's, for the batched and the staged form (small_1k: the plain
  form too).
* uneven_100k (99,999 reads of 300-500 nt, the headline workload): the
  oracle cannot run all 5e9 pairs in a test, so in the batched form
  - the survivors of 48 rows (the first, evenly spaced, random, the last
    rows) equal the oracle's, pair for pair and bit for bit;
  - every survivor passes the threshold and the list is in stage order;
  - for a 20,000-pair sample of the survivors, the oracle's distance
    decides whether the pair is in genDist's chunks, and the chunks carry
    exactly the oracle's distance for it;
  - every chunk is ascending, chunk sizes follow the 589,824 rule;
  - the staged form gives the same survivors and chunks as the batched.
Reference semantics: kmerCPU.cpp:24-58 / kmerKernel.cu:19-51 (counts),
kmerMain.cpp:161-216 (threshold, stage order), genCPU.cpp:290-466 (band DP),
genCUDA.cu:150-254 (windows, chunk flush, sort).
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def release_after(engine):
    yield
    engine.trim()


def _stage_order_key(pairs, n):
    a = cg.array_dim(n)
    sd = (n + a - 1) // a
    sx = pairs[:, 0].astype(np.int64) // a
    sy = pairs[:, 1].astype(np.int64) // a
    stage = sx * sd - sx * (sx - 1) // 2 + (sy - sx)
    return (stage * a + pairs[:, 0] % a) * a + pairs[:, 1] % a


def _passes(d, thr):
    t = np.float32(thr)
    return (d < t) | (np.abs((d - t).astype(np.float32)).astype(np.float64) < 1e-5)


def _same_chunks(got, want):
    assert len(got) == len(want), f"{len(got)} chunks, oracle {len(want)}"
    for (ci, p, d), (wi, wp, wd) in zip(got, want):
        assert ci == wi
        assert np.array_equal(p, wp), f"chunk {ci}: pairs differ"
        assert np.array_equal(d.view(np.uint32), wd.view(np.uint32)), f"chunk {ci}: distances differ"


@pytest.mark.parametrize("workload,modes", [
    ("small_1k", (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN)),
    ("plain_20k", (cg.MODE_BATCHED, cg.MODE_STAGED)),
])
def test_full_config_vs_oracle(engine, workload, modes):
    reads = synth.make_read_set(workload)
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    k, band = 6, 10
    thr_k = cg.default_threshold(n, -1.0, 0)
    thr_g = cg.default_threshold(n, -1.0, 1)
    assert thr_k == oracle.default_threshold(n, -1.0, 2)
    assert thr_g == oracle.default_threshold(n, -1.0, 1)
    want_p, want_d = oracle.kmer_all(buf, offs, lens, k, thr_k)
    assert len(want_p) > 0
    od, _, _, _ = oracle.gen_all(buf, offs, lens, want_p, band)
    want_chunks = oracle.gen_chunks(want_p, od, thr_g)
    engine.kmer_prepare(buf, offs, lens, k)
    for mode in modes:
        cnt = engine.kmer_run(thr_k, mode, True)
        p, d = engine.kmer_fetch(cnt, True)
        assert np.array_equal(p, want_p), f"mode {mode}: kmer pairs differ"
        assert np.array_equal(d.view(np.uint32), want_d.view(np.uint32)), f"mode {mode}: kmer distances differ"
        engine.gen_prepare_from_kmer()
        _same_chunks(engine.gen_run_from_kmer(band, thr_g, mode), want_chunks)


@pytest.fixture(scope="module")
def uneven():
    reads = synth.make_read_set("uneven_100k")
    return reads, synth.pack_reads(reads)


def test_uneven_100k_sampled_vs_oracle(engine, uneven):
    reads, (buf, offs, lens) = uneven
    n = len(lens)
    k, band = 6, 10
    thr_k = cg.default_threshold(n, -1.0, 0)
    thr_g = cg.default_threshold(n, -1.0, 1)
    engine.kmer_prepare(buf, offs, lens, k)
    cnt = engine.kmer_run(thr_k, cg.MODE_BATCHED, True)
    pairs, d = engine.kmer_fetch(cnt, True)
    assert cnt == len(pairs) > 0
    assert np.all(pairs[:, 0] < pairs[:, 1]) and np.all(pairs[:, 1] < n)
    assert np.all(np.diff(_stage_order_key(pairs, n)) > 0), "survivors are not in stage order"
    assert np.all(_passes(d, thr_k)), "a survivor fails the threshold"

    rng = np.random.default_rng(2024)
    rows = set(range(0, 4)) | set(np.linspace(0, n - 2, 16).astype(int).tolist())
    rows |= set(rng.integers(0, n - 1, 20).tolist()) | set(range(n - 9, n - 1))
    # a stage row boundary (arrayDim 1536) and its neighbours
    a = cg.array_dim(n)
    rows |= {a - 1, a, 7 * a - 1, 7 * a}
    rows = sorted(r for r in rows if 0 <= r < n - 1)
    assert len(rows) >= 48
    for r in rows:
        want_p, want_d = oracle.kmer_rows(buf, offs, lens, k, thr_k, r, r + 1)
        sel = pairs[:, 0] == r
        gp, gd = pairs[sel], d[sel]
        o = np.argsort(gp[:, 1], kind="stable")
        assert np.array_equal(gp[o], want_p), f"row {r}"
        assert np.array_equal(gd[o].view(np.uint32), want_d.view(np.uint32)), f"row {r}"

    engine.gen_prepare_from_kmer()
    chunks = engine.gen_run_from_kmer(band, thr_g, cg.MODE_BATCHED)
    assert chunks, "no genDist survivors"
    for i, (ci, p, dd) in enumerate(chunks):
        assert ci == i and np.all(np.diff(dd) >= 0), "chunk not ascending"
    # chunk boundaries: every chunk but the last holds at least one window's
    # worth of survivors (flushes happen at window ends)
    for ci, p, dd in chunks[:-1]:
        assert len(dd) >= cg.GEN_WINDOW
    got_p = np.concatenate([c[1] for c in chunks]).astype(np.int64)
    got_d = np.concatenate([c[2] for c in chunks])
    got_key = (got_p[:, 0] << 32) | got_p[:, 1]
    o = np.argsort(got_key)
    got_key, got_d = got_key[o], got_d[o]
    assert np.all(np.diff(got_key) > 0), "a pair appears twice in the chunks"

    sample = pairs[np.sort(rng.choice(len(pairs), size=min(20000, len(pairs)), replace=False))]
    od, _, _, _ = oracle.gen_all(buf, offs, lens, sample, band)
    skey = (sample[:, 0].astype(np.int64) << 32) | sample[:, 1].astype(np.int64)
    at = np.searchsorted(got_key, skey)
    at_c = np.minimum(at, len(got_key) - 1)
    present = got_key[at_c] == skey
    want_in = _passes(od, thr_g)
    assert np.array_equal(present, want_in), "chunk membership differs from the oracle's threshold"
    assert np.array_equal(got_d[at_c[present]].view(np.uint32), od[want_in].view(np.uint32))

    # the staged form (per-stage / per-window launches) gives the same bits
    cnt_s = engine.kmer_run(thr_k, cg.MODE_STAGED, True)
    ps, ds = engine.kmer_fetch(cnt_s, True)
    assert np.array_equal(ps, pairs) and np.array_equal(ds.view(np.uint32), d.view(np.uint32))
    engine.gen_prepare_from_kmer()
    staged = engine.gen_run_from_kmer(band, thr_g, cg.MODE_STAGED)
    assert len(staged) == len(chunks)
    for (ci, p, dd), (si, sp, sdd) in zip(chunks, staged):
        assert ci == si and np.array_equal(p, sp) and np.array_equal(dd.view(np.uint32), sdd.view(np.uint32))
