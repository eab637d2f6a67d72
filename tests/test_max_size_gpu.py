"""The reference's largest read set: 1,048,576 reads (MAX_NUM_READS,
kmerMain.h:28-30), k = 6, band 10, default thresholds, batched form.

At this size the oracle cannot run the whole triangle, so the checks are:
* the survivors of two slices of 16 rows (the first rows, against about a
  million columns each, and 16 rows near the end) equal the oracle's for
  those rows, pair for pair and bit for bit;
* every survivor's distance passes the threshold, and the survivor list is
  in stage order;
* genDist over all the survivors: its chunks are each ascending, flushed at
  the 589,824-pair rule, and hold exactly the survivors whose per-pair
  distance (crispy_gen_align) passes; a 20,000-pair sample of those
  distances equals the oracle's;
* one read more is refused.
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu

N_MAX = cg.MAX_NUM_READS


@pytest.fixture(scope="module")
def max_set():
    # about 1.07M raw reads from 20,000 centroids; after deduplication and
    # the (length, bytes) order, the first 2^20
    reads = synth.make_read_set(synth.ReadSetSpec(1_075_000, 20000, 260, "normal", 250, 15, 6, 2099))
    assert len(reads) >= N_MAX
    return synth.pack_reads(reads[:N_MAX])


@pytest.fixture(scope="module", autouse=True)
def release_after(engine):
    yield
    engine.trim()   # the session's engine keeps no multi-GB buffers for later tests


def _stage_order_key(pairs, n):
    a = cg.array_dim(n)
    sd = (n + a - 1) // a
    sx = pairs[:, 0].astype(np.int64) // a
    sy = pairs[:, 1].astype(np.int64) // a
    stage = sx * sd - sx * (sx - 1) // 2 + (sy - sx)      # row-major upper triangle
    return (stage * a + pairs[:, 0] % a) * a + pairs[:, 1] % a


def test_max_reads_kmer_and_gen(engine, max_set):
    buf, offs, lens = max_set
    n = len(lens)
    assert n == N_MAX
    thr_k = cg.default_threshold(n, -1.0, 0)
    engine.kmer_prepare(buf, offs, lens, 6)
    cnt = engine.kmer_run(thr_k, cg.MODE_BATCHED, True)
    pairs, d = engine.kmer_fetch(cnt, True)
    assert cnt == len(pairs) > 0
    assert np.all(pairs[:, 0] < pairs[:, 1]) and np.all(pairs[:, 1] < n)
    key = _stage_order_key(pairs, n)
    assert np.all(np.diff(key) > 0), "survivors are not in stage order"
    t = np.float32(thr_k)
    ok = (d < t) | (np.abs((d - t).astype(np.float32)).astype(np.float64) < 1e-5)
    assert np.all(ok)
    for lo in (0, n - 4096):
        hi = lo + 16
        want_p, want_d = oracle.kmer_rows(buf, offs, lens, 6, thr_k, lo, hi)
        sel = (pairs[:, 0] >= lo) & (pairs[:, 0] < hi)
        gp, gd = pairs[sel], d[sel]
        o = np.lexsort((gp[:, 1], gp[:, 0]))
        assert np.array_equal(gp[o], want_p)
        assert np.array_equal(gd[o].view(np.uint32), want_d.view(np.uint32))

    # genDist over every survivor, from the reads already on the device
    engine.gen_prepare_from_kmer()
    thr_g = cg.default_threshold(n, -1.0, 1)
    chunks = engine.gen_run_from_kmer(10, thr_g, cg.MODE_BATCHED)
    got = np.concatenate([c[1] for c in chunks]) if chunks else np.zeros((0, 2), np.uint32)
    for i, c in enumerate(chunks):
        assert c[0] == i
        assert np.all(np.diff(c[2]) >= 0), "chunk not ascending"
        if i + 1 < len(chunks):
            assert len(c[2]) >= cg.GEN_WINDOW
    dist, _, _, _ = engine.gen_align(pairs, 10)
    t = np.float32(thr_g)
    passing = (dist < t) | (np.abs((dist - t).astype(np.float32)).astype(np.float64) < 1e-5)

    def keys(p):
        return np.sort((p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64))
    assert np.array_equal(keys(got), keys(pairs[passing]))
    rng = np.random.default_rng(7)
    sample = pairs[rng.choice(len(pairs), size=min(20000, len(pairs)), replace=False)]
    od, _, _, _ = oracle.gen_all(buf, offs, lens, sample, 10)
    gd2, _, _, _ = engine.gen_align(sample, 10)
    assert np.array_equal(gd2.view(np.uint32), od.view(np.uint32))


def test_one_read_more_is_refused(engine, max_set):
    buf, offs, lens = max_set
    offs2 = np.concatenate([offs, offs[-1:]])
    lens2 = np.concatenate([lens, lens[-1:]])
    with pytest.raises(cg.CrispyError) as e:
        engine.kmer_prepare(buf, offs2, lens2, 6)
    assert e.value.code == cg.E_UNSUPPORTED
