"""The stress read set at full size: 496,820 reads of N(250, 30) nt from 5,000
centroids, k = 8, band 5, batched form.

K = 8 runs on reads sorted by H key and splits the pairs between two tile
kernels; the largest key group holds about 30 % of the reads.  The oracle
cannot run the whole triangle, so the checks are:
* the survivors of 24 rows equal the oracle's, pair for pair and bit for
  bit: rows of the largest key group, random rows and the last rows;
* every survivor passes the threshold and the list is in stage order;
* a 20,000-pair sample of genDist distances over the survivors equals the
  oracle's, and genDist's chunks hold exactly the passing pairs.
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu

_CODE = np.zeros(256, np.uint32)
_CODE[ord("G")], _CODE[ord("T")], _CODE[ord("C")] = 1, 2, 3


def _h_key(s: bytes) -> int:
    """(largest 8-mer >= 0x8000) << 16 | its count, 0 without one."""
    a = _CODE[np.frombuffer(s, np.uint8)]
    t = len(a) - 7
    v = np.zeros(t, np.uint32)
    for q in range(8):
        v = (v << 2) | a[q:q + t]
    h = v[v >= 0x8000]
    if len(h) == 0:
        return 0
    m = int(h.max())
    return (m << 16) | int((v == m).sum())


@pytest.fixture(scope="module")
def stress_set():
    reads = synth.make_read_set("stress_500k")
    return reads, synth.pack_reads(reads)


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


def test_stress_k8_rows_and_gen(engine, stress_set):
    reads, (buf, offs, lens) = stress_set
    n = len(lens)
    thr_k = cg.default_threshold(n, -1.0, 0)
    engine.kmer_prepare(buf, offs, lens, 8)
    cnt = engine.kmer_run(thr_k, cg.MODE_BATCHED, True)
    pairs, d = engine.kmer_fetch(cnt, True)
    assert cnt == len(pairs) > 0
    assert np.all(pairs[:, 0] < pairs[:, 1]) and np.all(pairs[:, 1] < n)
    assert np.all(np.diff(_stage_order_key(pairs, n)) > 0), "survivors are not in stage order"
    t = np.float32(thr_k)
    assert np.all((d < t) | (np.abs((d - t).astype(np.float32)).astype(np.float64) < 1e-5))

    # rows: 8 of the largest key group among the first 3,000 reads, 8 random, the last 8
    keys = np.array([_h_key(s) for s in reads[:3000]], np.uint64)
    vals, counts = np.unique(keys, return_counts=True)
    big = np.flatnonzero(keys == vals[np.argmax(counts)])
    assert len(big) > 300   # the set's largest group holds about 30 % of the reads
    rng = np.random.default_rng(5)
    rows = sorted(set(big[:: len(big) // 8][:8].tolist()) | set(rng.integers(0, n - 1, 8).tolist())
                  | set(range(n - 9, n - 1)))
    for r in rows:
        want_p, want_d = oracle.kmer_rows(buf, offs, lens, 8, thr_k, r, r + 1)
        sel = pairs[:, 0] == r
        gp, gd = pairs[sel], d[sel]
        o = np.argsort(gp[:, 1], kind="stable")
        assert np.array_equal(gp[o], want_p), f"row {r}"
        assert np.array_equal(gd[o].view(np.uint32), want_d.view(np.uint32)), f"row {r}"

    # genDist over every survivor, from the reads already on the device
    engine.gen_prepare_from_kmer()
    thr_g = cg.default_threshold(n, -1.0, 1)
    chunks = engine.gen_run_from_kmer(5, thr_g, cg.MODE_BATCHED)
    got = np.concatenate([c[1] for c in chunks]) if chunks else np.zeros((0, 2), np.uint32)
    for i, c in enumerate(chunks):
        assert c[0] == i and np.all(np.diff(c[2]) >= 0), "chunk not ascending"
    dist, _, _, _ = engine.gen_align(pairs, 5)
    tg = np.float32(thr_g)
    passing = (dist < tg) | (np.abs((dist - tg).astype(np.float32)).astype(np.float64) < 1e-5)

    def keyset(p):
        return np.sort((p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64))
    assert np.array_equal(keyset(got), keyset(pairs[passing]))
    sample = pairs[rng.choice(len(pairs), size=min(20000, len(pairs)), replace=False)]
    od, _, _, _ = oracle.gen_all(buf, offs, lens, sample, 5)
    gd2, _, _, _ = engine.gen_align(sample, 5)
    assert np.array_equal(gd2.view(np.uint32), od.view(np.uint32))
