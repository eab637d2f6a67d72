"""kmerDist on the GPU vs the oracle: survivors, order and distances bit-exact.

Cases follow what the reference handles: default and user thresholds, every
K in 1..8 (K = 8 carries the signed-sort merge quirk), read counts that give
each stage tile size (arrayDim 4, 32, 256, 1536), reads with K-mer
multiplicities beyond the shared-memory level budget, reads of length K-1
(no tuples), plain and batched modes.
"""
import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu


def _reads(n, seed, root=260, cents=20, dist="normal", a=250, b=15, k=6):
    return synth.make_read_set(synth.ReadSetSpec(n, cents, root, dist, a, b, k, seed))


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


@pytest.mark.parametrize("mode", [cg.MODE_PLAIN, cg.MODE_STAGED, cg.MODE_BATCHED])
@pytest.mark.parametrize("k", [4, 5, 6, 7, 8])
def test_kmer_k_modes(engine, k, mode):
    reads = _reads(400, 100 + k, k=k)
    thr = 0.45 if k < 8 else 0.6
    assert _check(engine, reads, k, thr, mode) > 0


@pytest.mark.parametrize("n", [10, 37, 99, 150, 1200])
def test_kmer_tile_sizes_default_threshold(engine, n):
    reads = _reads(n + n // 10 + 5, 7 + n)[:n]
    t = cg.default_threshold(len(reads), -1.0, 0)
    for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN):
        _check(engine, reads, 6, t, mode)


def test_kmer_k1_k3(engine):
    reads = _reads(120, 5)
    for k in (1, 2, 3):
        _check(engine, reads, k, 0.2, cg.MODE_BATCHED)


def test_kmer_heavy_multiplicity(engine):
    # homopolymer runs push one 6-mer's count far past the level budget (12)
    rng = np.random.default_rng(3)
    reads = _reads(200, 9)
    heavy = []
    for i in range(40):
        s = bytearray(reads[i])
        run = 20 + (i % 30)
        s[10:10 + run] = b"A" * run
        heavy.append(bytes(s))
    reads = synth.preprocess_order(reads[40:] + heavy)
    for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN):
        _check(engine, reads, 6, 0.5, mode)
    # long degenerate reads: counts above 255
    long = [b"A" * (400 + i) for i in range(5)] + [b"AC" * (150 + i) for i in range(5)]
    _check(engine, synth.preprocess_order(long + reads[:30]), 6, 0.9, cg.MODE_BATCHED)


def test_kmer_short_reads_no_tuples(engine):
    reads = synth.preprocess_order([b"ACGTA", b"ACGTC", b"GGGGGG", b"ACGTACGTAA"] + _reads(40, 11))
    _check(engine, reads, 6, 1.0, cg.MODE_BATCHED)
    # K = 8: reads of 7 (no tuple, H key "none") and 8 (one tuple) nt
    reads8 = synth.preprocess_order([b"ACGTACG", b"CCCCCCC", b"TTTTTTTT", b"ACGTACGTA"] + _reads(40, 12, k=8))
    for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN):
        _check(engine, reads8, 8, 1.0, mode)


def test_kmer_long_reads(engine):
    reads = _reads(150, 21, root=2100, dist="uniform", a=1500, b=2048, cents=6)
    _check(engine, reads, 6, 0.5, cg.MODE_BATCHED)
    # K = 8 counts of 11 bits: the two-phase kernel's 16-warp form
    assert _check(engine, reads, 8, 0.7, cg.MODE_BATCHED) == _check(engine, reads, 8, 0.7, cg.MODE_STAGED)


def test_kmer_uneven_lengths(engine):
    reads = _reads(3000, 31, root=520, dist="uniform", a=300, b=500, cents=60)
    t = cg.default_threshold(len(reads), -1.0, 0)
    a = _check(engine, reads, 6, t, cg.MODE_BATCHED)
    b = _check(engine, reads, 6, t, cg.MODE_PLAIN)
    c = _check(engine, reads, 6, t, cg.MODE_STAGED)
    assert a == b == c
    # the batched form again: its launch sequences replay as CUDA graphs
    assert _check(engine, reads, 6, t, cg.MODE_BATCHED) == a
    assert engine.stats()["graph_launches"] > 0


def test_kmer_nonacgt(engine):
    reads = _reads(100, 41)
    mixed = []
    for i, s in enumerate(reads):
        s = bytearray(s)
        s[5 + i % 50] = ord("N")
        s[80 + i % 20] = ord("a")
        mixed.append(bytes(s))
    _check(engine, synth.preprocess_order(mixed), 6, 0.4, cg.MODE_BATCHED)


def test_kmer_k8_quirk_tiles(engine):
    # K = 8 runs the 16-row tile kernel in the batched and staged forms: H / L
    # halves of the signed-sort quirk, reads without H K-mers (only A/G, so
    # [same] holds between two of them), repeated K-mers through the hash,
    # uneven lengths across group edges
    rng = np.random.default_rng(88)
    base = _reads(900, 808, root=520, dist="uniform", a=200, b=500, cents=30, k=8)
    ag = [bytes(rng.choice(np.frombuffer(b"AG", np.uint8), 150 + (i % 40)).astype(np.uint8).tobytes())
          for i in range(40)]
    rep = []
    for i in range(40):
        s = bytearray(base[i])
        s[20:20 + 30 + i] = b"C" * (30 + i)
        rep.append(bytes(s))
    reads = synth.preprocess_order(base[40:] + ag + rep)
    t = cg.default_threshold(len(reads), -1.0, 0)
    counts = [_check(engine, reads, 8, thr, mode)
              for thr in (t, 0.7) for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN)]
    assert counts[0] == counts[1] == counts[2] and counts[3] == counts[4] == counts[5] > 0


@pytest.mark.parametrize("kind", ["no_h", "one_key", "random"])
def test_kmer_k8_key_groups(engine, kind):
    # K = 8 orders the reads by H key and splits the batched form into the
    # H-only kernel (pairs of different keys) and the 16-row kernel over each
    # row block's same-key range; these sets put every read in one key group
    # (no H K-mer at all, or the same largest H K-mer once) or give mostly
    # distinct keys
    rng = np.random.default_rng({"no_h": 81, "one_key": 82, "random": 83}[kind])
    reads = []
    for i in range(520):
        L = int(rng.integers(120, 300))
        if kind == "no_h":       # A and G only: every K-mer is below 0x8000
            s = rng.choice(np.frombuffer(b"AG", np.uint8), L).tobytes()
        elif kind == "one_key":  # CCCCCCCC (0xFFFF, the largest K-mer) once, elsewhere no C
            s = bytearray(rng.choice(np.frombuffer(b"AGT", np.uint8), L).tobytes())
            p = int(rng.integers(0, L - 8))
            s[p:p + 8] = b"CCCCCCCC"
            s = bytes(s)
        else:
            s = rng.choice(np.frombuffer(b"ACGT", np.uint8), L).tobytes()
        reads.append(s)
    # a few near-copies so that pairs pass the threshold
    reads += [bytes(r[:-3]) + b"AAA" for r in reads[:60]]
    reads = synth.preprocess_order(reads)
    counts = [_check(engine, reads, 8, thr, mode) for thr in (0.75, 0.3)
              for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN)]
    assert counts[0] == counts[1] == counts[2] > 0


@pytest.mark.parametrize("n", [10, 37, 99, 150])
def test_kmer_k8_small_sets(engine, n):
    # stage tiles (arrayDim 4 and 32) narrower than the K = 8 kernels' 32-row
    # blocks, partial row and column groups, every form
    reads = _reads(n + n // 10 + 5, 300 + n, k=8)[:n]
    t = cg.default_threshold(len(reads), -1.0, 0)
    counts = [_check(engine, reads, 8, thr, mode) for thr in (t, 0.75)
              for mode in (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN)]
    assert counts[0] == counts[1] == counts[2] and counts[3] == counts[4] == counts[5]


def test_kmer_k8_one_kernel_form(engine, monkeypatch):
    # the batched K = 8 form without the split (the two-phase kernel over
    # every column, as when the H keys are not in order) gives the same
    # survivors as the split form and the oracle
    reads = _reads(700, 812, root=520, dist="uniform", a=200, b=480, cents=25, k=8)
    t = cg.default_threshold(len(reads), -1.0, 0)
    split = _check(engine, reads, 8, t, cg.MODE_BATCHED)
    monkeypatch.setenv("CRISPY_KMER_K8_SPLIT", "0")
    assert _check(engine, reads, 8, t, cg.MODE_BATCHED) == split
