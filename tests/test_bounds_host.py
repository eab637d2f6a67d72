"""The count bounds the k-mer tile kernels skip work on, checked on the CPU.

Every pair is counted exactly by the reference's rule (m = sum of minima of
the K-mer counts; at K = 8 the signed-sort quirk m = minsum(H) + [same] *
minsum(L), kmerMain.cpp:275-278 against kmerKernel.cu:37-45).  The kernels
may skip a pair only when a bound proves it cannot pass the cut
(dist < thr or |dist - thr| < 1e-5, kmerMain.cpp:180).  These tests compute
the bounds the kernels use from the same level entries and check, for all
pairs of small seeded read sets, that no pair that passes would be skipped:

* K <= 6 bound pass: with section 0 the level entries whose word index
  hashes below the split, m <= m0 + Ta - a0, and a pair with Tb >= Ta passes
  only if m0 >= mmin[Ta] - Ta + a0;
* K = 8, pairs without [same]: m = minsum(H) <= min(|H_a|, |H_b|), so the
  shorter read of a passing pair is H-heavy (|H| >= mmin[T]);
* K = 8, pairs with [same]: m <= mH + |L_a|, so with Tb >= Ta a passing pair
  has mH >= mmin[Ta] - |L_a|.
"""
import numpy as np
import pytest

from crispy_gb300 import synth

CODE = np.zeros(256, np.int64)
CODE[ord("G")], CODE[ord("T")], CODE[ord("C")] = 1, 2, 3


def _kmers(read: bytes, k: int) -> np.ndarray:
    s = CODE[np.frombuffer(read, np.uint8)]
    km = np.zeros(len(s) - k + 1, np.int64)
    for q in range(k):
        km = km * 4 + s[q:len(s) - k + 1 + q]
    return km


def _mmin_table(thr: float, max_t: int) -> np.ndarray:
    """Smallest passing m for each min(Ta, Tb), in the reference's types."""
    thr32 = np.float32(thr)
    out = np.full(max_t + 1, 1 << 30, np.int64)
    for t in range(1, max_t + 1):
        m = np.arange(t + 1)
        d = np.float32(1.0) - m.astype(np.float32) / np.float32(t)
        ok = (d < thr32) | (np.abs((d - thr32).astype(np.float32)).astype(np.float64) < 1e-5)
        if ok.any():
            out[t] = int(np.argmax(ok))
    return out


def _section0(words: np.ndarray, split: int) -> np.ndarray:
    h = (((words >> 3).astype(np.uint64) * np.uint64(0x9E3779B1)) & np.uint64(0xFFFFFFFF)) >> np.uint64(24)
    return h < split


def test_bound_pass_never_skips_a_passing_pair():
    k, k4 = 6, 4096
    reads = synth.make_read_set(synth.ReadSetSpec(260, 5, 520, "uniform", 300, 500, k, 71))
    counts = np.stack([np.bincount(_kmers(r, k), minlength=k4) for r in reads])
    n = len(reads)
    t = counts.sum(1)
    splits, thrs = (64, 112, 160), (0.05, 0.12, 0.3)
    mmins = {thr: _mmin_table(thr, int(t.max())) for thr in thrs}
    # dense level entries 1..2 (level t of K-mer v: word (t-1) * 4^K + v)
    s0 = {sp: _section0(np.arange(2 * k4), sp).reshape(2, k4) for sp in splits}
    a0 = {sp: ((counts >= 1) & s0[sp][0]).sum(1) + ((counts >= 2) & s0[sp][1]).sum(1) for sp in splits}
    passing = {thr: 0 for thr in thrs}
    for a in range(n - 1):
        mn = np.minimum(counts[a][None, :], counts[a + 1:])
        m = mn.sum(1)
        lv1, lv2 = mn >= 1, mn >= 2
        tb = t[a + 1:]
        for sp in splits:
            m0 = (lv1 & s0[sp][0]).sum(1) + (lv2 & s0[sp][1]).sum(1)
            assert np.all(m <= m0 + t[a] - a0[sp][a])
            for thr in thrs:
                mmin = mmins[thr]
                passes = m >= mmin[np.minimum(t[a], tb)]
                keep = (m0 >= mmin[t[a]] - t[a] + a0[sp][a]) | (tb < t[a])
                assert not np.any(passes & ~keep)
                passing[thr] += int(passes.sum())
    assert all(v > 0 for v in passing.values())


def _k8_parts(read: bytes):
    km = _kmers(read, 8)
    cnt = np.bincount(km, minlength=65536)
    h = cnt[0x8000:]
    hv = np.nonzero(h)[0]
    key = (int(hv.max()) + 0x8000, int(h[hv.max()])) if len(hv) else None
    return cnt, len(km), key


def test_k8_bounds_never_skip_a_passing_pair():
    reads = synth.make_read_set(synth.ReadSetSpec(240, 4, 260, "normal", 250, 30, 8, 72))
    rng = np.random.default_rng(72)
    # reads rich in T and C: H-heavy at any threshold
    reads += [rng.choice(np.frombuffer(b"TCTCTCTCAG", np.uint8), size=250).tobytes() for _ in range(8)]
    parts = [_k8_parts(r) for r in reads]
    cnt = np.stack([p[0] for p in parts])
    t = np.array([p[1] for p in parts])
    keys = [p[2] for p in parts]
    n = len(reads)
    thrs = (0.105, 0.3, 0.5, 0.55)
    mmins = {thr: _mmin_table(thr, int(t.max())) for thr in thrs}
    nh = cnt[:, 0x8000:].sum(1)
    nl = cnt[:, :0x8000].sum(1)
    passing = {thr: 0 for thr in thrs}
    for a in range(n - 1):
        bs = np.arange(a + 1, n)
        mh = np.minimum(cnt[a, 0x8000:][None, :], cnt[bs, 0x8000:]).sum(1)
        ml_all = np.minimum(cnt[a, :0x8000][None, :], cnt[bs, :0x8000]).sum(1)
        same = np.array([keys[a] == keys[b] for b in bs])
        m = mh + np.where(same, ml_all, 0)
        row = np.where(t[a] <= t[bs], a, bs)   # the shorter read
        for thr in thrs:
            mmin = mmins[thr]
            heavy = nh >= mmin[t]
            passes = m >= mmin[np.minimum(t[a], t[bs])]
            passing[thr] += int(passes.sum())
            # the count bound of the pairs without [same]
            assert np.all(~passes | same | heavy[a] | heavy[bs])
            # the bound after the H sums
            assert np.all(~(passes & same) | (mh >= mmin[t[row]] - nl[row]))
    assert all(v > 0 for v in passing.values())
