"""The oracle against the reference's own outputs (committed golden files).

The golden files were produced by the reference's CPU code compiled from
source (tests/golden/make_golden.py).  Its kmerDist CPU path writes pairs in
(row, col) order with one thread; the GPU path the oracle restates writes
them in stage order, so the k-mer check compares the oracle's survivors
re-sorted by (row, col).  genDist goldens came from the same .kpair input,
so the oracle's chunk files must match byte for byte.
"""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(GOLD, "MANIFEST.json")))


def _cases(kind):
    for name, s in MANIFEST["sets"].items():
        for run in s[kind]:
            yield name, run


def test_manifest_hashes():
    import hashlib

    for name, s in MANIFEST["sets"].items():
        for f, h in s["files"].items():
            data = open(os.path.join(GOLD, name, f), "rb").read()
            assert hashlib.sha256(data).hexdigest() == h, f


@pytest.mark.parametrize("name,run", list(_cases("kmer")), ids=lambda x: str(x) if isinstance(x, str) else x["tag"])
def test_oracle_kmer_matches_reference(name, run):
    fa = os.path.join(GOLD, name, name + "_Clean")
    buf, offs, lens = oracle.read_fasta(fa, 0)
    thr = oracle.default_threshold(len(lens), -1.0 if run["thr"] is None else run["thr"], 2)
    pairs, dists = oracle.kmer_all(buf, offs, lens, run["k"], thr)
    gp = np.fromfile(f"{fa}.{run['tag']}.kpair", np.int32).reshape(-1, 2)
    gd = np.fromfile(f"{fa}.{run['tag']}.kdist", np.float32)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    assert np.array_equal(pairs[order], gp)
    assert np.array_equal(dists[order].view(np.uint32), gd.view(np.uint32))


@pytest.mark.parametrize("name,run", list(_cases("gen")), ids=lambda x: str(x) if isinstance(x, str) else x["tag"])
def test_oracle_gen_matches_reference(name, run):
    fa = os.path.join(GOLD, name, name + "_Clean")
    buf, offs, lens = oracle.read_fasta(fa, 1)
    pairs = np.fromfile(f"{fa}.{run['kpair']}.kpair", np.int32).reshape(-1, 2)
    thr = oracle.default_threshold(len(lens), -1.0 if run["thr"] is None else run["thr"], 1)
    d, _, _, _ = oracle.gen_all(buf, offs, lens, pairs, run["band"])
    chunks = oracle.gen_chunks(pairs, d, thr)
    c = 0
    while os.path.exists(f"{fa}.{run['tag']}.npair_{c}"):
        gp = np.fromfile(f"{fa}.{run['tag']}.npair_{c}", np.uint32).reshape(-1, 2)
        gd = np.fromfile(f"{fa}.{run['tag']}.ndist_{c}", np.float32)
        assert np.array_equal(chunks[c][1], gp)
        assert np.array_equal(chunks[c][2].view(np.uint32), gd.view(np.uint32))
        c += 1
    assert c == len(chunks) and c > 0


def test_oracle_kmer_quirk_k8():
    # K = 8: tuples >= 0x8000 sort first (signed compare) while the merge
    # compares unsigned; the count is then not the multiset min-sum.
    a = b"TTTTTTTTACGTACGTA"   # holds 8-mers >= 0x8000 (T = 2 -> high bits 10)
    b = b"TTTTTTTTACGTACGTT"
    m = oracle.kmer_matches(a, b, 8)
    assert 0 <= m <= min(len(a), len(b)) - 7
