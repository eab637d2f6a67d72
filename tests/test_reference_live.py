"""Live comparison with the reference's CPU code where it can be built.

Runs only where the reference tree exists (never on the GPU machine): the
reference's kmerDist/genDist CPU path is compiled from its own sources into
oracle/_ref/ and run on the reference's sample FASTA and on fresh synthetic
sets; the oracle must agree with it exactly.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from crispy_gb300 import synth

REF = os.environ.get("CRISPY_REFERENCE", "/root/reference")
HAVE_REF = os.path.isdir(os.path.join(REF, "src", "kmerDist"))
pytestmark = pytest.mark.skipif(not HAVE_REF, reason="reference tree not present")


@pytest.fixture(scope="module")
def refbin():
    subprocess.run(["make", "-s", "-C", oracle.HERE, "ref", f"REF={REF}"], check=True)
    return oracle.REF_DIR


def _ref_kmer(refbin, d, name, k, thr):
    cmd = [os.path.join(refbin, "kmerDist"), "-i", name, "-k", str(k), "-c", "-n", "1", "-d"]
    if thr is not None:
        cmd += ["-t", str(thr)]
    subprocess.run(cmd, cwd=d, check=True, stdout=subprocess.DEVNULL)
    p = np.fromfile(os.path.join(d, name + ".kpair"), np.int32).reshape(-1, 2)
    q = np.fromfile(os.path.join(d, name + ".kdist"), np.float32)
    return p, q


def _prep(tmp_path, reads, name="setx"):
    d = str(tmp_path)
    with open(os.path.join(d, name), "wb") as f:
        for i, s in enumerate(reads):
            f.write(b">r%d\n%s\n" % (i, s))
    subprocess.run([os.path.join(oracle.REF_DIR, "preprocess"), "-i", name], cwd=d,
                   stdout=subprocess.DEVNULL)
    return d, name + "_Clean"


def test_sample_fasta(refbin, tmp_path):
    src = os.path.join(REF, "data", "V2Mice_sample1000")
    if not os.path.exists(src):
        pytest.skip("sample data absent")
    d = str(tmp_path)
    shutil.copy(src, os.path.join(d, "sample"))
    subprocess.run([os.path.join(refbin, "preprocess"), "-i", "sample"], cwd=d, stdout=subprocess.DEVNULL)
    name = "sample_Clean"
    rp, rd = _ref_kmer(refbin, d, name, 6, None)
    buf, offs, lens = oracle.read_fasta(os.path.join(d, name), 0)
    assert len(lens) == 585 and len(rp) == 8404
    thr = oracle.default_threshold(len(lens), -1.0, 2)
    op, od = oracle.kmer_all(buf, offs, lens, 6, thr)
    o = np.lexsort((op[:, 1], op[:, 0]))
    assert np.array_equal(op[o], rp) and np.array_equal(od[o].view(np.uint32), rd.view(np.uint32))
    for band in (10, 2, 1):
        for f in os.listdir(d):
            if ".npair_" in f or ".ndist_" in f:
                os.remove(os.path.join(d, f))
        subprocess.run([os.path.join(refbin, "genDist"), "-i", name, "-b", str(band), "-c", "-n", "1"],
                       cwd=d, check=True, stdout=subprocess.DEVNULL)
        gbuf, goffs, glens = oracle.read_fasta(os.path.join(d, name), 1)
        dist, _, _, _ = oracle.gen_all(gbuf, goffs, glens, rp, band)
        ch = oracle.gen_chunks(rp, dist, oracle.default_threshold(len(glens), -1.0, 1))
        gp = np.fromfile(os.path.join(d, name + ".npair_0"), np.uint32).reshape(-1, 2)
        gd = np.fromfile(os.path.join(d, name + ".ndist_0"), np.float32)
        assert np.array_equal(ch[0][1], gp) and np.array_equal(ch[0][2].view(np.uint32), gd.view(np.uint32))


@pytest.mark.parametrize("k", [1, 2, 3, 5, 7, 8])
def test_kmer_all_k(refbin, tmp_path, k):
    reads = synth.generate(synth.ReadSetSpec(160, 8, 260, "normal", 250, 15, k, 300 + k))
    d, name = _prep(tmp_path, reads)
    thr = {1: 0.05, 2: 0.1, 3: 0.15}.get(k, 0.5)
    rp, rd = _ref_kmer(refbin, d, name, k, thr)
    buf, offs, lens = oracle.read_fasta(os.path.join(d, name), 0)
    op, od = oracle.kmer_all(buf, offs, lens, k, thr)
    o = np.lexsort((op[:, 1], op[:, 0]))
    assert np.array_equal(op[o], rp) and np.array_equal(od[o].view(np.uint32), rd.view(np.uint32))


def test_fasta_quirks(refbin, tmp_path):
    # blank lines inside a record, CRLF, lowercase, N runs, long wrapped lines,
    # trailing non-ACGT characters; parsed by the reference stages themselves
    d = str(tmp_path)
    rng = np.random.default_rng(5)
    recs = []
    for i in range(60):
        s = rng.choice(np.frombuffer(b"ACGT", np.uint8), 240).tobytes()
        if i % 5 == 0:
            s = s[:50] + b"NNNN" + s[54:]
        if i % 7 == 0:
            s = s[:100] + s[100:140].lower() + s[140:]
        recs.append(s)
    with open(os.path.join(d, "quirk"), "wb") as f:
        for i, s in enumerate(recs):
            nl = b"\r\n" if i % 3 == 0 else b"\n"
            f.write(b">q%d some description" % i + nl)
            if i % 4 == 0:
                f.write(s[:120] + nl + nl + s[120:] + b"NN-" + nl)
            else:
                f.write(s + nl)
    name = "quirk"
    rp, rd = _ref_kmer(refbin, d, name, 6, 0.9)
    buf, offs, lens = oracle.read_fasta(os.path.join(d, name), 0)
    op, od = oracle.kmer_all(buf, offs, lens, 6, 0.9)
    o = np.lexsort((op[:, 1], op[:, 0]))
    assert np.array_equal(op[o], rp) and np.array_equal(od[o].view(np.uint32), rd.view(np.uint32))
    subprocess.run([os.path.join(refbin, "genDist"), "-i", name, "-b", "10", "-c", "-n", "1", "-t", "0.9"],
                   cwd=d, check=True, stdout=subprocess.DEVNULL)
    gbuf, goffs, glens = oracle.read_fasta(os.path.join(d, name), 1)
    dist, _, _, _ = oracle.gen_all(gbuf, goffs, glens, rp, 10)
    ch = oracle.gen_chunks(rp, dist, 0.9)
    gp = np.fromfile(os.path.join(d, name + ".npair_0"), np.uint32).reshape(-1, 2)
    gd = np.fromfile(os.path.join(d, name + ".ndist_0"), np.float32)
    # the CPU path compares raw characters where the GPU path compares 2-bit
    # codes: with N / lowercase present the two reference paths can differ,
    # so only the pairs whose reads are plain ACGT are compared here
    plain = np.array([all(c in b"ACGT" for c in gbuf[goffs[r]:goffs[r] + glens[r]].tobytes())
                      for r in range(len(glens))])
    want = {(int(a), int(b)): float(x) for (a, b), x in zip(gp, gd) if plain[a] and plain[b]}
    got = {(int(a), int(b)): float(x) for (a, b), x in zip(ch[0][1], ch[0][2]) if plain[a] and plain[b]}
    assert want == got


def _raw_set(path, seed, n, dup_frac=0.3, noise=True):
    """A raw FASTA with planted duplicates, N's, lower case and wrapped lines."""
    reads = synth.generate(synth.ReadSetSpec(n, max(4, n // 60), 260, "normal", 200, 12, 6, seed))
    rng = np.random.default_rng(seed)
    reads = reads + [reads[i] for i in rng.integers(0, len(reads), size=int(n * dup_frac))]
    reads = [bytearray(reads[i]) for i in rng.permutation(len(reads))]
    if noise:
        for r in reads:
            u = rng.random()
            if u < 0.03:
                r[rng.integers(0, len(r))] = ord("N")
            elif u < 0.05:
                a = rng.integers(0, len(r))
                r[a:a + 4] = r[a:a + 4].lower()
    with open(path, "wb") as f:
        for i, s in enumerate(reads):
            f.write(b">r%d desc %d\n" % (i, i % 13))
            for a in range(0, len(s), 70):
                f.write(bytes(s[a:a + 70]) + b"\n")
    return bytes(reads[0][:22]).upper()


@pytest.mark.parametrize("seed,n,args", [
    (41, 3000, []),
    (42, 3000, ["-s", "1.0"]),
    (43, 2000, ["-s", "1.5", "-m", "3", "-p"]),
    (44, 2000, ["-m", "1", "-p"]),
])
def test_preprocess_oracle_vs_reference(refbin, tmp_path, seed, n, args):
    d = str(tmp_path)
    primer = _raw_set(os.path.join(d, "raw.fa"), seed, n)
    argv = list(args)
    if argv and argv[-1] == "-p":
        with open(os.path.join(d, "primer.txt"), "wb") as f:
            f.write(primer + b"\n")
        argv.append("primer.txt")
    p = subprocess.run([os.path.join(refbin, "preprocess"), "-i", "raw.fa"] + argv, cwd=d,
                       stdout=subprocess.PIPE)
    assert p.returncode == 1
    sd = float(argv[argv.index("-s") + 1]) if "-s" in argv else None
    mm = int(argv[argv.index("-m") + 1]) if "-m" in argv else 2
    oracle.preprocess(os.path.join(d, "raw.fa"), os.path.join(d, "oracle_out"), sd=sd,
                      primer=primer if "-p" in argv else None, max_mm=mm)
    for ext in ("", ".frq"):
        assert open(os.path.join(d, "oracle_out" + ext), "rb").read() == \
            open(os.path.join(d, "raw.fa_Clean" + ext), "rb").read()
