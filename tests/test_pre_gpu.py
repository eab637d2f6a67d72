"""Preprocess on the GPU against the reference fixtures and the oracle.

* The drop-in `preprocess` executable reproduces every fixture of
  tests/golden/pre/ byte for byte (both output files), with the reference's
  "Total numReads" line and exit status 1.
* crispy_preprocess (through Engine.preprocess) gives the oracle's files on
  seeded sets with planted duplicates at sizes around the sort's tile
  boundaries and with each option (-s, -p, -m), and on degenerate sets.
"""
import json
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle
from crispy_gb300 import synth

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pre")
MANIFEST = json.load(open(os.path.join(GOLD, "MANIFEST.json")))
EXE = os.path.join(cg.BIN_DIR, "preprocess")


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_cli_matches_reference_fixture(tmp_path, name):
    case = MANIFEST[name]
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLD, name), d)
    want = {e: open(str(d / case["output"]) + e, "rb").read() for e in ("", ".frq")}
    for e in ("", ".frq"):
        os.remove(str(d / case["output"]) + e)
    p = subprocess.run([EXE] + case["args"], cwd=d, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    assert p.returncode == 1, p.stdout
    m = re.search(rb"Total numReads: (-?\d+)\. Preprocessed numReads: (-?\d+)", p.stdout)
    assert m and (int(m.group(1)), int(m.group(2))) == (case["total"], case["preprocessed"])
    for e in ("", ".frq"):
        assert open(str(d / case["output"]) + e, "rb").read() == want[e]


def _raw(path, seed, n, dup_frac=0.3, lo=200, sd=12, root=260, noise=True):
    reads = synth.generate(synth.ReadSetSpec(n, max(4, n // 60), root, "normal", lo, sd, 6, seed))
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


def _engine_vs_oracle(engine, d, name, sd=None, primer=None, max_mm=2):
    raw = cg.RawReads(os.path.join(d, name))
    idx, freq, st = engine.preprocess(raw, sd=sd, primer=primer, max_mm=max_mm)
    raw.write(idx, freq, os.path.join(d, "gpu_out"))
    c = oracle.preprocess(os.path.join(d, name), os.path.join(d, "oracle_out"), sd=sd, primer=primer,
                          max_mm=max_mm)
    for e in ("", ".frq"):
        assert open(os.path.join(d, "gpu_out" + e), "rb").read() == \
            open(os.path.join(d, "oracle_out" + e), "rb").read()
    assert (st["length_discards"], st["primer_discards"], st["merges"], st["kept"]) == \
        (c["length_discards"], c["primer_discards"], c["merges"], c["kept"])
    assert raw.records == c["records"]
    return st


# sizes around the 2048-read bitonic tiles and the merge passes
@pytest.mark.parametrize("n", [1, 2, 3, 100, 1500, 1600, 3100, 7000, 20000])
def test_engine_merge_sizes(engine, tmp_path, n):
    d = str(tmp_path)
    _raw(os.path.join(d, "raw.fa"), 500 + n, n)
    _engine_vs_oracle(engine, d, "raw.fa")


@pytest.mark.parametrize("sd", [1.0, 0.25, 3.0, -1.0])
def test_engine_length_filter(engine, tmp_path, sd):
    d = str(tmp_path)
    _raw(os.path.join(d, "raw.fa"), 71, 4000)
    st = _engine_vs_oracle(engine, d, "raw.fa", sd=sd)
    assert st["length_reads"] > 0


@pytest.mark.parametrize("mm", [0, 1, 2, 4])
def test_engine_primer(engine, tmp_path, mm):
    d = str(tmp_path)
    primer = _raw(os.path.join(d, "raw.fa"), 90 + mm, 3000)
    _engine_vs_oracle(engine, d, "raw.fa", primer=primer, max_mm=mm)
    _engine_vs_oracle(engine, d, "raw.fa", sd=1.0, primer=primer[:12], max_mm=mm)


def test_engine_long_reads_and_heavy_duplicates(engine, tmp_path):
    # 2,000-base reads (125 words per comparison), 80 % duplicates
    d = str(tmp_path)
    _raw(os.path.join(d, "raw.fa"), 17, 1500, dup_frac=4.0, lo=1800, sd=100, root=2100, noise=False)
    _engine_vs_oracle(engine, d, "raw.fa")


def test_engine_all_identical(engine, tmp_path):
    d = str(tmp_path)
    with open(os.path.join(d, "raw.fa"), "wb") as f:
        for i in range(5000):
            f.write(b">same%d\nACGTACGTTTGACCA\n" % i)
    st = _engine_vs_oracle(engine, d, "raw.fa")
    assert st["kept"] == 1 and st["merges"] == 4999


def test_engine_nothing_left(engine, tmp_path):
    d = str(tmp_path)
    with open(os.path.join(d, "raw.fa"), "wb") as f:
        for i in range(50):
            f.write(b">n%d\nACGNACGT%s\n" % (i, b"A" * i))
    st = _engine_vs_oracle(engine, d, "raw.fa", sd=1.0)
    assert st["kept"] == 0


def test_engine_primer_limit(engine, tmp_path):
    d = str(tmp_path)
    _raw(os.path.join(d, "raw.fa"), 3, 50)
    raw = cg.RawReads(os.path.join(d, "raw.fa"))
    with pytest.raises(cg.CrispyError) as e:
        engine.preprocess(raw, primer=b"A" * 257)
    assert e.value.code == cg.E_UNSUPPORTED
    # the context stays usable
    _engine_vs_oracle(engine, d, "raw.fa", primer=b"A" * 256)


def _run(cmd, cwd, ok=(0,)):
    p = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    assert p.returncode in ok, p.stdout
    return p.stdout


def _four_programs(d, name, k, band, cut=None):
    """crispy.sh:18-24 with the drop-in executables."""
    clean = name + "_Clean"
    _run([EXE, "-i", name], d, ok=(1,))
    _run([os.path.join(cg.BIN_DIR, "kmerDist"), "-i", clean, "-k", str(k)], d)
    _run([os.path.join(cg.BIN_DIR, "genDist"), "-i", clean, "-b", str(band)], d)
    num_reads = sum(1 for line in open(os.path.join(d, clean), "rb") if b">" in line)
    num_files = sum(1 for f in os.listdir(d) if f.startswith(clean + ".ndist"))
    _run([os.path.join(cg.BIN_DIR, "aveclust"), "-i", clean, "-n", str(num_reads), "-f", str(num_files)], d)
    if cut:
        _run([os.path.join(cg.BIN_DIR, "sparsecut"), "-i", clean, "-n", str(num_reads), "-c", cut], d)


def _outputs(d):
    return {f: open(os.path.join(d, f), "rb").read() for f in sorted(os.listdir(d))
            if "_Clean" in f}


def _whitespace_set(path):
    # a blank line and a run of spaces inside records: the kept reads then
    # hold whitespace and the stages have to read the _Clean file
    with open(path, "wb") as f:
        rng = np.random.default_rng(8)
        base = rng.choice(np.frombuffer(b"ACGT", np.uint8), size=300).tobytes()
        for i in range(40):
            s = bytearray(base)
            for p in rng.integers(0, 300, size=12):
                s[p] = ord("ACGT"[rng.integers(0, 4)])
            f.write(b">w%d\n%s\n" % (i, bytes(s[:150])))
            if i % 9 == 0:
                f.write(b"\n")
            elif i % 11 == 0:
                f.write(b"   \n")
            f.write(bytes(s[150:]) + (b"NN\n" if i % 4 == 0 else b"\n"))


@pytest.mark.parametrize("case,k,band", [
    ("dups", 6, 10), ("dups", 8, 5), ("uneven", 6, 10), ("trailing_n", 7, 2), ("whitespace", 6, 10)])
def test_crispyrun_matches_four_programs(tmp_path, case, k, band):
    a, b = tmp_path / "three", tmp_path / "one"
    a.mkdir()
    b.mkdir()
    raw = os.path.join(str(a), "raw.fa")
    if case == "dups":
        _raw(raw, 61, 3000)
    elif case == "uneven":
        _raw(raw, 62, 4000, lo=400, sd=50, root=520)
    elif case == "trailing_n":
        _raw(raw, 63, 2000)
        data = open(raw, "rb").read().replace(b"\n>", b"NNn\n>")   # trailing N's on most reads
        open(raw, "wb").write(data)
    else:
        _whitespace_set(raw)
    shutil.copy(raw, os.path.join(str(b), "raw.fa"))
    # with a cutoff file (the changepoint step's output) the sparsecut step
    # runs too, and rewrites .Cluster / .Cluster_List at those cutoffs
    cut = None
    if case in ("dups", "uneven") and k == 6:
        cut = "cut.txt"
        for d in (a, b):
            open(os.path.join(str(d), cut), "w").write("0.01\n0.02\n0.03\n0.05\n")
    _four_programs(str(a), "raw.fa", k, band, cut)
    out = _run([os.path.join(cg.BIN_DIR, "crispyRun"), "raw.fa", str(k), str(band)] + ([cut] if cut else []),
               str(b))
    assert b"totalNumPairs" in out
    if cut:
        assert b"sparsecut: 4 cutoffs" in out
        assert open(os.path.join(str(b), "raw.fa_Clean.Cluster_List")).read().startswith(" 0.010000 ")
    want, got = _outputs(str(a)), _outputs(str(b))
    assert sorted(want) == sorted(got)
    assert any(".npair_" in f for f in got) and "raw.fa_Clean_Merge" in got
    for f in want:
        assert got[f] == want[f], f


def test_prepare_from_pre_matches_file(engine, tmp_path):
    d = str(tmp_path)
    _raw(os.path.join(d, "raw.fa"), 64, 2500)
    raw = cg.RawReads(os.path.join(d, "raw.fa"))
    idx, freq, st = engine.preprocess(raw)
    raw.write(idx, freq, os.path.join(d, "raw.fa_Clean"))
    engine.kmer_prepare_from_pre(raw, 6)
    thr = cg.default_threshold(st["kept"], -1.0, 0)
    n1 = engine.kmer_run(thr)
    p1, d1 = engine.kmer_fetch(n1)
    engine.gen_prepare_from_pre(raw)
    a1 = engine.gen_align(p1[:5000], 10)
    kb, ko, kl = cg.read_fasta(os.path.join(d, "raw.fa_Clean"), 0)
    engine.kmer_prepare(kb, ko, kl, 6)
    n2 = engine.kmer_run(thr)
    p2, d2 = engine.kmer_fetch(n2)
    assert n1 == n2 and np.array_equal(p1, p2) and np.array_equal(d1.view(np.uint32), d2.view(np.uint32))
    gb, go, gl = cg.read_fasta(os.path.join(d, "raw.fa_Clean"), 1)
    engine.gen_prepare(gb, go, gl)
    a2 = engine.gen_align(p2[:5000], 10)
    for x, y in zip(a1, a2):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))


def test_prepare_from_pre_declines_whitespace(engine, tmp_path):
    d = str(tmp_path)
    _whitespace_set(os.path.join(d, "raw.fa"))
    raw = cg.RawReads(os.path.join(d, "raw.fa"))
    engine.preprocess(raw)
    with pytest.raises(cg.CrispyError) as e:
        engine.kmer_prepare_from_pre(raw, 6)
    assert e.value.code == cg.E_UNSUPPORTED
    other = cg.RawReads(os.path.join(GOLD, "dollar", "dollar.fa"))
    with pytest.raises(cg.CrispyError) as e:
        engine.gen_prepare_from_pre(other)
    assert e.value.code == cg.E_INPUT
