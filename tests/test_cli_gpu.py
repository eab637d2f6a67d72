"""The drop-in executables (crispy_gb300/bin/kmerDist, genDist) against the
golden files the reference wrote, byte for byte.

genDist is fed the reference's own .kpair, so its .npair_N/.ndist_N must be
identical to the reference's.  kmerDist writes the GPU path's stage order,
checked byte-exact against the oracle and as a set against the reference's
CPU-order file.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(GOLD, "MANIFEST.json")))
BIN = cg.BIN_DIR


def _cases(kind):
    for name, s in MANIFEST["sets"].items():
        for run in s[kind]:
            for mode in ("batched", "staged", "plain"):
                yield name, run, mode


def _env(mode):
    e = dict(os.environ)
    e["CRISPY_MODE"] = mode
    return e


@pytest.mark.parametrize("name,run,mode", list(_cases("kmer")),
                         ids=lambda x: x if isinstance(x, str) else x["tag"])
def test_kmerdist_cli(tmp_path, name, run, mode):
    src = os.path.join(GOLD, name, name + "_Clean")
    fa = str(tmp_path / (name + "_Clean"))
    shutil.copy(src, fa)
    cmd = [os.path.join(BIN, "kmerDist"), "-i", fa, "-k", str(run["k"]), "-d"]
    if run["thr"] is not None:
        cmd += ["-t", str(run["thr"])]
    r = subprocess.run(cmd, env=_env(mode), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    got_p = np.fromfile(fa + ".kpair", np.int32).reshape(-1, 2)
    got_d = np.fromfile(fa + ".kdist", np.float32)
    buf, offs, lens = oracle.read_fasta(fa, 0)
    thr = oracle.default_threshold(len(lens), -1.0 if run["thr"] is None else run["thr"], 2)
    op, od = oracle.kmer_all(buf, offs, lens, run["k"], thr)
    assert np.array_equal(got_p, op) and np.array_equal(got_d.view(np.uint32), od.view(np.uint32))
    gp = np.fromfile(f"{src}.{run['tag']}.kpair", np.int32).reshape(-1, 2)
    o = np.lexsort((got_p[:, 1], got_p[:, 0]))
    assert np.array_equal(got_p[o], gp)
    assert f"totalNumPairs: {len(gp)}" in r.stdout


@pytest.mark.parametrize("name,run,mode", list(_cases("gen")),
                         ids=lambda x: x if isinstance(x, str) else x["tag"])
def test_gendist_cli(tmp_path, name, run, mode):
    src = os.path.join(GOLD, name, name + "_Clean")
    fa = str(tmp_path / (name + "_Clean"))
    shutil.copy(src, fa)
    shutil.copy(f"{src}.{run['kpair']}.kpair", fa + ".kpair")
    cmd = [os.path.join(BIN, "genDist"), "-i", fa, "-b", str(run["band"])]
    if run["thr"] is not None:
        cmd += ["-t", str(run["thr"])]
    r = subprocess.run(cmd, env=_env(mode), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    c = 0
    total = 0
    while os.path.exists(f"{src}.{run['tag']}.npair_{c}"):
        for ext in ("npair", "ndist"):
            want = open(f"{src}.{run['tag']}.{ext}_{c}", "rb").read()
            got = open(f"{fa}.{ext}_{c}", "rb").read()
            assert got == want, f"{ext}_{c} differs"
        total += os.path.getsize(f"{fa}.ndist_{c}") // 4
        c += 1
    assert not os.path.exists(f"{fa}.npair_{c}")
    assert f"\n{total}\n" in r.stdout


def test_cli_errors(tmp_path):
    # missing input, not-FASTA input, missing .kpair: non-zero exit, no crash
    bad = str(tmp_path / "notfasta")
    open(bad, "w").write("ACGT\n")
    for exe, extra in (("kmerDist", []), ("genDist", ["-b", "10"])):
        r = subprocess.run([os.path.join(BIN, exe), "-i", bad] + extra, stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT)
        assert r.returncode != 0
    fa = str(tmp_path / "ok_Clean")
    open(fa, "w").write(">a\nACGTACGTAC\n>b\nACGTACGTAA\n")
    r = subprocess.run([os.path.join(BIN, "genDist"), "-i", fa], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT)
    assert r.returncode != 0   # no .kpair next to it


def _run(args, cwd=None, mode="batched"):
    r = subprocess.run(args, env=_env(mode), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       cwd=cwd)
    assert r.returncode == 0, r.stdout
    return r.stdout


def _outputs(base):
    d = os.path.dirname(base)
    stem = os.path.basename(base)
    return {f[len(stem):]: open(os.path.join(d, f), "rb").read()
            for f in sorted(os.listdir(d)) if f.startswith(stem + ".")}


def _fused_vs_two(tmp_path, src, k, band, mode):
    a, b = tmp_path / "two", tmp_path / "fused"
    a.mkdir(); b.mkdir()
    fa, fb = str(a / "reads_Clean"), str(b / "reads_Clean")
    shutil.copy(src, fa)
    shutil.copy(src, fb)
    _run([os.path.join(BIN, "kmerDist"), "-i", fa, "-k", str(k), "-d"], mode=mode)
    _run([os.path.join(BIN, "genDist"), "-i", fa, "-b", str(band)], mode=mode)
    out = _run([os.path.join(BIN, "crispyDist"), "-i", fb, "-k", str(k), "-b", str(band), "-p", "-d"], mode=mode)
    want, got = _outputs(fa), _outputs(fb)
    assert sorted(got) == sorted(want) and ".npair_0" in got
    for ext in want:
        assert got[ext] == want[ext], f"{ext} differs"
    return out


@pytest.mark.parametrize("name", sorted(MANIFEST["sets"]))
@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_crispydist_matches_two_programs(tmp_path, name, mode):
    # one process, survivors handed over in HBM: the same files as kmerDist -d
    # followed by genDist
    s = MANIFEST["sets"][name]
    src = os.path.join(GOLD, name, name + "_Clean")
    _fused_vs_two(tmp_path, src, s["kmer"][0]["k"], s["gen"][0]["band"], mode)


def test_crispydist_reads_parsed_differently(tmp_path):
    # trailing N: kmerDist trims it, genDist keeps it, so the fused tool
    # uploads genDist's own parse instead of reusing the k-mer stage's reads
    rng = np.random.default_rng(5)
    base = "".join(rng.choice(list("ACGT"), 240))
    lines = []
    for i in range(60):
        s = list(base)
        for p in rng.integers(0, 240, 6):
            s[p] = rng.choice(list("ACGT"))
        seq = "".join(s)[: 200 + i % 30]
        if i % 7 == 0:
            seq += "NN"
        lines.append(f">r{i}\n{seq}\n")
    src = str(tmp_path / "src_Clean")
    open(src, "w").write("".join(lines))
    _fused_vs_two(tmp_path, src, 6, 10, "batched")


@pytest.mark.parametrize("mode", ["batched", "staged"])
def test_crispydist_k8_matches_two_programs(tmp_path, mode):
    # k = 8: kmerDist's read order stays inside the process; genDist takes the
    # survivors by read ID, as from the .kpair file
    src = os.path.join(GOLD, "syn600", "syn600_Clean")
    _fused_vs_two(tmp_path, src, 8, 5, mode)
