"""sparsecut (cutting the aveclust dendrogram at given distances); host code,
no GPU.

* The drop-in `sparsecut` executable and crispy_sparsecut give the same
  clusters as the reference's sparsecut at every cutoff of every fixture of
  tests/golden/cut/ (made from src/sparsecut/sparsecut.cpp by
  tests/golden/cut/make_cut_golden.py).  The reference lists a level's
  clusters in pointer-hash order, this engine by root ID, so each level line
  compares as a set of clusters; each cluster's member order is the
  reference's.
* Cutoffs on merge distances, exactly and within / beyond the reference's
  EPSILON (1e-5), are among the fixtures.
* Where the reference tree exists, dendrograms of fresh seeded sets (written
  by crispy_aveclust) are cut by the reference binary itself.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import crispy_gb300 as cg
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "cut")
MANIFEST = json.load(open(os.path.join(GOLD, "MANIFEST.json")))
EXE = os.path.join(cg.BIN_DIR, "sparsecut")
REF = os.environ.get("CRISPY_REFERENCE", "/root/reference")


def cluster_sets(path):
    """Per level line: (level, sorted list of '|'-separated clusters)."""
    out = []
    for line in open(path):
        head, _, rest = line.partition("|")
        out.append((head.strip(), sorted(p for p in rest.strip().split("|") if p)))
    return out


def size_sets(path):
    return [(l.split()[0], sorted(l.split()[1:])) for l in open(path)]


def same_clusters(a_base, b_base):
    assert cluster_sets(a_base + ".Cluster") == cluster_sets(b_base + ".Cluster")
    assert size_sets(a_base + ".Cluster_List") == size_sets(b_base + ".Cluster_List")


def read_cutoffs(path):
    return [float(t) for t in open(path).read().split()]


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_cli_matches_reference_fixture(tmp_path, name):
    case = MANIFEST[name]
    d = str(tmp_path / name)
    shutil.copytree(os.path.join(GOLD, name), d)
    for ext in (".Cluster", ".Cluster_List"):
        shutil.move(os.path.join(d, "in" + ext), os.path.join(d, "ref" + ext))
    subprocess.run([EXE] + case["args"], cwd=d, check=True, stdout=subprocess.DEVNULL)
    same_clusters(os.path.join(d, "in"), os.path.join(d, "ref"))


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_api_matches_reference_fixture(tmp_path, name):
    case = MANIFEST[name]
    d = str(tmp_path / name)
    shutil.copytree(os.path.join(GOLD, name), d)
    cut = read_cutoffs(os.path.join(d, "cutoffs.txt"))
    shutil.copy(os.path.join(d, "in_Merge"), os.path.join(d, "api_Merge"))
    st = cg.sparsecut(os.path.join(d, "api"), case["num_reads"], cut)
    same_clusters(os.path.join(d, "api"), os.path.join(d, "in"))
    assert st["merges"] == sum(1 for _ in open(os.path.join(d, "in_Merge")))
    assert st["report"].count("Dist: ") == len(cut)


def _aveclust_levels(end_level):
    """The levels aveclust's float loop visits (step = endLevel / 10)."""
    end = np.float32(end_level)
    step = np.float32(end / np.float32(10))
    out, level = [], step
    while level < end or abs(float(np.float32(level - end))) < 1e-6:
        out.append(level)
        level = np.float32(level + step)
    return np.array(out, np.float32)


def test_cut_levels_equal_aveclust_levels(tmp_path):
    """At aveclust's own levels, cutting its _Merge gives aveclust's clusters.
    The two share printClusters; they differ in EPSILON (1e-6 against 1e-5)
    and sparsecut reads the distances as _Merge prints them (6 decimals), so
    the seed is one whose merge distances all lie 2e-5 or more from a level."""
    rng = np.random.default_rng(1)
    n = 400
    a = rng.integers(0, n, 1500)
    b = rng.integers(0, n, 1500)
    keep = a < b
    pairs = np.unique(np.stack([a[keep], b[keep]], 1), axis=0)
    d = rng.uniform(0, 0.12, len(pairs)).astype(np.float32)
    o = np.argsort(d, kind="stable")
    base = str(tmp_path / "x")
    st = cg.aveclust([(pairs[o].astype(np.uint32), d[o])], n, base)
    lv = _aveclust_levels(st["end_level"])
    md = np.array([float(l.split()[2]) for l in open(base + "_Merge")], np.float32)
    assert len(md) > 300 and np.min(np.abs(md[:, None] - lv[None, :])) > 2e-5
    shutil.copy(base + "_Merge", str(tmp_path / "y_Merge"))
    cg.sparsecut(str(tmp_path / "y"), n, lv)
    same_clusters(base, str(tmp_path / "y"))
    assert st["merges"] == len(md)


def test_bad_input(tmp_path):
    base = str(tmp_path / "m")
    with pytest.raises(cg.CrispyError):
        cg.sparsecut(base, 10, [0.1])                 # no _Merge file
    for bad in ("1 2 0.1\n1 3 0.2\n",                 # read 1 merged twice
                "1 12 0.1\n",                         # node 12 does not exist yet
                "0 2 0.1\n"):                         # IDs are 1-based
        open(base + "_Merge", "w").write(bad)
        with pytest.raises(cg.CrispyError) as e:
            cg.sparsecut(base, 10, [0.1])
        assert e.value.code == cg.E_INPUT
    open(base + "_Merge", "w").write("1 2 0.1\n3 11 0.2\n")
    st = cg.sparsecut(base, 10, [0.15, 0.3])
    assert st["merges"] == 2 and st["roots"] == 1 and st["singletons"] == 7
    # one root: the reference's output byte for byte (larger-ID child first,
    # the cut's nodes in push_front order, then the singletons)
    assert open(base + ".Cluster").read() == (" 0.150000 |2|1 0|3|4|5|6|7|8|9|\n"
                                              " 0.300000 |1 0 2|3|4|5|6|7|8|9|\n")
    assert open(base + ".Cluster_List").read() == (" 0.150000 1 2 1 1 1 1 1 1 1 \n"
                                                   " 0.300000 3 1 1 1 1 1 1 1 \n")
    # a cutoff file that is not numbers is refused by the executable
    open(str(tmp_path / "c.txt"), "w").write("0.1\nabc\n")
    r = subprocess.run([EXE, "-i", base, "-n", "10", "-c", str(tmp_path / "c.txt")], stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
    assert r.returncode != 0


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "sparsecut")), reason="reference tree not present")
@pytest.mark.parametrize("seed", [21, 22])
def test_reference_live(tmp_path, seed):
    subprocess.run(["make", "-s", "-C", oracle.HERE, "ref", f"REF={REF}"], check=True)
    rng = np.random.default_rng(seed)
    n = 1500
    a = rng.integers(0, n, 12000)
    b = np.minimum(n - 1, a + rng.integers(1, 40, 12000))
    keep = a < b
    pairs = np.unique(np.stack([a[keep], b[keep]], 1), axis=0)
    dist = (rng.integers(0, 40, len(pairs)) * 0.005).astype(np.float32)
    o = np.argsort(dist, kind="stable")
    d = str(tmp_path)
    cg.aveclust([(pairs[o].astype(np.uint32), dist[o])], n, os.path.join(d, "in"), end_level=0.2)
    md = sorted(set(float(l.split()[2]) for l in open(os.path.join(d, "in_Merge"))))
    cut = [0.01, 0.02, md[len(md) // 2], md[-1] - 4e-6, 0.1, 0.15]
    with open(os.path.join(d, "cut.txt"), "w") as f:
        f.write("\n".join("%.9g" % v for v in cut) + "\n")
    shutil.copy(os.path.join(d, "in_Merge"), os.path.join(d, "eng_Merge"))
    subprocess.run([os.path.join(oracle.REF_DIR, "sparsecut"), "-i", "in", "-n", str(n), "-c", "cut.txt"],
                   cwd=d, check=True, stdout=subprocess.DEVNULL)
    subprocess.run([EXE, "-i", "eng", "-n", str(n), "-c", "cut.txt"], cwd=d, check=True, stdout=subprocess.DEVNULL)
    same_clusters(os.path.join(d, "eng"), os.path.join(d, "in"))
