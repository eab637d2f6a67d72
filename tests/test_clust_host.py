"""aveclust (sparse average-linkage clustering) checks; host code, no GPU.

* The drop-in `aveclust` executable and crispy_aveclust reproduce the
  reference's _Merge file (and the -o edge files) byte for byte on every
  fixture of tests/golden/clust/ (made from src/aveclust/aveclust.cpp by
  tests/golden/clust/make_clust_golden.py), and the same clusters at every
  distance level of .Cluster / .Cluster_List (the reference lists them in
  pointer-hash order, this engine by root ID, so lines compare as sets).
* The oracle's restatement (oracle/oracle_clust.cpp) reproduces the same
  _Merge files, and so does the engine on seeded chunk sets against the
  oracle.
* Where the reference tree exists, fresh seeded sets run through the
  reference binary itself.
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
GOLD = os.path.join(HERE, "golden", "clust")
MANIFEST = json.load(open(os.path.join(GOLD, "MANIFEST.json")))
EXE = os.path.join(cg.BIN_DIR, "aveclust")
REF = os.environ.get("CRISPY_REFERENCE", "/root/reference")


def cluster_sets(path):
    """Per level line: (level, sorted list of '|'-separated OTU strings)."""
    out = []
    for line in open(path):
        head, _, rest = line.partition("|")
        out.append((head.strip(), sorted(p for p in rest.strip().split("|") if p)))
    return out


def size_sets(path):
    return [(l.split()[0], sorted(l.split()[1:])) for l in open(path)]


def _chunks(d, nchunks):
    return [(np.fromfile(os.path.join(d, f"in.npair_{f}"), np.uint32).reshape(-1, 2),
             np.fromfile(os.path.join(d, f"in.ndist_{f}"), np.float32)) for f in range(nchunks)]


def _same_clusters(a_base, b_base):
    assert cluster_sets(a_base + ".Cluster") == cluster_sets(b_base + ".Cluster")
    assert size_sets(a_base + ".Cluster_List") == size_sets(b_base + ".Cluster_List")


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_cli_matches_reference_fixture(tmp_path, name):
    case = MANIFEST[name]
    d = str(tmp_path / name)
    shutil.copytree(os.path.join(GOLD, name), d)
    want = {o: open(os.path.join(d, o), "rb").read() for o in case["outputs"]}
    shutil.copy(os.path.join(d, "in.Cluster"), os.path.join(d, "ref.Cluster"))
    shutil.copy(os.path.join(d, "in.Cluster_List"), os.path.join(d, "ref.Cluster_List"))
    for o in case["outputs"]:
        os.remove(os.path.join(d, o))
    subprocess.run([EXE] + case["args"], cwd=d, check=True, stdout=subprocess.DEVNULL)
    assert open(os.path.join(d, "in_Merge"), "rb").read() == want["in_Merge"]
    for o in ("edges", "edges_Index1"):
        if o in want:
            assert open(os.path.join(d, o), "rb").read() == want[o]
    _same_clusters(os.path.join(d, "in"), os.path.join(d, "ref"))


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_api_and_oracle_match_fixture(tmp_path, name):
    case = MANIFEST[name]
    d = os.path.join(GOLD, name)
    chunks = _chunks(d, case["chunks"])
    args = case["args"]
    level = float(args[args.index("-e") + 1]) if "-e" in args else -1.0
    st = cg.aveclust(chunks, case["num_reads"], str(tmp_path / "api"), end_level=level)
    want = open(os.path.join(d, "in_Merge"), "rb").read()
    assert open(str(tmp_path / "api_Merge"), "rb").read() == want
    assert st["merges"] == want.count(b"\n")
    _same_clusters(str(tmp_path / "api"), os.path.join(d, "in"))
    m = oracle.aveclust(chunks, case["num_reads"], str(tmp_path / "oracle_Merge"), end_level=level)
    assert open(str(tmp_path / "oracle_Merge"), "rb").read() == want and m == st["merges"]


def _seeded(seed, n, edges, chunks, grid, hi, sparse=False):
    rng = np.random.default_rng(seed)
    if sparse:   # clusters of nearby read IDs, links only inside them
        a = rng.integers(0, n, size=edges)
        b = np.minimum(n - 1, a + rng.integers(1, 12, size=edges))
    else:
        a = rng.integers(0, n, size=edges)
        b = rng.integers(0, n, size=edges)
    keep = a < b
    pairs = np.unique(np.stack([a[keep], b[keep]], 1), axis=0)
    rng.shuffle(pairs)
    d = (rng.integers(0, grid, size=len(pairs)) * (hi / grid)).astype(np.float32)
    out = []
    for idx in np.array_split(np.arange(len(pairs)), chunks):
        o = np.argsort(d[idx], kind="stable")
        out.append((pairs[idx][o].astype(np.uint32), d[idx][o]))
    return out


@pytest.mark.parametrize("seed,n,edges,chunks,grid,hi,sparse,level", [
    (1, 300, 2500, 1, 9, 0.1, False, -1.0),
    (2, 2000, 9000, 4, 30, 0.3, True, -1.0),
    (3, 5000, 30000, 3, 50, 0.2, True, 0.05),
    (4, 800, 20000, 6, 4, 0.2, False, 0.12),    # heavy ties, edge cap doublings
    (5, 1500, 4000, 2, 1000, 0.5, True, 0.6),
])
def test_engine_vs_oracle_seeded(tmp_path, seed, n, edges, chunks, grid, hi, sparse, level):
    ch = _seeded(seed, n, edges, chunks, grid, hi, sparse)
    st = cg.aveclust(ch, n, str(tmp_path / "api"), end_level=level)
    m = oracle.aveclust(ch, n, str(tmp_path / "oracle_Merge"), end_level=level)
    assert open(str(tmp_path / "api_Merge"), "rb").read() == open(str(tmp_path / "oracle_Merge"), "rb").read()
    assert m == st["merges"]


def test_bad_input(tmp_path):
    ch = [(np.array([[0, 5]], np.uint32), np.array([0.1], np.float32))]
    with pytest.raises(cg.CrispyError):
        cg.aveclust(ch, 4, str(tmp_path / "x"))   # read 5 of 4
    with pytest.raises(cg.CrispyError):
        cg.aveclust([], 4, str(tmp_path / "x"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "aveclust")), reason="reference tree not present")
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_reference_live(tmp_path, seed):
    subprocess.run(["make", "-s", "-C", oracle.HERE, "ref", f"REF={REF}"], check=True)
    n = 1200
    ch = _seeded(seed, n, 9000, 3, 25, 0.25, sparse=seed % 2 == 1)
    d = str(tmp_path)
    for f, (p, dist) in enumerate(ch):
        p.tofile(os.path.join(d, f"in.npair_{f}"))
        dist.tofile(os.path.join(d, f"in.ndist_{f}"))
    subprocess.run([os.path.join(oracle.REF_DIR, "aveclust"), "-i", "in", "-n", str(n), "-f", str(len(ch)),
                    "-o", "edges"], cwd=d, check=True, stdout=subprocess.DEVNULL)
    cg.aveclust(ch, n, os.path.join(d, "api"), edge_out=os.path.join(d, "api_edges"))
    assert open(os.path.join(d, "api_Merge"), "rb").read() == open(os.path.join(d, "in_Merge"), "rb").read()
    assert open(os.path.join(d, "api_edges"), "rb").read() == open(os.path.join(d, "edges"), "rb").read()
    _same_clusters(os.path.join(d, "api"), os.path.join(d, "in"))
