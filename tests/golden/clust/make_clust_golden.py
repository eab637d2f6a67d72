"""Regenerate the aveclust fixtures from the reference's own aveclust.

Needs the reference tree: `make -C oracle ref` compiles
src/aveclust/aveclust.cpp as it lies into oracle/_ref/aveclust.  Each case
is a set of genDist-style chunk files (<name>.npair_<f> / .ndist_<f>, each
ascending by distance) plus a command line; the reference's <name>_Merge,
<name>.Cluster and <name>.Cluster_List (and the -o edge files) are kept
under tests/golden/clust/<case>/, listed in MANIFEST.json with SHA-256.

Inputs: the genDist fixtures of tests/golden (syn600, uneven: one chunk each,
as genDist wrote them) and seeded chunk sets made here: several chunks with
distances on a coarse grid, so that equal distances meet across chunks
(the multimap order) and inside link maps (ties in the minimum search).

Run:  python tests/golden/clust/make_clust_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.dirname(HERE)
ROOT = os.path.dirname(os.path.dirname(GOLD))
REF = os.path.join(ROOT, "oracle", "_ref", "aveclust")


def seeded_chunks(seed: int, n: int, edges: int, chunks: int, grid: int, hi: float):
    """`chunks` sorted chunks of distinct random read pairs; distances on a grid."""
    rng = np.random.default_rng(seed)
    a = rng.integers(0, n, size=edges * 2)
    b = rng.integers(0, n, size=edges * 2)
    keep = a < b
    pairs = np.unique(np.stack([a[keep], b[keep]], 1), axis=0)[:edges]
    rng.shuffle(pairs)
    d = (rng.integers(0, grid, size=len(pairs)) * (hi / grid)).astype(np.float32)
    out = []
    for c, idx in enumerate(np.array_split(np.arange(len(pairs)), chunks)):
        o = np.argsort(d[idx], kind="stable")
        out.append((pairs[idx][o].astype(np.uint32), d[idx][o]))
    return out


def golden_chunks(set_name: str, tag: str):
    base = os.path.join(GOLD, set_name, f"{set_name}_Clean.{tag}")
    p = np.fromfile(base + ".npair_0", np.uint32).reshape(-1, 2)
    d = np.fromfile(base + ".ndist_0", np.float32)
    n = sum(1 for line in open(os.path.join(GOLD, set_name, f"{set_name}_Clean"), "rb") if line.startswith(b">"))
    return [(p, d)], n


CASES = {
    # name: (chunks builder -> (chunks, n), extra argv)
    "syn600_b10": (lambda: golden_chunks("syn600", "b10"), []),
    "uneven_b3": (lambda: golden_chunks("uneven", "b3"), []),
    "uneven_b10_e": (lambda: golden_chunks("uneven", "b10"), ["-e", "0.3"]),
    "ties_3chunks": (lambda: (seeded_chunks(5, 400, 3000, 3, 12, 0.12), 400), []),
    "ties_5chunks_o": (lambda: (seeded_chunks(6, 700, 6000, 5, 20, 0.2), 700), ["-o", "edges"]),
    "dense_small": (lambda: (seeded_chunks(7, 60, 1500, 2, 6, 0.3), 60), ["-e", "0.25"]),
}


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/aveclust is not built: make -C oracle ref (needs the reference tree)")
    manifest = {}
    for name, (build, extra) in CASES.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        chunks, n = build()
        tmp = tempfile.mkdtemp()
        try:
            files = []
            for f, (p, dist) in enumerate(chunks):
                for ext, arr in (("npair", p), ("ndist", dist)):
                    fn = f"in.{ext}_{f}"
                    arr.tofile(os.path.join(tmp, fn))
                    files.append(fn)
            args = ["-i", "in", "-n", str(n), "-f", str(len(chunks))] + extra
            proc = subprocess.run([REF] + args, cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if proc.returncode != 0:
                raise RuntimeError(f"{name}: reference returned {proc.returncode}")
            outs = ["in_Merge", "in.Cluster", "in.Cluster_List"]
            if "-o" in extra:
                outs += ["edges", "edges_Index1"]
            for fn in files + outs:
                shutil.copy(os.path.join(tmp, fn), os.path.join(d, fn))
            manifest[name] = {"args": args, "num_reads": n, "chunks": len(chunks), "outputs": outs,
                              "files": {fn: hashlib.sha256(open(os.path.join(d, fn), "rb").read()).hexdigest()
                                        for fn in files + outs}}
        finally:
            shutil.rmtree(tmp)
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("wrote", len(manifest), "cases")


if __name__ == "__main__":
    main()
