"""Regenerate the sparsecut fixtures from the reference's own sparsecut.

Needs the reference tree: `make -C oracle ref` compiles
src/sparsecut/sparsecut.cpp as it lies into oracle/_ref/sparsecut.  Each case
takes the _Merge dendrogram of one aveclust fixture (tests/golden/clust/,
written by the reference's aveclust) and a cutoff file, and keeps the
reference's <name>.Cluster and <name>.Cluster_List under
tests/golden/cut/<case>/, listed in MANIFEST.json with SHA-256.

Cutoff files: an even grid of levels, and levels placed on merge distances
of the dendrogram itself, exactly and 5e-6 / 2e-5 away (inside and outside
the reference's EPSILON of 1e-5).  The text varies (trailing newline or not,
blank lines, exponent notation) as the reference's "%f\\n" loop reads it.

Run:  python tests/golden/cut/make_cut_golden.py
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
REF = os.path.join(ROOT, "oracle", "_ref", "sparsecut")
CLUST = os.path.join(GOLD, "clust")


def merge_dists(path):
    return np.array([float(line.split()[2]) for line in open(path)], np.float32)


def grid_text(levels, tail="\n"):
    return "\n".join("%g" % v for v in levels) + tail


def tie_levels(d, seed):
    """Levels on merge distances: exact, +-5e-6 (inside EPSILON), +-2e-5 (outside)."""
    rng = np.random.default_rng(seed)
    picks = np.sort(rng.choice(np.unique(d), size=min(4, len(np.unique(d))), replace=False))
    out = []
    for v in picks:
        out += [float(v), float(v) + 5e-6, float(v) - 5e-6, float(v) + 2e-5]
    return out


CASES = {
    # name: (aveclust fixture, cutoff text builder(merge distances))
    "syn600_grid": ("syn600_b10", lambda d: grid_text([0.01, 0.02, 0.03, 0.05, 0.08, 0.1, 0.15])),
    "syn600_ties": ("syn600_b10", lambda d: "\n".join("%.9g" % v for v in tie_levels(d, 1)) + "\n\n\n"),
    "uneven_b3_grid": ("uneven_b3", lambda d: grid_text([0.005, 0.01, 0.02, 0.04], tail="")),
    "uneven_b10_ties": ("uneven_b10_e", lambda d: "\n".join("%.9g" % v for v in tie_levels(d, 2))),
    "ties_3chunks": ("ties_3chunks", lambda d: "1e-2\n3.0e-2\n  0.05\n0.07\n0.1\n"),
    "ties_5chunks": ("ties_5chunks_o", lambda d: "\n".join("%.9g" % v for v in tie_levels(d, 3)) + "\n"),
    "dense_small": ("dense_small", lambda d: grid_text([0.0, 0.05, 0.1, 0.2, 0.25, 0.5, 1.0])),
}


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/sparsecut is not built: make -C oracle ref (needs the reference tree)")
    clust = json.load(open(os.path.join(CLUST, "MANIFEST.json")))
    manifest = {}
    for name, (src, cut_text) in CASES.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        n = clust[src]["num_reads"]
        tmp = tempfile.mkdtemp()
        try:
            shutil.copy(os.path.join(CLUST, src, "in_Merge"), os.path.join(tmp, "in_Merge"))
            with open(os.path.join(tmp, "cutoffs.txt"), "w") as f:
                f.write(cut_text(merge_dists(os.path.join(tmp, "in_Merge"))))
            args = ["-i", "in", "-n", str(n), "-c", "cutoffs.txt"]
            proc = subprocess.run([REF] + args, cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if proc.returncode != 0:
                raise RuntimeError(f"{name}: reference returned {proc.returncode}")
            files = ["in_Merge", "cutoffs.txt", "in.Cluster", "in.Cluster_List"]
            for fn in files:
                shutil.copy(os.path.join(tmp, fn), os.path.join(d, fn))
            manifest[name] = {"args": args, "num_reads": n, "from": src,
                              "files": {fn: hashlib.sha256(open(os.path.join(d, fn), "rb").read()).hexdigest()
                                        for fn in files}}
        finally:
            shutil.rmtree(tmp)
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("wrote", len(manifest), "cases")


if __name__ == "__main__":
    main()
