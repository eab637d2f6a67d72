"""Regenerate the golden fixtures from the reference's own CPU code.

Needs the reference tree (its CPU path is compiled from source by
`make -C oracle ref`, outputs in oracle/_ref/).  Each fixture set is a
seeded synthetic read set, run exactly as crispy.sh runs it:
    preprocess -i <set>            -> <set>_Clean           (dedup + length sort)
    kmerDist -i <set>_Clean ... -c -n 1 -d                  -> .kpair / .kdist
    genDist  -i <set>_Clean -b B -c -n 1                    -> .npair_0 / .ndist_0
-n 1 keeps the reference CPU path deterministic: its .kpair is then in
(row, col) order, and genDist's chunk keeps input order among equal
distances.  The files are renamed per parameter set (e.g. .k6.kpair,
.b10.npair_0) and listed with their SHA-256 in MANIFEST.json.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crispy_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")

# name -> (generator spec, kmer runs [(tag, k, thr)], gen runs [(tag, band, thr)])
SETS = {
    # > 500 reads: log2 default thresholds, arrayDim 32; the sample-sized case
    "syn600": (synth.ReadSetSpec(700, 30, 260, "normal", 250, 15, 6, 2024),
               [("k6", 6, None), ("k8", 8, 0.45), ("k4", 4, 0.15)],
               [("b10", 10, None), ("b2", 2, None), ("b1", 1, 0.2), ("b5", 5, 0.3)]),
    # uneven lengths 300-500 from a 520-long root
    "uneven": (synth.ReadSetSpec(260, 12, 520, "uniform", 300, 500, 6, 77),
               [("k6", 6, 0.3), ("k7", 7, 0.4)],
               [("b10", 10, 0.25), ("b3", 3, 0.25)]),
}


def _run(cmd, cwd, ok=(0,)):
    p = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode not in ok:
        raise RuntimeError(f"{cmd} failed:\n{p.stdout}")
    return p.stdout


def _raw_fasta(path, reads):
    with open(path, "wb") as f:
        for i, s in enumerate(reads):
            f.write(b">read_%d synthetic\n" % i)
            # wrap at 60 columns like common FASTA writers; preprocess joins lines
            for a in range(0, len(s), 60):
                f.write(s[a:a + 60] + b"\n")


def make_set(name, spec, kruns, gruns, out_dir):
    tmp = tempfile.mkdtemp()
    try:
        raw = os.path.join(tmp, name)
        _raw_fasta(raw, synth.generate(spec))
        # preprocess ends with `return 1` on success (preprocess.cpp:725)
        _run([os.path.join(REF_BIN, "preprocess"), "-i", name], tmp, ok=(0, 1))
        clean = name + "_Clean"
        shutil.copy(os.path.join(tmp, clean), os.path.join(out_dir, clean))
        files = [clean]
        for tag, k, thr in kruns:
            cmd = [os.path.join(REF_BIN, "kmerDist"), "-i", clean, "-k", str(k), "-c", "-n", "1", "-d"]
            if thr is not None:
                cmd += ["-t", str(thr)]
            _run(cmd, tmp)
            for ext in ("kpair", "kdist"):
                dst = f"{clean}.{tag}.{ext}"
                shutil.copy(os.path.join(tmp, f"{clean}.{ext}"), os.path.join(out_dir, dst))
                files.append(dst)
        # genDist reads <clean>.kpair: use the k=6 run's pairs
        k6 = [t for t, k, _ in kruns if k == 6][0]
        shutil.copy(os.path.join(out_dir, f"{clean}.{k6}.kpair"), os.path.join(tmp, f"{clean}.kpair"))
        for tag, band, thr in gruns:
            for f in os.listdir(tmp):
                if ".npair_" in f or ".ndist_" in f:
                    os.remove(os.path.join(tmp, f))
            cmd = [os.path.join(REF_BIN, "genDist"), "-i", clean, "-b", str(band), "-c", "-n", "1"]
            if thr is not None:
                cmd += ["-t", str(thr)]
            _run(cmd, tmp)
            c = 0
            while os.path.exists(os.path.join(tmp, f"{clean}.npair_{c}")):
                for ext in ("npair", "ndist"):
                    dst = f"{clean}.{tag}.{ext}_{c}"
                    shutil.copy(os.path.join(tmp, f"{clean}.{ext}_{c}"), os.path.join(out_dir, dst))
                    files.append(dst)
                c += 1
        return files
    finally:
        shutil.rmtree(tmp)


def main():
    for exe in ("preprocess", "kmerDist", "genDist"):
        if not os.path.exists(os.path.join(REF_BIN, exe)):
            sys.exit("oracle/_ref is not built: make -C oracle ref (needs the reference tree)")
    manifest = {"generator": "crispy_gb300.synth (numpy PCG64)", "sets": {}}
    for name, (spec, kruns, gruns) in SETS.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        files = make_set(name, spec, kruns, gruns, d)
        manifest["sets"][name] = {
            "spec": spec.__dict__,
            "kmer": [{"tag": t, "k": k, "thr": thr} for t, k, thr in kruns],
            "gen": [{"tag": t, "band": b, "thr": thr, "kpair": "k6"} for t, b, thr in gruns],
            "files": {f: hashlib.sha256(open(os.path.join(d, f), "rb").read()).hexdigest()
                      for f in files},
        }
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("wrote", sum(len(s["files"]) for s in manifest["sets"].values()), "files")


if __name__ == "__main__":
    main()
