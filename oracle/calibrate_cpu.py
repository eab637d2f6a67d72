"""Times the oracle port beside the reference's own CPU path on one host.

TEST INFRASTRUCTURE ONLY.  The timed CPU baseline of the benchmark is the
oracle port (oracle_cli), because the reference's sources are not on the
machines the benchmark runs on.  This script runs both on the same seeded
sample where the reference binaries exist (oracle/_ref, built by
`make -C oracle ref`), checks that they produce the same survivors and
chunks, and prints their wall times, so that the port's rate can be read
as the reference's.

    python -m oracle.calibrate_cpu [--workload uneven_100k] [--reads 4000] [--threads N]

Output: one JSON line (times in seconds, threads used, identical flags).
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from crispy_gb300 import synth  # noqa: E402


def _run(cmd, cwd):
    t0 = time.perf_counter()
    subprocess.run(cmd, check=True, cwd=cwd, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return time.perf_counter() - t0


def _pairs(path):
    p = np.fromfile(path, np.int32).reshape(-1, 2)
    return set(map(tuple, p.tolist()))


def _chunks(base):
    """Per chunk: the set of (pair, distance) and the distance sequence.  The
    reference's CPU genDist orders pairs of equal distance by its threads'
    order (its GPU path, which the engine follows, by a stable device sort),
    so pairs compare as sets."""
    out = []
    for f in sorted(glob.glob(base + ".ndist_*"), key=lambda x: int(x.rsplit("_", 1)[1])):
        i = f.rsplit("_", 1)[1]
        p = np.fromfile(base + ".npair_" + i, np.uint32).reshape(-1, 2)
        d = np.fromfile(f, np.float32)
        out.append((set(zip(map(tuple, p.tolist()), d.view(np.uint32).tolist())), d.tobytes()))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="uneven_100k")
    ap.add_argument("--reads", type=int, default=4000)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--k", type=int, default=6)
    ap.add_argument("--band", type=int, default=10)
    args = ap.parse_args()
    ref_kmer = os.path.join(oracle.REF_DIR, "kmerDist")
    ref_gen = os.path.join(oracle.REF_DIR, "genDist")
    if not (os.path.exists(ref_kmer) and os.path.exists(ref_gen)):
        print(json.dumps({"unavailable": "oracle/_ref not built (the reference sources are absent here)"}))
        return
    if not os.path.exists(oracle.CLI_PATH):
        oracle.build()
    reads = synth.make_read_set(args.workload)
    rng = np.random.default_rng(1234)
    idx = np.sort(rng.choice(len(reads), size=min(args.reads, len(reads)), replace=False))
    sub = [reads[i] for i in idx]
    tk = oracle.default_threshold(len(reads), -1.0, 2)
    tg = oracle.default_threshold(len(reads), -1.0, 1)
    out = {"workload": args.workload, "sample_reads": len(sub), "threads": args.threads,
           "k": args.k, "band": args.band}
    with tempfile.TemporaryDirectory() as td:
        for who in ("port", "reference"):
            d = os.path.join(td, who)
            os.makedirs(d)
            fa = os.path.join(d, "s_Clean")
            synth.write_fasta(fa, sub)
            if who == "port":
                kc = [oracle.CLI_PATH, "kmer", "-i", fa, "-k", str(args.k), "-t", repr(tk), "-n", str(args.threads)]
                gc = [oracle.CLI_PATH, "gen", "-i", fa, "-b", str(args.band), "-t", repr(tg), "-n", str(args.threads)]
            else:
                kc = [ref_kmer, "-i", fa, "-k", str(args.k), "-t", repr(tk), "-c", "-n", str(args.threads)]
                gc = [ref_gen, "-i", fa, "-b", str(args.band), "-t", repr(tg), "-c", "-n", str(args.threads)]
            out[who + "_kmer_s"] = _run(kc, d)
            if who == "reference":
                # the reference's multi-threaded CPU kmerDist writes pairs in
                # thread order; genDist reads them in that order, so hand it
                # the port's stage-ordered file for a like-for-like genDist
                os.replace(fa + ".kpair", fa + ".kpair_ref")
                with open(fa + ".kpair", "wb") as f:
                    f.write(open(os.path.join(td, "port", "s_Clean.kpair"), "rb").read())
            out[who + "_gen_s"] = _run(gc, d)
        pp = _pairs(os.path.join(td, "port", "s_Clean.kpair"))
        rp = _pairs(os.path.join(td, "reference", "s_Clean.kpair_ref"))
        out["kmer_survivors"] = len(pp)
        out["kmer_survivors_identical"] = pp == rp
        out["gen_chunks_identical"] = (_chunks(os.path.join(td, "port", "s_Clean")) ==
                                       _chunks(os.path.join(td, "reference", "s_Clean")))
    out["kmer_time_ratio_port_over_reference"] = out["port_kmer_s"] / out["reference_kmer_s"]
    out["gen_time_ratio_port_over_reference"] = out["port_gen_s"] / out["reference_gen_s"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
