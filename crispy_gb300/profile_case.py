"""One pass of the hot path on a named workload, for profiler captures.

    python -m crispy_gb300.profile_case --workload uneven_100k [--stage kmer|gen|both] [--reads N]

Reads are generated and uploaded first; then one batched kmerDist run and one
batched genDist run over its survivors, nothing else.  Run it with
CRISPY_AUTOTUNE=0 so that the first genDist launches are the real ones.
"""
import argparse

import crispy_gb300 as cg
from crispy_gb300 import synth

WORKLOADS = {"uneven_100k": (6, 10), "plain_20k": (6, 10), "small_1k": (6, 10), "stress_500k": (8, 5)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="uneven_100k", choices=sorted(WORKLOADS))
    ap.add_argument("--stage", default="both", choices=["kmer", "gen", "both"])
    ap.add_argument("--reads", type=int, default=0, help="keep the first N reads (0: all)")
    args = ap.parse_args()
    k, band = WORKLOADS[args.workload]
    reads = synth.make_read_set(args.workload)
    if args.reads:
        reads = reads[:args.reads]
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    with cg.Engine(0) as eng:
        eng.kmer_prepare(buf, offs, lens, k)
        eng.gen_prepare(buf, offs, lens)
        kp = eng.kmer_run(cg.default_threshold(n, -1.0, 0), cg.MODE_BATCHED, False)
        if args.stage in ("gen", "both"):
            chunks = eng.gen_run_from_kmer(band, cg.default_threshold(n, -1.0, 1), cg.MODE_BATCHED)
            print(f"{n} reads, {kp} k-mer survivors, {sum(len(c[2]) for c in chunks)} genetic survivors")
        else:
            print(f"{n} reads, {kp} k-mer survivors")


if __name__ == "__main__":
    main()
