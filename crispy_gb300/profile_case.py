"""One pass of the hot path on a named workload, for profiler captures.

    python -m crispy_gb300.profile_case --workload uneven_100k [--stage kmer|gen|both|pre] [--reads N]

Reads are generated and uploaded first; then one batched kmerDist run and one
batched genDist run over its survivors, nothing else.  Run it with
CRISPY_AUTOTUNE=0 so that the first genDist launches are the real ones.
--stage pre instead writes the workload's raw reads (before deduplication,
60 columns per line) to a temporary FASTA and runs crispy_preprocess on
them twice.
"""
import argparse
import os
import tempfile

import crispy_gb300 as cg
from crispy_gb300 import synth

WORKLOADS = {"uneven_100k": (6, 10), "plain_20k": (6, 10), "small_1k": (6, 10), "stress_500k": (8, 5)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="uneven_100k", choices=sorted(WORKLOADS))
    ap.add_argument("--stage", default="both", choices=["kmer", "gen", "both", "pre"])
    ap.add_argument("--reads", type=int, default=0, help="keep the first N reads (0: all)")
    args = ap.parse_args()
    k, band = WORKLOADS[args.workload]
    if args.stage == "pre":
        raw_reads = synth.generate(synth.WORKLOADS[args.workload])
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "raw.fa")
            with open(path, "wb") as f:
                for i, s in enumerate(raw_reads):
                    f.write(b">read_%d synthetic\n" % i)
                    for a in range(0, len(s), 60):
                        f.write(s[a:a + 60] + b"\n")
            raw = cg.RawReads(path)
            with cg.Engine(0) as eng:
                for _ in range(2):
                    _, _, st = eng.preprocess(raw)
            raw.close()
        print(f"{len(raw_reads)} raw reads, {st['kept']} kept")
        return
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
