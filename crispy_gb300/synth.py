"""Seeded synthetic 16S-like read sets.

The generator follows the workload definition the reference pipeline is
benchmarked on: a random ACGT root, OTU centroids at 3-15 % per-site
substitution divergence, reads copied from a uniformly chosen centroid with
0-3 % substitutions plus homopolymer-length indels (0.25 % delete and 0.25 %
duplicate per base), truncated to a drawn length.  The result is then
deduplicated and ordered by (length, byte order) exactly as the reference's
preprocess step orders its ``_Clean`` output (preprocess.cpp:42-50, 244-280,
562-601), so read IDs match what kmerDist/genDist see in the real pipeline.

Everything is numpy (PCG64) and fully determined by the seed.
"""
from __future__ import annotations

import dataclasses
import numpy as np

_ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


@dataclasses.dataclass(frozen=True)
class ReadSetSpec:
    n_reads: int            # reads drawn before deduplication
    n_centroids: int
    root_len: int = 260
    length_dist: str = "normal"   # "normal" or "uniform"
    length_a: float = 250.0       # mean (normal) or low bound (uniform)
    length_b: float = 15.0        # sd (normal) or high bound (uniform)
    k: int = 6
    seed: int = 1


# Named workloads (k-mer size / band are stage parameters, listed for reference).
WORKLOADS = {
    "small_1k": ReadSetSpec(1000, 40, 260, "normal", 250, 15, 6, 11),
    "plain_20k": ReadSetSpec(20000, 400, 260, "normal", 250, 15, 6, 12),
    "uneven_100k": ReadSetSpec(100000, 1500, 520, "uniform", 300, 500, 6, 13),
    "stress_500k": ReadSetSpec(500000, 5000, 260, "normal", 250, 30, 8, 15),
}


def _substitute(rng, seqs: np.ndarray, rate: np.ndarray) -> np.ndarray:
    """Per-site substitution; a substituted base becomes one of the other 3."""
    hit = rng.random(seqs.shape) < rate[:, None]
    shift = rng.integers(1, 4, size=seqs.shape, dtype=np.uint8)
    codes = seqs.copy()
    codes[hit] = (codes[hit] + shift[hit]) % 4
    return codes


def generate(spec: ReadSetSpec) -> list[bytes]:
    """Raw reads (before dedup/sort) as ASCII byte strings."""
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    root = rng.integers(0, 4, size=spec.root_len, dtype=np.uint8)
    cdiv = rng.uniform(0.03, 0.15, size=spec.n_centroids)
    cents = _substitute(rng, np.broadcast_to(root, (spec.n_centroids, spec.root_len)), cdiv)
    pick = rng.integers(0, spec.n_centroids, size=spec.n_reads)
    rdiv = rng.uniform(0.0, 0.03, size=spec.n_reads)
    reads = _substitute(rng, cents[pick], rdiv)
    # homopolymer-length indels: each base kept once, dropped, or doubled
    u = rng.random(reads.shape)
    reps = np.where(u < 0.0025, 0, np.where(u < 0.005, 2, 1)).astype(np.int64)
    flat = np.repeat(reads.reshape(-1), reps.reshape(-1))
    row_len = reps.sum(axis=1)
    if spec.length_dist == "normal":
        want = np.rint(rng.normal(spec.length_a, spec.length_b, size=spec.n_reads))
    else:
        want = rng.integers(int(spec.length_a), int(spec.length_b) + 1, size=spec.n_reads)
    want = np.clip(want, spec.k + 1, 2048).astype(np.int64)
    take = np.minimum(want, row_len)
    starts = np.concatenate(([0], np.cumsum(row_len)[:-1]))
    ascii_all = _ACGT[flat].tobytes()
    return [ascii_all[s:s + t] for s, t in zip(starts.tolist(), take.tolist())]


def preprocess_order(reads: list[bytes]) -> list[bytes]:
    """Deduplicate and order by (length, strcmp) like the reference preprocess."""
    return sorted(set(reads), key=lambda s: (len(s), s))


def make_read_set(spec: ReadSetSpec | str) -> list[bytes]:
    if isinstance(spec, str):
        spec = WORKLOADS[spec]
    return preprocess_order(generate(spec))


def write_fasta(path: str, reads: list[bytes]) -> None:
    """FASTA in the layout of the preprocess output ("> label" then one line)."""
    with open(path, "wb") as f:
        for i, s in enumerate(reads):
            f.write(b"> r%d\n" % i)
            f.write(s)
            f.write(b"\n")


def pack_reads(reads: list[bytes]):
    """Concatenate reads: (uint8 buffer, int64 offsets, int32 lengths)."""
    lens = np.fromiter((len(s) for s in reads), dtype=np.int32, count=len(reads))
    offs = np.zeros(len(reads), dtype=np.int64)
    if len(reads) > 1:
        offs[1:] = np.cumsum(lens[:-1], dtype=np.int64)
    buf = np.frombuffer(b"".join(reads), dtype=np.uint8).copy()
    return buf, offs, lens
