"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the reference results are compared
with or as the timed CPU baseline, never as a substitute for the GPU engine.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
CLI_PATH = os.path.join(HERE, "oracle_cli")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.oracle_fasta_read.argtypes = [C.c_char_p, C.c_int, C.POINTER(P)]
        L.oracle_fasta_read.restype = C.c_int
        L.oracle_fasta_get.argtypes = [P, C.POINTER(C.c_char_p), C.POINTER(C.POINTER(C.c_int64)),
                                       C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.c_int32)]
        L.oracle_fasta_free.argtypes = [P]
        L.oracle_default_threshold.argtypes = [C.c_int, C.c_float, C.c_int]
        L.oracle_default_threshold.restype = C.c_float
        L.oracle_array_dim.argtypes = [C.c_int]
        L.oracle_array_dim.restype = C.c_int
        L.oracle_kmer_matches.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int]
        L.oracle_kmer_matches.restype = C.c_int
        L.oracle_kmer_all.argtypes = [P, P, P, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, P, P,
                                      C.c_int64]
        L.oracle_kmer_all.restype = C.c_int64
        L.oracle_gen_pair.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int, P, P, P]
        L.oracle_gen_pair.restype = C.c_float
        L.oracle_gen_all.argtypes = [P, P, P, C.c_int, P, C.c_int64, C.c_int, C.c_int, P, P, P, P]
        L.oracle_gen_all.restype = None
        L.oracle_band_cells.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oracle_band_cells.restype = C.c_int64
        L.oracle_gen_chunks.argtypes = [P, P, C.c_int64, C.c_float, P, P, P, C.c_int]
        L.oracle_gen_chunks.restype = C.c_int
        L.oracle_preprocess.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_double,
                                        C.c_char_p, C.c_int, P]
        L.oracle_preprocess.restype = C.c_int
        L.oracle_aveclust.argtypes = [C.POINTER(P), C.POINTER(P), P, C.c_int, C.c_int, C.c_float,
                                      C.c_char_p, P]
        L.oracle_aveclust.restype = C.c_int
        L.oracle_kmer_rows.argtypes = [P, P, P, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int,
                                       P, P, C.c_int64]
        L.oracle_kmer_rows.restype = C.c_int64
        _lib = L
    return _lib


def read_fasta(path: str, flavour: int):
    L = lib()
    h = C.c_void_p()
    n = L.oracle_fasta_read(path.encode(), flavour, C.byref(h))
    if n < 0:
        raise OSError(f"oracle cannot read {path} ({n})")
    buf = C.c_char_p()
    off = C.POINTER(C.c_int64)()
    ln = C.POINTER(C.c_int32)()
    mx = C.c_int32()
    L.oracle_fasta_get(h, C.byref(buf), C.byref(off), C.byref(ln), C.byref(mx))
    offs = np.ctypeslib.as_array(off, shape=(n,)).copy() if n else np.zeros(0, np.int64)
    lens = np.ctypeslib.as_array(ln, shape=(n,)).copy() if n else np.zeros(0, np.int32)
    total = int(offs[-1] + lens[-1]) if n else 0
    data = np.frombuffer(C.string_at(buf, total), dtype=np.uint8).copy()
    L.oracle_fasta_free(h)
    return data, offs, lens


def kmer_rows(buf, offs, lens, k: int, thr: float, row_lo: int, row_hi: int, nthreads: int = 0):
    """Survivors of rows [row_lo, row_hi) against all later columns, (row, col) order."""
    L = lib()
    buf = np.ascontiguousarray(buf, np.uint8)
    offs = np.ascontiguousarray(offs, np.int64)
    lens = np.ascontiguousarray(lens, np.int32)
    cap = 1 << 16
    while True:
        pairs = np.empty((cap, 2), np.int32)
        d = np.empty(cap, np.float32)
        tot = L.oracle_kmer_rows(buf.ctypes.data, offs.ctypes.data, lens.ctypes.data, len(lens), k, thr,
                                 row_lo, row_hi, nthreads, pairs.ctypes.data, d.ctypes.data, cap)
        if tot < 0:
            raise ValueError("oracle_kmer_rows failed")
        if tot <= cap:
            return pairs[:tot], d[:tot]
        cap = tot


def default_threshold(n: int, user_thr: float, num: int) -> float:
    return float(lib().oracle_default_threshold(n, user_thr, num))


def array_dim(n: int) -> int:
    return int(lib().oracle_array_dim(n))


def kmer_all(buf, offs, lens, k: int, thr: float, nthreads: int = 0):
    """Survivor pairs and distances in the GPU path's stage order."""
    L = lib()
    buf = np.ascontiguousarray(buf, np.uint8)
    offs = np.ascontiguousarray(offs, np.int64)
    lens = np.ascontiguousarray(lens, np.int32)
    n = len(lens)
    A = array_dim(n)
    cap = 1 << 16
    while True:
        pairs = np.empty((cap, 2), np.int32)
        d = np.empty(cap, np.float32)
        tot = L.oracle_kmer_all(buf.ctypes.data, offs.ctypes.data, lens.ctypes.data, n, k, thr, A,
                                nthreads, pairs.ctypes.data, d.ctypes.data, cap)
        if tot < 0:
            raise ValueError("oracle_kmer_all failed")
        if tot <= cap:
            return pairs[:tot], d[:tot]
        cap = tot


def kmer_matches(a: bytes, b: bytes, k: int) -> int:
    return int(lib().oracle_kmer_matches(a, len(a), b, len(b), k))


def gen_all(buf, offs, lens, pairs, band: int, nthreads: int = 0):
    L = lib()
    buf = np.ascontiguousarray(buf, np.uint8)
    offs = np.ascontiguousarray(offs, np.int64)
    lens = np.ascontiguousarray(lens, np.int32)
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    n = len(pairs)
    dist = np.empty(max(n, 1), np.float32)
    score = np.empty(max(n, 1), np.int32)
    ml = np.empty(max(n, 1), np.int32)
    al = np.empty(max(n, 1), np.int32)
    L.oracle_gen_all(buf.ctypes.data, offs.ctypes.data, lens.ctypes.data, len(lens),
                     pairs.ctypes.data, n, band, nthreads, dist.ctypes.data, score.ctypes.data,
                     ml.ctypes.data, al.ctypes.data)
    return dist[:n], score[:n], ml[:n], al[:n]


def band_cells(l1: int, l2: int, band: int) -> int:
    return int(lib().oracle_band_cells(l1, l2, band))


def gen_chunks(pairs, dists, thr: float):
    """[(chunk_id, uint32 pairs, float32 dists)] of genCUDA.cu's writer."""
    L = lib()
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    dists = np.ascontiguousarray(dists, np.float32)
    n = len(dists)
    op = np.empty((max(n, 1), 2), np.uint32)
    od = np.empty(max(n, 1), np.float32)
    maxc = n // 589824 + 4
    sizes = np.empty(maxc, np.int64)
    nc = L.oracle_gen_chunks(pairs.ctypes.data, dists.ctypes.data, n, thr, op.ctypes.data,
                             od.ctypes.data, sizes.ctypes.data, maxc)
    out, at = [], 0
    for c in range(nc):
        s = int(sizes[c])
        out.append((c, op[at:at + s].copy(), od[at:at + s].copy()))
        at += s
    return out


def preprocess(in_path: str, out_path: str, fastq: bool = False, sd: float | None = None,
               primer: bytes | None = None, max_mm: int = 2) -> dict:
    """The oracle's preprocess: writes out_path and out_path.frq, returns the counts."""
    counts = np.zeros(5, np.int64)
    rc = lib().oracle_preprocess(in_path.encode(), out_path.encode(), int(fastq),
                                 int(sd is not None), float(sd if sd is not None else 1.0),
                                 primer, int(max_mm), counts.ctypes.data)
    if rc != 0:
        raise OSError(f"oracle preprocess failed on {in_path} ({rc})")
    return dict(zip(["records", "length_discards", "primer_discards", "merges", "kept"],
                    counts.tolist()))


def aveclust(chunks, num_reads: int, merge_path: str, end_level: float = -1.0) -> int:
    """The oracle's aveclust: writes merge_path (the _Merge lines); returns the merge count."""
    keep = [(np.ascontiguousarray(p, dtype=np.uint32).reshape(-1, 2), np.ascontiguousarray(d, dtype=np.float32))
            for p, d in chunks]
    k = len(keep)
    pp = (C.c_void_p * max(k, 1))(*[p.ctypes.data for p, _ in keep])
    dd = (C.c_void_p * max(k, 1))(*[d.ctypes.data for _, d in keep])
    counts = np.array([len(d) for _, d in keep] or [0], np.int64)
    m = np.zeros(1, np.int64)
    rc = lib().oracle_aveclust(pp, dd, counts.ctypes.data, k, num_reads, end_level, merge_path.encode(),
                               m.ctypes.data)
    if rc != 0:
        raise OSError(f"oracle aveclust failed ({rc})")
    return int(m[0])
