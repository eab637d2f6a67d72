"""crispy_gb300 -- GB300 (sm_103a) engine for CRiSPy's kmerDist and genDist.

The engine is the C-ABI library ``lib/libcrispy_gb300.so`` (declared in
``include/crispy_gb300.h``); this module binds it with ctypes, the same way
a Python caller of the reference's stages would.  There is no CPU fallback:
if the library is missing or cannot reach an sm_103a GPU, every call raises.

Stage mirror of the reference (src/kmerDist, src/genDist):
    compute_kmer_dist(fasta, k, thr, dists)   -> writes <fasta>.kpair [.kdist]
    compute_gen_dist(fasta, band, thr)        -> writes <fasta>.npair_N / .ndist_N
and the lower-level ``Engine`` for device-resident work.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libcrispy_gb300.so")
BIN_DIR = os.path.join(_PKG, "bin")

OK, E_INPUT, E_OOM, E_DEVICE, E_TIMEOUT, E_STATE, E_IO, E_UNSUPPORTED = range(8)
MODE_PLAIN, MODE_BATCHED, MODE_STAGED = 0, 1, 2
GEN_WINDOW = 589824
MAX_READ_LEN = 2048
MAX_NUM_READS = 1024 * 1024

_STATUS = {0: "OK", 1: "E_INPUT", 2: "E_OOM", 3: "E_DEVICE", 4: "E_TIMEOUT", 5: "E_STATE",
           6: "E_IO", 7: "E_UNSUPPORTED"}


class CrispyError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


SINK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_float), C.c_int64)


class Stats(C.Structure):
    _fields_ = [("kmer_kernel_ms", C.c_double), ("kmer_launches", C.c_int64),
                ("gen_kernel_ms", C.c_double), ("gen_launches", C.c_int64),
                ("total_ms", C.c_double), ("kmer_pairs", C.c_int64),
                ("kmer_survivors", C.c_int64), ("gen_pairs", C.c_int64),
                ("gen_cells", C.c_int64), ("gen_survivors", C.c_int64),
                ("kernels_launched", C.c_int64), ("graph_launches", C.c_int64),
                ("kmer_spilled", C.c_int64), ("kmer_bound_entries", C.c_int64),
                ("kmer_full_entries", C.c_int64), ("kmer_full_columns", C.c_int64),
                ("kmer_rounds", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_P = C.c_void_p
_i64p = C.POINTER(C.c_int64)


class ClustStats(C.Structure):
    _fields_ = [("pairs_read", C.c_int64), ("merges", C.c_int64), ("roots", C.c_int32),
                ("singletons", C.c_int32), ("end_level", C.c_float), ("report", C.c_char * 2048),
                ("ms_edges", C.c_double), ("ms_update", C.c_double), ("ms_merges", C.c_double),
                ("ms_output", C.c_double)]


class PreOpts(C.Structure):
    _fields_ = [("length_check", C.c_int), ("sd_allowed", C.c_double), ("primer", C.c_char_p),
                ("max_mismatches", C.c_int)]


class PreStats(C.Structure):
    _fields_ = [("length_discards", C.c_int32), ("primer_discards", C.c_int32),
                ("merges", C.c_int32), ("kept", C.c_int32), ("length_reads", C.c_int32),
                ("min_len0", C.c_int32), ("max_len0", C.c_int32), ("min_len", C.c_int32),
                ("max_len", C.c_int32), ("ave_len", C.c_double), ("sd", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}

# name -> (restype, argtypes); exactly the declarations of include/crispy_gb300.h
PROTOTYPES = {
    "crispy_version": (C.c_char_p, []),
    "crispy_last_error": (C.c_char_p, [_P]),
    "crispy_ctx_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "crispy_ctx_destroy": (C.c_int, [_P]),
    "crispy_ctx_set_stream": (C.c_int, [_P, _P]),
    "crispy_reads_load_fasta": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
    "crispy_reads_view": (C.c_int, [_P, C.POINTER(C.c_char_p), C.POINTER(_i64p),
                                    C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32)]),
    "crispy_reads_free": (None, [_P]),
    "crispy_default_threshold": (C.c_float, [C.c_int, C.c_float, C.c_int]),
    "crispy_array_dim": (C.c_int, [C.c_int]),
    "crispy_kmer_prepare": (C.c_int, [_P, _P, _P, _P, C.c_int, C.c_int]),
    "crispy_kmer_rebuild": (C.c_int, [_P]),
    "crispy_kmer_run": (C.c_int, [_P, C.c_float, C.c_int, C.c_int, _i64p]),
    "crispy_kmer_fetch": (C.c_int, [_P, _P, _P, C.c_int64, _i64p]),
    "crispy_kmer_stream": (C.c_int, [_P, SINK, _P]),
    "crispy_gen_prepare": (C.c_int, [_P, _P, _P, _P, C.c_int]),
    "crispy_gen_prepare_from_kmer": (C.c_int, [_P]),
    "crispy_gen_run": (C.c_int, [_P, _P, C.c_int64, C.c_int, C.c_float, C.c_int, SINK, _P, _i64p]),
    "crispy_gen_run_from_kmer": (C.c_int, [_P, C.c_int, C.c_float, C.c_int, SINK, _P, _i64p]),
    "crispy_gen_align": (C.c_int, [_P, _P, C.c_int64, C.c_int, C.c_int, _P, _P, _P, _P]),
    "crispy_gen_align_noalloc": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, _P, C.c_int64, C.c_int,
                                           _P, _P, _P, _P, _P]),
    "crispy_raw_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
    "crispy_raw_view": (C.c_int, [_P, C.POINTER(C.c_char_p), C.POINTER(_i64p),
                                  C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_uint8)),
                                  C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "crispy_raw_label": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_int32)]),
    "crispy_raw_free": (None, [_P]),
    "crispy_preprocess": (C.c_int, [_P, _P, _P, _P, _P, C.c_int32, C.POINTER(PreOpts), _P, _P,
                                    C.POINTER(PreStats)]),
    "crispy_pre_write": (C.c_int, [_P, _P, _P, C.c_int32, C.c_char_p, C.c_int]),
    "crispy_kmer_prepare_from_pre": (C.c_int, [_P, _P, C.c_int]),
    "crispy_gen_prepare_from_pre": (C.c_int, [_P, _P]),
    "crispy_aveclust": (C.c_int, [C.POINTER(_P), C.POINTER(_P), _P, C.c_int, C.c_int, C.c_float,
                                  C.c_char_p, C.c_char_p, C.POINTER(ClustStats)]),
    "crispy_sparsecut": (C.c_int, [C.c_char_p, C.c_int, _P, C.c_int, C.POINTER(ClustStats)]),
    "crispy_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "crispy_set_timing": (C.c_int, [_P, C.c_int]),
    "crispy_probe_int32": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "crispy_probe_lds128": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "crispy_tune_report": (C.c_int, [C.c_char_p, C.c_size_t]),
    "crispy_ctx_set_mem_cap": (C.c_int, [_P, C.c_size_t]),
    "crispy_ctx_mem_in_use": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "crispy_ctx_trim": (C.c_int, [_P]),
    "crispy_server_create": (C.c_int, [C.c_int, C.c_size_t, C.c_int, C.POINTER(_P)]),
    "crispy_server_destroy": (C.c_int, [_P]),
    "crispy_server_submit": (C.c_int, [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_float,
                                       C.c_float, C.POINTER(C.c_uint64)]),
    "crispy_server_wait": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(C.c_int)]),
    "crispy_server_result": (C.c_int, [_P, C.c_uint64, SINK, _P, _i64p, _i64p]),
    "crispy_server_cancel": (C.c_int, [_P, C.c_uint64]),
    "crispy_server_job_memory": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                                           C.POINTER(C.c_int)]),
    "crispy_server_job_bytes": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_size_t)]),
    "crispy_server_stats": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), _i64p, _i64p]),
    "crispy_server_stats_reset": (C.c_int, [_P]),
    "crispy_server_last_error": (C.c_char_p, [_P]),
}

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, JOB_CANCELLED = range(5)

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load the engine; raise (never fall back) when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CrispyError(E_DEVICE, f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def default_threshold(n: int, user_thr: float = -1.0, stage: int = 0) -> float:
    return float(load_library().crispy_default_threshold(n, user_thr, stage))


def array_dim(n: int) -> int:
    return int(load_library().crispy_array_dim(n))


def tune_report() -> list:
    """The autotuner's cached choices (list of dicts)."""
    import json

    buf = C.create_string_buffer(1 << 16)
    load_library().crispy_tune_report(buf, len(buf))
    return json.loads(buf.value.decode() or "[]")


def read_fasta(path: str, flavour: int = 0):
    """Parse like the reference's readFile: (bytes buffer, offsets, lengths)."""
    lib = load_library()
    h = _P()
    rc = lib.crispy_reads_load_fasta(path.encode(), flavour, C.byref(h))
    if rc != OK:
        raise CrispyError(rc, lib.crispy_last_error(None).decode())
    try:
        buf = C.c_char_p()
        off = _i64p()
        ln = C.POINTER(C.c_int32)()
        n = C.c_int32()
        mx = C.c_int32()
        lib.crispy_reads_view(h, C.byref(buf), C.byref(off), C.byref(ln), C.byref(n), C.byref(mx))
        cnt = n.value
        offs = np.ctypeslib.as_array(off, shape=(cnt,)).copy() if cnt else np.zeros(0, np.int64)
        lens = np.ctypeslib.as_array(ln, shape=(cnt,)).copy() if cnt else np.zeros(0, np.int32)
        total = int(offs[-1] + lens[-1]) if cnt else 0
        data = np.frombuffer(C.string_at(buf, total), dtype=np.uint8).copy()
    finally:
        lib.crispy_reads_free(h)
    return data, offs, lens


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


class RawReads:
    """Records of a raw FASTA / FASTQ file as preprocess's readFile collects
    them (crispy_raw_load); the handle owns the memory."""

    def __init__(self, path: str, fastq: bool = False):
        self.lib = load_library()
        self.fastq = bool(fastq)
        h = _P()
        rc = self.lib.crispy_raw_load(path.encode(), 1 if fastq else 0, C.byref(h))
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_last_error(None).decode())
        self.h = h
        buf = C.c_char_p()
        off = _i64p()
        ln = C.POINTER(C.c_int32)()
        fr = C.POINTER(C.c_uint8)()
        n = C.c_int32()
        rec = C.c_int32()
        self.lib.crispy_raw_view(h, C.byref(buf), C.byref(off), C.byref(ln), C.byref(fr), C.byref(n),
                                 C.byref(rec))
        self.n, self.records = n.value, rec.value
        # views into the handle's memory (valid while it lives)
        self._buf_addr = C.cast(buf, C.c_void_p).value
        self.offsets = np.ctypeslib.as_array(off, shape=(self.n,)) if self.n else np.zeros(0, np.int64)
        self.lengths = np.ctypeslib.as_array(ln, shape=(self.n,)) if self.n else np.zeros(0, np.int32)
        self.freq = np.ctypeslib.as_array(fr, shape=(self.n,)) if self.n else np.zeros(0, np.uint8)

    def seq(self, i: int) -> bytes:
        return C.string_at(self._buf_addr + int(self.offsets[i]), int(self.lengths[i]))

    def label(self, i: int) -> bytes:
        p = C.c_char_p()
        n = C.c_int32()
        rc = self.lib.crispy_raw_label(self.h, i, C.byref(p), C.byref(n))
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_last_error(None).decode())
        return C.string_at(C.cast(p, C.c_void_p).value, n.value) if n.value else b""

    def write(self, index: np.ndarray, freq: np.ndarray, out_path: str):
        index = np.ascontiguousarray(index, dtype=np.int32)
        freq = np.ascontiguousarray(freq, dtype=np.int32)
        rc = self.lib.crispy_pre_write(self.h, _ptr(index), _ptr(freq), len(index), out_path.encode(),
                                       1 if self.fastq else 0)
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_last_error(None).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.crispy_raw_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """One context on one GPU (the C ABI's crispy_ctx)."""

    def __init__(self, device: int = 0, timing: bool = False):
        self.lib = load_library()
        h = _P()
        rc = self.lib.crispy_ctx_create(device, C.byref(h))
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_last_error(None).decode())
        self.h = h
        if timing:
            self.lib.crispy_set_timing(self.h, 1)

    def close(self):
        if getattr(self, "h", None):
            self.lib.crispy_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_last_error(self.h).decode())

    def set_mem_cap(self, nbytes: int):
        self._check(self.lib.crispy_ctx_set_mem_cap(self.h, nbytes))

    def mem_in_use(self) -> int:
        v = C.c_size_t()
        self._check(self.lib.crispy_ctx_mem_in_use(self.h, C.byref(v)))
        return v.value

    def trim(self):
        self._check(self.lib.crispy_ctx_trim(self.h))

    def set_stream(self, stream_handle: int | None):
        self._check(self.lib.crispy_ctx_set_stream(self.h, stream_handle))

    def set_timing(self, on: bool):
        self._check(self.lib.crispy_set_timing(self.h, 1 if on else 0))

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.crispy_get_stats(self.h, C.byref(s)))
        return s.as_dict()

    # ---- kmerDist ----
    def kmer_prepare(self, buf: np.ndarray, offs: np.ndarray, lens: np.ndarray, k: int = 6):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        lens = np.ascontiguousarray(lens, dtype=np.int32)
        self._check(self.lib.crispy_kmer_prepare(self.h, _ptr(buf), _ptr(offs), _ptr(lens),
                                                 len(lens), k))

    def kmer_rebuild(self):
        self._check(self.lib.crispy_kmer_rebuild(self.h))

    def probe_int32_gops(self) -> float:
        g = C.c_double()
        self._check(self.lib.crispy_probe_int32(self.h, C.byref(g)))
        return g.value

    def probe_lds128_wavefronts(self) -> float:
        """Conflict-free 128-bit shared-load throughput, L1 wavefronts/s."""
        w = C.c_double()
        self._check(self.lib.crispy_probe_lds128(self.h, C.byref(w)))
        return w.value

    def kmer_run(self, thr: float, mode: int = MODE_BATCHED, dists: bool = True) -> int:
        n = C.c_int64()
        self._check(self.lib.crispy_kmer_run(self.h, thr, mode, 1 if dists else 0, C.byref(n)))
        return n.value

    def kmer_fetch(self, count: int, dists: bool = True):
        pairs = np.empty((max(count, 1), 2), dtype=np.int32)
        d = np.empty(max(count, 1), dtype=np.float32) if dists else None
        got = C.c_int64()
        self._check(self.lib.crispy_kmer_fetch(self.h, _ptr(pairs), _ptr(d), count, C.byref(got)))
        return pairs[:got.value], (d[:got.value] if dists else None)

    # ---- preprocess ----
    def preprocess(self, raw: "RawReads", sd: float | None = None, primer: bytes | None = None,
                   max_mm: int = 2):
        """Filters and duplicate merge on the device (crispy_preprocess).
        Returns (record index, merged frequency, stats dict) in _Clean order."""
        n = raw.n
        index = np.empty(max(n, 1), np.int32)
        freq = np.empty(max(n, 1), np.int32)
        opts = PreOpts(1 if sd is not None else 0, float(sd if sd is not None else 1.0), primer, int(max_mm))
        st = PreStats()
        self._check(self.lib.crispy_preprocess(self.h, raw._buf_addr, _ptr(raw.offsets), _ptr(raw.lengths),
                                               _ptr(raw.freq), n, C.byref(opts), _ptr(index), _ptr(freq),
                                               C.byref(st)))
        k = st.kept
        return index[:k].copy(), freq[:k].copy(), st.as_dict()

    def kmer_prepare_from_pre(self, raw: "RawReads", k: int = 6):
        """kmer_prepare on the reads the last preprocess kept (no file, no upload)."""
        self._check(self.lib.crispy_kmer_prepare_from_pre(self.h, raw.h, k))

    def gen_prepare_from_pre(self, raw: "RawReads"):
        self._check(self.lib.crispy_gen_prepare_from_pre(self.h, raw.h))

    # ---- genDist ----
    def gen_prepare(self, buf: np.ndarray, offs: np.ndarray, lens: np.ndarray):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        lens = np.ascontiguousarray(lens, dtype=np.int32)
        self._check(self.lib.crispy_gen_prepare(self.h, _ptr(buf), _ptr(offs), _ptr(lens), len(lens)))

    def gen_prepare_from_kmer(self):
        """Pack the reads the last kmer_prepare left on the device (no second upload)."""
        self._check(self.lib.crispy_gen_prepare_from_kmer(self.h))

    def gen_align(self, pairs: np.ndarray, band: int, mode: int = MODE_BATCHED):
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        n = len(pairs)
        dist = np.empty(max(n, 1), np.float32)
        score = np.empty(max(n, 1), np.int32)
        ml = np.empty(max(n, 1), np.int32)
        al = np.empty(max(n, 1), np.int32)
        self._check(self.lib.crispy_gen_align(self.h, _ptr(pairs), n, band, mode, _ptr(dist),
                                              _ptr(score), _ptr(ml), _ptr(al)))
        return dist[:n], score[:n], ml[:n], al[:n]

    def _collect(self):
        chunks = []

        def cb(user, chunk_id, pairs, dists, count):
            p = np.ctypeslib.as_array(C.cast(pairs, C.POINTER(C.c_uint32)), shape=(count, 2)).copy() if count else np.zeros((0, 2), np.uint32)
            d = np.ctypeslib.as_array(dists, shape=(count,)).copy() if count else np.zeros(0, np.float32)
            chunks.append((chunk_id, p, d))
            return 0

        return chunks, SINK(cb)

    def gen_run(self, pairs: np.ndarray, band: int, thr: float, mode: int = MODE_BATCHED):
        """Returns the list of chunks [(chunk_id, uint32 pairs[N,2], float32 dists[N])]."""
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        chunks, cb = self._collect()
        ns = C.c_int64()
        self._check(self.lib.crispy_gen_run(self.h, _ptr(pairs), len(pairs), band, thr, mode, cb,
                                            None, C.byref(ns)))
        return chunks

    def gen_run_from_kmer(self, band: int, thr: float, mode: int = MODE_BATCHED):
        chunks, cb = self._collect()
        ns = C.c_int64()
        self._check(self.lib.crispy_gen_run_from_kmer(self.h, band, thr, mode, cb, None, C.byref(ns)))
        return chunks


class Server:
    """Continuous-batching job server (crispy_server_* of the C ABI)."""

    def __init__(self, device: int = 0, budget_bytes: int = 0, slots: int = 4):
        self.lib = load_library()
        h = _P()
        rc = self.lib.crispy_server_create(device, budget_bytes, slots, C.byref(h))
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.crispy_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != OK:
            raise CrispyError(rc, self.lib.crispy_server_last_error(self.h).decode())

    def submit(self, buf, offs, lens, k=6, band=10, kmer_thr=-1.0, gen_thr=-1.0) -> int:
        buf = np.ascontiguousarray(buf, np.uint8)
        offs = np.ascontiguousarray(offs, np.int64)
        lens = np.ascontiguousarray(lens, np.int32)
        jid = C.c_uint64()
        self._check(self.lib.crispy_server_submit(self.h, _ptr(buf), _ptr(offs), _ptr(lens), len(lens),
                                                  k, band, kmer_thr, gen_thr, C.byref(jid)))
        return jid.value

    def wait(self, job: int, timeout_ms: int = -1) -> int:
        st = C.c_int()
        rc = self.lib.crispy_server_wait(self.h, job, timeout_ms, C.byref(st))
        if rc == E_TIMEOUT:
            return st.value
        self._check(rc)
        return st.value

    def result(self, job: int):
        """(kmer survivor count, [(chunk_id, pairs, dists)]) of a finished job."""
        chunks = []

        def cb(user, chunk_id, pairs, dists, count):
            p = np.ctypeslib.as_array(C.cast(pairs, C.POINTER(C.c_uint32)), shape=(count, 2)).copy() if count else np.zeros((0, 2), np.uint32)
            d = np.ctypeslib.as_array(dists, shape=(count,)).copy() if count else np.zeros(0, np.float32)
            chunks.append((chunk_id, p, d))
            return 0

        f = SINK(cb)
        kp = C.c_int64()
        gp = C.c_int64()
        self._check(self.lib.crispy_server_result(self.h, job, f, None, C.byref(kp), C.byref(gp)))
        return kp.value, chunks

    def job_memory(self, job: int) -> dict:
        """Memory of the run that served a finished job (call before result())."""
        r = C.c_size_t()
        nd = C.c_size_t()
        cs = C.c_int()
        self._check(self.lib.crispy_server_job_memory(self.h, job, C.byref(r), C.byref(nd), C.byref(cs)))
        return {"reserved": r.value, "needed": nd.value, "cohort_size": cs.value}

    def cancel(self, job: int):
        self._check(self.lib.crispy_server_cancel(self.h, job))

    def stats(self) -> dict:
        p50 = C.c_double()
        p99 = C.c_double()
        nj = C.c_int64()
        npairs = C.c_int64()
        self._check(self.lib.crispy_server_stats(self.h, C.byref(p50), C.byref(p99), C.byref(nj),
                                                 C.byref(npairs)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "jobs": nj.value, "pairs": npairs.value}

    def reset_stats(self):
        self._check(self.lib.crispy_server_stats_reset(self.h))


def server_job_bytes(lens, k: int = 6) -> int:
    """Device bytes the server's admission reserves for a job with these read lengths."""
    lens = np.ascontiguousarray(lens, dtype=np.int32)
    b = C.c_size_t()
    rc = load_library().crispy_server_job_bytes(_ptr(lens), len(lens), k, C.byref(b))
    if rc != OK:
        raise CrispyError(rc, "server_job_bytes")
    return b.value


def compute_kmer_dist(fasta: str, k: int = 6, thr: float = -1.0, dists: bool = False,
                      mode: int = MODE_BATCHED, engine: Engine | None = None) -> int:
    """kmerDist -i fasta -k k [-t thr] [-d]: writes <fasta>.kpair (and .kdist)."""
    buf, offs, lens = read_fasta(fasta, 0)
    t = default_threshold(len(lens), thr, 0)
    eng = engine or Engine()
    eng.kmer_prepare(buf, offs, lens, k)
    n = eng.kmer_run(t, mode, dists)
    pairs, d = eng.kmer_fetch(n, dists)
    pairs.astype(np.int32).tofile(fasta + ".kpair")
    if dists:
        d.astype(np.float32).tofile(fasta + ".kdist")
    return n


def compute_gen_dist(fasta: str, band: int = 2, thr: float = -1.0, mode: int = MODE_BATCHED,
                     engine: Engine | None = None) -> int:
    """genDist -i fasta -b band [-t thr]: writes <fasta>.npair_N / .ndist_N."""
    buf, offs, lens = read_fasta(fasta, 1)
    t = default_threshold(len(lens), thr, 1)
    raw = np.fromfile(fasta + ".kpair", dtype=np.int32)
    pairs = raw[: (len(raw) // 2) * 2].reshape(-1, 2)
    eng = engine or Engine()
    eng.gen_prepare(buf, offs, lens)
    total = 0
    for cid, p, d in eng.gen_run(pairs, band if band > 0 else 2, t, mode):
        p.astype(np.uint32).tofile(f"{fasta}.npair_{cid}")
        d.astype(np.float32).tofile(f"{fasta}.ndist_{cid}")
        total += len(d)
    return total


def aveclust(chunks, num_reads: int, out_base: str, end_level: float = -1.0,
             edge_out: str | None = None) -> dict:
    """Average-linkage clustering of genDist chunks [(uint32 pairs[N,2], float32 dists[N])]
    (crispy_aveclust); writes out_base_Merge, .Cluster, .Cluster_List."""
    lib = load_library()
    keep = [(np.ascontiguousarray(p, dtype=np.uint32).reshape(-1, 2), np.ascontiguousarray(d, dtype=np.float32))
            for p, d in chunks]
    k = len(keep)
    pp = (_P * max(k, 1))(*[p.ctypes.data for p, _ in keep])
    dd = (_P * max(k, 1))(*[d.ctypes.data for _, d in keep])
    counts = np.array([len(d) for _, d in keep] or [0], np.int64)
    st = ClustStats()
    rc = lib.crispy_aveclust(pp, dd, counts.ctypes.data, k, num_reads, end_level, out_base.encode(),
                             edge_out.encode() if edge_out else None, C.byref(st))
    if rc != OK:
        raise CrispyError(rc, lib.crispy_last_error(None).decode())
    return {"pairs_read": st.pairs_read, "merges": st.merges, "roots": st.roots,
            "singletons": st.singletons, "end_level": st.end_level, "report": st.report.decode(),
            "ms_edges": st.ms_edges, "ms_update": st.ms_update, "ms_merges": st.ms_merges,
            "ms_output": st.ms_output}


def sparsecut(in_base: str, num_reads: int, cutoffs) -> dict:
    """Clusters of the dendrogram in_base_Merge at each cutoff distance
    (crispy_sparsecut); writes in_base.Cluster and in_base.Cluster_List."""
    lib = load_library()
    cut = np.ascontiguousarray(cutoffs, dtype=np.float32).reshape(-1)
    st = ClustStats()
    rc = lib.crispy_sparsecut(in_base.encode(), num_reads, cut.ctypes.data if len(cut) else None, len(cut),
                              C.byref(st))
    if rc != OK:
        raise CrispyError(rc, lib.crispy_last_error(None).decode())
    return {"merges": st.merges, "roots": st.roots, "singletons": st.singletons, "report": st.report.decode()}
