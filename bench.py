#!/usr/bin/env python
"""Throughput of the kmerDist -> genDist hot path on GB300.

One step = one pass of both stages over one synthetic read set:
  kmerDist  all-pairs k-mer distance + fused threshold/compaction, survivors
            ordered as the reference orders .kpair;
  genDist   banded NW over those survivors, threshold, 589,824-pair windows,
            chunk flush, stable per-chunk sort, chunks delivered to host memory.

value  = all-pairs count n(n-1)/2 / step time, batched form, reads resident in
         HBM (the device rebuilds the k-mer structures inside the step).
e2e    = the same through the public C ABI from pinned host buffers, in the
         fused one-process form (crispyDist): the reads go up once, the
         kmerDist survivors reach genDist in HBM, and every genDist chunk
         comes back to host memory.  e2e_two_program adds the .kpair
         hand-over of the two-program form (survivor pairs fetched to the
         host and uploaded again to genDist), minus disk I/O.
plain  = the same pipeline with the plain from-scratch kernels (one thread
         per pair, one launch per reference stage / load window);
staged = the GB300 kernels launched the plain way (per stage / window),
         which splits the batched-vs-plain ratio into kernel design and
         scheduling.  The bits of all three forms are compared in every run
         and the comparison is reported.

--impl reference times the reference's CPU algorithm (the oracle port,
OpenMP on every host core) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from crispy_gb300 import synth  # noqa: E402

METRIC = "banded-NW GCUPS & k-mer pairs/s, batched vs plain; serve p50/p99, bit-exact"
UNIT = "k-mer pairs/s"
KMER_OPS_NOTE = "kmer: (Ta+Tb) int ops per pair; genDist: 10 int ops per band cell"

WORKLOADS = {
    # name: (synth workload, k, band)
    "uneven_100k": ("uneven_100k", 6, 10),
    "plain_20k": ("plain_20k", 6, 10),
    "small_1k": ("small_1k", 6, 10),
    "stress_500k": ("stress_500k", 8, 5),
}


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group(backend="gloo")
        return dist, ws, rank, local
    return None, 1, 0, local


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _read_set(name: str, rank: int):
    spec = synth.WORKLOADS[WORKLOADS[name][0]]
    if rank:
        spec = synth.ReadSetSpec(**{**spec.__dict__, "seed": spec.seed + 1000 * rank})
    return synth.make_read_set(spec)


# ---------------------------------------------------------------------------
# CPU baseline (the oracle port of the reference's CPU path)
# ---------------------------------------------------------------------------

def _cpu_sample(reads, k, band, m, workdir):
    """Run the oracle CLI on a deterministic subset of m reads; returns
    (kmer pairs/s, band-GCUPS, cores, description, seconds).

    Only oracle/ code runs here: the thresholds come from the oracle's
    restatement of kmerMain.cpp:43-48 / genMain.cpp:42-47, so the product
    library is never loaded by this leg."""
    import oracle

    if not os.path.exists(oracle.CLI_PATH):
        oracle.build()
    rng = np.random.default_rng(1234)
    idx = np.sort(rng.choice(len(reads), size=min(m, len(reads)), replace=False))
    sub = [reads[i] for i in idx]
    fa = os.path.join(workdir, "cpu_sample_Clean")
    synth.write_fasta(fa, sub)
    cores = os.cpu_count() or 1
    n = len(sub)
    # the full workload's thresholds (the subset keeps its read lengths)
    tk = oracle.default_threshold(len(reads), -1.0, 2)
    tg = oracle.default_threshold(len(reads), -1.0, 1)
    t0 = time.perf_counter()
    subprocess.run([oracle.CLI_PATH, "kmer", "-i", fa, "-k", str(k), "-t", repr(tk), "-n", str(cores)],
                   check=True, stdout=subprocess.DEVNULL)
    tkmer = time.perf_counter() - t0
    pairs = np.fromfile(fa + ".kpair", np.int32).reshape(-1, 2)
    lens = np.array([len(s) for s in sub])
    t0 = time.perf_counter()
    subprocess.run([oracle.CLI_PATH, "gen", "-i", fa, "-b", str(band), "-t", repr(tg), "-n", str(cores)],
                   check=True, stdout=subprocess.DEVNULL)
    tgen = time.perf_counter() - t0
    cells = sum(oracle.band_cells(int(lens[a]), int(lens[b]), band) for a, b in pairs) if len(pairs) else 0
    kpps = n * (n - 1) / 2 / tkmer
    gcups = cells / tgen / 1e9 if cells else None
    desc = (f"{n} of {len(reads)} reads (seeded subset), all {n*(n-1)//2} k-mer pairs "
            f"({tkmer:.2f} s) + genDist on its {len(pairs)} survivors ({cells} cells, {tgen:.2f} s)")
    return kpps, gcups, cores, desc, tkmer + tgen


def _cpu_pipeline_rate(n_sample_reads, seconds):
    """All-pairs rate of the whole pipeline, extrapolated from the sample.

    A uniform random subset of m of the n reads keeps each pair with
    probability m(m-1) / (n(n-1)), and the thresholds are the full set's, so
    both the all-pairs work and the survivors genDist aligns scale by the
    same factor: the full run takes about seconds * n(n-1) / (m(m-1)), and
    its all-pairs rate is the sample's own, m(m-1)/2 / seconds."""
    m = n_sample_reads
    return m * (m - 1) / 2 / seconds


def _config(workload: str, n: int, k: int, band: int, thr_k: float, thr_g: float, ws: int) -> dict:
    """The workload description both arms print."""
    return {"workload": workload, "n_reads": n, "k": k, "band": band,
            "kmer_threshold": thr_k, "gen_threshold": thr_g,
            "l2": "GPU arm: flushed (512 MB write) before every timed step",
            "parallelism": f"replicas x{ws}"}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args, dist, ws, rank, local):
    import torch

    import crispy_gb300 as cg

    torch.cuda.set_device(local)
    reads = _read_set(args.workload, rank)
    _, k, band = WORKLOADS[args.workload]
    buf, offs, lens = synth.pack_reads(reads)
    n = len(lens)
    n_pairs = n * (n - 1) // 2
    thr_k = cg.default_threshold(n, -1.0, 0)
    thr_g = cg.default_threshold(n, -1.0, 1)

    eng = cg.Engine(local, timing=True)
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    eng.kmer_prepare(buf, offs, lens, k)
    eng.gen_prepare(buf, offs, lens)
    int_peak_gops = eng.probe_int32_gops()
    lds_peak_gwf = eng.probe_lds128_wavefronts() / 1e9
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def pipeline(mode):
        eng.kmer_rebuild()
        kp = eng.kmer_run(thr_k, mode, False)
        st_k = eng.stats()
        chunks = eng.gen_run_from_kmer(band, thr_g, mode)
        st_g = eng.stats()
        return kp, chunks, st_k, st_g

    def timed(mode, steps, warm):
        for _ in range(warm):
            pipeline(mode)
        torch.cuda.synchronize()
        _barrier(dist)
        torch.cuda.synchronize()
        ms, kms, gms, launches, last = [], [], [], 0, None
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()          # L2 flush between timed iterations
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
            last = pipeline(mode)
            with torch.cuda.stream(stream):
                b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
            kms.append(last[2]["kmer_kernel_ms"])
            gms.append(last[3]["gen_kernel_ms"])
            launches += last[2]["kernels_launched"] + last[3]["kernels_launched"]
        torch.cuda.synchronize()
        _barrier(dist)
        return ms, kms, gms, launches, last

    clocks = ClockSampler(local)
    clocks.start()
    ms_b, kms_b, gms_b, launches_b, last_b = timed(cg.MODE_BATCHED, args.steps, args.warmup)
    clk = clocks.stop()
    other_steps = max(1, min(args.steps, 3))
    ms_s, kms_s, gms_s, _, last_s = timed(cg.MODE_STAGED, other_steps, 1)
    # the plain form takes tens of seconds per step beyond 2e10 pairs: one step
    big = n_pairs > 2e10
    ms_p, kms_p, gms_p, _, last_p = timed(cg.MODE_PLAIN, 1 if big else other_steps, 0 if big else 1)

    kp, chunks, st_k, st_g = last_b
    survivors = sum(len(c[2]) for c in chunks)

    def same(other):
        if kp != other[0] or len(chunks) != len(other[1]):
            return False
        return all(np.array_equal(a[1], b[1]) and np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
                   for a, b in zip(chunks, other[1]))

    # the bits of the three forms, compared here and reported as found
    identical = {"staged_vs_batched": bool(same(last_s)), "plain_vs_batched": bool(same(last_p))}
    if not all(identical.values()):
        print(f"bench: forms disagree: {identical}", file=sys.stderr)
    cells = st_g["gen_cells"]
    mean_t = float(np.mean(np.maximum(np.array(lens) - k + 1, 0)))

    step_s = _max_over_ranks(dist, float(np.mean(ms_b)) / 1e3)
    value = ws * n_pairs / step_s
    kmer_s = float(np.mean(kms_b)) / 1e3
    gen_s = float(np.mean(gms_b)) / 1e3
    plain_s = float(np.mean(ms_p)) / 1e3
    staged_s = float(np.mean(ms_s)) / 1e3

    # e2e through the public API from pinned host buffers: reads up once,
    # kmerDist survivors handed to genDist in HBM, genDist chunks read back
    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return t, v
    _keep = [pinned(buf), pinned(offs), pinned(lens)]
    pbuf, poffs, plens = (x[1] for x in _keep)

    def e2e_step():
        eng.kmer_prepare(pbuf, poffs, plens, k)
        c = eng.kmer_run(thr_k, cg.MODE_BATCHED, False)
        eng.gen_prepare_from_kmer()
        out = eng.gen_run_from_kmer(band, thr_g, cg.MODE_BATCHED)
        return c, out

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c, out = e2e_step()
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = _max_over_ranks(dist, float(np.mean(e2e_ms)) / 1e3)
    e2e_same = c == kp and len(out) == len(chunks) and all(
        np.array_equal(a[1], b[1]) and np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
        for a, b in zip(out, chunks))

    # the two-program hand-over (kmerDist writes .kpair, genDist reads it):
    # survivor pairs fetched to pinned host memory and uploaded again
    def e2e_two_program_step():
        eng.kmer_prepare(pbuf, poffs, plens, k)
        cnt = eng.kmer_run(thr_k, cg.MODE_BATCHED, False)
        kpairs, _ = eng.kmer_fetch(cnt, False)
        eng.gen_prepare(pbuf, poffs, plens)
        return kpairs, eng.gen_run(kpairs, band, thr_g, cg.MODE_BATCHED)

    e2e_two_program_step()
    two_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kpairs, out2 = e2e_two_program_step()
        torch.cuda.synchronize()
        two_ms.append((time.perf_counter() - t0) * 1e3)
    two_s = _max_over_ranks(dist, float(np.mean(two_ms)) / 1e3)
    # reads and offsets, per-read tuple counts, lengths and word offsets, per-group layouts
    h2d = buf.nbytes + offs.nbytes + n * 16 + (n // 32 + 1) * 40
    d2h = sum(len(o[2]) for o in out) * 12 + n * 8                  # chunks + per-read multiplicities

    kmer_ops = n_pairs * 2 * mean_t            # frozen: (Ta + Tb) per pair
    tune = []
    try:
        tune = cg.tune_report() or []
    except Exception:   # the report is informative only
        tune = []
    gen_kernel_name = ("gen16_kernel" if any(t.get("kernel") == "gen16_kernel" for t in tune)
                       else "gen_warp_kernel")
    gen_ops = cells * 10                        # frozen: 10 per band cell
    tile_kernel = ("kmer_tile8h_kernel + kmer_tile8_kernel" if k == 8 else "kmer_tile_kernel" if k == 7
                   else "kmer_tile128_kernel")
    # The tile kernels are bound by the L1 data pipe: one conflict-free
    # shared gather per column entry serves a block's row reads (128 rows of
    # 128-bit words at k <= 6, 64 of 64-bit words at k = 7, 32 of 32-bit words
    # at k = 8), and a warp's gather moves 32 x 16 / 8 / 4 bytes in 4 / 2 / 1
    # wavefronts, so one pass over a column's entries costs T_col / 1024
    # wavefronts per pair.  At k <= 6 the batched kernel's bound pass
    # gathers section 0 of every column and the full entries of the columns
    # left alive only: its work is those entries, a gather each (1/8
    # wavefront per lane), as the kernel counts them.
    single_wf = n_pairs * mean_t / 1024
    kb, kf = st_k.get("kmer_bound_entries", 0), st_k.get("kmer_full_entries", 0)
    bound_pass = kb > 0
    kmer_wf = (kb + kf) / 8 if bound_pass else single_wf
    work = (f"{kmer_wf / n_pairs:.4f} L1 wavefronts per k-mer pair: the level entries the bound pass "
            f"(section 0 of every column) and the full passes (the columns left alive) gather, "
            f"a 128-bit gather per entry and 128 row reads" if bound_pass
            else f"{mean_t / 1024:.4f} L1 wavefronts per k-mer pair (T_col / 1024)")
    roof_k = {"kernel": tile_kernel, "bound": "l1_shared", "unit": "Gwavefront/s",
              "achieved": kmer_wf / kmer_s / 1e9, "peak": lds_peak_gwf,
              "frac": kmer_wf / kmer_s / 1e9 / lds_peak_gwf,
              "work_per_unit": work, "traffic": None,
              "peak_source": "measured: crispy_probe_lds128 (conflict-free 128-bit shared gathers), this run"}
    if bound_pass:
        rg = (n + 127) // 128
        items = sum(n - 128 * r for r in range(rg))     # (128-row group, column) pairs
        roof_k["bound_pass"] = {
            "bound_entries": int(kb), "full_entries": int(kf),
            "full_columns": int(st_k.get("kmer_full_columns", 0)), "rounds": int(st_k.get("kmer_rounds", 0)),
            "row_group_columns": int(items),
            "alive_fraction": st_k.get("kmer_full_columns", 0) / max(1, items),
            "note": "per (128-row group, column): section 0 of the column's entries, then all of them "
                    "where a row may still pass (m <= m0 + Ta - a0)"}
        roof_k["single_pass_view"] = {
            "work_per_unit": f"{mean_t / 1024:.4f} L1 wavefronts per k-mer pair (T_col / 1024), every "
                             "entry of every column",
            "achieved": single_wf / kmer_s / 1e9, "frac": single_wf / kmer_s / 1e9 / lds_peak_gwf,
            "note": "the one-pass algorithm's work over this kernel's time: above the bound pass's own "
                    "fraction by the work the bound pass skips"}
    roof_k["frozen_scalar_view"] = {
        "work_per_unit": f"{2*mean_t:.1f} int ops per k-mer pair (Ta + Tb)", "unit": "Gop/s",
        "achieved": kmer_ops / kmer_s / 1e9, "peak": int_peak_gops,
        "frac": kmer_ops / kmer_s / 1e9 / int_peak_gops,
        "note": "the sorted-merge work model; the bit-sliced kernel serves many rows per op, so this "
                "view exceeds 1 and is not a roofline"}
    roof_g = {"kernel": gen_kernel_name, "bound": "int32", "unit": "Gop/s",
              "achieved": gen_ops / gen_s / 1e9, "peak": int_peak_gops,
              "frac": gen_ops / gen_s / 1e9 / int_peak_gops,
              "work_per_unit": "10 ops per band cell", "traffic": None,
              "peak_source": "measured: crispy_probe_int32 (IADD3/LOP3 chains), this run"}
    # the dense count-vector formulation: 4^k/4 packed count words per read,
    # 2 ops per word and pair (a min and an add)
    dense_ops = (4 ** k) // 4 * 2
    roof_k["frozen_scalar_view"]["dense_count_vector_view"] = {
        "work_per_unit": f"{dense_ops} ops per k-mer pair", "unit": "Gop/s",
        "achieved": n_pairs * dense_ops / kmer_s / 1e9, "peak": int_peak_gops,
        "frac": n_pairs * dense_ops / kmer_s / 1e9 / int_peak_gops}
    dominant = roof_g if gen_s >= kmer_s else roof_k
    _attach_traffic(roof_k, roof_g, n_pairs, cells, k)
    _attach_hbm_view(roof_k, kmer_s)
    _attach_hbm_view(roof_g, gen_s)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded 16S-like generator, preprocess order)",
        "config": _config(args.workload, n, k, band, thr_k, thr_g, ws),
        "mode": "batched",
        "kmer_pairs_per_s": n_pairs / kmer_s, "kmer_survivors": kp,
        "gen_gcups": cells / gen_s / 1e9, "gen_cells": cells, "gen_survivors": survivors,
        "kmer_kernel_ms": kmer_s * 1e3, "gen_kernel_ms": gen_s * 1e3,
        "plain": {"kernels": "one thread per pair, launched per reference stage / load window",
                  "ms_per_step": plain_s * 1e3, "value": n_pairs / plain_s,
                  "kmer_kernel_ms": float(np.mean(kms_p)), "gen_kernel_ms": float(np.mean(gms_p))},
        "staged": {"kernels": "bit-sliced tiles + warp DP, launched per stage / window",
                   "ms_per_step": staged_s * 1e3, "value": n_pairs / staged_s,
                   "kmer_kernel_ms": float(np.mean(kms_s)), "gen_kernel_ms": float(np.mean(gms_s))},
        "batched_over_plain": plain_s / step_s,
        "batched_over_staged": staged_s / step_s,
        "outputs_identical_across_forms": identical,
        "e2e": {"value": ws * n_pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                "path": "fused one-process form (crispyDist): survivors handed to genDist in HBM",
                "outputs_identical_to_value_run": bool(e2e_same)},
        "e2e_two_program": {
            "value": ws * n_pairs / two_s, "unit": UNIT, "ms_per_step": two_s * 1e3,
            "h2d_bytes_per_step": int(h2d + buf.nbytes + offs.nbytes + n * 4 + kpairs.nbytes),
            "d2h_bytes_per_step": int(kpairs.nbytes + sum(len(o[2]) for o in out2) * 12),
            "path": "kmerDist then genDist as two programs minus disk I/O: .kpair pairs fetched "
                    "to the host and uploaded to genDist with the reads",
            "outputs_identical_to_value_run": bool(
                len(out2) == len(chunks) and all(np.array_equal(a[1], b[1]) for a, b in zip(out2, chunks)))},
        "gpu_launches": int(launches_b),
        "roofline": dominant, "roofline_kmer": roof_k, "roofline_gen": roof_g,
        "clocks": clk,
    }
    line["autotune"] = tune
    if not args.no_serve:
        line["serve"] = serve_bench(args, local)
    if rank == 0 and not args.no_configs:
        line["configs"] = config_bench(args, local)
    if rank == 0 and not args.no_pre:
        line["preprocess"] = preprocess_bench(args, local)
        line["aveclust"] = clust_bench(args, local, chunks, n)
        line["crispy_run"] = run_bench(args)
    if rank == 0 and not args.no_cpu_baseline:
        with tempfile.TemporaryDirectory() as td:
            kpps, gcups, cores, desc, secs = _cpu_sample(reads, k, band, args.cpu_sample_reads, td)
        m = min(args.cpu_sample_reads, n)
        line["cpu_baseline"] = {"value": _cpu_pipeline_rate(m, secs), "unit": UNIT,
                                "cores": cores, "kind": "port", "sample": desc,
                                "kmer_pairs_per_s": kpps, "gen_gcups": gcups,
                                "note": "all-pairs rate of the sample's kmerDist + genDist run; a random "
                                        "subset keeps every pair with the same probability, so the full "
                                        "run's rate is the sample's"}
    eng.close()
    return line


def config_bench(args, local: int) -> dict:
    """The other benchmark read sets, timed beside the headline one:
    plain_20k (20,000 reads, k = 6, band 10) in the batched, staged and plain
    forms, and the stress set (496,820 reads, k = 8, band 5) in the batched
    and staged forms (its plain form takes about a minute per step).  Per
    form: CUDA-event step time over a few steps (L2 flushed before each) and
    the all-pairs rate; the forms' outputs are compared bit for bit."""
    import torch

    import crispy_gb300 as cg

    out = {}
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    names = {cg.MODE_BATCHED: "batched", cg.MODE_STAGED: "staged", cg.MODE_PLAIN: "plain"}
    for name, forms in (("plain_20k", (cg.MODE_BATCHED, cg.MODE_STAGED, cg.MODE_PLAIN)),
                        ("stress_500k", (cg.MODE_BATCHED, cg.MODE_STAGED))):
        _, k, band = WORKLOADS[name]
        reads = synth.make_read_set(name)
        buf, offs, lens = synth.pack_reads(reads)
        n = len(lens)
        n_pairs = n * (n - 1) // 2
        thr_k = cg.default_threshold(n, -1.0, 0)
        thr_g = cg.default_threshold(n, -1.0, 1)
        res = {"n_reads": n, "k": k, "band": band}
        outputs = {}
        with cg.Engine(local, timing=True) as eng:
            stream = torch.cuda.Stream()
            eng.set_stream(stream.cuda_stream)
            eng.kmer_prepare(buf, offs, lens, k)
            eng.gen_prepare_from_kmer()
            for mode in forms:
                steps, warm = (3, 2) if mode == cg.MODE_BATCHED else (2, 1) if mode == cg.MODE_STAGED else (1, 0)
                times, last = [], None
                for it in range(warm + steps):
                    with torch.cuda.stream(stream):
                        flush.zero_()
                        a = torch.cuda.Event(enable_timing=True)
                        b = torch.cuda.Event(enable_timing=True)
                        a.record(stream)
                    eng.kmer_rebuild()
                    kp = eng.kmer_run(thr_k, mode, False)
                    chunks = eng.gen_run_from_kmer(band, thr_g, mode)
                    with torch.cuda.stream(stream):
                        b.record(stream)
                    b.synchronize()
                    if it >= warm:
                        times.append(a.elapsed_time(b))
                    last = (kp, chunks)
                ms = float(np.mean(times))
                res[names[mode]] = {"ms_per_step": ms, "value": n_pairs / (ms / 1e3), "steps": steps}
                outputs[names[mode]] = last
        b_kp, b_ch = outputs["batched"]
        res["kmer_survivors"] = b_kp
        res["gen_survivors"] = int(sum(len(c[2]) for c in b_ch))
        for label, (kp, ch) in outputs.items():
            if label == "batched":
                continue
            res[f"{label}_identical_to_batched"] = bool(
                kp == b_kp and len(ch) == len(b_ch) and
                all(np.array_equal(x[1], y[1]) and np.array_equal(x[2].view(np.uint32), y[2].view(np.uint32))
                    for x, y in zip(ch, b_ch)))
            res[f"batched_over_{label}"] = res[label]["ms_per_step"] / res["batched"]["ms_per_step"]
        out[name] = res
    return out


def preprocess_bench(args, local: int) -> dict:
    """preprocess (the step before kmerDist) on the workload's raw reads.

    The raw FASTA is the generator's reads before deduplication, 60 columns
    per line.  Timed per run: the record parse on the host
    (crispy_raw_load), crispy_preprocess on the GPU (upload, filters, sort,
    duplicate merge, download of the kept order) and the _Clean / .frq
    writer; against the oracle's single-threaded restatement of the
    reference (std::list-style stable sort of strings, fprintf output) on
    the same file.  Both outputs are compared byte for byte.
    """
    import crispy_gb300 as cg
    import oracle

    reads = synth.generate(synth.WORKLOADS[WORKLOADS[args.workload][0]])
    out = {"input_reads": len(reads)}
    with tempfile.TemporaryDirectory() as td:
        raw_path = os.path.join(td, "raw.fa")
        with open(raw_path, "wb") as f:
            for i, s in enumerate(reads):
                f.write(b">read_%d synthetic\n" % i)
                for a in range(0, len(s), 60):
                    f.write(s[a:a + 60] + b"\n")
        out["input_bytes"] = os.path.getsize(raw_path)
        eng = cg.Engine(local)
        times = []
        for it in range(4):
            t0 = time.perf_counter()
            raw = cg.RawReads(raw_path)
            t1 = time.perf_counter()
            idx, freq, st = eng.preprocess(raw)
            t2 = time.perf_counter()
            raw.write(idx, freq, os.path.join(td, "gpu_Clean"))
            t3 = time.perf_counter()
            raw.close()
            if it:   # the first run is the warm-up
                times.append((t1 - t0, t2 - t1, t3 - t2, t3 - t0))
        eng.close()
        parse_s, dev_s, write_s, e2e_s = (float(np.mean(x)) for x in zip(*times))
        t0 = time.perf_counter()
        c = oracle.preprocess(raw_path, os.path.join(td, "cpu_Clean"))
        cpu_s = time.perf_counter() - t0
        same = all(open(os.path.join(td, "gpu_Clean" + e), "rb").read() ==
                   open(os.path.join(td, "cpu_Clean" + e), "rb").read() for e in ("", ".frq"))
    out.update({"kept_reads": int(st["kept"]), "merges": int(st["merges"]),
                "e2e_ms": e2e_s * 1e3, "parse_ms": parse_s * 1e3,
                "device_ms": dev_s * 1e3, "write_ms": write_s * 1e3,
                "reads_per_s": len(reads) / e2e_s,
                "cpu_baseline": {"ms": cpu_s * 1e3, "cores": 1, "kind": "port",
                                 "sample": "the whole raw file"},
                "outputs_identical": bool(same and c["kept"] == st["kept"])})
    return out


def clust_bench(args, local: int, chunks, n: int) -> dict:
    """aveclust (the step after genDist) on genDist's chunks.

    Timed: crispy_aveclust on this workload's chunks, and on the chunks of
    plain_20k (19,954 reads) beside the oracle's step-by-step restatement of
    the reference (which scans every node per merge: it would take minutes
    on 100,000 reads, so the CPU comparison uses the 20k set).  The _Merge
    files of the engine and the oracle are compared byte for byte.
    """
    import crispy_gb300 as cg
    import oracle

    out = {}
    with tempfile.TemporaryDirectory() as td:
        ch = [(c[1], c[2]) for c in chunks]
        t0 = time.perf_counter()
        st = cg.aveclust(ch, n, os.path.join(td, "wl"))
        out[args.workload] = {"reads": n, "edges": int(sum(len(c[1]) for c in ch)),
                              "merges": int(st["merges"]), "ms": (time.perf_counter() - t0) * 1e3,
                              "phases_ms": {"edges": st["ms_edges"], "update_min": st["ms_update"],
                                            "merges": st["ms_merges"], "levels_and_output": st["ms_output"]}}
        reads = synth.make_read_set("plain_20k")
        buf, offs, lens = synth.pack_reads(reads)
        m = len(lens)
        with cg.Engine(local) as eng:
            eng.kmer_prepare(buf, offs, lens, 6)
            eng.kmer_run(cg.default_threshold(m, -1.0, 0), cg.MODE_BATCHED, False)
            eng.gen_prepare_from_kmer()
            ch20 = [(c[1], c[2]) for c in eng.gen_run_from_kmer(10, cg.default_threshold(m, -1.0, 1))]
        t0 = time.perf_counter()
        st20 = cg.aveclust(ch20, m, os.path.join(td, "p20"))
        ours = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        om = oracle.aveclust(ch20, m, os.path.join(td, "oracle_Merge"))
        cpu = (time.perf_counter() - t0) * 1e3
        same = open(os.path.join(td, "p20_Merge"), "rb").read() == open(os.path.join(td, "oracle_Merge"), "rb").read()
        out["plain_20k"] = {"reads": m, "edges": int(sum(len(c[1]) for c in ch20)), "merges": int(st20["merges"]),
                            "ms": ours, "cpu_baseline": {"ms": cpu, "cores": 1, "kind": "port",
                                                         "sample": "the whole 20k-read chunk set"},
                            "merge_file_identical": bool(same and om == st20["merges"])}
    return out


def run_bench(args) -> dict:
    """crispyRun: crispy.sh from the raw FASTA through aveclust in one
    process (preprocess, kmerDist, genDist, aveclust; every file written).
    Wall time of the executable on the workload's raw reads, best of 2 after
    one warm-up, and the time it prints itself."""
    import subprocess as sp

    import crispy_gb300 as cg

    reads = synth.generate(synth.WORKLOADS[WORKLOADS[args.workload][0]])
    _, k, band = WORKLOADS[args.workload]
    out = {"input_reads": len(reads), "k": k, "band": band}
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "raw.fa"), "wb") as f:
            for i, s in enumerate(reads):
                f.write(b">read_%d synthetic\n" % i)
                for a in range(0, len(s), 60):
                    f.write(s[a:a + 60] + b"\n")
        walls = []
        for it in range(3):
            t0 = time.perf_counter()
            p = sp.run([os.path.join(cg.BIN_DIR, "crispyRun"), "raw.fa", str(k), str(band)], cwd=td,
                       stdout=sp.PIPE, stderr=sp.STDOUT)
            if p.returncode != 0:
                return {"error": p.stdout.decode(errors="replace")[-300:]}
            if it:
                walls.append(time.perf_counter() - t0)
        files = sorted(f for f in os.listdir(td) if f != "raw.fa")
        out.update({"wall_ms": min(walls) * 1e3, "files": files,
                    "stdout_tail": p.stdout.decode(errors="replace").strip().splitlines()[-3:]})
    return out


def serve_bench(args, local: int) -> dict:
    """Continuous-batching server on a Poisson stream of clustering jobs.

    Jobs: read counts log-uniform in [500, 50000], lengths N(250, 20), k = 6,
    band 1/10, default thresholds, 120 GB HBM admission budget.  Saturated
    throughput comes from a closed loop (all jobs queued at once); latency
    percentiles from open-loop Poisson arrivals at 50 % and 90 % of it.
    """
    import crispy_gb300 as cg

    rng = np.random.default_rng(4242)
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), size=args.serve_jobs)).astype(int)
    pool = []
    for i, n in enumerate(sizes):
        spec = synth.ReadSetSpec(int(n), max(4, int(n) // 50), 260, "normal", 250, 20, 6, 9000 + i)
        pool.append(synth.pack_reads(synth.make_read_set(spec)))
    pairs = [len(p[2]) * (len(p[2]) - 1) // 2 for p in pool]
    out = {"jobs": len(pool), "slots": args.serve_slots, "hbm_budget_gb": 120,
           "reads_per_job": {"min": int(min(len(p[2]) for p in pool)),
                             "max": int(max(len(p[2]) for p in pool))}}
    with cg.Server(local, 120 << 30, args.serve_slots) as srv:
        # warm-up: one small and one large job
        for p in (pool[int(np.argmin(sizes))], pool[int(np.argmax(sizes))]):
            j = srv.submit(*p)
            srv.wait(j)
            srv.result(j)
        srv.reset_stats()
        t0 = time.perf_counter()
        ids = [srv.submit(*p) for p in pool]
        for j in ids:
            srv.wait(j)
            srv.result(j)
        sat_s = time.perf_counter() - t0
        sat = srv.stats()
        rate = len(pool) / sat_s
        out["saturated"] = {"jobs_per_s": rate, "pairs_per_s": sum(pairs) / sat_s,
                            "p50_ms": sat["p50_ms"], "p99_ms": sat["p99_ms"]}
        for frac in (0.5, 0.9):
            srv.reset_stats()
            gaps = rng.exponential(1.0 / (frac * rate), size=len(pool))
            ids = []
            t0 = time.perf_counter()
            nxt = t0
            for p, g in zip(pool, gaps):
                nxt += g
                delay = nxt - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                ids.append(srv.submit(*p))
            for j in ids:
                srv.wait(j)
                srv.result(j)
            el = time.perf_counter() - t0
            st = srv.stats()
            out[f"load_{int(frac * 100)}"] = {"offered_jobs_per_s": frac * rate,
                                              "jobs_per_s": len(pool) / el,
                                              "pairs_per_s": sum(pairs) / el,
                                              "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"]}
    return out


def _attach_hbm_view(roof, seconds):
    """The same launch against the measured HBM copy bandwidth: its DRAM
    traffic per launch over its duration.  Shows how far from HBM-bound the
    kernel is (neither stage is: their binding pipes are integer / L1)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if roof.get("traffic") is None or not os.path.exists(p) or seconds <= 0:
        return
    try:
        peak = float(json.load(open(p))["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return
    gbs = roof["traffic"] / seconds / 1e9
    roof["hbm_view"] = {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "peak_source": "measured: MEASURED_PEAKS.json hbm_gbs"}


def _attach_traffic(roof_k, roof_g, n_pairs, cells, k):
    """DRAM bytes per launch from a committed ncu summary, scaled by units
    (k = 8 has kmerDist figures of its own, from the stress set)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(p):
        return
    try:
        t = json.load(open(p))
    except (OSError, ValueError):
        return
    tk = t.get("k8", t) if k == 8 else t
    if "kmer_bytes_per_pair" in tk:
        roof_k["traffic"] = tk["kmer_bytes_per_pair"] * n_pairs
        roof_k["traffic_source"] = tk.get("source")
    if "gen_bytes_per_cell" in t:
        roof_g["traffic"] = t["gen_bytes_per_cell"] * cells
        roof_g["traffic_source"] = t.get("source")
    if "kmer_shared_wavefronts_per_pair" in tk:
        roof_k["ncu_shared_wavefronts_per_pair"] = tk["kmer_shared_wavefronts_per_pair"]
    # the hardware pipe each kernel saturates, from the same ncu captures
    if "kmer_binding_pipe" in tk:
        roof_k["ncu_binding_pipe"] = tk["kmer_binding_pipe"]
    if "gen_binding_pipe" in t:
        roof_g["ncu_binding_pipe"] = t["gen_binding_pipe"]


def run_reference(args, dist, ws, rank):
    """The reference's CPU algorithm on this host's cores (oracle port,
    OpenMP), each step a bounded sample of the workload: a seeded subset of
    the reads, all of its pairs through kmerDist and the survivors through
    genDist.  Only oracle/ code runs (the product library is never loaded);
    the line's config is the GPU arm's, thresholds included."""
    if rank != 0:
        return None
    import oracle

    reads = _read_set(args.workload, 0)
    _, k, band = WORKLOADS[args.workload]
    n = len(reads)
    m = min(args.cpu_sample_reads, n)
    thr_k = oracle.default_threshold(n, -1.0, 2)
    thr_g = oracle.default_threshold(n, -1.0, 1)
    rates = []
    with tempfile.TemporaryDirectory() as td:
        for i in range(args.warmup + args.steps):
            kpps, gcups, cores, desc, secs = _cpu_sample(reads, k, band, m, td)
            if i >= args.warmup:
                rates.append((kpps, gcups, secs))
    kpps = float(np.mean([r[0] for r in rates]))
    gcups_list = [r[1] for r in rates if r[1]]
    gcups = float(np.mean(gcups_list)) if gcups_list else None
    secs = float(np.mean([r[2] for r in rates]))
    value = _cpu_pipeline_rate(m, secs)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": secs * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded 16S-like generator, preprocess order)",
            "config": _config(args.workload, n, k, band, thr_k, thr_g, ws),
            "mode": "reference CPU algorithm (oracle port), one sample per step",
            "kmer_pairs_per_s": kpps, "gen_gcups": gcups,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": desc,
                             "note": "all-pairs rate of the sample's kmerDist + genDist run; a random "
                                     "subset keeps every pair with the same probability, so the full "
                                     "run's rate is the sample's"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("CRISPY_BENCH_WORKLOAD", "uneven_100k"),
                    choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-sample-reads", type=int, default=_env_int("CRISPY_CPU_SAMPLE", 12000))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-pre", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the plain_20k / stress_500k lines")
    ap.add_argument("--serve-jobs", type=int, default=240)
    ap.add_argument("--serve-slots", type=int, default=4)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist, ws, rank, local = _dist()
    if args.impl == "reference":
        line = run_reference(args, dist, ws, rank)
    else:
        line = run_ours(args, dist, ws, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
