"""Build libcrispy_gb300.so and the drop-in kmerDist / genDist executables.

Everything is compiled in-tree for sm_103a only:
    crispy_gb300/lib/libcrispy_gb300.so
    crispy_gb300/bin/kmerDist, crispy_gb300/bin/genDist, crispy_gb300/bin/crispyDist,
    crispy_gb300/bin/preprocess, crispy_gb300/bin/crispyRun, crispy_gb300/bin/aveclust
Translation units compile in parallel; nothing here needs cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libcrispy_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")

CU_SOURCES = ["ctx.cu", "sort.cu", "kmer.cu", "gen.cu", "gen16.cu", "serve.cu", "noalloc.cu", "pre.cu"]
CXX_SOURCES = ["fasta.cpp", "pre_io.cpp", "clust.cpp"]
CLI = {"kmerDist": "cli_kmer.cpp", "genDist": "cli_gen.cpp", "crispyDist": "cli_pipe.cpp",
       "preprocess": "cli_pre.cpp", "crispyRun": "cli_run.cpp", "aveclust": "cli_clust.cpp",
       "sparsecut": "cli_cut.cpp"}

NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I", os.path.join(ROOT, "include"),
]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off",
             "-I", os.path.join(CUDA_HOME, "include"), "-I", os.path.join(ROOT, "include")]


def _run(cmd: list[str]) -> str:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(ROOT, "include", "crispy_gb300.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([NVCC] + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"])
    for exe, src in CLI.items():
        s = os.path.join(CSRC, src)
        out = os.path.join(BINDIR, exe)
        if _stale(out, [s, LIB] + hdrs):
            _run(["g++"] + CXX_FLAGS + [s, "-o", out, "-L", LIBDIR, "-lcrispy_gb300",
                                        "-Wl,-rpath,$ORIGIN/../lib"])
    text = "".join(logs)
    if verbose and text:
        print(text)
    return text


def build_oracle(with_reference: bool | None = None) -> None:
    """Compile the oracle (oracle/) and, where the reference tree exists,
    the reference's own CPU path into oracle/_ref/."""
    odir = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", odir])
    ref = os.environ.get("CRISPY_REFERENCE", "/root/reference")
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(ref, "src", "kmerDist"))
    if with_reference and shutil.which("g++"):
        _run(["make", "-s", "-C", odir, "ref", f"REF={ref}"])


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    build_oracle()
    print("built", LIB)
