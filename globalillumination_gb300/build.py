"""Builds libgishadow.so in-tree with nvcc (sm_103a) and g++.

The CUDA translation units are compiled with -fmad=false and IEEE division /
square root (nvcc defaults without --use_fast_math) and the host units with
-ffp-contract=off, so every FP32 operation of the passes rounds once in the
order the source writes it; the CPU oracle relies on the same rule.
Objects go to globalillumination_gb300/_build/, the library next to this
file.  Files are recompiled only when a source or header is newer than the
object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgishadow.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgishadow.so")


def _cuda_include(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh", ".inc")):
            hs.append(os.path.join(CSRC, f))
    return hs


def _stale(obj: str, src: str, headers: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if r.stdout.strip() and os.environ.get("GI_BUILD_VERBOSE"):
        sys.stdout.write(r.stdout)


def build_library(verbose: bool = False, extra_nvcc: list[str] | None = None) -> str:
    """Compiles every source under csrc/ and links libgishadow.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                         "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                         "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-I", CSRC, "-I", INCLUDE, *(extra_nvcc or []),
                         "-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", CSRC, "-I", INCLUDE, "-I", _cuda_include(nvcc),
                         "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def ptxas_report() -> str:
    """Registers / spills of every kernel (nvcc -Xptxas -v), for tuning."""
    nvcc = _nvcc()
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu"):
            r = subprocess.run([nvcc, *ARCH, "-O3", "-std=c++17", "-fmad=false", "-Xptxas", "-v",
                                "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE, "-c",
                                os.path.join(CSRC, f), "-o", os.devnull],
                               stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            out.append(r.stdout)
    return "\n".join(out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "ptxas":
        print(ptxas_report())
    else:
        build_library(verbose=True)
