"""Build libhsgb300.so and the drop-in command-line programs for sm_103a.

Usage:  python -m heterosync_gb300.build [--force]

Outputs stay in the source tree (git-ignored):
  heterosync_gb300/lib/libhsgb300.so      the C-ABI library (include/hs/hs.h)
  heterosync_gb300/bin/allSyncPrims-1kernel
Translation units compile in parallel; an object is rebuilt only when a source
or header is newer than it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
LIBNAME = "libhsgb300.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", ARCH, "-Xcompiler", "-fPIC", "-I" + INC]

# CUDA translation units of the library
CU_SOURCES = [
    "hs_syncprims.cu",
    "hs_api.cu",
    "hs_probe.cu",
    "hs_cohort.cu",
    "hs_noalloc.cu",
    "hs_relaxed.cu",
    "hs_relaxed_api.cu",
    "hs_uts.cu",
    "hs_batch.cu",
    "hs_exchange.cu",
    "hs_serve.cu",
    "hs_uts_geo.cu",
]
# command-line programs: (output name, source)
PROGRAMS = [
    ("allSyncPrims-1kernel", "allSyncPrims.cpp"),
    ("hs-relaxed", "relaxed_cli.cpp"),
]
# names the multi-call relaxed-atomics/UTS program answers to (the reference's binaries)
RELAXED_NAMES = ["refCounter", "splitCounter", "seqlocks", "flags", "uts"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _headers() -> list[str]:
    out = []
    for d in (CSRC, os.path.join(INC, "hs")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s" % (" ".join(cmd), r.stdout))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile everything; return the library path."""
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    for d in (BUILD, LIB, BIN):
        os.makedirs(d, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = os.path.join(LIB, LIBNAME)
    if force or jobs or _stale(lib, objs):
        _run([nvcc, ARCH, "-shared", "-o", lib] + objs)
    for name, src in PROGRAMS:
        exe = os.path.join(BIN, name)
        s = os.path.join(CSRC, src)
        if force or _stale(exe, [s, lib] + headers):
            _run(["g++", "-std=c++17", "-O2", "-I" + INC, s, "-o", exe, "-L" + LIB, "-lhsgb300",
                  "-Wl,-rpath,$ORIGIN/../lib"])
    for alias in RELAXED_NAMES:
        dst = os.path.join(BIN, alias)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(os.path.join(BIN, "hs-relaxed")):
            if os.path.lexists(dst):
                os.remove(dst)
            shutil.copy2(os.path.join(BIN, "hs-relaxed"), dst)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
