"""ORACLE -- test infrastructure only.

CPU restatements of the reference's algorithms, used as the checker by tests/,
by ``__graft_entry__.smoke()`` and by bench.py's CPU-baseline leg.  Nothing in
the product (heterosync_gb300/) imports, links or runs anything from here.

  golden.c   the SyncPrims host golden (heterosync cuda/syncPrims/uvm/main.cu:33-51,
             1283-1308, 1633-1788) and the SLICE workload replay
  twins.cpp  std::thread / std::atomic runs of the same lock, semaphore and
             barrier algorithms (the host-thread CPU baseline)
  uts.c      the UTS binary-tree generator and its golden (cuda/uts/uvm/uts.cu:290-339)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or any(
                os.path.getmtime(os.path.join(HERE, f)) > os.path.getmtime(LIB)
                for f in os.listdir(HERE) if f.endswith((".c", ".cpp", ".h"))):
            build()
        L = ctypes.CDLL(LIB)
        L.hs_oracle_locs_mult.restype = ctypes.c_long
        L.hs_oracle_storage_words.restype = ctypes.c_long
        L.hs_oracle_golden.argtypes = [ctypes.c_int] * 8 + [ctypes.c_void_p, ctypes.c_long]
        L.hs_oracle_slice.argtypes = [ctypes.c_int] * 6 + [ctypes.c_void_p, ctypes.c_long]
        _lib = L
    return _lib


def storage_words(prim: int, T: int, L: int, num_tbs: int, nsm: int) -> int:
    return int(lib().hs_oracle_storage_words(prim, T, L, num_tbs, nsm))


def golden(prim: int, T: int, L: int, num_tbs: int, iters: int, repeats: int, nsm: int, inc: bool,
           init: np.ndarray) -> np.ndarray:
    """Reference golden replay of `init` (uint32 words; float bits in ref mode)."""
    s = np.array(init, dtype=np.uint32, copy=True)
    rc = lib().hs_oracle_golden(prim, T, L, num_tbs, iters, repeats, nsm, int(inc), s.ctypes.data, s.size)
    if rc:
        raise ValueError("oracle golden rejected the configuration")
    return s


def slice_replay(uniq: bool, L: int, num_tbs: int, iters: int, repeats: int, nsm: int,
                 init: np.ndarray) -> np.ndarray:
    s = np.array(init, dtype=np.uint32, copy=True)
    rc = lib().hs_oracle_slice(int(uniq), L, num_tbs, iters, repeats, nsm, s.ctypes.data, s.size)
    if rc:
        raise ValueError("oracle slice replay rejected the configuration")
    return s
