"""ORACLE -- test infrastructure only.

CPU restatements of the reference's algorithms, used as the checker by tests/,
by ``__graft_entry__.smoke()`` and by bench.py's CPU-baseline leg.  Nothing in
the product (heterosync_gb300/) imports, links or runs anything from here.

  golden.c   the SyncPrims host golden (heterosync cuda/syncPrims/uvm/main.cu:33-51,
             1283-1308, 1633-1788) and the SLICE workload replay
  twins.cpp  std::thread / std::atomic runs of the same lock, semaphore and
             barrier algorithms (the host-thread CPU baseline)
  uts.c      the UTS binary-tree generator and its golden (cuda/uts/uvm/uts.cu:290-339)
  uts_geo.c  geometric UTS tree with a SHA-1 node generator, counted depth-first
             (no reference implementation: parity unpinned; SHA-1 checked
             against hashlib)
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
        # pointers always as void*: without argtypes ctypes passes a Python int as a 32-bit C int
        L.hs_oracle_uts_tree.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.hs_oracle_uts_frontier.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]
        L.hs_oracle_storage_words.restype = ctypes.c_long
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


# ---------------------------------------------------------------------------
# The reference's own kernels (oracle/_ref/*.cubin, built by build_ref.sh from
# the unmodified reference sources) run through oracle/ref_runner.cpp.
# ---------------------------------------------------------------------------
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(HERE, "_build", "libhsref.so")
_ref = None


def ref_module(threads: int) -> str:
    return os.path.join(REF_DIR, "syncprims_t%d_sm100.cubin" % threads)


def ref_available(threads: int = 32) -> bool:
    return os.path.exists(ref_module(threads)) and os.path.exists(REF_LIB)


def _reflib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            build()
        L = ctypes.CDLL(REF_LIB)
        L.hs_ref_last_error.restype = ctypes.c_char_p
        L.hs_ref_run.argtypes = [ctypes.c_char_p] + [ctypes.c_int] * 7 + [ctypes.c_void_p, ctypes.c_long,
                                                                           ctypes.POINTER(ctypes.c_float)]
        _ref = L
    return _ref


def ref_device():
    n, t = ctypes.c_int(), ctypes.c_int()
    rc = _reflib().hs_ref_device(ctypes.byref(n), ctypes.byref(t))
    if rc:
        raise RuntimeError(_reflib().hs_ref_last_error().decode())
    return n.value, t.value


def ref_run(prim: int, T: int, L: int, num_tbs: int, iters: int, repeats: int, init: np.ndarray,
            sync_each: bool = True):
    """Run the reference kernel; returns (final storage uint32, elapsed ms over all repeats).
    Raises RuntimeError when the runner refuses (a launch that would deadlock) or fails."""
    if not os.path.exists(ref_module(T)):
        raise FileNotFoundError("no reference module for %d threads per TB" % T)
    s = np.array(init, dtype=np.uint32, copy=True)
    ms = ctypes.c_float()
    rc = _reflib().hs_ref_run(ref_module(T).encode(), T, prim, L, num_tbs, iters, repeats, int(sync_each),
                              s.ctypes.data, s.size, ctypes.byref(ms))
    if rc:
        raise RuntimeError("reference run refused/failed (%d): %s" % (rc, _reflib().hs_ref_last_error().decode()))
    return s, float(ms.value)


def ref_refcounter_module() -> str:
    return os.path.join(REF_DIR, "refcounter_sm100.cubin")


def ref_refcounter(num_sharers: int, num_tbs: int, tb_size: int, num_repeats: int):
    """The reference's own refCounter kernel (one launch, refCounter.cu:24-82);
    returns (counters0, counters1, del0, del1, ms)."""
    if not os.path.exists(ref_refcounter_module()):
        raise FileNotFoundError("no reference refCounter module")
    L = _reflib()
    if not hasattr(L, "_rc_ready"):
        L.hs_ref_refcounter.argtypes = [ctypes.c_char_p] + [ctypes.c_int] * 4 + [ctypes.c_void_p] * 4 + \
            [ctypes.POINTER(ctypes.c_float)]
        L._rc_ready = True
    thrs = num_tbs * tb_size
    nc = thrs // num_sharers
    c0, c1 = np.zeros(nc, np.uint32), np.zeros(nc, np.uint32)
    d0, d1 = np.zeros(thrs, np.uint32), np.zeros(thrs, np.uint32)
    ms = ctypes.c_float()
    rc = L.hs_ref_refcounter(ref_refcounter_module().encode(), num_sharers, num_tbs, tb_size, num_repeats,
                             c0.ctypes.data, c1.ctypes.data, d0.ctypes.data, d1.ctypes.data, ctypes.byref(ms))
    if rc:
        raise RuntimeError("reference refCounter run refused/failed (%d): %s" % (rc, L.hs_ref_last_error().decode()))
    return c0, c1, d0, d1, float(ms.value)


def twin_run(prim: int, T: int, L: int, num_tbs: int, iters: int, repeats: int, nsm: int, mode: int,
             init: np.ndarray, threads: int = 0):
    """Host std::thread run of the same algorithm; returns (final storage, seconds)."""
    L_ = lib()
    if not hasattr(L_, "_twin_ready"):
        L_.hs_twin_run.argtypes = [ctypes.c_int] * 8 + [ctypes.c_void_p, ctypes.c_long, ctypes.c_int,
                                                         ctypes.POINTER(ctypes.c_double)]
        L_._twin_ready = True
    s = np.array(init, dtype=np.uint32, copy=True)
    secs = ctypes.c_double()
    rc = L_.hs_twin_run(prim, T, L, num_tbs, iters, repeats, nsm, mode, s.ctypes.data, s.size, threads,
                        ctypes.byref(secs))
    if rc:
        raise ValueError("twin rejected the configuration")
    return s, float(secs.value)


# ---------------------------------------------------------------------------
# UTS (uts.c): reference tree generator, golden and initial frontier.
# ---------------------------------------------------------------------------
UTS_NODE = np.dtype([("value", "<u4"), ("depth", "<u4"), ("to_add", "<u4"), ("child_a", "<i4"), ("child_b", "<i4")])


def uts_tree(num_nodes: int, fertility: int, seed: int = 200):
    L_ = lib()
    tree = np.zeros(num_nodes, dtype=UTS_NODE)
    lv, ls, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
    rc = L_.hs_oracle_uts_tree(num_nodes, fertility, seed, tree.ctypes.data, ctypes.byref(lv),
                               ctypes.byref(ls), ctypes.byref(rs))
    if rc:
        raise ValueError("bad UTS tree size")
    return tree, lv.value, ls.value, rs.value


def uts_frontier(tree, cores_used: int):
    L_ = lib()
    fr = np.zeros(cores_used * 16 + 2, dtype=np.int32)
    cnt, proc = ctypes.c_int(), ctypes.c_uint()
    rc = L_.hs_oracle_uts_frontier(tree.ctypes.data, tree.size, cores_used, fr.ctypes.data, ctypes.byref(cnt),
                                   ctypes.byref(proc))
    if rc:
        raise ValueError("frontier cannot be filled")
    return fr[:cnt.value].copy(), proc.value


def exchange_expected(buffers: np.ndarray, episodes: int) -> np.ndarray:
    """Tree barrier with local exchange: each episode moves CTA b's buffer to
    CTA (b + 1) mod n (the exchange phase of main.cu:153-270 works on the data
    of another TB between two barriers), so after `episodes` episodes CTA b
    holds the initial buffer of CTA (b - episodes) mod n."""
    n = buffers.shape[0]
    return np.roll(buffers, episodes % n if n else 0, axis=0)


# Geometric SHA-1 UTS (uts_geo.c).
def sha1(msg: bytes) -> bytes:
    assert len(msg) <= 55
    out = ctypes.create_string_buffer(20)
    lib().hs_oracle_sha1.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
    lib().hs_oracle_sha1(msg, len(msg), out)
    return out.raw


def geo_table(b: float, n: int = 128):
    t = np.zeros(n, dtype=np.uint32)
    lib().hs_oracle_geo_table.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
    nz = lib().hs_oracle_geo_table(b, t.ctypes.data, n)
    return t, nz


def geo_root(seed: int) -> bytes:
    out = ctypes.create_string_buffer(20)
    lib().hs_oracle_geo_root.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
    lib().hs_oracle_geo_root(seed, out)
    return out.raw


def geo_child(parent: bytes, i: int) -> bytes:
    out = ctypes.create_string_buffer(20)
    lib().hs_oracle_geo_child.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_void_p]
    lib().hs_oracle_geo_child(parent, i, out)
    return out.raw


def geo_count(seed: int, depth_limit: int, b: float = 4.0):
    """(nodes, leaves, deepest level) of the geometric tree."""
    n, lv, md = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_int()
    lib().hs_oracle_geo_count.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
    rc = lib().hs_oracle_geo_count(seed, depth_limit, b, ctypes.byref(n), ctypes.byref(lv), ctypes.byref(md))
    if rc:
        raise ValueError("bad geometric tree parameters")
    return n.value, lv.value, md.value
