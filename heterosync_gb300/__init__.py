"""heterosync_gb300 -- GB300-native (sm_103a) HeteroSync hot path.

Python mirror of the C ABI in include/hs/hs.h (libhsgb300.so, loaded with
ctypes).  The names follow the reference (heterosync cuda/syncPrims/uvm/main.cu):
primitives are addressed by the same strings as the ``allSyncPrims-1kernel``
command line ("faMutex", "spinSemEBO10", "lfTreeBarrUniqLocalExch", ...), and a
run takes the same four numbers (numLdSt, numTBs, numCSIters plus the threads
per TB the reference fixes at compile time).

There is no CPU fallback: if the CUDA library has not been built, importing
works (so the host-side helpers stay usable) but every call that needs the
library raises ``HsLibraryMissing``.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional

__all__ = [
    "HsError", "HsLibraryMissing", "RunConfig", "RunResult", "PRIM_NAMES", "prim_id", "prim_name",
    "prim_label", "storage_words", "expected_storage", "run", "lib", "lib_path", "launch_count",
    "device_info", "MODE_REF", "MODE_INC", "MODE_SLICE",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_PKG, "lib", "libhsgb300.so")

MODE_REF, MODE_INC, MODE_SLICE = 0, 1, 2
_MODES = {"ref": MODE_REF, "inc": MODE_INC, "slice": MODE_SLICE}

HS_OK, HS_EINVAL, HS_ETIMEDOUT, HS_ENORES, HS_ECUDA, HS_ENODEV, HS_EMISMATCH = range(7)
RUN_SYNC_EACH, RUN_KEEP_STATE, RUN_NO_CLUSTER, RUN_REGISTER_CS, RUN_GRAPH, RUN_NO_COHORT = 1, 2, 4, 8, 16, 32
RUN_CLUSTER_CS = 64
RUN_NO_GROUP_CTA = 128

# Reference names and ids, main.cu:1224-1256.
PRIM_NAMES = {
    "atomicTreeBarrUniq": 0, "atomicTreeBarrUniqLocalExch": 1, "lfTreeBarrUniq": 2,
    "lfTreeBarrUniqLocalExch": 3, "spinMutex": 4, "spinMutexEBO": 5, "sleepMutex": 6, "faMutex": 7,
    "spinSem1": 8, "spinSem2": 9, "spinSem10": 10, "spinSem120": 11, "spinSemEBO1": 12,
    "spinSemEBO2": 13, "spinSemEBO10": 14, "spinSemEBO120": 15, "spinMutexUniq": 20,
    "spinMutexEBOUniq": 21, "sleepMutexUniq": 22, "faMutexUniq": 23, "spinSemUniq1": 24,
    "spinSemUniq2": 25, "spinSemUniq10": 26, "spinSemUniq120": 27, "spinSemEBOUniq1": 28,
    "spinSemEBOUniq2": 29, "spinSemEBOUniq10": 30, "spinSemEBOUniq120": 31,
}
# The HIP build's extra primitives (hip/syncPrims/uvm/main.hip.cpp:2056-2083):
# priority semaphores and sense-reversing atomic tree barriers, run on the CUDA
# primitive's kernel (hs_prim_base) with the same final storage.
HIP_PRIM_NAMES = {
    "PRspinSem1": 16, "PRspinSem2": 17, "PRspinSem10": 18, "PRspinSem120": 19,
    "PRspinSemEBO1": 32, "PRspinSemEBO2": 33, "PRspinSemEBO10": 34, "PRspinSemEBO120": 35,
    "atomicTreeBarrUniqSRB": 37, "atomicTreeBarrUniqLocalExchSRB": 38, "atomicTreeBarrUniqNaiveSRB": 39,
    "atomicTreeBarrUniqLocalExchNaiveSRB": 40, "atomicTreeBarrUniqNaiveAllSRB": 41,
    "atomicTreeBarrUniqLocalExchNaiveAllSRB": 42,
}
_ID_TO_NAME = {v: k for k, v in list(PRIM_NAMES.items()) + list(HIP_PRIM_NAMES.items())}


class HsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class HsLibraryMissing(HsError):
    pass


class _RunConfig(ctypes.Structure):
    _fields_ = [
        ("prim", ctypes.c_int), ("num_ldst", ctypes.c_int), ("num_tbs", ctypes.c_int),
        ("num_iters", ctypes.c_int), ("threads", ctypes.c_int), ("repeats", ctypes.c_int),
        ("mode", ctypes.c_int), ("nsm", ctypes.c_int), ("backoff_min_ns", ctypes.c_uint),
        ("backoff_max_ns", ctypes.c_uint), ("backoff_unit_ns", ctypes.c_uint),
        ("timeout_ns", ctypes.c_ulonglong), ("skip_tb", ctypes.c_int), ("flags", ctypes.c_int),
    ]


class _RunResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int), ("dev_error_bits", ctypes.c_uint), ("dev_error_site", ctypes.c_uint),
        ("elapsed_ms", ctypes.c_float), ("avg_ms", ctypes.c_float), ("h2d_ms", ctypes.c_float),
        ("d2h_ms", ctypes.c_float), ("ops", ctypes.c_ulonglong), ("launches", ctypes.c_uint),
        ("cluster", ctypes.c_int), ("cohort", ctypes.c_int), ("tbs_per_cta", ctypes.c_int),
    ]


_lib = None
_ctx = None


def lib_path() -> str:
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    """The loaded libhsgb300.so (raises HsLibraryMissing if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise HsLibraryMissing(HS_ENODEV, "libhsgb300.so not built: run `python -m heterosync_gb300.build` "
                                   "(expected at %s)" % _LIB_PATH)
        L = ctypes.CDLL(_LIB_PATH)
        L.hs_last_error.restype = ctypes.c_char_p
        L.hs_status_string.restype = ctypes.c_char_p
        L.hs_prim_name.restype = ctypes.c_char_p
        L.hs_launch_count.restype = ctypes.c_ulonglong
        L.hs_prim_id.argtypes = [ctypes.c_char_p]
        L.hs_storage_words.argtypes = [ctypes.POINTER(_RunConfig), ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
        L.hs_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(_RunConfig), ctypes.c_void_p, ctypes.c_int,
                             ctypes.c_void_p, ctypes.POINTER(_RunResult)]
        L.hs_expected_storage.argtypes = [ctypes.POINTER(_RunConfig), ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_size_t]
        L.hs_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.hs_ctx_destroy.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _err(status: int) -> HsError:
    L = lib()
    return HsError(status, "%s: %s" % (L.hs_status_string(status).decode(), L.hs_last_error().decode()))


def launch_count() -> int:
    """Kernels launched by the library in this process."""
    return int(lib().hs_launch_count())


def device_info(device: int = 0) -> dict:
    vals = [ctypes.c_int() for _ in range(4)]
    s = lib().hs_device_info(device, *[ctypes.byref(v) for v in vals])
    if s:
        raise _err(s)
    return {"nsm": vals[0].value, "cc": (vals[1].value, vals[2].value), "max_threads_per_block": vals[3].value}


def prim_id(name) -> int:
    if isinstance(name, int):
        if name not in _ID_TO_NAME:
            raise ValueError("unknown syncPrim id %d" % name)
        return name
    if name in PRIM_NAMES:
        return PRIM_NAMES[name]
    if name in HIP_PRIM_NAMES:
        return HIP_PRIM_NAMES[name]
    raise ValueError("ERROR: Unknown synchronization primitive: %s" % name)


def prim_base(prim) -> tuple:
    """(CUDA base primitive id, variant) a primitive runs as."""
    v = ctypes.c_int()
    lib().hs_prim_base.argtypes = [ctypes.c_int, ctypes.c_void_p]
    b = lib().hs_prim_base(prim_id(prim), ctypes.byref(v))
    return b, v.value


def prim_name(pid: int) -> str:
    return _ID_TO_NAME[pid]


def prim_label(prim, num_iters: int) -> str:
    buf = ctypes.create_string_buffer(128)
    lib().hs_prim_label(prim_id(prim), num_iters, buf, 128)
    return buf.value.decode()


def is_barrier(prim) -> bool:
    return prim_id(prim) <= 3


def is_semaphore(prim) -> bool:
    p = prim_id(prim)
    return 8 <= p <= 15 or 24 <= p <= 31


def sem_count(prim) -> int:
    name = prim_name(prim_id(prim))
    for n in ("120", "10", "2", "1"):
        if ("Sem" in name) and name.endswith(n):
            return int(n)
    return 0


@dataclass
class RunConfig:
    """One run: `repeats` launches of `num_tbs` TBs x `threads` threads, each TB
    doing `num_iters` critical sections (or barrier episodes) of `num_ldst`
    loads/stores per thread.  Defaults are the reference's (T=32, 10 repeats)."""
    prim: object = "faMutex"
    num_ldst: int = 10
    num_tbs: int = 8
    num_iters: int = 100
    threads: int = 32
    repeats: int = 10
    mode: object = "ref"
    nsm: int = 0
    backoff_min_ns: int = 1
    backoff_max_ns: int = 1024
    backoff_unit_ns: int = 0
    timeout_ns: int = 0
    skip_tb: int = -1
    flags: int = 0

    def to_c(self) -> _RunConfig:
        mode = _MODES[self.mode] if isinstance(self.mode, str) else int(self.mode)
        return _RunConfig(prim_id(self.prim), self.num_ldst, self.num_tbs, self.num_iters, self.threads,
                          self.repeats, mode, self.nsm, self.backoff_min_ns, self.backoff_max_ns,
                          self.backoff_unit_ns, self.timeout_ns, self.skip_tb, self.flags)


@dataclass
class RunResult:
    status: int
    dev_error_bits: int
    dev_error_site: int
    elapsed_ms: float
    avg_ms: float
    h2d_ms: float
    d2h_ms: float
    ops: int
    launches: int
    cluster: int = 1
    cohort: int = 0
    tbs_per_cta: int = 1

    @property
    def ops_per_s(self) -> float:
        return self.ops / (self.elapsed_ms * 1e-3) if self.elapsed_ms > 0 else float("inf")


def storage_words(cfg: RunConfig, nsm: int = 0) -> int:
    w = ctypes.c_size_t()
    c = cfg.to_c()
    s = lib().hs_storage_words(ctypes.byref(c), nsm, ctypes.byref(w))
    if s:
        raise _err(s)
    return int(w.value)


def expected_storage(cfg: RunConfig, init, nsm: int = 0):
    """Expected final storage (numpy uint32) from the initial contents."""
    import numpy as np
    init = np.ascontiguousarray(init, dtype=np.uint32)
    out = np.empty_like(init)
    c = cfg.to_c()
    s = lib().hs_expected_storage(ctypes.byref(c), nsm, init.ctypes.data, out.ctypes.data, init.size)
    if s:
        raise _err(s)
    return out


def _context():
    global _ctx
    if _ctx is None:
        h = ctypes.c_void_p()
        s = lib().hs_ctx_create(0, ctypes.byref(h))
        if s:
            raise _err(s)
        _ctx = h
    return _ctx


def run(cfg: RunConfig, storage, stream: Optional[int] = None, check: bool = True) -> RunResult:
    """Run one primitive on `storage`: a numpy uint32/float32 array (host; copied
    in and out inside the call) or a CUDA tensor (device; used in place).
    `stream` is a raw cudaStream_t (defaults to torch's current stream for
    tensors, the legacy default stream otherwise)."""
    c = cfg.to_c()
    need = storage_words(cfg)
    on_device = 0
    if hasattr(storage, "data_ptr"):  # torch tensor
        if not storage.is_cuda:
            raise ValueError("torch storage must be a CUDA tensor (use numpy for host storage)")
        if storage.numel() * storage.element_size() < need * 4 or storage.element_size() != 4:
            raise ValueError("storage needs %d 32-bit words" % need)
        if not storage.is_contiguous():
            raise ValueError("storage must be contiguous")
        ptr = storage.data_ptr()
        on_device = 1
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(storage.device).cuda_stream
    else:
        import numpy as np
        if not isinstance(storage, np.ndarray) or storage.dtype.itemsize != 4 or not storage.flags.c_contiguous:
            raise ValueError("host storage must be a contiguous numpy array of 32-bit words")
        if storage.size < need:
            raise ValueError("storage needs %d 32-bit words" % need)
        ptr = storage.ctypes.data
    r = _RunResult()
    s = lib().hs_run(_context(), ctypes.byref(c), ctypes.c_void_p(ptr), on_device,
                     ctypes.c_void_p(stream or 0), ctypes.byref(r))
    res = RunResult(r.status, r.dev_error_bits, r.dev_error_site, r.elapsed_ms, r.avg_ms, r.h2d_ms, r.d2h_ms,
                    r.ops, r.launches, r.cluster, r.cohort, r.tbs_per_cta)
    if check and s:
        raise _err(s)
    return res


# ---------------------------------------------------------------------------
# Relaxed-atomics microbenchmarks and UTS (include/hs/hs.h)
# ---------------------------------------------------------------------------
class _RelaxedResult(ctypes.Structure):
    _fields_ = [("elapsed_ms", ctypes.c_float), ("ops", ctypes.c_ulonglong), ("dev_error_bits", ctypes.c_uint),
                ("dev_error_site", ctypes.c_uint)]


class _UtsResult(ctypes.Structure):
    _fields_ = [("nodes_processed", ctypes.c_uint), ("leaves_found", ctypes.c_uint), ("leaf_sum", ctypes.c_uint),
                ("elapsed_ms", ctypes.c_float), ("dev_error_bits", ctypes.c_uint)]


def _np():
    import numpy as np
    return np


def _relaxed_err(s):
    L = lib()
    L.hs_relaxed_last_error.restype = ctypes.c_char_p
    return HsError(s, L.hs_relaxed_last_error().decode())


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def refcounter(num_sharers: int, num_tbs: int, tb_size: int, num_repeats: int):
    """refCounter.cu: returns (counters0, counters1, del0, del1, result)."""
    np = _np()
    thr = num_tbs * tb_size
    nc = thr // num_sharers
    c0, c1 = np.zeros(nc, np.uint32), np.zeros(nc, np.uint32)
    d0, d1 = np.zeros(thr, np.uint32), np.zeros(thr, np.uint32)
    r = _RelaxedResult()
    s = lib().hs_refcounter(num_sharers, num_tbs, tb_size, num_repeats, _p(c0), _p(c1), _p(d0), _p(d1), ctypes.byref(r))
    if s:
        raise _relaxed_err(s)
    return c0, c1, d0, d1, r


def splitcounter(num_tbs: int, tb_size: int):
    """splitCounter.cu: returns (counters, outArr, result)."""
    np = _np()
    thr = num_tbs * tb_size
    c, o = np.zeros(thr // 2, np.uint32), np.zeros(thr, np.uint32)
    r = _RelaxedResult()
    s = lib().hs_splitcounter(num_tbs, tb_size, _p(c), _p(o), ctypes.byref(r))
    if s:
        raise _relaxed_err(s)
    return c, o, r


def seqlocks(num_tbs: int, tb_size: int, group_size: int, use_tfs: bool = False, timeout_ns: int = 0):
    """seqlocks.cu: returns (seqlock, data0, data1, outArr, result)."""
    np = _np()
    seq = np.zeros(max(num_tbs // group_size, 1), np.uint32)
    d0, d1 = np.zeros(32, np.int32), np.zeros(32, np.int32)
    o = np.full(num_tbs * tb_size, -1, np.int32)
    r = _RelaxedResult()
    lib().hs_seqlocks.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 4 + [ctypes.c_ulonglong, ctypes.c_void_p]
    s = lib().hs_seqlocks(num_tbs, tb_size, group_size, int(use_tfs), _p(seq), _p(d0), _p(d1), _p(o), timeout_ns,
                          ctypes.byref(r))
    if s:
        raise _relaxed_err(s)
    return seq, d0, d1, o, r


def flags(num_tbs: int, tb_size: int, num_accs: int, num_repeats: int, cutoff: float, num_iters: int, rand_arr):
    """flags.cu: returns (outArr, dirty, result)."""
    np = _np()
    rand_arr = np.ascontiguousarray(rand_arr, dtype=np.float32)
    o = np.zeros(num_tbs * tb_size, np.uint32)
    dirty = ctypes.c_uint()
    r = _RelaxedResult()
    lib().hs_flags.argtypes = [ctypes.c_int] * 4 + [ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_ulonglong,
                                                     ctypes.c_void_p]
    s = lib().hs_flags(num_tbs, tb_size, num_accs, num_repeats, cutoff, num_iters, _p(rand_arr), rand_arr.size, _p(o),
                       ctypes.byref(dirty), 0, ctypes.byref(r))
    if s:
        raise _relaxed_err(s)
    return o, dirty.value, r


UTS_NODE_FIELDS = [("value", "<u4"), ("depth", "<u4"), ("to_add", "<u4"), ("child_a", "<i4"), ("child_b", "<i4")]


def uts_tree(num_nodes: int, fertility: int, seed: int = 200):
    """uts.cu:290-339: (tree, golden leaves, golden leaf sum, restarts)."""
    np = _np()
    tree = np.zeros(num_nodes, dtype=np.dtype(UTS_NODE_FIELDS))
    lv, ls, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
    s = lib().hs_uts_tree_build(num_nodes, fertility, ctypes.c_uint(seed), _p(tree), ctypes.byref(lv),
                                ctypes.byref(ls), ctypes.byref(rs))
    if s:
        raise HsError(s, "uts tree")
    return tree, lv.value, ls.value, rs.value


def uts_frontier(tree, cores_used: int):
    np = _np()
    fr = np.zeros(cores_used * 16 + 2, dtype=np.int32)
    cnt, proc = ctypes.c_int(), ctypes.c_uint()
    s = lib().hs_uts_frontier(_p(tree), tree.size, cores_used, _p(fr), ctypes.byref(cnt), ctypes.byref(proc))
    if s:
        raise HsError(s, "uts frontier")
    return fr[:cnt.value].copy(), proc.value


def uts_run(tree, frontier, host_processed: int, blocks: int, threads: int = 128, timeout_ns: int = 0):
    np = _np()
    frontier = np.ascontiguousarray(frontier, dtype=np.int32)
    r = _UtsResult()
    lib().hs_uts_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_void_p]
    s = lib().hs_uts_run(_p(tree), tree.size, _p(frontier), frontier.size, host_processed, blocks, threads,
                         timeout_ns, ctypes.byref(r))
    if s:
        raise HsError(s, "uts run")
    return r


# ---------------------------------------------------------------------------
# Geometric UTS with a SHA-1 node generator (hs_uts_geo_*)
# ---------------------------------------------------------------------------
class _GeoResult(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_ulonglong), ("leaves", ctypes.c_ulonglong), ("max_depth", ctypes.c_uint),
                ("elapsed_ms", ctypes.c_float), ("dev_error_bits", ctypes.c_uint)]


def uts_geo_table(branching: float = 4.0, n: int = 128):
    np = _np()
    t = np.zeros(n, dtype=np.uint32)
    lib().hs_uts_geo_table.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
    nz = lib().hs_uts_geo_table(branching, _p(t), n)
    if nz < 0:
        raise HsError(1, "geo table")
    return t, nz


def uts_geo_run(seed: int, depth_limit: int, branching: float = 4.0, blocks: int = 0, threads: int = 256,
                timeout_ns: int = 0):
    """Count the geometric tree on the GPU: (nodes, leaves, deepest level, ms)."""
    blocks = blocks or device_info()["nsm"] * 4
    r = _GeoResult()
    L = lib()
    L.hs_uts_geo_last_error.restype = ctypes.c_char_p
    L.hs_uts_geo_run.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_ulonglong, ctypes.c_void_p]
    s = L.hs_uts_geo_run(seed, depth_limit, branching, blocks, threads, timeout_ns, ctypes.byref(r))
    if s:
        raise HsError(s, L.hs_uts_geo_last_error().decode())
    return r.nodes, r.leaves, r.max_depth, r.elapsed_ms


class _LatencyResult(ctypes.Structure):
    _fields_ = [("handoff_ns_median", ctypes.c_double), ("handoff_ns_min", ctypes.c_double),
                ("handoff_ns_max", ctypes.c_double), ("atomic_rtt_ns", ctypes.c_double),
                ("load_rtt_ns", ctypes.c_double), ("partners", ctypes.c_int), ("dev_error_bits", ctypes.c_uint)]


def probe_latency(rounds: int = 256) -> dict:
    """Lock hand-off latencies on this GPU (hs_probe_latency): flag ping-pong
    between SMs (one hand-off = half a round trip; median, min, max over the
    SMs), dependent L2 atomics and dependent L2 loads, in ns."""
    r = _LatencyResult()
    lib().hs_probe_latency.argtypes = [ctypes.c_int, ctypes.c_void_p]
    s = lib().hs_probe_latency(rounds, ctypes.byref(r))
    if s:
        raise HsError(s, "hs_probe_latency failed")
    return {f: getattr(r, f) for f, _ in _LatencyResult._fields_}


class _CoopResult(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_ulonglong), ("leaves", ctypes.c_ulonglong), ("max_depth", ctypes.c_uint),
                ("gpu_nodes", ctypes.c_ulonglong), ("host_nodes", ctypes.c_ulonglong),
                ("to_host", ctypes.c_ulonglong), ("to_gpu", ctypes.c_ulonglong), ("host_threads", ctypes.c_int),
                ("elapsed_ms", ctypes.c_float), ("dev_error_bits", ctypes.c_uint)]


def uts_geo_coop_run(seed: int, depth_limit: int, branching: float = 4.0, blocks: int | None = None,
                     threads: int = 256, host_threads: int = -1, timeout_ns: int = 0) -> dict:
    """Walk the geometric tree with GPU CTAs and host threads together
    (hs_uts_geo_coop_run).  blocks None: 2 CTAs per SM; blocks 0: host threads
    only (no CUDA call).  host_threads -1: the host's cores minus one.
    Returns the counts, each side's share and the items that crossed the link."""
    if blocks is None:
        blocks = device_info()["nsm"] * 2
    r = _CoopResult()
    L = lib()
    L.hs_uts_geo_last_error.restype = ctypes.c_char_p
    L.hs_uts_geo_coop_run.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_ulonglong, ctypes.c_void_p]
    s = L.hs_uts_geo_coop_run(seed, depth_limit, branching, blocks, threads, host_threads, timeout_ns,
                              ctypes.byref(r))
    if s:
        raise HsError(s, L.hs_uts_geo_last_error().decode())
    return {f: getattr(r, f) for f, _ in _CoopResult._fields_}


# ---------------------------------------------------------------------------
# Tree barrier with local exchange on thread-block clusters (hs_exchange_*)
# ---------------------------------------------------------------------------
class _ExchResult(ctypes.Structure):
    _fields_ = [("elapsed_ms", ctypes.c_float), ("episodes_per_s", ctypes.c_double),
                ("exchange_gbs", ctypes.c_double), ("clusters", ctypes.c_int), ("dev_error_bits", ctypes.c_uint),
                ("wait_site", ctypes.c_uint)]


def exchange_fill(seed: int, n: int, elems: int):
    """(n, elems) uint32 words holding fp32 values uniform in [-1, 1) drawn
    from std::mt19937_64(seed)."""
    np = _np()
    out = np.empty((n, elems), dtype=np.uint32)
    lib().hs_exchange_fill.argtypes = [ctypes.c_ulonglong, ctypes.c_size_t, ctypes.c_void_p]
    s = lib().hs_exchange_fill(seed, out.size, _p(out))
    if s:
        raise HsError(s, "exchange fill")
    return out


def exchange_run(buffers, cluster: int, lf: bool, episodes: int, timeout_ns: int = 0):
    """Rotate the (n, elems) buffers by `episodes` CTAs, one tree barrier per
    episode, clusters of `cluster` CTAs.  Returns (final buffers, result)."""
    np = _np()
    buffers = np.ascontiguousarray(buffers, dtype=np.uint32)
    if buffers.ndim != 2:
        raise ValueError("buffers must be (n, elems)")
    out = np.empty_like(buffers)
    r = _ExchResult()
    L = lib()
    L.hs_exchange_last_error.restype = ctypes.c_char_p
    L.hs_exchange_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_void_p]
    s = L.hs_exchange_run(_p(buffers), _p(out), buffers.shape[0], buffers.shape[1], cluster, 1 if lf else 0,
                          episodes, timeout_ns, ctypes.byref(r))
    if s:
        raise HsError(s, L.hs_exchange_last_error().decode())
    return out, r


# ---------------------------------------------------------------------------
# Served request loop (hs_serve_*)
# ---------------------------------------------------------------------------
REQ_SYNCPRIM, REQ_UTS_GEO = 0, 1


class _ServeRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("prim", ctypes.c_int), ("num_ldst", ctypes.c_int),
                ("num_tbs", ctypes.c_int), ("num_iters", ctypes.c_int), ("seed", ctypes.c_uint),
                ("depth_limit", ctypes.c_int), ("branching", ctypes.c_double)]


def _request(inst):
    """A request from (prim, num_ldst, num_tbs, num_iters) or ("uts", seed, depth_limit, branching)."""
    if inst[0] == "uts":
        _, seed, depth, b = inst
        return _ServeRequest(REQ_UTS_GEO, 0, 0, 0, 0, seed, depth, b)
    p, L, G, I = inst
    return _ServeRequest(REQ_SYNCPRIM, prim_id(p) if isinstance(p, str) else p, L, G, I, 0, 0, 0.0)


def serve_request_words(inst, nsm: int = 0) -> int:
    nsm = nsm or device_info()["nsm"]
    r = _request(inst)
    w = ctypes.c_size_t()
    lib().hs_serve_request_words.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    s = lib().hs_serve_request_words(ctypes.byref(r), nsm, ctypes.byref(w))
    if s:
        raise HsError(s, "request words")
    return int(w.value)


def serve_uts_counts(final_words):
    """(nodes, leaves, deepest level) from a tree-search request's final state."""
    np = _np()
    a = np.ascontiguousarray(final_words, dtype=np.uint32)
    n, lv, d = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_uint()
    lib().hs_serve_uts_geo_counts.argtypes = [ctypes.c_void_p, ctypes.c_size_t] + [ctypes.c_void_p] * 3
    s = lib().hs_serve_uts_geo_counts(_p(a), a.size, ctypes.byref(n), ctypes.byref(lv), ctypes.byref(d))
    if s:
        raise HsError(s, "tree-search counts")
    return n.value, lv.value, d.value


class _ServeCompletion(ctypes.Structure):
    _fields_ = [("id", ctypes.c_ulonglong), ("status", ctypes.c_int), ("dev_error_bits", ctypes.c_uint),
                ("wait_site", ctypes.c_uint), ("latency_us", ctypes.c_double), ("service_us", ctypes.c_double),
                ("admit_to_end_us", ctypes.c_double)]


def _comp_dict(c):
    return {"id": c.id, "status": c.status, "dev_error_bits": c.dev_error_bits, "wait_site": c.wait_site,
            "latency_us": c.latency_us, "service_us": c.service_us, "admit_to_end_us": c.admit_to_end_us}


class Server:
    """A persistent server kernel admitting SyncPrims requests as they arrive.
    While it runs, make no synchronising CUDA calls in this process."""

    def __init__(self, slots: int = 32, gang: int = 8, arena_bytes: int = 1 << 30, staging_bytes: int = 1 << 30,
                 idle_timeout_s: float = 60.0):
        L = lib()
        L.hs_serve_last_error.restype = ctypes.c_char_p
        L.hs_serve_start.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_ulonglong,
                                     ctypes.c_double, ctypes.c_void_p]
        L.hs_serve_submit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.hs_serve_poll.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.hs_serve_pending.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.hs_serve_stop.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.hs_serve_destroy.argtypes = [ctypes.c_void_p]
        L.hs_serve_drive.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                     ctypes.c_void_p]
        L.hs_serve_request_words.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        h = ctypes.c_void_p()
        s = L.hs_serve_start(slots, gang, arena_bytes, staging_bytes, idle_timeout_s, ctypes.byref(h))
        if s:
            raise HsError(s, L.hs_serve_last_error().decode())
        self.h = h
        self.slots, self.gang = slots, gang
        self._keep = {}

    def _check(self, s):
        if s:
            raise HsError(s, lib().hs_serve_last_error().decode())

    @staticmethod
    def request_words(prim, num_ldst, num_tbs, num_iters, nsm: int = 0):
        return serve_request_words((prim, num_ldst, num_tbs, num_iters), nsm)

    def submit(self, inst, init=None):
        """inst = (prim, num_ldst, num_tbs, num_iters) with init = the initial
        storage (uint32), or ("uts", seed, depth_limit, branching) with no
        init.  Returns (id, output array filled at completion)."""
        np = _np()
        r = _request(inst)
        if inst[0] == "uts":
            out = np.zeros(serve_request_words(inst), dtype=np.uint32)
            init_p = None
        else:
            init = np.ascontiguousarray(init, dtype=np.uint32)
            out = np.zeros_like(init)
            init_p = _p(init)
        rid = ctypes.c_ulonglong()
        self._check(lib().hs_serve_submit(self.h, ctypes.byref(r), init_p, _p(out), ctypes.byref(rid)))
        self._keep[rid.value] = out
        return rid.value, out

    def poll(self, max_n: int = 256):
        buf = (_ServeCompletion * max_n)()
        n = ctypes.c_int()
        self._check(lib().hs_serve_poll(self.h, buf, max_n, ctypes.byref(n)))
        res = []
        for i in range(n.value):
            d = _comp_dict(buf[i])
            self._keep.pop(d["id"], None)
            res.append(d)
        return res

    def wait(self, n: int, timeout_s: float = 120.0):
        """Poll until n completions arrived (or the timeout)."""
        import time
        got, t0 = [], time.time()
        while len(got) < n:
            got += self.poll()
            if time.time() - t0 > timeout_s:
                raise HsError(2, "%d of %d completions after %.0f s" % (len(got), n, timeout_s))
        return got

    def drive(self, insts, inits, arrival_s, timeout_s: float = 300.0):
        """Open-loop run: request i published at arrival_s[i]; returns
        (outputs, completions in request order, wall seconds)."""
        np = _np()
        n = len(insts)
        reqs = (_ServeRequest * n)(*[_request(x) for x in insts])
        ins = [None if x[0] == "uts" else np.ascontiguousarray(a, dtype=np.uint32) for x, a in zip(insts, inits)]
        outs = [np.zeros(serve_request_words(x), dtype=np.uint32) if x[0] == "uts" else np.zeros_like(a)
                for x, a in zip(insts, ins)]
        in_p = (ctypes.c_void_p * n)(*[None if a is None else a.ctypes.data for a in ins])
        out_p = (ctypes.c_void_p * n)(*[x.ctypes.data for x in outs])
        arr = np.ascontiguousarray(arrival_s, dtype=np.float64)
        comps = (_ServeCompletion * n)()
        wall = ctypes.c_double()
        self._check(lib().hs_serve_drive(self.h, reqs, n, in_p, out_p, _p(arr), timeout_s, comps,
                                         ctypes.byref(wall)))
        return outs, [_comp_dict(c) for c in comps], wall.value

    def stop(self, timeout_s: float = 120.0):
        if self.h:
            self._check(lib().hs_serve_stop(self.h, timeout_s))

    def close(self):
        if self.h:
            lib().hs_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


# ---------------------------------------------------------------------------
# Batched mixed instances (hs_batch_*)
# ---------------------------------------------------------------------------
class _BatchInst(ctypes.Structure):
    _fields_ = [("prim", ctypes.c_int), ("num_ldst", ctypes.c_int), ("num_tbs", ctypes.c_int),
                ("num_iters", ctypes.c_int)]


class _BatchResult(ctypes.Structure):
    _fields_ = [("elapsed_ms", ctypes.c_float), ("ops", ctypes.c_ulonglong), ("launches", ctypes.c_uint),
                ("grid", ctypes.c_int), ("tbs_per_cta", ctypes.c_int), ("dev_error_bits", ctypes.c_uint),
                ("failed_instance", ctypes.c_int)]


BATCH_REFCOUNTER, BATCH_SPLITCOUNTER, BATCH_SEQLOCK, BATCH_FLAGS = 60, 61, 62, 63
BATCH_KIND_NAMES = {60: "RefCounter", 61: "SplitCounter", 62: "Seqlock", 63: "Flags"}


def batch_instance_words(inst, nsm: int = 0) -> int:
    """Storage words of one (prim, num_ldst, num_tbs, num_iters) instance."""
    nsm = nsm or device_info()["nsm"]
    x = _BatchInst(*inst)
    w = ctypes.c_size_t()
    lib().hs_batch_instance_words.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    s = lib().hs_batch_instance_words(ctypes.byref(x), nsm, ctypes.byref(w))
    if s:
        raise HsError(s, "instance words")
    return int(w.value)


def batch_expected(inst, init, nsm: int = 0, mode: str = "inc"):
    """Closed-form final storage of one batch or served instance (any kind)."""
    np = _np()
    nsm = nsm or device_info()["nsm"]
    init = np.ascontiguousarray(init, dtype=np.uint32)
    out = np.empty_like(init)
    x = _BatchInst(*inst)
    lib().hs_batch_expected_storage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_size_t]
    s = lib().hs_batch_expected_storage(ctypes.byref(x), nsm, _MODES[mode], _p(init), _p(out), init.size)
    if s:
        raise HsError(s, "batch expected storage")
    return out


def batch_generate(seed: int, n: int = 64, nsm: int = 0, iter_div: int = 1):
    """The mixed batch: list of (prim, num_ldst, num_tbs, num_iters); prim is
    a SyncPrims id or one of the BATCH_* relaxed-atomics kinds."""
    nsm = nsm or device_info()["nsm"]
    arr = (_BatchInst * n)()
    s = lib().hs_batch_generate(ctypes.c_ulonglong(seed), n, nsm, iter_div, arr)
    if s:
        raise HsError(s, "batch generate")
    return [(a.prim, a.num_ldst, a.num_tbs, a.num_iters) for a in arr]


def plan_cache_path() -> str:
    """Where tuned batch plans are kept: $HS_PLAN_CACHE, else
    ~/.cache/heterosync_gb300/batch_plans.json."""
    return os.environ.get("HS_PLAN_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "heterosync_gb300",
                                                           "batch_plans.json")


def plan_cache_key(instances, mode: str, device: Optional[dict] = None) -> str:
    """A batch's cache key: the instances (kind, numLdSt, numTBs, numCSIters),
    the data mode and the device (SM count, compute capability, max threads per
    block); a plan tuned for one of them says nothing about another."""
    import hashlib
    import json
    dev = device if device is not None else device_info()
    blob = json.dumps({"instances": [list(map(int, x)) for x in instances], "mode": mode,
                       "device": [int(dev["nsm"]), int(dev["cc"][0]), int(dev["cc"][1]),
                                  int(dev["max_threads_per_block"])], "plan_format": 1}, sort_keys=True)
    return hashlib.sha256(blob.encode()).hexdigest()


def plan_cache_load(path: str, key: str):
    import json
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def plan_cache_store(path: str, key: str, entry: dict) -> None:
    """Add one plan to the cache file (written to a temporary file and renamed,
    so a reader never sees half a file)."""
    import json
    import tempfile
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        try:
            with open(path) as f:
                data = json.load(f)
        except (OSError, ValueError):
            data = {}
        data[key] = entry
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path) or ".", suffix=".tmp")
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass  # an unwritable cache only costs the next run its trials


class Batch:
    """Instances run in one persistent, graph-replayed launch (run) or one
    standalone launch each (run_serial)."""

    def __init__(self, instances, mode: str = "inc"):
        L = lib()
        L.hs_batch_last_error.restype = ctypes.c_char_p
        L.hs_batch_storage_words.restype = ctypes.c_size_t
        L.hs_batch_storage_words.argtypes = [ctypes.c_void_p, ctypes.c_int]
        for f in ("hs_batch_set_storage", "hs_batch_get_storage"):
            getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        for f in ("hs_batch_run", "hs_batch_run_serial"):
            getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.hs_batch_plan.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.hs_batch_plan_ex.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p]
        L.hs_batch_get_plan.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 4
        L.hs_batch_autotune.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.hs_batch_destroy.argtypes = [ctypes.c_void_p]
        self.instances = list(instances)
        arr = (_BatchInst * len(self.instances))(*[_BatchInst(*x) for x in self.instances])
        h = ctypes.c_void_p()
        s = L.hs_batch_create(arr, len(self.instances), 256, _MODES[mode], ctypes.byref(h))
        if s:
            raise HsError(s, L.hs_batch_last_error().decode())
        self.h = h
        self.mode = mode

    def _check(self, s):
        if s:
            raise HsError(s, lib().hs_batch_last_error().decode())

    def words(self, i):
        return int(lib().hs_batch_storage_words(self.h, i))

    def set_storage(self, i, arr):
        import numpy as np
        a = np.ascontiguousarray(arr, dtype=np.uint32)
        self._check(lib().hs_batch_set_storage(self.h, i, a.ctypes.data))

    def get_storage(self, i):
        import numpy as np
        a = np.empty(self.words(i), dtype=np.uint32)
        self._check(lib().hs_batch_get_storage(self.h, i, a.ctypes.data))
        return a

    def plan(self, v):
        grid, cap = ctypes.c_int(), ctypes.c_int()
        s = lib().hs_batch_plan(self.h, v, ctypes.byref(grid), ctypes.byref(cap))
        return s, grid.value, cap.value

    def plan_ex(self, cl: int, serial_execs: int, v: int):
        """Clusters of cl CTAs per operation; serial_execs clusters for each
        instance serialised on one lock or semaphore (0 = ceil(numTBs / v)),
        ceil(numTBs / v) clusters for the others."""
        grid, cap = ctypes.c_int(), ctypes.c_int()
        s = lib().hs_batch_plan_ex(self.h, cl, serial_execs, v, ctypes.byref(grid), ctypes.byref(cap))
        return s, grid.value, cap.value

    def get_plan(self):
        """(cluster size, serialised-instance clusters, v, grid) of the current plan."""
        a, b, c, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(lib().hs_batch_get_plan(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                            ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def set_backoff(self, bo_min: int, bo_max: int):
        """EBO bounds (ns) of the batched launch; invalidates the plan."""
        lib().hs_batch_set_backoff.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
        self._check(lib().hs_batch_set_backoff(self.h, bo_min, bo_max))

    def get_backoff(self):
        a, b = ctypes.c_uint(), ctypes.c_uint()
        lib().hs_batch_get_backoff.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        self._check(lib().hs_batch_get_backoff(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def get_stage(self) -> int:
        lib().hs_batch_get_stage.argtypes = [ctypes.c_void_p]
        lib().hs_batch_get_stage.restype = ctypes.c_uint
        return int(lib().hs_batch_get_stage(self.h))

    def tuned_settings(self):
        """(cluster, serial executors, v, staging bytes, backoff cap, backoff start) of the current plan."""
        cl, se, v, _ = self.get_plan()
        bo_min, bo_max = self.get_backoff()
        return cl, se, v, self.get_stage(), bo_max, bo_min

    def apply_settings(self, settings):
        """Apply tuned_settings() of another batch (e.g. one tuned on fewer iterations)."""
        cl, se, v, stage, bo = settings[:5]
        bo_min = settings[5] if len(settings) > 5 else 1
        self.set_stage(stage)
        self.set_backoff(bo_min, bo)
        return self.plan_ex(cl, se, v)

    def set_stage(self, nbytes: int):
        """Staging bytes per CTA (0 = whole chunks); invalidates the plan."""
        lib().hs_batch_set_stage.argtypes = [ctypes.c_void_p, ctypes.c_uint]
        self._check(lib().hs_batch_set_stage(self.h, nbytes))

    def autotune(self, cache: Optional[str] = ""):
        """Choose the launch plan (hs_batch_autotune) and apply it; returns
        (v, ms of the best trial).  The plan is kept in a cache file keyed by
        the instances, the data mode and the device (plan_cache_path(); None
        disables it): a batch tuned before on this device gets its plan back
        without any trial.  self.last_tune tells which happened."""
        path = plan_cache_path() if cache == "" else cache
        key = plan_cache_key(self.instances, self.mode) if path else None
        if path:
            hit = plan_cache_load(path, key)
            if hit is not None:
                s, _, _ = self.apply_settings(hit["settings"])
                if s == 0:
                    self.last_tune = {"cache": "hit", "path": path, "key": key[:16]}
                    return self.get_plan()[2], float(hit["ms"])
        v, ms = ctypes.c_int(), ctypes.c_float()
        self._check(lib().hs_batch_autotune(self.h, None, ctypes.byref(v), ctypes.byref(ms)))
        self.last_tune = {"cache": "miss" if path else "off", "path": path, "key": key[:16] if key else None}
        if path:
            plan_cache_store(path, key, {"settings": list(self.tuned_settings()), "ms": float(ms.value)})
        return v.value, ms.value

    def run(self):
        r = _BatchResult()
        self._check(lib().hs_batch_run(self.h, None, ctypes.byref(r)))
        return r

    def run_serial(self):
        r = _BatchResult()
        self._check(lib().hs_batch_run_serial(self.h, None, ctypes.byref(r)))
        return r

    def close(self):
        if self.h:
            lib().hs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
