"""hs_run_noalloc: the SyncPrims run for callers that cannot allocate device
memory (host frameworks that own all device memory, fixed memory budgets,
loops that cannot take cudaMalloc's device-wide synchronisation).  It keeps its
lock state in a fixed device array instead of cudaMalloc'd buffers.

Called through the C ABI and compared with the existing entry point, hs_run,
bit for bit (the tolerance every parity test here uses), on two calls in a row:
the array keeps the previous call's contents, so the second call also checks
that each call clears what must start at zero.  Collected last so that a run
stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # (prim, mode, threads, numLdSt, numTBs, iters, repeats, nsm)
    ("faMutex", "slice", 256, 10, 8, 100, 1, 0),
    ("sleepMutex", "ref", 64, 30, 8, 2, 2, 4),
    ("spinSemEBO10", "inc", 32, 12, 12, 3, 1, 4),
    ("atomicTreeBarrUniqLocalExch", "ref", 64, 20, 8, 3, 2, 4),
    ("faMutexUniq", "inc", 32, 9, 10, 4, 1, 4),
    # numLdSt > 32: critical sections staged through shared memory by bulk copies
    ("spinMutex", "inc", 256, 40, 8, 3, 1, 4),
    ("spinSemEBO2", "ref", 256, 48, 12, 2, 1, 4),
    ("faMutex", "ref", 128, 100, 6, 2, 2, 0),
]


def _call_noalloc(hs, cfg, tensor):
    L = hs.lib()
    L.hs_run_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.hs_noalloc_last_error.restype = ctypes.c_char_p
    import torch
    c = cfg.to_c()
    res = hs._RunResult()
    stream = torch.cuda.current_stream().cuda_stream
    s = L.hs_run_noalloc(ctypes.byref(c), ctypes.c_void_p(tensor.data_ptr()), ctypes.c_void_p(stream),
                         ctypes.byref(res))
    return s, res, L.hs_noalloc_last_error().decode()


def test_noalloc_matches_hs_run_on_two_calls(hs):
    torch = pytest.importorskip("torch")
    for call in range(2):
        for i, (prim, mode, T, L, G, iters, reps, nsm) in enumerate(CASES):
            cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=reps,
                               mode=mode, nsm=nsm)
            n = hs.storage_words(cfg)
            rng = np.random.default_rng(1000 * call + i)
            init = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
            a = torch.from_numpy(init.view(np.int32).copy()).cuda()
            b = torch.from_numpy(init.view(np.int32).copy()).cuda()
            hs.run(cfg, a)                                   # existing entry point
            s, res, err = _call_noalloc(hs, cfg, b)          # the entry point that allocates nothing
            torch.cuda.synchronize()
            assert s == 0, (prim, err)
            assert res.launches == reps and res.ops == G * iters * reps
            got_a = a.cpu().numpy().view(np.uint32)
            got_b = b.cpu().numpy().view(np.uint32)
            assert np.array_equal(got_b, got_a), (call, prim)
            assert np.array_equal(got_b, hs.expected_storage(cfg, init)), (call, prim)


def test_noalloc_rejects_state_beyond_the_array(hs):
    torch = pytest.importorskip("torch")
    # per-SM ring mutexes for 4096 TBs need ~152 rings x 4097 slots x 32 B, far beyond the array
    cfg = hs.RunConfig(prim="sleepMutexUniq", num_ldst=1, num_tbs=4096, num_iters=1, threads=32, repeats=1)
    t = torch.zeros(hs.storage_words(cfg), dtype=torch.int32, device="cuda")
    s, res, err = _call_noalloc(hs, cfg, t)
    assert s == 1  # HS_EINVAL, before anything is launched
    assert res.launches == 0
    assert "at most" in err


def _pair(hs, torch, cfg, seed):
    n = hs.storage_words(cfg)
    init = np.random.default_rng(seed).integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    a = torch.from_numpy(init.view(np.int32).copy()).cuda()
    b = torch.from_numpy(init.view(np.int32).copy()).cuda()
    return init, a, b


def test_noalloc_barrier_with_shared_memory_tiles(hs):
    """A tree barrier at four TBs per SM whose critical sections go through
    shared-memory tiles (numLdSt 64): launched with the same tiles as hs_run and
    bit-identical to it, on two calls in a row."""
    torch = pytest.importorskip("torch")
    nsm = hs.device_info()["nsm"]
    for call in range(2):
        cfg = hs.RunConfig(prim="atomicTreeBarrUniq", num_ldst=64, num_tbs=4 * nsm, num_iters=3, threads=256,
                           repeats=1, mode="inc", timeout_ns=2_000_000_000)
        init, a, b = _pair(hs, torch, cfg, 77 + call)
        hs.run(cfg, a)
        s, res, err = _call_noalloc(hs, cfg, b)
        torch.cuda.synchronize()
        assert s == 0, err
        got_b = b.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_b, a.cpu().numpy().view(np.uint32))
        assert np.array_equal(got_b, hs.expected_storage(cfg, init))


def test_noalloc_refuses_barriers_that_cannot_be_resident(hs):
    """Co-residency is judged with the shared memory the barrier launches with:
    walking numTBs = k * NUM_SM + 1 upwards (256 threads, numLdSt 40), every shape
    hs_run accepts runs bit-identically here, and the first one hs_run refuses is
    refused here too with HS_ENORES, before any launch."""
    torch = pytest.importorskip("torch")
    nsm = hs.device_info()["nsm"]
    refused = False
    for k in range(3, 9):
        cfg = hs.RunConfig(prim="lfTreeBarrUniq", num_ldst=40, num_tbs=k * nsm + 1, num_iters=1, threads=256,
                           repeats=1, mode="inc", timeout_ns=2_000_000_000)
        init, a, b = _pair(hs, torch, cfg, 900 + k)
        ra = hs.run(cfg, a, check=False)
        s, res, err = _call_noalloc(hs, cfg, b)
        torch.cuda.synchronize()
        if ra.status == 3:  # HS_ENORES
            assert s == 3, (k, s, err)
            assert res.launches == 0 and "co-resident" in err
            refused = True
            break
        assert ra.status == 0 and s == 0, (k, ra.status, s, err)
        assert np.array_equal(b.cpu().numpy().view(np.uint32), a.cpu().numpy().view(np.uint32)), k
    assert refused


def test_noalloc_rejects_flags_it_cannot_honour(hs):
    torch = pytest.importorskip("torch")
    for flag in (2, 16, 64):  # HS_RUN_KEEP_STATE, HS_RUN_GRAPH, HS_RUN_CLUSTER_CS
        cfg = hs.RunConfig(prim="spinMutex", num_ldst=4, num_tbs=4, num_iters=2, threads=32, repeats=1, flags=flag)
        t = torch.zeros(hs.storage_words(cfg), dtype=torch.int32, device="cuda")
        s, res, err = _call_noalloc(hs, cfg, t)
        assert s == 1 and res.launches == 0, (flag, s)
        assert "HS_RUN_SYNC_EACH" in err
    # the flags it honours: one host synchronisation per launch, flat form, register path
    cfg = hs.RunConfig(prim="spinMutex", num_ldst=40, num_tbs=6, num_iters=3, threads=256, repeats=2, mode="inc",
                       nsm=4, flags=1 | 4 | 8 | 32)
    init, a, b = _pair(hs, torch, cfg, 5)
    hs.run(cfg, a)
    s, res, err = _call_noalloc(hs, cfg, b)
    torch.cuda.synchronize()
    assert s == 0 and res.launches == 2, err
    assert np.array_equal(b.cpu().numpy().view(np.uint32), hs.expected_storage(cfg, init))
