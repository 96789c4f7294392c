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
