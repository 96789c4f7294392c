"""Served request loop: host-side contract without a GPU (arguments rejected
before any device call, request sizing)."""
import ctypes

import pytest


def test_start_rejects_bad_arguments(hs):
    L = hs.lib()
    L.hs_serve_start.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_ulonglong,
                                 ctypes.c_double, ctypes.c_void_p]
    h = ctypes.c_void_p()
    for args in [(0, 4, 1 << 30, 1 << 20, 1.0), (4, 0, 1 << 30, 1 << 20, 1.0), (4, 4, 1000, 1 << 20, 1.0),
                 (4, 4, 1 << 30, 100, 1.0), (4, 4, 1 << 30, 1 << 20, 0.0)]:
        assert L.hs_serve_start(*args, ctypes.byref(h)) == 1


def test_request_words_match_storage_words(hs):
    for inst in [(4, 10, 8, 3), (1, 100, 152, 2), (24, 7, 304, 5), (6, 33, 17, 4)]:
        p, L, G, I = inst
        cfg = hs.RunConfig(prim=p, num_ldst=L, num_tbs=G, num_iters=I, threads=256, repeats=1, mode="inc")
        assert hs.Server.request_words(*inst, nsm=152) == hs.storage_words(cfg, nsm=152)


def test_submit_without_server_is_rejected(hs):
    L = hs.lib()
    L.hs_serve_submit.argtypes = [ctypes.c_void_p] * 5
    assert L.hs_serve_submit(None, None, None, None, None) == 1


def test_window_rates_ignore_the_drain():
    """A server that keeps up completes requests as fast as they arrive inside
    the middle of the arrival window, however long the last ones take; one that
    falls behind completes fewer there than arrive."""
    import numpy as np
    from heterosync_gb300.served import poisson_arrivals, window_rates
    arr = poisson_arrivals(1000.0, 4000, seed=3)
    assert abs((len(arr) - 1) / arr[-1] - 1000.0) < 60
    lat = np.full(arr.size, 2000.0)          # 2 ms each, constant: keeps up
    lat[-5:] = 200000.0                      # a slow drain at the end does not count
    arrived, completed = window_rates(arr, lat)
    assert abs(completed / arrived - 1.0) < 0.01
    behind = (np.arange(arr.size) / 500.0 - arr) * 1e6 + 2000.0   # completions at 500/s
    arrived, completed = window_rates(arr, np.maximum(behind, 2000.0))
    assert completed < 0.7 * arrived
