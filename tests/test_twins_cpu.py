"""The host std::thread twins (CPU baseline) produce the oracle golden's final
storage for every primitive; this pins the CPU baseline to the same algorithm."""
import os

import numpy as np
import pytest

ALL_PRIMS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15,
             20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]


@pytest.mark.parametrize("prim", ALL_PRIMS)
@pytest.mark.parametrize("mode", [0, 1])
def test_twin_matches_golden(oracle, prim, mode):
    rng = np.random.default_rng(prim + 31 * mode)
    for (T, L, G, iters, reps, nsm, nt) in [(32, 30, 8, 2, 2, 4, 3), (16, 12, 12, 1, 2, 4, 5), (64, 9, 5, 1, 1, 8, 2)]:
        n = oracle.storage_words(prim, T, L, G, nsm)
        init = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
        got, secs = oracle.twin_run(prim, T, L, G, iters, reps, nsm, mode, init, threads=nt)
        want = oracle.golden(prim, T, L, G, iters, reps, nsm, mode == 1, init)
        assert np.array_equal(got, want), (prim, mode, T, L, G)
        assert secs >= 0


@pytest.mark.parametrize("prim", [4, 5, 6, 7, 20, 21, 22, 23])
def test_twin_slice_mode(oracle, prim):
    L, G, iters, reps, nsm = 10, 8, 100, 1, 152
    init = (np.arange(G * L) % 1000).astype(np.uint32)
    got, _ = oracle.twin_run(prim, 256, L, G, iters, reps, nsm, 2, init, threads=4)
    assert np.array_equal(got, oracle.slice_replay(prim >= 20, L, G, iters, reps, nsm, init))
