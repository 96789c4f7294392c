"""CPU checks of the oracle (the reference golden restated in C) against an
independent pure-Python restatement, and of the product's closed-form
expectation (hs_expected_storage) against the oracle."""
import itertools

import numpy as np
import pytest

ALL_PRIMS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15,
             20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]


def py_golden(prim, T, L, G, iters, repeats, nsm, inc, s):
    """Pure-Python restatement of main.cu:1637-1788 (small sizes only)."""
    s = list(int(x) for x in s)
    U = T * (L + 1)
    k = -(-G // nsm)

    def acc(loc):
        if loc % (16 * (L + 1)) >= 16:
            s[loc] = (s[loc] + 1) & 0xFFFFFFFF if inc else s[loc - 16]

    for _ in range(repeats):
        for j in range(iters):
            if prim < 4:
                N = G * U
                for i in range(N - 1, -1, -1):
                    acc((i + j * U) % N)
                if prim in (1, 3) and k > 1:
                    for i in range(N - 1, -1, -1):
                        acc(((i + k * U) % N + j * U) % N)
            elif prim <= 7:
                for _b in range(G):
                    for i in range(U - 1, -1, -1):
                        acc(i)
            elif prim <= 19:
                nS = min(G, nsm)
                for tb in range(G):
                    if tb // nS == (tb % nS) % k:
                        for kk in range(k):
                            for i in range(U - 1, -1, -1):
                                acc((i + kk * U) % len(s))
            elif prim <= 23:
                for i in range(G * U - 1, -1, -1):
                    acc(i % (nsm * U))
            else:
                for i in range(G * U - 1, -1, -1):
                    acc(i)
    return np.array(s, dtype=np.uint32)


@pytest.mark.parametrize("prim", ALL_PRIMS)
@pytest.mark.parametrize("inc", [False, True])
def test_oracle_matches_python_restatement(oracle, prim, inc):
    rng = np.random.default_rng(prim * 7 + inc)
    for (T, L, G, iters, reps, nsm) in [(16, 2, 3, 2, 1, 2), (32, 3, 5, 1, 2, 4), (16, 1, 4, 3, 1, 4)]:
        n = oracle.storage_words(prim, T, L, G, nsm)
        init = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
        a = oracle.golden(prim, T, L, G, iters, reps, nsm, inc, init)
        b = py_golden(prim, T, L, G, iters, reps, nsm, inc, init)
        assert np.array_equal(a, b), (prim, T, L, G, iters, reps, nsm)


@pytest.mark.parametrize("prim", ALL_PRIMS)
def test_closed_form_matches_oracle(hs, oracle, prim):
    """The product's O(size) expectation equals the reference's literal replay
    on even configurations (numTBs a multiple of NUM_SM or below it)."""
    rng = np.random.default_rng(1000 + prim)
    for (T, L, G, iters, reps, nsm), mode in itertools.product(
            [(16, 5, 4, 2, 2, 2), (32, 12, 8, 1, 3, 4), (16, 3, 3, 2, 1, 4), (64, 40, 6, 1, 1, 3),
             (16, 2, 12, 3, 1, 4), (32, 7, 1, 4, 2, 4)],
            ["ref", "inc"]):
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=reps,
                           mode=mode, nsm=nsm)
        n = hs.storage_words(cfg, nsm)
        assert n == oracle.storage_words(prim, T, L, G, nsm)
        init = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
        want = oracle.golden(prim, T, L, G, iters, reps, nsm, mode == "inc", init)
        got = hs.expected_storage(cfg, init, nsm)
        assert np.array_equal(got, want), (prim, T, L, G, iters, reps, nsm, mode)


@pytest.mark.parametrize("prim,uniq", [(4, False), (7, False), (20, True), (23, True)])
def test_slice_closed_form(hs, oracle, prim, uniq):
    rng = np.random.default_rng(prim)
    for (L, G, iters, reps, nsm) in [(10, 8, 100, 1, 152), (3, 9, 7, 2, 4), (5, 13, 4, 3, 5)]:
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=256, repeats=reps,
                           mode="slice", nsm=nsm)
        n = hs.storage_words(cfg, nsm)
        assert n == G * L
        init = rng.integers(0, 1000, size=n).astype(np.uint32)
        want = oracle.slice_replay(uniq, L, G, iters, reps, nsm, init)
        assert np.array_equal(hs.expected_storage(cfg, init, nsm), want)
        # every slice sees exactly repeats*iters increments
        assert np.array_equal(want - init, np.full(n, reps * iters, dtype=np.uint32))


def test_copy_shift_converges(oracle):
    """After >= numLdSt shifts every line of a region equals its first line
    (why the reference golden alone is weak, and why the parity tests keep the
    number of shifts below numLdSt)."""
    T, L = 32, 4
    n = oracle.storage_words(7, T, L, 1, 4)
    init = np.arange(n, dtype=np.uint32)
    out = oracle.golden(7, T, L, 2, 1, 2, 4, False, init)  # 4 shifts
    reg = out.reshape(-1, L + 1, 16)
    assert np.array_equal(reg, np.repeat(init.reshape(-1, L + 1, 16)[:, :1, :], L + 1, axis=1))
