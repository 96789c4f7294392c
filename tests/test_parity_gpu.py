"""GPU parity: every SyncPrims primitive, through the C ABI, against the oracle
(the reference golden restated in C), bit-exact.

Sizes keep the number of copy shifts per region below numLdSt, so the
reference-mode result pins the exact number of critical sections (the
reference golden alone converges after numLdSt shifts).  NUM_SM is overridden
to small values so that few TBs still form multi-TB logical-SM groups.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALL_PRIMS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15,
             20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]

# (threads, numLdSt, numTBs, iters, repeats, nsm): even group sizes
CASES = [
    (32, 40, 8, 2, 2, 4),     # 2 TBs per logical SM, multi-pass shift (40 > 32 lines)
    (256, 10, 6, 1, 1, 3),    # 256 threads per TB
    (64, 25, 5, 2, 1, 8),     # fewer TBs than SMs
    (16, 12, 12, 1, 1, 4),    # 3 TBs per logical SM, half-warp TBs
    (256, 100, 4, 2, 1, 2),   # 100 KB chunks: bulk-copy (TMA) critical sections
]


def _init(n, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("prim", ALL_PRIMS)
@pytest.mark.parametrize("mode", ["ref", "inc"])
def test_parity_host_storage(hs, oracle, prim, mode):
    for ci, (T, L, G, iters, reps, nsm) in enumerate(CASES):
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=reps,
                           mode=mode, nsm=nsm, timeout_ns=5_000_000_000)
        n = hs.storage_words(cfg)
        init = _init(n, prim * 100 + ci)
        st = init.copy()
        res = hs.run(cfg, st)
        want = oracle.golden(prim, T, L, G, iters, reps, nsm, mode == "inc", init)
        assert res.status == 0 and res.launches == reps
        bad = np.flatnonzero(st != want)
        assert bad.size == 0, "prim %d mode %s case %d: %d words differ, first %s" % (
            prim, mode, ci, bad.size, bad[:8])


@pytest.mark.parametrize("prim", [4, 5, 6, 7, 20, 21, 22, 23])
def test_slice_mode(hs, oracle, prim):
    """The slice workload: uint32[numTBs*numLdSt] seeded in [0,1000), +1 per critical section."""
    for (T, L, G, iters, reps, nsm) in [(256, 10, 8, 100, 1, 0), (64, 7, 24, 20, 2, 4), (32, 33, 17, 9, 1, 5)]:
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=reps,
                           mode="slice", nsm=nsm)
        n = hs.storage_words(cfg)
        rng = np.random.default_rng(20260101)
        init = (rng.integers(0, 2**63, size=n, dtype=np.uint64) % 1000).astype(np.uint32)
        st = init.copy()
        hs.run(cfg, st)
        nsm_eff = nsm or hs.device_info()["nsm"]
        want = oracle.slice_replay(prim >= 20, L, G, iters, reps, nsm_eff, init)
        assert np.array_equal(st, want)


def test_device_storage_torch(hs, oracle):
    torch = pytest.importorskip("torch")
    cfg = hs.RunConfig(prim="faMutex", num_ldst=30, num_tbs=8, num_iters=3, threads=256, repeats=1, mode="ref")
    n = hs.storage_words(cfg)
    init = _init(n, 7)
    t = torch.from_numpy(init.view(np.int32).copy()).cuda()
    res = hs.run(cfg, t)
    torch.cuda.synchronize()
    got = t.cpu().numpy().view(np.uint32)
    want = oracle.golden(7, 256, 30, 8, 3, 1, hs.device_info()["nsm"], False, init)
    assert np.array_equal(got, want)
    assert res.ops == 8 * 3


@pytest.mark.parametrize("prim", [0, 2])
def test_barrier_timeout_is_reported(hs, prim):
    """A TB that never arrives makes the others' bounded waits run out: the run
    returns HS_ETIMEDOUT, nothing hangs, and the context stays usable."""
    cfg = hs.RunConfig(prim=prim, num_ldst=4, num_tbs=16, num_iters=4, threads=64, repeats=1, mode="inc",
                       nsm=8, timeout_ns=20_000_000, skip_tb=5)
    st = np.zeros(hs.storage_words(cfg), dtype=np.uint32)
    res = hs.run(cfg, st, check=False)
    assert res.status == 2  # HS_ETIMEDOUT
    assert res.dev_error_bits & 1
    assert res.dev_error_site in (6, 7, 8, 9)
    ok = hs.RunConfig(prim=prim, num_ldst=4, num_tbs=16, num_iters=4, threads=64, repeats=1, mode="inc", nsm=8)
    st = np.zeros(hs.storage_words(ok), dtype=np.uint32)
    assert hs.run(ok, st).status == 0


def test_barrier_co_residency_rejected(hs):
    nsm = hs.device_info()["nsm"]
    cfg = hs.RunConfig(prim="atomicTreeBarrUniq", num_ldst=1, num_tbs=nsm * 64, num_iters=1, threads=1024,
                       repeats=1)
    st = np.zeros(hs.storage_words(cfg), dtype=np.uint32)
    res = hs.run(cfg, st, check=False)
    assert res.status == 3  # HS_ENORES, rejected before launch
    assert res.launches == 0


def test_uneven_barrier_groups_complete(hs, oracle):
    """numTBs not a multiple of NUM_SM: the reference kernels deadlock here
    (README.txt:80); these barriers count each group's real members."""
    for prim in (0, 2):
        cfg = hs.RunConfig(prim=prim, num_ldst=20, num_tbs=11, num_iters=3, threads=32, repeats=2, mode="inc",
                           nsm=4, timeout_ns=2_000_000_000)
        n = hs.storage_words(cfg)
        init = _init(n, 11)
        st = init.copy()
        hs.run(cfg, st)
        want = oracle.golden(prim, 32, 20, 11, 3, 2, 4, True, init)
        assert np.array_equal(st, want)


@pytest.mark.parametrize("prim", [0, 1, 2, 3])
@pytest.mark.parametrize("mult", [2, 4])
@pytest.mark.parametrize("L", [10, 64, 100])
def test_barrier_groups_on_clusters(hs, oracle, prim, mult, L):
    """numTBs = mult * NUM_SM: each logical-SM group runs as one CTA of mult x
    256 threads (the local stage is the CTA barrier; register path up to
    numLdSt 64, two bulk-copy buffers above), or as one thread-block cluster
    (local stage = hardware cluster barrier), or flat; every form's result
    equals the golden's, on the register path and the tiled bulk-copy path."""
    nsm = hs.device_info()["nsm"]
    G = mult * nsm
    outs = []
    for flags in (0, hs.RUN_NO_GROUP_CTA, hs.RUN_NO_CLUSTER):
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=4, threads=256, repeats=2, mode="inc",
                           flags=flags, timeout_ns=5_000_000_000)
        init = _init(hs.storage_words(cfg), prim + 7 * mult)
        st = init.copy()
        res = hs.run(cfg, st)
        assert res.status == 0
        if flags == 0:
            assert res.tbs_per_cta == mult and res.cluster == 1   # one CTA per logical-SM group
        else:
            assert res.tbs_per_cta == 1
            # clusters of `mult` are used when numTBs / mult of them can be resident
            # (at 4 per SM the GPCs do not hold every cluster of 4: flat launch)
            assert res.cluster in ((mult, 1) if flags != hs.RUN_NO_CLUSTER else (1,))
            if mult == 2 and flags != hs.RUN_NO_CLUSTER:
                assert res.cluster == 2
        assert np.array_equal(st, hs.expected_storage(cfg, init))
        outs.append(st)
    want = oracle.golden(prim, 256, L, G, 4, 2, nsm, True, init)
    for o in outs:
        assert np.array_equal(o, want)


@pytest.mark.parametrize("prim", [0, 1, 2, 3])
@pytest.mark.parametrize("T,mult,nsm", [(128, 8, 0), (64, 4, 6), (32, 16, 5), (256, 2, 3), (16, 3, 4)])
@pytest.mark.parametrize("mode", ["ref", "inc"])
def test_barrier_group_cta_shapes(hs, oracle, prim, T, mult, nsm, mode):
    """The group-CTA form at other shapes: up to 16 logical TBs per CTA,
    half-warp TBs, logical NUM_SM below the device's, reference and INC data
    modes; three launches (the generations carry across launches); equal to the
    literal golden."""
    dev_nsm = hs.device_info()["nsm"]
    n = nsm or dev_nsm
    cfg = hs.RunConfig(prim=prim, num_ldst=9, num_tbs=mult * n, num_iters=5, threads=T, repeats=3, mode=mode,
                       nsm=nsm, timeout_ns=5_000_000_000)
    init = _init(hs.storage_words(cfg), 31 * prim + mult)
    st = init.copy()
    res = hs.run(cfg, st)
    assert res.status == 0 and res.tbs_per_cta == mult
    assert np.array_equal(st, oracle.golden(prim, T, 9, mult * n, 5, 3, n, mode == "inc", init))


@pytest.mark.parametrize("prim", [0, 1, 2, 3])
@pytest.mark.parametrize("T,mult,nsm,L", [(256, 2, 0, 100), (256, 4, 7, 127), (128, 8, 6, 65), (64, 15, 5, 80),
                                          (256, 3, 4, 100), (32, 8, 6, 70)])
@pytest.mark.parametrize("mode", ["ref", "inc"])
def test_barrier_group_cta_bulk_copies(hs, oracle, prim, T, mult, nsm, L, mode):
    """The group-CTA form above numLdSt 64: the group's chunks go through two
    bulk-copy buffers (tiles that split a chunk at numLdSt 127, many small
    chunks at 64 threads), three launches; equal to the literal golden and to
    the one-CTA-per-TB form."""
    dev_nsm = hs.device_info()["nsm"]
    n = nsm or dev_nsm
    outs = []
    for flags in (0, hs.RUN_NO_GROUP_CTA):
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=mult * n, num_iters=4, threads=T, repeats=3, mode=mode,
                           nsm=nsm, flags=flags, timeout_ns=5_000_000_000)
        init = _init(hs.storage_words(cfg), 17 * prim + mult + L)
        st = init.copy()
        res = hs.run(cfg, st)
        assert res.status == 0 and res.tbs_per_cta == (mult if flags == 0 else 1)
        outs.append(st)
    want = oracle.golden(prim, T, L, mult * n, 4, 3, n, mode == "inc", init)
    for o in outs:
        assert np.array_equal(o, want)


@pytest.mark.parametrize("prim", [20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31])
@pytest.mark.parametrize("mult,L", [(2, 10), (4, 40), (8, 7)])
@pytest.mark.parametrize("mode", ["inc", "ref"])
def test_uniq_groups_on_clusters(hs, oracle, prim, mult, L, mode):
    """Per-SM (Uniq) mutexes and semaphores with numTBs = mult * NUM_SM: each
    group is one cluster and its lock word lives in distributed shared memory;
    the result equals the flat launch's and the golden's."""
    nsm = 16  # logical SMs: small groups keep the golden fast
    G = mult * nsm
    outs = []
    for flags in (0, hs.RUN_NO_CLUSTER):
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=3, threads=64, repeats=2, mode=mode, nsm=nsm,
                           flags=flags, timeout_ns=5_000_000_000)
        init = _init(hs.storage_words(cfg), prim * 10 + mult)
        st = init.copy()
        res = hs.run(cfg, st)
        # clusters when all nsm of them fit at once (always at 16 logical SMs)
        assert res.status == 0 and res.cluster == (mult if flags == 0 else 1)
        outs.append(st)
    want = oracle.golden(prim, 64, L, G, 3, 2, nsm, mode == "inc", init)
    assert np.array_equal(outs[0], want) and np.array_equal(outs[1], want)


@pytest.mark.parametrize("prim", [20, 23])
def test_uniq_slice_on_clusters(hs, oracle, prim):
    cfg = hs.RunConfig(prim=prim, num_ldst=5, num_tbs=64, num_iters=4, threads=32, repeats=2, mode="slice", nsm=16)
    init = _init(hs.storage_words(cfg), prim)
    st = init.copy()
    res = hs.run(cfg, st)
    assert res.cluster == 4
    assert np.array_equal(st, oracle.slice_replay(True, 5, 64, 4, 2, 16, init))


@pytest.mark.parametrize("name,base", [("PRspinSem1", 8), ("PRspinSem120", 11), ("PRspinSemEBO2", 13),
                                       ("PRspinSemEBO10", 14), ("atomicTreeBarrUniqSRB", 0),
                                       ("atomicTreeBarrUniqLocalExchSRB", 1), ("atomicTreeBarrUniqNaiveSRB", 0),
                                       ("atomicTreeBarrUniqLocalExchNaiveSRB", 1),
                                       ("atomicTreeBarrUniqNaiveAllSRB", 0),
                                       ("atomicTreeBarrUniqLocalExchNaiveAllSRB", 1)])
@pytest.mark.parametrize("mode", ["ref", "inc"])
def test_hip_extension_primitives(hs, oracle, name, base, mode):
    """The HIP build's priority semaphores and sense-reversing barriers: the
    final storage is the CUDA base primitive's golden."""
    for ci, (T, L, G, iters, reps, nsm) in enumerate(CASES[:4]):
        cfg = hs.RunConfig(prim=name, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=reps, mode=mode,
                           nsm=nsm, timeout_ns=5_000_000_000)
        init = _init(hs.storage_words(cfg), base * 7 + ci)
        st = init.copy()
        res = hs.run(cfg, st)
        assert res.status == 0
        assert np.array_equal(st, oracle.golden(base, T, L, G, iters, reps, nsm, mode == "inc", init)), (name, ci)
