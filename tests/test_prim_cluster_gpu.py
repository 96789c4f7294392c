"""GPU: global mutexes and semaphores with a bulk-copy critical section
(numLdSt > 32) run one thread-block cluster per logical TB, the critical
section split over the cluster's SMs (HS_RUN_CLUSTER_CS for every such run;
by default semaphores whose writers own 4 or more chunks).  Final storage
must equal the flat launch's (HS_RUN_NO_CLUSTER), the golden's closed form
and, on small cases, the oracle's literal golden replay; the cluster size
follows the TB's half-warp regions (8 at 256 threads, 4 at 64, 2 at 32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GLOBAL = [4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15]


def _init(n, seed):
    return np.random.default_rng(seed).integers(0, 1000, size=n).astype(np.uint32)


@pytest.mark.parametrize("prim", GLOBAL)
@pytest.mark.parametrize("mode", ["inc", "ref"])
def test_cluster_equals_flat(hs, prim, mode):
    nsm = hs.device_info()["nsm"]
    for L, G in [(33, nsm), (64, 2 * nsm + 7), (100, 4 * nsm)]:
        outs = []
        for flags in (hs.RUN_CLUSTER_CS, hs.RUN_NO_CLUSTER):
            cfg = hs.RunConfig(prim, L, G, 5, threads=256, repeats=2, mode=mode, flags=flags)
            init = _init(hs.storage_words(cfg), prim * 100 + L)
            st = init.copy()
            r = hs.run(cfg, st)
            assert r.cluster == (8 if flags == hs.RUN_CLUSTER_CS else 1), (prim, L, G)
            assert np.array_equal(st, hs.expected_storage(cfg, init)), (prim, L, G, flags)
            outs.append(st)
        assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("threads,m", [(32, 2), (64, 4), (112, 4), (208, 8)])
def test_cluster_sizes_follow_regions(hs, threads, m):
    nsm = hs.device_info()["nsm"]
    for prim in (4, 7, 8, 14):
        cfg = hs.RunConfig(prim, 40, 2 * nsm, 4, threads=threads, repeats=1, mode="inc", flags=hs.RUN_CLUSTER_CS)
        init = _init(hs.storage_words(cfg), threads + prim)
        st = init.copy()
        r = hs.run(cfg, st)
        assert r.cluster == m
        assert np.array_equal(st, hs.expected_storage(cfg, init)), (prim, threads)


@pytest.mark.parametrize("prim", [4, 6, 7, 9, 13])
def test_cluster_against_oracle_golden(hs, oracle, prim):
    nsm = 16
    cfg = hs.RunConfig(prim, 40, 48, 3, threads=64, repeats=2, mode="ref", nsm=nsm, flags=hs.RUN_CLUSTER_CS)
    init = _init(hs.storage_words(cfg), prim)
    st = init.copy()
    r = hs.run(cfg, st)
    assert r.cluster == 4
    assert np.array_equal(st, oracle.golden(prim, 64, 40, 48, 3, 2, nsm, False, init))


def test_cluster_in_a_graph(hs):
    nsm = hs.device_info()["nsm"]
    cfg = hs.RunConfig("spinSem2", 100, 2 * nsm, 5, threads=256, repeats=3, mode="inc",
                       flags=hs.RUN_GRAPH | hs.RUN_CLUSTER_CS)
    init = _init(hs.storage_words(cfg), 11)
    for _ in range(2):
        st = init.copy()
        r = hs.run(cfg, st)
        assert r.cluster == 8 and np.array_equal(st, hs.expected_storage(cfg, init))


def test_default_choice(hs):
    """By default only semaphores whose writers own 4 or more chunks take clusters."""
    nsm = hs.device_info()["nsm"]
    for prim, G, want in [("spinSem1", 4 * nsm, 8), ("spinSemEBO120", 5 * nsm, 8), ("spinSem10", 2 * nsm, 1),
                          ("faMutex", 4 * nsm, 1), ("spinMutex", nsm, 1)]:
        cfg = hs.RunConfig(prim, 100, G, 3, threads=256, repeats=1, mode="ref")
        init = _init(hs.storage_words(cfg), G)
        st = init.copy()
        r = hs.run(cfg, st)
        assert r.cluster == want, (prim, G)
        assert np.array_equal(st, hs.expected_storage(cfg, init))
