"""Closed forms of the batch's relaxed-atomics instance kinds against a
direct restatement of their operations (no GPU)."""
import numpy as np
import pytest

T = 256
NSM = 152


def _init(n, seed):
    return np.random.default_rng(seed).integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("L,G,I", [(1, 4, 10), (7, 33, 12), (128, 512, 3), (100, 5, 77)])
def test_refcounter(hs, L, G, I):
    x = (hs.BATCH_REFCOUNTER, L, G, I)
    n = hs.batch_instance_words(x, NSM)
    assert n == 2 * L
    init = _init(n, L + G)
    total = np.zeros(L, dtype=np.uint64)
    for b in range(G):
        for j in range(I):
            idx = (b + j + np.arange(T)) % L
            np.add.at(total, idx, 1)
    want = init.copy()
    want[L:] = (init[L:].astype(np.uint64) + total).astype(np.uint32)
    assert np.array_equal(hs.batch_expected(x, init, NSM), want)


@pytest.mark.parametrize("L,G,I", [(1, 4, 10), (9, 200, 7), (128, 512, 5000)])
def test_splitcounter(hs, L, G, I):
    x = (hs.BATCH_SPLITCOUNTER, L, G, I)
    init = _init(hs.batch_instance_words(x, NSM), G)
    part = init.view(np.uint64).copy()
    for b in range(G):
        part[b % NSM] += np.uint64(I * T * L)
    assert np.array_equal(hs.batch_expected(x, init, NSM).view(np.uint64), part)


@pytest.mark.parametrize("G,I", [(4, 10), (5, 3), (511, 2)])
def test_seqlock(hs, G, I):
    x = (hs.BATCH_SEQLOCK, 3, G, I)
    init = _init(hs.batch_instance_words(x, NSM), G)
    writers = sum(1 for b in range(G) if b % 4 == 0)
    seq = 2 * writers * I
    pay = [(seq * 0x9E3779B97F4A7C15 + i) % 2 ** 64 for i in range(4)]
    want = init.copy()
    want[:8] = np.array(pay, dtype=np.uint64).view(np.uint32)
    assert np.array_equal(hs.batch_expected(x, init, NSM), want)


@pytest.mark.parametrize("L,G,I", [(1, 4, 10), (64, 100, 33)])
def test_flags(hs, L, G, I):
    x = (hs.BATCH_FLAGS, L, G, I)
    init = _init(hs.batch_instance_words(x, NSM), L)
    want = init.copy()
    want[:L] = I
    assert np.array_equal(hs.batch_expected(x, init, NSM), want)


def test_generator_draws_every_kind(hs):
    insts = hs.batch_generate(seed=20260101, n=512, nsm=NSM)
    kinds = {p for p, _, _, _ in insts}
    assert {60, 61, 62, 63} <= kinds and len(kinds) == 32


def test_syncprims_expected_matches_run_config_form(hs):
    for x in [(4, 10, 8, 3), (1, 20, 304, 2), (26, 7, 152, 4)]:
        p, L, G, I = x
        cfg = hs.RunConfig(prim=p, num_ldst=L, num_tbs=G, num_iters=I, threads=256, repeats=1, mode="inc", nsm=NSM)
        init = _init(hs.storage_words(cfg), p)
        assert np.array_equal(hs.batch_expected(x, init, NSM), hs.expected_storage(cfg, init, NSM))


def test_plan_cache_keys_and_round_trip(tmp_path):
    """Tuned batch plans are cached per (instances, mode, device): the key
    changes with any of them; a stored plan reads back; a missing or broken
    file reads as no plan."""
    import heterosync_gb300 as hs
    dev = {"nsm": 152, "cc": (10, 3), "max_threads_per_block": 1024}
    insts = [(4, 10, 8, 100), (62, 4, 32, 5)]
    k = hs.plan_cache_key(insts, "inc", dev)
    assert k == hs.plan_cache_key([tuple(x) for x in insts], "inc", dict(dev))
    assert k != hs.plan_cache_key(insts, "ref", dev)
    assert k != hs.plan_cache_key(insts[:1], "inc", dev)
    assert k != hs.plan_cache_key(insts, "inc", dict(dev, nsm=148))
    path = str(tmp_path / "sub" / "plans.json")
    assert hs.plan_cache_load(path, k) is None
    hs.plan_cache_store(path, k, {"settings": [8, 8, 32, 57344, 1024, 1], "ms": 12.5})
    hs.plan_cache_store(path, "other", {"settings": [1, 16, 128, 57344, 32, 8], "ms": 3.0})
    assert hs.plan_cache_load(path, k) == {"settings": [8, 8, 32, 57344, 1024, 1], "ms": 12.5}
    with open(path, "w") as f:
        f.write("{not json")
    assert hs.plan_cache_load(path, k) is None
