"""GPU: mixed-instance batches (one persistent graph-replayed launch) against
one launch per instance; every instance bit-exact against the closed form of
the reference golden in both forms."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _expected(hs, inst, init, mode):
    return hs.batch_expected(inst, init, mode=mode)


def _run_both(hs, insts, mode="inc"):
    b = hs.Batch(insts, mode=mode)
    rng = np.random.default_rng(5)
    inits = [rng.integers(0, 2**32, size=b.words(i), dtype=np.uint64).astype(np.uint32) for i in range(len(insts))]
    for i, a in enumerate(inits):
        b.set_storage(i, a)
    rs = b.run_serial()
    for i, a in enumerate(inits):
        assert np.array_equal(b.get_storage(i), _expected(hs, insts[i], a, mode)), ("serial", i, insts[i])
        b.set_storage(i, a)
    v, _ = b.autotune()
    for i, a in enumerate(inits):
        b.set_storage(i, a)
    rb = b.run()
    for i, a in enumerate(inits):
        assert np.array_equal(b.get_storage(i), _expected(hs, insts[i], a, mode)), ("batched", i, insts[i])
    b.close()
    return rs, rb, v


def test_every_primitive_once(hs):
    insts = [(p, 7 + (p % 5) * 9, 3 + p % 13, 6 + p % 4) for p in
             [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31,
              60, 61, 62, 63]]
    rs, rb, v = _run_both(hs, insts)
    assert rb.grid > 0 and rb.ops == rs.ops
    assert rs.launches >= len(insts)


def test_generated_mixed_batch(hs):
    insts = hs.batch_generate(seed=20260101, n=64, iter_div=100)
    assert len(insts) == 64
    rs, rb, v = _run_both(hs, insts)
    assert rb.ops == rs.ops == sum(G * I for _, _, G, I in insts)


def test_ref_mode_batch(hs):
    insts = hs.batch_generate(seed=7, n=16, iter_div=500)
    insts = [(p, max(L, 10), G, min(I, 3)) for (p, L, G, I) in insts]
    _run_both(hs, insts, mode="ref")


def test_plan_rejects_non_co_resident_gangs(hs):
    insts = [(7, 4, 512, 2)] * 8  # 4096 logical TBs
    b = hs.Batch(insts)
    s, grid, cap = b.plan(1)
    assert grid == 4096 and (s == 3) == (grid > cap)
    b.close()


@pytest.mark.parametrize("cl", [2, 4, 8])
@pytest.mark.parametrize("mode", ["inc", "ref"])
def test_cluster_plans_bit_exact(hs, cl, mode):
    """Clusters of cl CTAs execute each mutex/semaphore operation together (the
    leader holds the lock, every rank moves a slice of the regions)."""
    insts = [(p, 5 + (p % 7) * 13, 2 + p % 11, 3 + p % 3) for p in
             [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]]
    b = hs.Batch(insts, mode=mode)
    rng = np.random.default_rng(11 + cl)
    inits = [rng.integers(0, 2**32, size=b.words(i), dtype=np.uint64).astype(np.uint32) for i in range(len(insts))]
    for se in (1, 2, 0):
        s, grid, cap = b.plan_ex(cl, se, 1)
        if s == 3:
            continue
        assert s == 0 and grid % cl == 0
        assert b.get_plan()[:3] == (cl, se, 1)
        for i, a in enumerate(inits):
            b.set_storage(i, a)
        r = b.run()
        assert r.dev_error_bits == 0
        for i, a in enumerate(inits):
            assert np.array_equal(b.get_storage(i), _expected(hs, insts[i], a, mode)), (cl, se, i, insts[i])
    b.close()



@pytest.mark.parametrize("kind", [60, 61, 62, 63])
def test_relaxed_kinds(hs, kind):
    """RefCounter, SplitCounter, Seqlock (4 x u64 payload) and Flags instances:
    final counters, payload and data exact, no torn seqlock read and no flag
    violation (those counts are part of the compared storage), batched and
    per-launch."""
    insts = [(kind, L, G, I) for (L, G, I) in [(1, 4, 50), (17, 64, 20), (128, 300, 8), (64, 512, 3)]]
    _run_both(hs, insts)
