"""GPU: the reference's own kernels (compiled from its unmodified sources into
oracle/_ref) against the oracle and against this build, on the same inputs.
This pins the oracle to the reference itself."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _need_ref(oracle, T):
    if not oracle.ref_available(T):
        pytest.skip("reference modules (oracle/_ref) not present")


@pytest.mark.parametrize("prim", [0, 1, 2, 3, 4, 5, 6, 7, 20, 21, 22, 23])
def test_reference_kernels_match_oracle_and_build(hs, oracle, prim):
    _need_ref(oracle, 32)
    nsm, _ = oracle.ref_device()
    T, reps = 32, 10
    if prim <= 3:
        G, L, iters = 2 * nsm, 45, 2
    elif prim <= 7:
        G, L, iters = 2, 25, 1
    else:
        G, L, iters = nsm + 8, 25, 1
    n = oracle.storage_words(prim, T, L, G, nsm)
    init = np.arange(n, dtype=np.float32).view(np.uint32)
    ref_final, _ = oracle.ref_run(prim, T, L, G, iters, reps, init)
    want = oracle.golden(prim, T, L, G, iters, reps, nsm, False, init)
    assert np.array_equal(ref_final, want), "reference kernels differ from the oracle"
    cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=reps, mode="ref")
    mine = init.copy()
    hs.run(cfg, mine)
    assert np.array_equal(mine, ref_final), "this build differs from the reference kernels"


def test_reference_t256_faMutex(hs, oracle):
    _need_ref(oracle, 256)
    init = np.arange(oracle.storage_words(7, 256, 30, 3, 152), dtype=np.float32).view(np.uint32)
    nsm, _ = oracle.ref_device()
    ref_final, ms = oracle.ref_run(7, 256, 30, 3, 1, 10, init)
    assert np.array_equal(ref_final, oracle.golden(7, 256, 30, 3, 1, 10, nsm, False, init))
    assert ms > 0


def test_reference_runner_refuses_deadlocking_barrier(oracle):
    _need_ref(oracle, 32)
    nsm, _ = oracle.ref_device()
    G = nsm + 3  # neither <= NUM_SM nor a multiple: the reference barrier would hang
    init = np.zeros(oracle.storage_words(0, 32, 2, G, nsm), dtype=np.uint32)
    with pytest.raises(RuntimeError, match="deadlock"):
        oracle.ref_run(0, 32, 2, G, 1, 1, init)


def test_reference_runner_refuses_uniq_semaphores(oracle):
    """The reference's per-SM semaphore kernels livelocked on GB300; the runner
    refuses them instead of launching them again."""
    _need_ref(oracle, 32)
    init = np.zeros(oracle.storage_words(24, 32, 2, 4, 152), dtype=np.uint32)
    with pytest.raises(RuntimeError, match="livelock"):
        oracle.ref_run(24, 32, 2, 4, 1, 1, init)


@pytest.mark.parametrize("prim", [8, 12])
def test_reference_runner_refuses_global_semaphores(oracle, prim):
    """The reference's global semaphore kernels can wait forever (maxSemCount is
    read from the live count at kernel start); the runner refuses them."""
    _need_ref(oracle, 32)
    init = np.zeros(oracle.storage_words(prim, 32, 2, 4, 152), dtype=np.uint32)
    with pytest.raises(RuntimeError, match="maxSemCount"):
        oracle.ref_run(prim, 32, 2, 4, 1, 1, init)


@pytest.mark.parametrize("case", [(32, 64, 32, 4), (1, 8, 256, 3), (4, 152, 128, 2), (2, 16, 64, 10)])
def test_reference_refcounter_matches_build(hs, oracle, case):
    """refCounter: the reference's own kernel (one launch, refCounter.cu:24-82)
    and this build leave the same final counters (all references dropped), and
    both set delete flags (refCounter.cu:86-120)."""
    import os
    if not os.path.exists(oracle.ref_refcounter_module()):
        pytest.skip("reference refCounter module not present")
    sharers, tbs, tb_size, reps = case
    r0, r1, rd0, rd1, _ = oracle.ref_refcounter(sharers, tbs, tb_size, reps)
    c0, c1, d0, d1, _ = hs.refcounter(sharers, tbs, tb_size, reps)
    assert np.array_equal(c0, r0) and np.array_equal(c1, r1)
    assert rd0.any() and rd1.any() and d0.any() and d1.any()
