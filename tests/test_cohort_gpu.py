"""GPU: the die-aware cohort global mutexes (spin, EBO, FA; the ring "sleep"
mutex stays plain).  Final storage
must be bit-exact against the golden's closed form with the cohort lock and
with HS_RUN_NO_COHORT, in every data mode and at every sweep size, including
repeats that keep the ticket state; the run must report which lock ran."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(hs, cfg, seed):
    init = np.random.default_rng(seed).integers(0, 1000, size=hs.storage_words(cfg)).astype(np.uint32)
    want = hs.expected_storage(cfg, init)
    st = init.copy()
    r = hs.run(cfg, st)
    assert np.array_equal(st, want), cfg
    return r


@pytest.mark.parametrize("prim", ["spinMutex", "spinMutexEBO", "sleepMutex", "faMutex"])
@pytest.mark.parametrize("mult,L", [(1, 10), (2, 10), (4, 100), (1, 100)])
@pytest.mark.parametrize("mode", ["inc", "ref"])
def test_cohort_exact(hs, prim, mult, L, mode):
    nsm = hs.device_info()["nsm"]
    cfg = hs.RunConfig(prim, L, mult * nsm, 40, threads=256, repeats=2, mode=mode)
    r = _check(hs, cfg, mult * 100 + L)
    plain = hs.RunConfig(prim, L, mult * nsm, 40, threads=256, repeats=2, mode=mode, flags=hs.RUN_NO_COHORT)
    r0 = _check(hs, plain, mult * 100 + L)
    assert r0.cohort == 0
    assert r.cohort in (0, 1)


def test_cohort_runs_on_this_part(hs):
    nsm = hs.device_info()["nsm"]
    r = _check(hs, hs.RunConfig("spinMutex", 10, nsm, 20, threads=256, repeats=1, mode="inc"), 1)
    assert r.cohort == 1  # GB300: two dies
    ring = _check(hs, hs.RunConfig("sleepMutex", 10, nsm, 20, threads=256, repeats=1, mode="inc"), 3)
    assert ring.cohort == 0  # a queue lock already: no die queue in front of it
    one = _check(hs, hs.RunConfig("spinMutex", 10, 1, 20, threads=256, repeats=1, mode="inc"), 2)
    assert one.cohort == 0  # a single TB needs no lock hand-off


@pytest.mark.parametrize("prim", ["spinMutex", "faMutex", "spinMutexEBO", "sleepMutex"])
def test_cohort_slice_and_reference_threads(hs, prim):
    nsm = hs.device_info()["nsm"]
    _check(hs, hs.RunConfig(prim, 10, 8, 100, threads=256, repeats=1, mode="slice"), 3)
    _check(hs, hs.RunConfig(prim, 10, 2 * nsm, 30, threads=32, repeats=10, mode="ref"), 4)


@pytest.mark.parametrize("prim", ["faMutex", "spinMutexEBO", "spinMutex"])
def test_cohort_ticket_state_kept_across_repeats(hs, prim):
    # die tickets and turns carry over from launch to launch
    nsm = hs.device_info()["nsm"]
    _check(hs, hs.RunConfig(prim, 10, nsm, 25, threads=256, repeats=1, mode="inc"), 4)  # initialises the state
    cfg = hs.RunConfig(prim, 10, nsm, 25, threads=256, repeats=3, mode="inc", flags=hs.RUN_KEEP_STATE)
    for seed in (5, 6):
        r = _check(hs, cfg, seed)
        assert r.cohort == 1
