"""Cooperative CPU+GPU geometric UTS, host side only (no GPU): with no CTAs
the library's host walkers walk the whole tree, sharing work through their
deque, and the counts must equal the oracle's depth-first walk for any number
of walkers; bad arguments are rejected before anything runs."""
import pytest


CASES = [(2, 6, 1), (3, 7, 4), (5, 9, 8), (7, 5, 3), (11, 8, 16), (4, 8, 2), (0, 0, 4)]


@pytest.mark.parametrize("seed,depth,walkers", CASES)
def test_host_walkers_count_exactly(hs, oracle, seed, depth, walkers):
    r = hs.uts_geo_coop_run(seed, depth, 4.0, blocks=0, host_threads=walkers)
    assert (r["nodes"], r["leaves"], r["max_depth"]) == oracle.geo_count(seed, depth, 4.0)
    assert r["gpu_nodes"] == 0 and r["host_nodes"] == r["nodes"]
    assert r["to_host"] == 0 and r["to_gpu"] == 0
    assert r["host_threads"] == walkers


def test_other_branching_factors(hs, oracle):
    for b in (1.5, 2.0, 6.0):
        r = hs.uts_geo_coop_run(9, 6, b, blocks=0, host_threads=3)
        assert (r["nodes"], r["leaves"], r["max_depth"]) == oracle.geo_count(9, 6, b)


@pytest.mark.parametrize("args", [
    dict(depth_limit=-1), dict(depth_limit=31), dict(branching=0.0), dict(host_threads=0),
    dict(host_threads=2000),
])
def test_rejects_bad_arguments(hs, args):
    kw = dict(seed=1, depth_limit=5, branching=4.0, blocks=0, host_threads=2)
    kw.update(args)
    with pytest.raises(hs.HsError) as e:
        hs.uts_geo_coop_run(**kw)
    assert e.value.status == hs.HS_EINVAL
