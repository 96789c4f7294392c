"""GPU: cooperative CPU+GPU geometric UTS.  GPU CTAs and host threads walk one
tree through the bridge rings in mapped pinned memory; the counts must equal
the oracle (and the GPU-only kernel) however the work was split, both sides
must have expanded nodes on a tree large enough to share, and the GPU-only
form of the cooperative kernel (no host walkers) must agree too."""
import pytest

pytestmark = pytest.mark.gpu


def _coop(hs, *args, **kw):
    try:
        return hs.uts_geo_coop_run(*args, **kw)
    except hs.HsError as e:
        if e.status == hs.HS_EINVAL and "native atomics" in str(e):
            pytest.skip("the host link has no native atomics")
        raise


@pytest.mark.parametrize("seed,depth,walkers", [(2, 6, 4), (3, 8, 2), (5, 9, -1), (7, 5, 3), (11, 9, 8)])
def test_counts_exact(hs, oracle, seed, depth, walkers):
    r = _coop(hs, seed, depth, 4.0, host_threads=walkers)
    assert (r["nodes"], r["leaves"], r["max_depth"]) == oracle.geo_count(seed, depth, 4.0)
    assert r["gpu_nodes"] + r["host_nodes"] == r["nodes"]


def test_both_sides_work_on_a_large_tree(hs):
    want = hs.uts_geo_run(2, 11, 4.0)[:3]
    for _ in range(2):
        r = _coop(hs, 2, 11, 4.0, host_threads=-1)
        assert (r["nodes"], r["leaves"], r["max_depth"]) == want
        assert r["to_host"] > 0 and r["host_nodes"] > 0 and r["gpu_nodes"] > 0
        assert r["dev_error_bits"] == 0


def test_gpu_side_alone_through_the_bridge(hs, oracle):
    r = _coop(hs, 3, 9, 4.0, host_threads=0)
    assert (r["nodes"], r["leaves"], r["max_depth"]) == oracle.geo_count(3, 9, 4.0)
    assert r["host_nodes"] == 0 and r["to_host"] == 0


def test_small_grids(hs, oracle):
    for blocks, threads in [(1, 32), (2, 64), (7, 96)]:
        r = _coop(hs, 4, 7, 4.0, blocks=blocks, threads=threads, host_threads=2)
        assert (r["nodes"], r["leaves"], r["max_depth"]) == oracle.geo_count(4, 7, 4.0)
