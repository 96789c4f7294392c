"""GPU: geometric SHA-1 UTS by work stealing over per-CTA lock-free queues;
node count, leaf count and deepest level exact against the oracle's
depth-first walk."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 2, 3, 4, 5, 7, 11, 13])
@pytest.mark.parametrize("limit", [4, 6, 8])
def test_counts_match_oracle(hs, oracle, seed, limit):
    nodes, leaves, deepest, ms = hs.uts_geo_run(seed, limit)
    assert (nodes, leaves, deepest) == oracle.geo_count(seed, limit)


@pytest.mark.parametrize("blocks,threads", [(1, 32), (3, 64), (152, 128), (608, 256)])
def test_launch_shapes(hs, oracle, blocks, threads):
    want = oracle.geo_count(2, 8)
    assert hs.uts_geo_run(2, 8, blocks=blocks, threads=threads)[:3] == want


def test_larger_tree_and_other_branching(hs, oracle):
    assert hs.uts_geo_run(4, 10)[:3] == oracle.geo_count(4, 10)
    assert hs.uts_geo_run(9, 6, branching=8.0)[:3] == oracle.geo_count(9, 6, 8.0)
    assert hs.uts_geo_run(11, 9, branching=2.0)[:3] == oracle.geo_count(11, 9, 2.0)
