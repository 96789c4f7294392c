"""GPU: the tree barrier with local exchange on thread-block clusters moves
every CTA's buffer to the next CTA once per episode; the final buffers are a
bit-exact rotation of the seeded fp32 input, for cluster sizes 1, 2, 4, 8 and
both global stages (generation counter; flags with a master scan)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cluster", [1, 2, 4, 8])
@pytest.mark.parametrize("lf", [False, True])
@pytest.mark.parametrize("episodes", [0, 1, 7, 1000])
def test_rotation_592_ctas(hs, oracle, cluster, lf, episodes):
    x = hs.exchange_fill(20260101, 592, 4096)
    out, r = hs.exchange_run(x, cluster, lf, episodes)
    assert r.dev_error_bits == 0 and r.clusters == 592 // cluster
    assert np.array_equal(out, oracle.exchange_expected(x, episodes))


@pytest.mark.parametrize("n,elems,cluster", [(8, 4, 8), (24, 1028, 4), (152, 8192, 2), (304, 16, 1)])
def test_rotation_other_shapes(hs, oracle, n, elems, cluster):
    x = hs.exchange_fill(7, n, elems)
    for episodes in (3, n + 5):
        out, r = hs.exchange_run(x, cluster, episodes % 2 == 1, episodes)
        assert np.array_equal(out, oracle.exchange_expected(x, episodes))
