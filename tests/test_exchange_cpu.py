"""Tree barrier with local exchange: the host-side contract without a GPU
(argument checks that return before any device call, the seeded fp32 input
generator, the rotation oracle)."""
import numpy as np
import pytest


def test_fill_is_seeded_uniform_and_exact(hs):
    a = hs.exchange_fill(20260101, 8, 4096)
    b = hs.exchange_fill(20260101, 8, 4096)
    c = hs.exchange_fill(20260102, 8, 4096)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    f = a.view(np.float32)
    assert f.min() >= -1.0 and f.max() < 1.0
    # (int32)(r >> 40) * 2^-23 - 1: every value is k * 2^-23 - 1 with 0 <= k < 2^24
    k = (f.astype(np.float64) + 1.0) * 2.0 ** 23
    assert np.array_equal(k, np.floor(k)) and k.min() >= 0 and k.max() < 2 ** 24
    assert abs(float(f.mean())) < 0.02


@pytest.mark.parametrize("n,elems,cluster", [(10, 4096, 4), (16, 4094, 2), (16, 4096, 3), (0, 4096, 1),
                                             (16, 40000, 2)])
def test_bad_shapes_rejected_before_launch(hs, n, elems, cluster):
    buf = np.zeros((max(n, 1), elems), np.uint32)[:n]
    with pytest.raises(hs.HsError) as e:
        hs.exchange_run(buf, cluster, False, 3)
    assert e.value.status == 1  # HS_EINVAL


def test_rotation_oracle(oracle):
    x = np.arange(6 * 4, dtype=np.uint32).reshape(6, 4)
    assert np.array_equal(oracle.exchange_expected(x, 0), x)
    assert np.array_equal(oracle.exchange_expected(x, 1)[1], x[0])
    assert np.array_equal(oracle.exchange_expected(x, 1)[0], x[5])
    assert np.array_equal(oracle.exchange_expected(x, 6 * 7 + 2), oracle.exchange_expected(x, 2))
