"""GPU: the roofline probes.  The L2 atomic rate, the L2-resident copy rate and
the lock hand-off latencies must come back finite, ordered and in physically
sensible ranges."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_l2_atomic_probe(hs):
    nsm = hs.device_info()["nsm"]
    v, same = ctypes.c_double(), ctypes.c_double()
    assert hs.lib().hs_probe_l2_atomics(nsm * 8, 256, 64, 0, ctypes.byref(v)) == 0
    assert hs.lib().hs_probe_l2_atomics(nsm, 32, 200, 1, ctypes.byref(same)) == 0
    assert v.value > same.value > 1e6


def test_latency_probe(hs):
    nsm = hs.device_info()["nsm"]
    r = hs.probe_latency(64)
    assert r["partners"] == nsm - 1 and r["dev_error_bits"] == 0
    assert 20 < r["handoff_ns_min"] <= r["handoff_ns_median"] <= r["handoff_ns_max"] < 100000
    assert 20 < r["atomic_rtt_ns"] < 100000
    assert 20 < r["load_rtt_ns"] < 100000


def test_latency_probe_rejects_bad_rounds(hs):
    r = ctypes.c_char * 64
    assert hs.lib().hs_probe_latency(0, ctypes.byref(r())) == hs.HS_EINVAL


def test_l2_bandwidth_probe(hs):
    lib = hs.lib()
    lib.hs_probe_l2_bandwidth.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    v = ctypes.c_double()
    assert lib.hs_probe_l2_bandwidth(48 << 20, 10, ctypes.byref(v)) == 0
    assert 100.0 < v.value < 100000.0  # GB/s
    assert lib.hs_probe_l2_bandwidth(1024, 10, ctypes.byref(v)) == hs.HS_EINVAL
    assert lib.hs_probe_l2_bandwidth(48 << 20, 0, ctypes.byref(v)) == hs.HS_EINVAL
