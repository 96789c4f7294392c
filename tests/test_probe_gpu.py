"""GPU: the roofline probes.  The L2 atomic rate and the lock hand-off
latencies must come back finite, ordered and in physically sensible ranges."""
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
