"""bench.py's lock-latency floors, from a stand-in probe and sweep records (no
GPU): a CAS lock's floor is hand-off + atomic + 2 x L2 load, a queue lock's
drops the atomic; each numLdSt-10 lock cell at NUM_SM TBs is reported as the
fraction of its floor; other cells are left out."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Probe:
    @staticmethod
    def probe_latency(rounds):
        assert rounds > 0
        return {"handoff_ns_median": 700.0, "handoff_ns_min": 400.0, "handoff_ns_max": 800.0,
                "atomic_rtt_ns": 300.0, "load_rtt_ns": 150.0, "partners": 151, "dev_error_bits": 0}


def _rec(prim, tbs, L, us_per_op, ops=1000):
    return {"prim": prim, "num_tbs": tbs, "num_ldst": L, "ops": ops, "ms": us_per_op * ops * 1e-3}


def test_floors_and_fractions():
    recs = [_rec("spinMutex", 152, 10, 1.6), _rec("spinMutex", 152, 10, 1.4), _rec("faMutex", 152, 10, 1.25),
            _rec("spinSem1", 152, 10, 2.6), _rec("spinMutex", 304, 10, 9.0), _rec("faMutex", 152, 100, 9.0),
            _rec("atomicTreeBarrUniq", 152, 10, 0.02)]
    out = bench.lock_latency(_Probe, recs, 152)
    assert out["floor_ns"] == {"cas_lock": 1300.0, "queue_lock": 1000.0}
    cells = out["cells_152x10"]
    assert set(cells) == {"spinMutex", "faMutex", "spinSem1"}
    assert cells["spinMutex"]["us_per_op"] == 1.5 and cells["spinMutex"]["floor_us"] == 1.3
    assert abs(cells["spinMutex"]["frac"] - 1.3 / 1.5) < 1e-3
    assert cells["faMutex"]["floor_us"] == 1.0 and abs(cells["faMutex"]["frac"] - 0.8) < 1e-3
    assert abs(cells["spinSem1"]["frac"] - 0.5) < 1e-3
    assert out["handoff_ns"] == {"median": 700.0, "min": 400.0, "max": 800.0, "partners": 151}


def test_every_lock_primitive_has_a_chain():
    locks = [p for p in bench.SWEEP_PRIMS if "Barr" not in p]
    assert sorted(locks) == sorted(bench.LOCK_CHAIN)
    assert {bench.LOCK_CHAIN[p] for p in ("faMutex", "sleepMutex")} == {"queue"}
