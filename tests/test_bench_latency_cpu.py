"""bench.py's latency roofline, from stand-ins for the probe and the runs (no
GPU): a lock's floor per op is one hand-off, two L2 loads and (for an op that
enters by CAS) one atomic, plus the extra time one uncontended TB spends on a larger numLdSt
than 10; the roofline fraction
is the floor-weighted ops over the measured time of the dominant kernel's
cells.  Also the sweep aggregate: each cell counts once at its mean time."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Res:
    def __init__(self, ops, ms):
        self.ops, self.elapsed_ms = ops, ms


class _HS:
    """Stand-in for the package: fixed probe figures, and 1-TB runs whose time
    per op is 2 us at numLdSt 10 and 4 us at 100."""

    class RunConfig:
        def __init__(self, **kw):
            self.__dict__.update(kw)

    @staticmethod
    def probe_latency(rounds):
        assert rounds > 0
        return {"handoff_ns_median": 700.0, "handoff_ns_min": 400.0, "handoff_ns_max": 800.0,
                "atomic_rtt_ns": 300.0, "load_rtt_ns": 150.0, "partners": 151, "dev_error_bits": 0}

    @staticmethod
    def storage_words(cfg):
        return 16

    @staticmethod
    def run(cfg, storage):
        assert cfg.num_tbs == 1
        us = 2.0 if cfg.num_ldst == 10 else 4.0
        return _Res(cfg.num_iters, us * cfg.num_iters * 1e-3)


def test_floors():
    floors, lat = bench.lock_floors(_HS, ["spinMutex", "faMutex", "spinSem1", "lfTreeBarrUniq"])
    assert set(floors) == {(p, L) for p in ("spinMutex", "faMutex", "spinSem1") for L in (10, 100)}
    # every mutex passes through a die queue: hand-off + 2 loads, no atomic
    assert abs(floors[("spinMutex", 10)] - (0.7 + 0.3)) < 1e-9
    assert abs(floors[("spinMutex", 100)] - (0.7 + 0.3 + 2.0)) < 1e-9
    assert abs(floors[("faMutex", 10)] - (0.7 + 0.3)) < 1e-9
    assert abs(floors[("faMutex", 100)] - (0.7 + 0.3 + 2.0)) < 1e-9
    # a semaphore's writers pass through the die queue, its readers enter by CAS
    w, r = floors[("spinSem1", 100)]["writer"], floors[("spinSem1", 100)]["reader"]
    assert abs(w - (0.7 + 0.3 + 2.0)) < 1e-9 and abs(r - (0.7 + 0.3 + 0.3 + 2.0)) < 1e-9
    assert lat["floor_ns"] == {"cas_lock": 1300.0, "queue_lock": 1000.0}
    assert lat["handoff_ns"] == {"median": 700.0, "min": 400.0, "max": 800.0, "partners": 151}


def test_semaphore_cell_floor_weights_writers_and_readers():
    floors = {("spinSem2", 10): {"writer": 1.0, "reader": 1.4}}
    cell = {"prim": "spinSem2", "num_ldst": 10}
    # numTBs <= NUM_SM: every TB a writer; 2 per SM: half; 4 per SM: one in four
    assert bench.cell_floor(dict(cell, num_tbs=100), floors, 152) == 1.0
    assert abs(bench.cell_floor(dict(cell, num_tbs=304), floors, 152) - 1.2) < 1e-9
    assert abs(bench.cell_floor(dict(cell, num_tbs=608), floors, 152) - 1.3) < 1e-9


def _rec(prim, tbs, L, us_per_op, ops=1000):
    return {"prim": prim, "num_tbs": tbs, "num_ldst": L, "ops": ops, "ms": us_per_op * ops * 1e-3, "wall_s": 0.01}


def test_aggregate_and_roofline():
    recs = [_rec("spinMutex", 152, 10, 3.0), _rec("spinMutex", 152, 10, 5.0), _rec("faMutex", 152, 10, 2.0),
            _rec("lfTreeBarrUniq", 152, 10, 0.01)]
    cells, value, e2e = bench.aggregate(recs)
    assert set(cells) == {"spinMutex@152/10", "faMutex@152/10", "lfTreeBarrUniq@152/10"}
    assert abs(cells["spinMutex@152/10"]["us_per_op"] - 4.0) < 1e-9       # mean of its two runs
    assert abs(value - 3000 / ((4.0 + 2.0 + 0.01) * 1e-3 * 1e3 * 1e-3)) < 1e-6
    assert abs(e2e - 3000 / 0.03) < 1e-6
    floors = {("spinMutex", 10): 2.0, ("faMutex", 10): 1.0}
    roof = bench.latency_roofline(cells, floors, ["spinMutex", "faMutex"], None)
    assert roof["bound"] == "latency"
    assert abs(roof["frac"] - (1000 * 2.0 + 1000 * 1.0) / (1000 * 4.0 + 1000 * 2.0)) < 1e-9
    assert roof["cells"]["spinMutex@152/10"]["frac"] == 0.5


def test_every_lock_primitive_has_a_chain():
    locks = [p for p in bench.SWEEP_PRIMS if "Barr" not in p]
    assert sorted(locks) == sorted(bench.LOCK_CHAIN)
    assert {bench.LOCK_CHAIN[p] for p in bench.HEAD_PRIMS if "Barr" not in p} == {"queue"}
    assert {bench.LOCK_CHAIN[p] for p in bench.SEM_PRIMS} == {"sem"}
    assert bench.HEAD_PRIMS == [p for p in bench.SWEEP_PRIMS if "Sem" not in p]
