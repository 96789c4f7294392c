"""Benchmark: sync ops/s of the SyncPrims hot path on GB300.

Headline workload (both arms run exactly this): the 8 SyncPrims the
reference's own CUDA build can run on GB300 -- spinMutex, spinMutexEBO,
sleepMutex, faMutex, atomicTreeBarrUniq(LocalExch), lfTreeBarrUniq(LocalExch)
-- at 256 threads/TB, numCSIters = 1000, numLdSt in {10, 100}, numTBs in
{1, 2, 4} x NUM_SM (148, 296, 592 on a 148-SM part; 152, 304, 608 here), seeded
uint32 shared data moved by the reference's critical section (bit-exact final
state checked after every run).  One step = one launch of each of the 8
primitives at one (numTBs, numLdSt) point; steps cycle through the 6 points.

  value  sync ops/s over the sweep: every (primitive, point) cell carries its
         numTBs * 1000 ops at its mean device time over the steps that ran it
         (so the figure does not depend on how often the step count visits each
         point); storage already resident in HBM, CUDA events on the launch stream
  e2e    the same, with each cell's wall time of the C-ABI call hs_run() on pinned
         HOST buffers (host->device copy, lock-state init, launch, device->host
         copy and status read-back inside the timed region)

  roofline      bound "latency": the dominant kernel (k_mutex) against its
                measured per-op floor, one lock hand-off plus one uncontended
                operation of the same primitive and numLdSt (see lock_floors)
  full_sweep    the 16-primitive sweep (the 8 above plus spinSem{1,2,10,120} and
                spinSemEBO{1,2,10,120}) once over the 6 points, outside the timed
                region; the reference's semaphore kernels cannot run on GB300
  per_cell_vs_reference  this arm's us/op against the reference arm's, per cell,
                when the reference arm ran on this machine just before

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Beside the sweep, outside its timed region, the line carries "fa_mutex_slice"
(faMutex, 8 TBs, numLdSt 10, 100 iterations: the one-launch slice workload),
"relaxed" (refCounter, splitCounter and seqlocks at 4 x NUM_SM TBs: ops/s and
the L2-atomic fraction), "exchange" (tree barrier with local exchange on thread-block clusters: 592
CTAs, fp32[4096] per CTA rotated every episode, 1000 episodes, cluster sizes
1/2/4/8), "batch" (the 64-instance mixed batch, one launch per instance against
the autotuned persistent graph-replayed launch), "serve" (the served request
loop: sustained request rate, p50/p99 latency and slowdown under Poisson
arrivals at 10-90% of it) and "uts_geo" (geometric SHA-1 UTS, depth 12,
nodes/s, on the GPU alone and with the host cores walking the same tree);
--no-extras skips them.

--impl reference runs the reference's own SyncPrims kernels (built from its
unmodified sources into oracle/_ref) on the same GPU, on the same cells, at the
same numCSIters = 1000 (no projection); without oracle/_ref it falls back to the
host std::thread port.  Multi-GPU: replicas only (each rank runs the whole
sweep on its own GPU; no data crosses GPUs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SWEEP_PRIMS = ["spinMutex", "spinMutexEBO", "sleepMutex", "faMutex",
               "spinSem1", "spinSem2", "spinSem10", "spinSem120",
               "spinSemEBO1", "spinSemEBO2", "spinSemEBO10", "spinSemEBO120",
               "atomicTreeBarrUniq", "atomicTreeBarrUniqLocalExch", "lfTreeBarrUniq", "lfTreeBarrUniqLocalExch"]
# The reference's global semaphore kernels are not run (they can wait forever
# on GB300: each CTA reads maxSemCount from the live count at kernel start), so
# the headline workload -- the one both arms run -- is the mutexes and barriers.
HEAD_PRIMS = [p for p in SWEEP_PRIMS if "Sem" not in p]
SEM_PRIMS = [p for p in SWEEP_PRIMS if "Sem" in p]
REF_EXCLUDED = ("not run: each CTA of the reference's semaphore kernels reads maxSemCount from the live "
                "count word at kernel start (main.cu:542-543, 695-696); a late writer that reads 0 can wait "
                "forever, and a run that launched them did not finish")
THREADS = 256
ITERS = 1000
WARM_ITERS = 20
LDST = (10, 100)
TB_MULT = (1, 2, 4)
SEED = 20260101
# where the reference arm leaves its per-cell times for the build arm run next on the same machine
REF_CELLS_FILE = os.path.join(tempfile.gettempdir(), "hs_reference_cells.json")


# DRAM bytes (read + write) of one launch of the dominant headline kernel, from
# one ncu capture (k_mutex, spinMutex, 152 TBs x 256 threads, numLdSt 100): the
# chunk and the lock word stay L2-resident, so DRAM traffic is the cold first
# read and does not grow with the launch's operations.
DRAM_BYTES_PER_LAUNCH = 184320 + 35840
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_mutex (spinMutex, 152 TBs x 256, numLdSt 100, "
                  "200 iterations); profiles/k_mutex_spinMutex_152tbs_L100.md")


def head_config(nsm):
    """The headline workload's description: the same object in both arms' lines."""
    return {"workload": "SyncPrims sweep: spinMutex, spinMutexEBO, sleepMutex, faMutex, atomicTreeBarrUniq(LocalExch), "
                        "lfTreeBarrUniq(LocalExch) x numTBs {%s} x numLdSt {10,100}, 256 threads/TB, numCSIters 1000, "
                        "reference critical section on seeded uint32 data"
                        % ",".join(str(m * nsm) for m in TB_MULT),
            "threads": THREADS, "num_iters": ITERS, "num_ldst": list(LDST),
            "num_tbs": [m * nsm for m in TB_MULT], "primitives": HEAD_PRIMS,
            "step": "one launch of each primitive at one (numTBs, numLdSt) point; steps cycle the 6 points; "
                    "each cell counts at its mean time over the steps that ran it",
            "l2": "flushed before every run (256 MiB write)"}


def sweep_points(nsm):
    return [(m * nsm, L) for m in TB_MULT for L in LDST]


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        busy = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def make_init(words, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=words, dtype=np.uint64).astype(np.uint32)


def pinned_like(arr):
    import torch
    t = torch.empty(arr.size, dtype=torch.int32, pin_memory=True)
    a = t.numpy().view(np.uint32)
    a[:] = arr
    return t, a


def run_cells(hs, prims, point, iters, check, flush):
    """Every primitive of `prims` at one (numTBs, numLdSt) point through hs_run
    with pinned host storage.  Returns per-run records."""
    G, L = point
    recs = []
    for name in prims:
        cfg = hs.RunConfig(prim=name, num_ldst=L, num_tbs=G, num_iters=iters, threads=THREADS, repeats=1,
                           mode="ref")
        words = hs.storage_words(cfg)
        init = make_init(words, SEED + G + L)
        _keep, host = pinned_like(init)
        flush()
        t0 = time.perf_counter()
        r = hs.run(cfg, host)
        wall = time.perf_counter() - t0
        if check:
            want = hs.expected_storage(cfg, init)
            if not np.array_equal(host, want):
                raise SystemExit("bench: %s numTBs=%d numLdSt=%d differs from the expected final state"
                                 % (name, G, L))
        recs.append({"prim": name, "num_tbs": G, "num_ldst": L, "iters": iters, "ops": r.ops,
                     "ms": r.elapsed_ms, "wall_s": wall, "bytes": words * 4, "launches": r.launches,
                     "cohort": r.cohort, "cluster": r.cluster})
    return recs


def cell_key(prim, G, L):
    return "%s@%d/%d" % (prim, G, L)


def aggregate(recs):
    """Per-cell means over the runs of each (primitive, numTBs, numLdSt) cell,
    and the sweep rate: sum of the cells' ops over the sum of their mean times."""
    cells = {}
    for r in recs:
        c = cells.setdefault(cell_key(r["prim"], r["num_tbs"], r["num_ldst"]),
                             {"prim": r["prim"], "num_tbs": r["num_tbs"], "num_ldst": r["num_ldst"], "ops": r["ops"],
                              "ms": [], "wall_s": []})
        c["ms"].append(r["ms"])
        c["wall_s"].append(r.get("wall_s", 0.0))
    for c in cells.values():
        c["mean_ms"] = sum(c["ms"]) / len(c["ms"])
        c["mean_wall_s"] = sum(c["wall_s"]) / len(c["wall_s"])
        c["us_per_op"] = c["mean_ms"] * 1e3 / c["ops"]
    ops = sum(c["ops"] for c in cells.values())
    ms = sum(c["mean_ms"] for c in cells.values())
    wall = sum(c["mean_wall_s"] for c in cells.values())
    return cells, (ops / (ms * 1e-3) if ms else None), (ops / wall if wall else None)


def cpu_baseline(nsm, prims=None, budget_s=15.0):
    """Host std::thread port (the oracle twins) on a bounded sample of the same
    sweep: every (primitive, numTBs, numLdSt) cell, each with an untimed
    5-iteration pilot and then a timed run whose iteration count spreads
    `budget_s` of CPU work evenly over the cells (at most 1000 iterations)."""
    import oracle
    import heterosync_gb300 as hs
    prims = prims or HEAD_PRIMS
    cores = os.cpu_count() or 1
    cells = [(name, G, L) for (G, L) in sweep_points(nsm) for name in prims]
    per_cell = budget_s / len(cells)
    total_ops, total_s, iters_used = 0, 0.0, []
    for name, G, L in cells:
        p = hs.prim_id(name)
        n = oracle.storage_words(p, THREADS, L, G, nsm)
        init = make_init(n, SEED)
        _, s5 = oracle.twin_run(p, THREADS, L, G, 5, 1, nsm, 0, init, threads=cores)
        it = int(max(5, min(ITERS, 5 * per_cell / max(s5, 1e-6))))
        _, secs = oracle.twin_run(p, THREADS, L, G, it, 1, nsm, 0, init, threads=cores)
        total_ops += G * ITERS                 # the cell's full-workload ops ...
        total_s += secs * ITERS / it           # ... at the sampled rate
        iters_used.append(it)
    return {"value": total_ops / total_s if total_s else None, "unit": "sync ops/s", "cores": cores,
            "kind": "port",
            "sample": "host std::thread twins over the %d cells of the headline sweep, numCSIters %d-%d per cell "
                      "(pilot-scaled, ~%.0f s of CPU work), each cell's rate projected to its numTBs*1000 ops"
                      % (len(cells), min(iters_used), max(iters_used), budget_s)}


L2_PROBE_BYTES = 48 << 20  # two 24 MiB buffers: well inside the 129 MB L2 (half of it per die)


def l2_bandwidth_peak(hs):
    """The L2-resident copy rate (hs_probe_l2_bandwidth), GB/s read + written."""
    import ctypes
    v = ctypes.c_double()
    hs.lib().hs_probe_l2_bandwidth.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    if hs.lib().hs_probe_l2_bandwidth(L2_PROBE_BYTES, 20, ctypes.byref(v)):
        return None
    return v.value


def l2_atomic_peak(hs):
    import ctypes
    v = ctypes.c_double()
    nsm = hs.device_info()["nsm"]
    if hs.lib().hs_probe_l2_atomics(nsm * 8, 256, 256, 0, ctypes.byref(v)):
        return None, None
    same = ctypes.c_double()
    hs.lib().hs_probe_l2_atomics(nsm * 4, 32, 2000, 1, ctypes.byref(same))
    return v.value, same.value


# The hand-off chain of each lock primitive as this build runs it on a two-die
# part: the spin, EBO and ticket mutexes are a die ticket queue in front of the
# primitive's lock (a pass is a release store, no atomic), the ring mutex hands
# its slot on (a queue lock), a semaphore's writers pass as the mutexes do while
# its readers enter by CAS
LOCK_CHAIN = {"spinMutex": "queue", "spinMutexEBO": "queue", "faMutex": "queue", "sleepMutex": "queue",
              "spinSem1": "sem", "spinSem2": "sem", "spinSem10": "sem", "spinSem120": "sem",
              "spinSemEBO1": "sem", "spinSemEBO2": "sem", "spinSemEBO10": "sem", "spinSemEBO120": "sem"}


def lock_floors(hs, prims):
    """The per-op latency floor of each serialised lock primitive at each
    numLdSt, from measurements on this GPU:

        floor(L) = hand-off + 2 x L2 load + (CAS entry ? atomic : 0) + (t1(L) - t1(10))

    The first three terms are the chain of one contended op at numLdSt 10: the
    next holder sees the release (the median one-way flag latency between two
    SMs), wins its atomic (an op that enters by CAS: a semaphore reader; a queue
    took its ticket ahead of time), loads its critical section and waits for
    its stores before releasing (two L2 round trips).  The last term is the
    extra critical-section time of a larger numLdSt: t1(L) is the time per op of
    the same primitive run by ONE TB (1000 uncontended rounds), so
    t1(L) - t1(10) is the data movement one SM adds, which no hand-off hides.
    A mutex's floor is a number; a semaphore's is {"writer": queue chain,
    "reader": CAS chain}, weighted per cell by its ops (cell_floor)."""
    lat = hs.probe_latency(256)
    h, a, ld = lat["handoff_ns_median"], lat["atomic_rtt_ns"], lat["load_rtt_ns"]
    t1 = {}
    for name in prims:
        if name not in LOCK_CHAIN:
            continue
        for L in LDST:
            cfg = hs.RunConfig(prim=name, num_ldst=L, num_tbs=1, num_iters=ITERS, threads=THREADS, repeats=1,
                               mode="ref")
            init = make_init(hs.storage_words(cfg), SEED)
            best = None
            for _ in range(3):
                r = hs.run(cfg, init.copy())
                us = r.elapsed_ms * 1e3 / r.ops
                best = us if best is None else min(best, us)
            t1[(name, L)] = best
    base = {"cas": h + a + 2 * ld, "queue": h + 2 * ld}
    floors = {}
    for (name, L), v in t1.items():
        extra = max(0.0, v - t1[(name, LDST[0])]) * 1e3 if (name, LDST[0]) in t1 else 0.0
        if LOCK_CHAIN[name] == "sem":
            floors[(name, L)] = {"writer": (base["queue"] + extra) * 1e-3, "reader": (base["cas"] + extra) * 1e-3}
        else:
            floors[(name, L)] = (base[LOCK_CHAIN[name]] + extra) * 1e-3
    return floors, {"handoff_ns": {"median": h, "min": lat["handoff_ns_min"], "max": lat["handoff_ns_max"],
                                   "partners": lat["partners"]},
                    "atomic_rtt_ns": a, "load_rtt_ns": ld,
                    "floor_ns": {"cas_lock": base["cas"], "queue_lock": base["queue"]},
                    "uncontended_us_per_op": {"%s/%d" % k: round(v, 4) for k, v in t1.items()},
                    "floor_us_per_op": {"%s/%d" % k: (round(v, 4) if not isinstance(v, dict) else
                                                      {r: round(x, 4) for r, x in v.items()})
                                        for k, v in floors.items()},
                    "model": "floor = hand-off + 2 x L2 load + (CAS entry: atomic) + t1(numLdSt) - t1(10); t1 = one "
                             "TB's uncontended time per op; mutexes and semaphore writers pass through die queues "
                             "or hand on a ring slot (no atomic), semaphore readers enter by CAS; a semaphore "
                             "cell's floor weights the two by its writer and reader ops"}


def cell_floor(c, floors, nsm):
    """The per-op floor of one cell: a mutex's floor, or a semaphore's writer
    and reader floors weighted by the cell's ops (one writer TB of the
    numTBs_perSM TBs of each logical SM, main.cu:554-555)."""
    f = floors[(c["prim"], c["num_ldst"])]
    if not isinstance(f, dict):
        return f
    k = -(-c["num_tbs"] // min(c["num_tbs"], nsm))
    return (f["writer"] + (k - 1) * f["reader"]) / k


def latency_roofline(cells, floors, kernel_prims, traffic, nsm=None, kernel="k_mutex"):
    """bound "latency": the dominant kernel's cells against their floors.
    achieved = its ops / its time; peak = the same ops at the floor per op."""
    sel = [c for c in cells.values() if c["prim"] in kernel_prims and (c["prim"], c["num_ldst"]) in floors]
    fl = {id(c): cell_floor(c, floors, nsm) for c in sel}
    ops = sum(c["ops"] for c in sel)
    ms = sum(c["mean_ms"] for c in sel)
    floor_ms = sum(c["ops"] * fl[id(c)] * 1e-3 for c in sel)
    achieved = ops / (ms * 1e-3)
    peak = ops / (floor_ms * 1e-3)
    return {"bound": "latency", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "sync ops/s",
            "frac": achieved / peak, "peak_source": "measured (hs_probe_latency hand-off + uncontended op)",
            "traffic": traffic, "traffic_source": TRAFFIC_SOURCE,
            "cells": {cell_key(c["prim"], c["num_tbs"], c["num_ldst"]):
                      {"us_per_op": round(c["us_per_op"], 4), "floor_us": round(fl[id(c)], 4),
                       "frac": round(fl[id(c)] / c["us_per_op"], 3)} for c in sel},
            "formula": "frac = sum(ops * floor_us) / sum(ops * us_per_op) over the dominant kernel's cells"}


# algorithmic L2 atomics per sync op (contention-free minimum of this build's
# implementation of each primitive): lock + unlock
ATOMICS_PER_OP = {"spinMutex": 2, "spinMutexEBO": 2, "sleepMutex": 3, "faMutex": 2,
                  "spinSem1": 2, "spinSem2": 2, "spinSem10": 2, "spinSem120": 2,
                  "spinSemEBO1": 2, "spinSemEBO2": 2, "spinSemEBO10": 2, "spinSemEBO120": 2,
                  "atomicTreeBarrUniq": 1, "atomicTreeBarrUniqLocalExch": 2, "lfTreeBarrUniq": 1,
                  "lfTreeBarrUniqLocalExch": 2}


def cs_bytes(name, G, L, nsm, iters=ITERS):
    """Algorithmic bytes one launch moves: 4-byte load + 4-byte store per element
    touched by a critical section (T*numLdSt elements per mutex op; the writer's
    numTBs_perSM chunks per semaphore writer op, T*numLdSt loads per reader op;
    per barrier episode every TB's chunk once, twice with local exchange)."""
    T = THREADS
    k = -(-G // nsm)
    if "Barr" in name:
        per = 2 if ("LocalExch" in name and k > 1) else 1
        return G * iters * T * L * 8 * per
    if "Sem" in name:
        numSM = min(G, nsm)
        writers = sum(1 for tb in range(G) if tb // numSM == (tb % numSM) % k)
        readers = G - writers
        return iters * (writers * k * T * L * 8 + readers * T * L * 4)
    return G * iters * T * L * 8


def secondary_bounds(hs, cells, nsm, dev_s):
    """The HBM, L2-bandwidth and L2-atomic fractions of the same cells (tiny for
    the serialised locks, which use neither bandwidth nor atomic rate), and the
    L2-bandwidth fraction of each tree-barrier cell at numLdSt 100, whose
    episodes move every TB's chunk through L2."""
    peak_gbs, peak_kind = load_peaks()
    byts = sum(cs_bytes(c["prim"], c["num_tbs"], c["num_ldst"], nsm) for c in cells.values())
    atom_peak, same_rate = l2_atomic_peak(hs)
    l2_gbs = l2_bandwidth_peak(hs)
    atom = sum(c["ops"] * ATOMICS_PER_OP[c["prim"]] for c in cells.values()) / dev_s
    barr = {}
    for k, c in cells.items():
        if "Barr" in c["prim"] and c["num_ldst"] == LDST[-1]:
            gbs = cs_bytes(c["prim"], c["num_tbs"], c["num_ldst"], nsm) / (c["mean_ms"] * 1e-3) / 1e9
            barr[k] = {"gbs": round(gbs, 1), "frac": round(gbs / l2_gbs, 3) if l2_gbs else None}
    return {"hbm": {"achieved": byts / dev_s / 1e9, "peak": peak_gbs, "unit": "GB/s",
                    "frac": byts / dev_s / 1e9 / peak_gbs, "peak_source": peak_kind,
                    "note": "critical-section bytes (L2-resident)"},
            "l2_bandwidth": {"achieved": byts / dev_s / 1e9, "peak": l2_gbs, "unit": "GB/s",
                             "frac": (byts / dev_s / 1e9 / l2_gbs) if l2_gbs else None,
                             "peak_source": "measured (hs_probe_l2_bandwidth: L2-resident copy, %d MiB, L1 bypassed)"
                                            % (L2_PROBE_BYTES >> 20),
                             "barrier_cells_numldst_%d" % LDST[-1]: barr},
            "l2_atomic": {"achieved": atom, "peak": atom_peak, "frac": (atom / atom_peak) if atom_peak else None,
                          "unit": "atomics/s", "same_address_rate": same_rate,
                          "note": "peak: contention-free red.add probe; same_address_rate: one word"}}


def fa_mutex_slice_extra(hs, nsm):
    """faMutex (ticket lock), one launch: numTBs 8 x 256 threads, numLdSt 10,
    numCSIters 100 on uint32[80] seeded in [0, 1000); every critical section
    adds 1 to a 10-word slice.  Device rate (median of 20 launches), e2e rate
    through hs_run with host storage, and the host std::thread run of the same
    algorithm (bit-exact with the GPU's result)."""
    import oracle
    cfg = hs.RunConfig(prim="faMutex", num_ldst=10, num_tbs=8, num_iters=100, threads=256, repeats=1, mode="slice")
    rng = np.random.default_rng(SEED)
    init = (rng.integers(0, 2 ** 63, size=hs.storage_words(cfg), dtype=np.uint64) % 1000).astype(np.uint32)
    want = hs.expected_storage(cfg, init)
    dev, wall = [], []
    for _ in range(20):
        st = init.copy()
        t0 = time.perf_counter()
        r = hs.run(cfg, st)
        wall.append(time.perf_counter() - t0)
        dev.append(r.elapsed_ms * 1e-3)
        if not np.array_equal(st, want):
            raise SystemExit("bench: faMutex slice result differs from the expected final state")
    ops = 8 * 100
    twin, secs = oracle.twin_run(7, 256, 10, 8, 100, 1, nsm, 2, init)
    return {"workload": "faMutex slice, numTBs 8 x 256, numLdSt 10, numCSIters 100, one launch",
            "ops_per_launch": ops, "sync_ops_per_s": ops / statistics.median(dev),
            "e2e_sync_ops_per_s": ops / statistics.median(wall), "us_per_op": statistics.median(dev) * 1e6 / ops,
            "cpu_baseline": {"sync_ops_per_s": ops / secs if secs > 0 else None, "kind": "port",
                             "cores": os.cpu_count(), "bit_exact_with_gpu": bool(np.array_equal(twin, want))}}


def exchange_extra(hs):
    """Tree barrier with local exchange on clusters: 592 resident CTAs x 256
    threads, a 4096-word fp32 buffer per CTA rotated to the next CTA every
    episode, 1000 episodes; cluster sizes 1 (flat), 2, 4, 8, both global stages;
    final buffers checked bit-exact against the rotation."""
    import oracle
    x = hs.exchange_fill(SEED, 592, 4096)
    rows = {}
    for lf in (False, True):
        for cl in (1, 2, 4, 8):
            out, r = hs.exchange_run(x, cl, lf, 1000)
            if not np.array_equal(out, oracle.exchange_expected(x, 1000)):
                raise SystemExit("bench: exchange cluster=%d lf=%s is not the expected rotation" % (cl, lf))
            rows["%s_cluster%d" % ("lf" if lf else "atomic", cl)] = {
                "episodes_per_s": round(r.episodes_per_s), "exchange_gbs": round(r.exchange_gbs, 1),
                "ms": round(r.elapsed_ms, 3)}
    l2_gbs = l2_bandwidth_peak(hs)
    best = max(rows.values(), key=lambda r: r["exchange_gbs"])
    return {"workload": "592 CTAs x 256 threads, fp32[4096] per CTA rotated to CTA b+1 each episode, "
                        "1000 episodes, one tree barrier per episode (bit-exact rotation checked)",
            "exchange_bytes_per_episode": 592 * 4096 * 4 * 2, "results": rows,
            "l2_bandwidth": {"peak_gbs": l2_gbs, "best_exchange_gbs": best["exchange_gbs"],
                             "frac": round(best["exchange_gbs"] / l2_gbs, 3) if l2_gbs else None,
                             "note": "most of the exchange moves SM to SM through distributed shared memory, so "
                                     "the L2 copy rate is a reference point, not its bound"}}


def relaxed_extra(hs, nsm):
    """The relaxed-atomics programs at GB300 sizes (4 x NUM_SM TBs of 256
    threads), each checked against its known answer: refCounter (every counter
    back to 0, refCounter.cu:86-98), splitCounter (every counter 1,
    splitCounter.cu:54-60) and seqlocks (each lock's final sequence number,
    seqlocks_kernel.cu:193-203).  Best of 3 kernel times; ops as the programs
    count them; refCounter against the L2 atomic rate (1 atomic per op: 2 adds
    and 2 decrements per thread and repeat); splitCounter's readers (numTBs
    relaxed 4-byte loads per reader thread, the reference's atomicAdd(0) reads
    of splitCounter_kernel.cu:50-61, which it says may be relaxed) against the
    L2-resident copy rate, its writers (1 red.add each) beside."""
    atom_peak, same_rate = l2_atomic_peak(hs)
    G, T = 4 * nsm, 256
    out = {"workload": "%d TBs x %d threads per program" % (G, T), "l2_atomic_peak": atom_peak,
           "l2_same_address_rate": same_rate, "programs": {}}

    def best(fn):
        rs = [fn() for _ in range(3)]
        return min(rs, key=lambda x: x[-1].elapsed_ms)

    c0, c1, d0, d1, r = best(lambda: hs.refcounter(32, G, T, 64))
    if c0.any() or c1.any():
        raise SystemExit("bench: refCounter counters not back to 0")
    s = r.elapsed_ms * 1e-3
    out["programs"]["refCounter"] = {"args": "32 sharers, %d TBs, %d threads, 64 repeats" % (G, T),
                                     "ms": r.elapsed_ms, "ops_per_s": r.ops / s, "atomics_per_s": r.ops / s,
                                     "l2_atomic_frac": (r.ops / s) / atom_peak if atom_peak else None}
    c, o, r = best(lambda: hs.splitcounter(G, T))
    if not np.array_equal(c, np.ones_like(c)):
        raise SystemExit("bench: splitCounter counters differ from 1")
    s = r.elapsed_ms * 1e-3
    thr = G * T
    read_bytes = (thr // 2) * G * 4
    l2_gbs = l2_bandwidth_peak(hs)
    out["programs"]["splitCounter"] = {"args": "%d TBs, %d threads" % (G, T), "ms": r.elapsed_ms,
                                       "ops_per_s": r.ops / s, "writer_atomics_per_s": (thr // 2) / s,
                                       "reader_gbs": read_bytes / s * 1e-9,
                                       "l2_copy_gbs": l2_gbs,
                                       "l2_frac": (read_bytes / s * 1e-9) / l2_gbs if l2_gbs else None}
    seq, dd0, dd1, so, r = best(lambda: hs.seqlocks(G, T, 4))
    for k in range(G // 4):
        if seq[k] != 2 * 10 * sum(1 for b in range(G) if b % 16 == 0 and b % 4 == k):
            raise SystemExit("bench: seqlocks sequence number %d differs from its known value" % k)
    s = r.elapsed_ms * 1e-3
    out["programs"]["seqlocks"] = {"args": "%d TBs, %d threads, group 4" % (G, T), "ms": r.elapsed_ms,
                                   "ops_per_s": r.ops / s, "note": "ops: 10 reader or writer rounds per TB"}
    return out


def batch_extra(hs):
    """The 64-instance mixed batch (numTBs log-uniform [4,512], numLdSt [1,128],
    numCSIters [10,5000]): one launch per instance against one persistent
    graph-replayed launch, plan chosen by the autotuner on the same batch with
    numCSIters / 25; every instance checked bit-exact after both."""
    insts = hs.batch_generate(seed=SEED, n=64, iter_div=1)
    small = hs.batch_generate(seed=SEED, n=64, iter_div=25)
    tb = hs.Batch(small, mode="inc")
    t0 = time.perf_counter()
    _, tune_ms = tb.autotune()
    first = dict(tb.last_tune, wall_s=time.perf_counter() - t0)
    tuned = tb.tuned_settings()
    tb.close()
    tb = hs.Batch(small, mode="inc")   # the same batch again: its plan comes from the cache
    t0 = time.perf_counter()
    tb.autotune()
    second = dict(tb.last_tune, wall_s=time.perf_counter() - t0)
    if tb.tuned_settings() != tuned:
        raise SystemExit("bench: the cached batch plan differs from the tuned one")
    tb.close()
    b = hs.Batch(insts, mode="inc")
    rng = np.random.default_rng(SEED)
    inits = [rng.integers(0, 1000, size=b.words(i)).astype(np.uint32) for i in range(len(insts))]

    def check(tag):
        for i, x in enumerate(insts):
            if not np.array_equal(b.get_storage(i), hs.batch_expected(x, inits[i])):
                raise SystemExit("bench: batch instance %d differs after the %s run" % (i, tag))

    for i, a in enumerate(inits):
        b.set_storage(i, a)
    rs = b.run_serial()
    check("per-launch")
    s, grid, cap = b.apply_settings(tuned)
    if s:
        raise SystemExit("bench: the tuned batch plan does not fit (status %d)" % s)
    for i, a in enumerate(inits):
        b.set_storage(i, a)
    rb = b.run()
    check("batched")
    b.close()
    return {"workload": "64 mixed instances (28 SyncPrims + RefCounter/SplitCounter/Seqlock/Flags, seed %d), "
                        "numCSIters [10,5000]" % SEED,
            "ops": rb.ops, "per_launch_ms": round(rs.elapsed_ms, 2), "per_launch_ops_per_s": rs.ops / (rs.elapsed_ms * 1e-3),
            "launches_per_instance_form": rs.launches, "batched_ms": round(rb.elapsed_ms, 2),
            "batched_ops_per_s": rb.ops / (rb.elapsed_ms * 1e-3), "ratio": rs.elapsed_ms / rb.elapsed_ms,
            "plan": {"cluster": tuned[0], "serial_executors": tuned[1], "tbs_per_executor": tuned[2],
                     "stage_bytes": tuned[3], "ctas_per_sm": {40 * 1024: 4, 56 * 1024: 3}.get(tuned[3]),
                     "backoff_min_ns": tuned[5], "backoff_max_ns": tuned[4], "cta_threads": 256,
                     "grid": grid, "capacity": cap,
                     "tuned_on": "numCSIters / 25 (best trial %.1f ms)" % tune_ms,
                     "cache": {"first": first, "second": second}}}


def uts_geo_extra(hs):
    """Geometric SHA-1 UTS (branching 4, depth limit 12) counted by work
    stealing on the GPU; node count checked against the host walk of the same
    tree at depth 9 (bounded CPU sample, also the host rate)."""
    import oracle
    rows = {}
    for seed in (2, 3):
        n, lv, md, ms = hs.uts_geo_run(seed, 12, 4.0, blocks=304, threads=256)
        rows["seed%d" % seed] = {"nodes": n, "leaves": lv, "deepest": md, "ms": round(ms, 3),
                                 "nodes_per_s": n / (ms * 1e-3)}
    want = oracle.geo_count(2, 9)
    got = hs.uts_geo_run(2, 9, 4.0, blocks=304, threads=256)[:3]
    if got != want:
        raise SystemExit("bench: geometric UTS depth 9 count differs from the host walk")
    t0 = time.perf_counter()
    oracle.geo_count(2, 9)
    host_s = time.perf_counter() - t0
    coop = {}
    for seed in (2, 3):  # the same trees walked by the GPU CTAs and the host cores together
        try:
            r = hs.uts_geo_coop_run(seed, 12, 4.0, blocks=304, threads=256, host_threads=-1)
        except hs.HsError as e:
            coop = {"unavailable": str(e)}
            break
        if (r["nodes"], r["leaves"], r["max_depth"]) != (rows["seed%d" % seed]["nodes"], rows["seed%d" % seed]["leaves"],
                                                         rows["seed%d" % seed]["deepest"]):
            raise SystemExit("bench: cooperative UTS counts differ from the GPU walk")
        coop["seed%d" % seed] = {"ms": round(r["elapsed_ms"], 3), "nodes_per_s": r["nodes"] / (r["elapsed_ms"] * 1e-3),
                                 "host_share": r["host_nodes"] / r["nodes"], "host_threads": r["host_threads"],
                                 "to_host": r["to_host"], "to_gpu": r["to_gpu"]}
    return {"workload": "geometric tree, SHA-1 node generator, branching 4, depth limit 12, 304 CTAs x 256",
            "results": rows, "cooperative": coop,
            "check": "depth 9, seed 2: %d nodes, equal to the host walk" % want[0],
            "cpu_baseline": {"nodes_per_s": want[0] / host_s, "cores": 1, "kind": "port",
                             "sample": "host depth-first walk of seed 2 at depth 9 (%d nodes)" % want[0]}}


def serve_extra(hs):
    """Served request loop: 256 requests from the mixed-instance generator
    (numCSIters / 50, every eighth a tree search), 64 slots of 8-CTA clusters;
    each request's latency alone, the burst rate, the sustainable peak (the
    highest Poisson rate the open-loop driver keeps up with), then Poisson
    arrivals at 10-90% of that peak: arrived and completed rates, p50/p99
    latency from each request's due time, and slowdown (latency over latency
    alone) overall and per request class; the offline batch of the same
    requests; every result bit-exact."""
    from heterosync_gb300.served import served_sweep
    r = served_sweep(seed=SEED, n=256, iter_div=50, slots=64, gang=8)
    if not r["bit_exact"]:
        raise SystemExit("bench: a served request's result differs from the expected final storage")
    return r


def combine_ranks(dist, dev_s, e2e_s, ops, device):
    """Whole-job figures of a replicas run: the slowest rank's device and wall
    times (max over ranks) and every rank's operations (sum)."""
    import torch
    t = torch.tensor([dev_s, e2e_s, float(ops)], device=device, dtype=torch.float64)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return mx[0].item(), mx[1].item(), int(sm[2].item())


def gpu_identity():
    try:
        import torch
        pr = torch.cuda.get_device_properties(torch.cuda.current_device())
        return "%s/%s" % (pr.name, getattr(pr, "uuid", ""))
    except Exception:  # noqa: BLE001
        return ""


def reference_arm(args, rank, flush):
    """The reference's own SyncPrims kernels (sm_100 build of its unmodified
    sources) on the headline cells, each run at numCSIters = 1000 and timed with
    CUDA events around its launch (the reference's ROI, main.cu:1494-1619)."""
    if rank != 0:
        return None
    import oracle
    import heterosync_gb300 as hs
    out = {"impl": "reference", "metric": "sync ops/s", "unit": "sync ops/s", "higher_is_better": True,
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
           "dtype": "u32", "scaling": "weak", "vs_baseline": None}
    if oracle.ref_available(THREADS):
        nsm, _ = oracle.ref_device()
        pts = sweep_points(nsm)
        recs = []
        t_start = time.perf_counter()
        for step in range(args.warmup + args.steps):
            G, L = pts[step % len(pts)]
            timed = step >= args.warmup
            it = ITERS if timed else WARM_ITERS
            for name in HEAD_PRIMS:
                p = hs.prim_id(name)
                n = oracle.storage_words(p, THREADS, L, G, nsm)
                init = make_init(n, SEED + G + L)
                flush()
                got, ms = oracle.ref_run(p, THREADS, L, G, it, 1, init)
                print("reference %s numTBs=%d numLdSt=%d iters=%d: %.3f ms" % (name, G, L, it, ms), file=sys.stderr,
                      flush=True)
                if timed:
                    cfg = hs.RunConfig(prim=name, num_ldst=L, num_tbs=G, num_iters=it, threads=THREADS, repeats=1,
                                       mode="ref")
                    if not args.no_check and not np.array_equal(got, hs.expected_storage(cfg, init)):
                        raise SystemExit("bench: the reference's %s numTBs=%d numLdSt=%d final state differs from "
                                         "the closed form" % (name, G, L))
                    recs.append({"prim": name, "num_tbs": G, "num_ldst": L, "ops": G * it, "ms": ms})
        cells, value, _ = aggregate(recs)
        per_cell = {k: round(c["us_per_op"], 4) for k, c in cells.items()}
        try:
            with open(REF_CELLS_FILE, "w") as f:
                json.dump({"gpu": gpu_identity(), "time": time.time(), "us_per_op": per_cell}, f)
        except OSError:
            pass
        out.update({"value": value, "ms_per_step": sum(r["ms"] for r in recs) / args.steps,
                    "config": head_config(nsm),
                    "reference_build": "reference SyncPrims kernels, sm_100 build of the unmodified sources "
                                       "(oracle/_ref), run through the driver API with the reference's launch shape",
                    "excluded": {"semaphores (spinSem*, spinSemEBO*)": REF_EXCLUDED},
                    "per_cell_us_per_op": per_cell,
                    "wall_s": time.perf_counter() - t_start,
                    "cpu_baseline": {"value": value, "unit": "sync ops/s", "cores": None, "kind": "reference",
                                     "sample": "the reference's CUDA kernels on this GPU (the reference has no CPU "
                                               "implementation of its primitives): every headline cell at "
                                               "numCSIters %d, no projection" % ITERS},
                    "e2e": {"value": value, "unit": "sync ops/s", "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}})
    else:
        nsm = hs.device_info()["nsm"]
        cb = cpu_baseline(nsm)
        out.update({"value": cb["value"], "ms_per_step": None, "config": head_config(nsm),
                    "reference_build": "absent: host std::thread port of the same algorithms",
                    "cpu_baseline": cb,
                    "e2e": {"value": cb["value"], "unit": "sync ops/s", "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}})
    return out


def reference_cells():
    """The per-cell us/op the reference arm measured on this GPU within the last
    hour (None when it did not run here)."""
    try:
        with open(REF_CELLS_FILE) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    if d.get("gpu") != gpu_identity() or time.time() - d.get("time", 0) > 3600:
        return None
    return d["us_per_op"]


def kernel_of(prim):
    if "Barr" in prim:
        return "k_barrier"
    return "k_sem" if "Sem" in prim else "k_mutex"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-check", action="store_true", help="skip the bit-exact check of every run")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-full-sweep", action="store_true", help="skip the 16-primitive sweep beside the headline")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the cluster exchange, batch, serving and UTS figures reported beside the sweep")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 256 MiB > L2

    def flush():
        flush_buf.zero_()
        torch.cuda.synchronize()

    if args.impl == "reference":
        out = reference_arm(args, rank, flush)
        if rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    import heterosync_gb300 as hs
    nsm = hs.device_info(local)["nsm"] if local == 0 else hs.device_info()["nsm"]
    pts = sweep_points(nsm)

    for s in range(args.warmup):
        run_cells(hs, HEAD_PRIMS, pts[s % len(pts)], WARM_ITERS, check=False, flush=flush)

    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    launches0 = hs.launch_count()
    t0 = time.perf_counter()
    recs = []
    for s in range(args.steps):
        recs += run_cells(hs, HEAD_PRIMS, pts[s % len(pts)], ITERS, check=not args.no_check, flush=flush)
    torch.cuda.synchronize()
    wall_total = time.perf_counter() - t0
    launches = hs.launch_count() - launches0
    ck = clocks.stop()

    cells, value, e2e_value = aggregate(recs)
    ops = sum(r["ops"] for r in recs)
    dev_s = sum(r["ms"] for r in recs) * 1e-3
    e2e_s = sum(r["wall_s"] for r in recs)
    if dist is not None:
        # replicas: each rank's sweep rate over the slowest rank's times, all ranks' ops
        cell_dev_s = sum(c["mean_ms"] for c in cells.values()) * 1e-3
        cell_e2e_s = sum(c["mean_wall_s"] for c in cells.values())
        cell_ops = sum(c["ops"] for c in cells.values())
        mx_dev, mx_e2e, all_ops = combine_ranks(dist, cell_dev_s, cell_e2e_s, cell_ops, "cuda")
        value, e2e_value = all_ops / mx_dev, all_ops / mx_e2e
        dev_s, e2e_s, _ = combine_ranks(dist, dev_s, e2e_s, ops, "cuda")

    if rank == 0:
        by_kernel = {}
        for c in cells.values():
            by_kernel[kernel_of(c["prim"])] = by_kernel.get(kernel_of(c["prim"]), 0.0) + c["mean_ms"]
        mutexes = [p for p in HEAD_PRIMS if p in LOCK_CHAIN]
        floors, lat = lock_floors(hs, SWEEP_PRIMS)
        roofline = latency_roofline(cells, floors, mutexes, DRAM_BYTES_PER_LAUNCH, nsm=nsm)
        roofline["share_of_device_time"] = by_kernel.get("k_mutex", 0.0) / sum(by_kernel.values())
        out = {
            "metric": "sync ops/s", "value": value, "unit": "sync ops/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded uint32 shared data, bit-exact final state checked every run)",
            "config": head_config(nsm),
            "e2e": {"value": e2e_value, "unit": "sync ops/s",
                    "h2d_bytes_per_step": int(sum(r["bytes"] for r in recs) / args.steps),
                    "d2h_bytes_per_step": int(sum(r["bytes"] for r in recs) / args.steps)},
            "gpu_launches": launches,
            "roofline": roofline,
            "secondary_bounds": secondary_bounds(hs, cells, nsm, sum(c["mean_ms"] for c in cells.values()) * 1e-3),
            "lock_latency": lat,
            "kernel_share": {k: round(v / sum(by_kernel.values()), 4) for k, v in by_kernel.items()},
            "per_prim": {p: {"ops_per_s": sum(c["ops"] for c in cells.values() if c["prim"] == p) /
                             (sum(c["mean_ms"] for c in cells.values() if c["prim"] == p) * 1e-3)}
                         for p in HEAD_PRIMS if any(c["prim"] == p for c in cells.values())},
            "per_cell_us_per_op": {k: round(c["us_per_op"], 4) for k, c in cells.items()},
            "parallelism": "replicas" if world > 1 else "single GPU",
            "wall_s": wall_total,
        }
        ref = reference_cells()
        if ref:
            cmp = {k: round(ref[k] / c["us_per_op"], 3) for k, c in cells.items() if k in ref}
            out["per_cell_vs_reference"] = {"speedup": cmp, "min": min(cmp.values()) if cmp else None,
                                            "source": "the reference arm's per-cell us/op on this GPU, run just "
                                                      "before (reference us/op / this build's us/op)"}
        if ck:
            out["clocks"] = ck
        if not args.no_full_sweep and world == 1:
            srecs = []
            for pt in pts:
                srecs += run_cells(hs, SEM_PRIMS, pt, ITERS, check=not args.no_check, flush=flush)
            scells, _, _ = aggregate(srecs)
            allc = dict(cells)
            allc.update(scells)
            fops = sum(c["ops"] for c in allc.values())
            fms = sum(c["mean_ms"] for c in allc.values())
            fwall = sum(c["mean_wall_s"] for c in allc.values())
            sk = {}
            for c in allc.values():
                sk[kernel_of(c["prim"])] = sk.get(kernel_of(c["prim"]), 0.0) + c["mean_ms"]
            sem_roof = latency_roofline(scells, floors, SEM_PRIMS, None, nsm=nsm, kernel="k_sem")
            sem_roof["traffic_source"] = None
            out["full_sweep"] = {
                "workload": "16 SyncPrims (the headline 8 plus spinSem{1,2,10,120}, spinSemEBO{1,2,10,120}) x the "
                            "same 6 points, numCSIters 1000; semaphore cells run once each after the timed steps",
                "value": fops / (fms * 1e-3), "e2e": fops / fwall, "unit": "sync ops/s",
                "kernel_share": {k: round(v / fms, 4) for k, v in sk.items()},
                "roofline": sem_roof,
                "per_cell_us_per_op": {k: round(c["us_per_op"], 4) for k, c in scells.items()},
                "note": "the reference's semaphore kernels cannot run on GB300: " + REF_EXCLUDED}
        if not args.no_extras and world == 1:
            for key, fn in (("fa_mutex_slice", lambda h: fa_mutex_slice_extra(h, nsm)), ("exchange", exchange_extra),
                            ("relaxed", lambda h: relaxed_extra(h, nsm)), ("batch", batch_extra),
                            ("serve", serve_extra), ("uts_geo", uts_geo_extra)):
                try:
                    out[key] = fn(hs)
                except SystemExit:
                    raise
                except Exception as e:  # noqa: BLE001
                    out[key] = {"error": str(e)}
        if not args.no_cpu_baseline and world == 1:
            try:
                out["cpu_baseline"] = cpu_baseline(nsm)
            except Exception as e:  # noqa: BLE001
                out["cpu_baseline"] = {"value": None, "error": str(e)}
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
