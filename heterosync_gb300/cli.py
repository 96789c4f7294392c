"""Command line for the workloads beside the drop-in programs.

  python -m heterosync_gb300.cli exchange [--ctas 592] [--elems 4096]
         [--cluster 8] [--lf] [--episodes 1000] [--seed 20260101]
      tree barrier with local exchange on thread-block clusters; prints one
      JSON line (episodes/s, exchange GB/s, bit-exact check of the rotation)

  python -m heterosync_gb300.cli serve [--n 256] [--iter-div 50] [--slots 64]
         [--gang 8] [--loads 10,30,50,70,90]
      the served request loop: peak request rate, then Poisson arrivals at
      each offered load; p50/p99 latency, throughput, the offline batch of the
      same requests, bit-exact check of every result

  python -m heterosync_gb300.cli uts-geo [--seed 2] [--depth 12] [--host-threads N]
         [--branching 4] [--blocks 304] [--threads 256]
      geometric SHA-1 UTS by work stealing; node, leaf and depth counts

  python -m heterosync_gb300.cli sweep [--prims "..."] [--num-ldst 10]
         [--num-tbs ...] [--iters 10] [--runs 1] [--graph]
      the results-script sweep through the drop-in program; one JSON line per
      (primitive, numLdSt, numTBs) with the parsed `average` durations
      (--graph: each point in this process, its repeats one CUDA graph)

  python -m heterosync_gb300.cli batch [--seed 20260101] [--n 64]
         [--iter-div 1] [--tune-div 25] [--plan cl,se,v,stage,bo]
      the mixed-instance batch: one launch per instance, then the autotuned
      persistent graph-replayed launch; prints one JSON line (both times, the
      ratio, the plan, bit-exact check of every instance)
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np

from . import (Batch, batch_expected, batch_generate, exchange_fill, exchange_run)


def _rotation(x, episodes):
    return np.roll(x, episodes % x.shape[0], axis=0)


def cmd_exchange(a):
    x = exchange_fill(a.seed, a.ctas, a.elems)
    out, r = exchange_run(x, a.cluster, a.lf, a.episodes)
    exact = bool(np.array_equal(out, _rotation(x, a.episodes)))
    print(json.dumps({"workload": "exchange", "ctas": a.ctas, "elems": a.elems, "cluster": a.cluster,
                      "global_stage": "lock-free flags" if a.lf else "atomic counter", "episodes": a.episodes,
                      "ms": r.elapsed_ms, "episodes_per_s": r.episodes_per_s, "exchange_gbs": r.exchange_gbs,
                      "bit_exact": exact}), flush=True)
    return 0 if exact else 1


def cmd_batch(a):
    insts = batch_generate(seed=a.seed, n=a.n, iter_div=a.iter_div)
    if a.plan:
        tuned = tuple(int(v) for v in a.plan.split(","))
    else:
        tb = Batch(batch_generate(seed=a.seed, n=a.n, iter_div=a.tune_div), mode="inc")
        tb.autotune()
        tuned = tb.tuned_settings()
        tb.close()
    b = Batch(insts, mode="inc")
    rng = np.random.default_rng(a.seed)
    inits = [rng.integers(0, 1000, size=b.words(i)).astype(np.uint32) for i in range(len(insts))]

    def exact():
        return all(np.array_equal(b.get_storage(i), batch_expected(x, inits[i])) for i, x in enumerate(insts))

    for i, x in enumerate(inits):
        b.set_storage(i, x)
    rs = b.run_serial()
    ok_serial = exact()
    b.apply_settings(tuned)
    for i, x in enumerate(inits):
        b.set_storage(i, x)
    rb = b.run()
    ok_batch = exact()
    b.close()
    print(json.dumps({"workload": "batch", "instances": len(insts), "ops": rb.ops,
                      "per_launch_ms": rs.elapsed_ms, "batched_ms": rb.elapsed_ms,
                      "ratio": rs.elapsed_ms / rb.elapsed_ms,
                      "plan": dict(zip(["cluster", "serial_executors", "tbs_per_executor", "stage_bytes", "backoff_max_ns"],
                                       tuned)), "grid": rb.grid,
                      "bit_exact": ok_serial and ok_batch}), flush=True)
    return 0 if ok_serial and ok_batch else 1


def cmd_uts_geo(a):
    from . import uts_geo_coop_run, uts_geo_run
    if a.host_threads is not None:  # cooperative: GPU CTAs and host threads on one tree
        r = uts_geo_coop_run(a.seed, a.depth, a.branching, blocks=a.blocks, threads=a.threads,
                             host_threads=a.host_threads)
        ms = r["elapsed_ms"]
        print(json.dumps({"workload": "uts-geo-coop", "seed": a.seed, "depth_limit": a.depth,
                          "branching": a.branching, **r,
                          "nodes_per_s": r["nodes"] / (ms * 1e-3) if ms > 0 else None}), flush=True)
        return 0
    nodes, leaves, deepest, ms = uts_geo_run(a.seed, a.depth, a.branching, blocks=a.blocks, threads=a.threads)
    print(json.dumps({"workload": "uts-geo", "seed": a.seed, "depth_limit": a.depth, "branching": a.branching,
                      "nodes": nodes, "leaves": leaves, "deepest": deepest, "ms": ms,
                      "nodes_per_s": nodes / (ms * 1e-3) if ms > 0 else None}), flush=True)
    return 0


SWEEP_PRIMS = ("atomicTreeBarrUniq atomicTreeBarrUniqLocalExch lfTreeBarrUniq lfTreeBarrUniqLocalExch spinMutex "
               "spinMutexEBO faMutex sleepMutex spinSem10 spinSemEBO10 spinMutexUniq spinMutexEBOUniq faMutexUniq "
               "sleepMutexUniq spinSemUniq10 spinSemEBOUniq10")


def cmd_sweep(a):
    """The results-script sweep (syncPrims_results.sh:1-59): every primitive x
    numLdSt x numTBs through the drop-in program, its `average` field parsed as
    the script parses it (third ':' field, up to 'm'); one JSON line per point."""
    import os
    import subprocess
    from . import device_info
    exe = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bin", "allSyncPrims-1kernel")
    nsm = device_info()["nsm"]
    tbs = [int(x) for x in a.num_tbs.split(",")] if a.num_tbs else [m * nsm for m in (1, 2, 4, 8)]
    ok = True
    for prim in a.prims.split():
        for L in (int(x) for x in a.num_ldst.split(",")):
            for G in tbs:
                durations = []
                if a.graph:
                    point_ok, durations = _graph_point(prim, L, G, a.iters, a.runs)
                    ok = ok and point_ok
                    vals = [d for d in durations if d is not None]
                    print(json.dumps({"syncPrim": prim, "numLdSt": L, "numTBs": G, "numCSIters": a.iters,
                                      "durations_ms": durations, "graph": True, "bit_exact": point_ok,
                                      "average_ms": sum(vals) / len(vals) if vals else None}), flush=True)
                    continue
                for _ in range(a.runs):
                    p = subprocess.run([exe, prim, str(L), str(G), str(a.iters)], capture_output=True, text=True)
                    line = next((x for x in p.stdout.splitlines() if "average" in x), "")
                    try:
                        durations.append(float(line.split(":")[2].split("m")[0]))
                    except (IndexError, ValueError):
                        durations.append(None)
                    ok = ok and p.returncode == 0 and "PASSED" in p.stdout
                vals = [d for d in durations if d is not None]
                print(json.dumps({"syncPrim": prim, "numLdSt": L, "numTBs": G, "numCSIters": a.iters,
                                  "durations_ms": durations,
                                  "average_ms": sum(vals) / len(vals) if vals else None}), flush=True)
    return 0 if ok else 1


def _graph_point(prim, num_ldst, num_tbs, iters, runs):
    """One sweep point in this process: the program's run (32 threads, 10
    repeats, the reference critical section) with the repeats replayed as one
    CUDA graph; each run's final storage checked against the golden's closed
    form.  Returns (all runs exact, per-run average launch ms)."""
    import numpy as np
    from . import RUN_GRAPH, HsError, RunConfig, expected_storage, run, storage_words
    cfg = RunConfig(prim, num_ldst, num_tbs, iters, threads=32, repeats=10, mode="ref", flags=RUN_GRAPH)
    try:
        words = storage_words(cfg)
    except HsError:
        return False, [None] * runs
    init = np.random.default_rng(20260101).integers(0, 1000, size=words).astype(np.uint32)
    want = expected_storage(cfg, init)
    ok, durations = True, []
    for _ in range(runs):
        st = init.copy()
        try:
            r = run(cfg, st)
        except HsError:
            ok = False
            durations.append(None)
            continue
        ok = ok and bool(np.array_equal(st, want))
        durations.append(r.avg_ms)
    return ok, durations


def cmd_serve(a):
    from .served import served_sweep
    loads = tuple(float(x) / 100.0 for x in a.loads.split(","))
    r = served_sweep(seed=a.seed, n=a.n, iter_div=a.iter_div, slots=a.slots, gang=a.gang, loads=loads,
                     offline=not a.no_offline)
    print(json.dumps({"workload": "serve", **r}), flush=True)
    return 0 if r["bit_exact"] else 1


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m heterosync_gb300.cli")
    sub = ap.add_subparsers(dest="cmd", required=True)
    e = sub.add_parser("exchange")
    e.add_argument("--ctas", type=int, default=592)
    e.add_argument("--elems", type=int, default=4096)
    e.add_argument("--cluster", type=int, default=8)
    e.add_argument("--lf", action="store_true")
    e.add_argument("--episodes", type=int, default=1000)
    e.add_argument("--seed", type=int, default=20260101)
    bt = sub.add_parser("batch")
    bt.add_argument("--seed", type=int, default=20260101)
    bt.add_argument("--n", type=int, default=64)
    bt.add_argument("--iter-div", type=int, default=1)
    bt.add_argument("--tune-div", type=int, default=25)
    bt.add_argument("--plan", default="", help="cluster,serial_executors,v,stage_bytes,backoff_max_ns: skip tuning")
    ug = sub.add_parser("uts-geo")
    ug.add_argument("--seed", type=int, default=2)
    ug.add_argument("--depth", type=int, default=12)
    ug.add_argument("--branching", type=float, default=4.0)
    ug.add_argument("--blocks", type=int, default=304)
    ug.add_argument("--threads", type=int, default=256)
    ug.add_argument("--host-threads", type=int, default=None,
                    help="walk cooperatively with this many host threads (-1: cores minus one; with --blocks 0 the "
                         "host walks alone)")
    sw = sub.add_parser("sweep")
    sw.add_argument("--prims", default=SWEEP_PRIMS)
    sw.add_argument("--num-ldst", default="10")
    sw.add_argument("--num-tbs", default="", help="comma list; default 1, 2, 4, 8 TBs per SM")
    sw.add_argument("--iters", type=int, default=10)
    sw.add_argument("--runs", type=int, default=1)
    sw.add_argument("--graph", action="store_true",
                    help="run each point in this process with its repeats replayed as one CUDA graph")
    sv = sub.add_parser("serve")
    sv.add_argument("--seed", type=int, default=20260101)
    sv.add_argument("--n", type=int, default=256)
    sv.add_argument("--iter-div", type=int, default=50)
    sv.add_argument("--slots", type=int, default=64)
    sv.add_argument("--gang", type=int, default=8)
    sv.add_argument("--loads", default="10,30,50,70,90", help="offered loads, percent of the measured peak")
    sv.add_argument("--no-offline", action="store_true")
    a = ap.parse_args(argv)
    return {"exchange": cmd_exchange, "batch": cmd_batch, "serve": cmd_serve, "uts-geo": cmd_uts_geo,
            "sweep": cmd_sweep}[a.cmd](a)


if __name__ == "__main__":
    sys.exit(main())
