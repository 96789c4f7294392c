"""Served-load measurement: the persistent server kernel under open-loop
Poisson arrivals.

The request mix is the mixed-instance generator's (primitive uniform over the
28 SyncPrims and the four relaxed-atomics kinds, numTBs log-uniform in [4, 512], numLdSt in [1, 128],
numCSIters in [10, 5000] divided by `iter_div`).  The peak request rate is the
highest Poisson rate the open-loop driver sustains (see served_sweep); each
offered load is a Poisson arrival process at a fraction of it over the same
requests, and slowdown compares each request's latency with its latency alone.
Every eighth request is a geometric SHA-1 tree search instead.  Latency runs
from a request's due time to the host seeing its completion, so time queued on
the host counts.  Every instance's output is checked bit-exact against the
closed form of the reference golden, every tree search's counts against the
standalone kernel's.
"""
from __future__ import annotations

import numpy as np

from . import (Batch, Server, batch_expected, batch_generate, batch_instance_words, device_info, serve_uts_counts,
               uts_geo_run)


def make_requests(seed: int, n: int, iter_div: int, tree_every: int = 8, tree_depth: int = 9):
    """n requests: the mixed-instance generator's, with every tree_every-th
    replaced by a geometric SHA-1 tree search (branching 4, the given depth
    limit, seed from the request stream)."""
    insts = batch_generate(seed=seed, n=n, iter_div=iter_div)
    nsm = device_info()["nsm"]
    rng = np.random.default_rng(seed)
    out, inits = [], []
    for k, x in enumerate(insts):
        if tree_every and k % tree_every == tree_every - 1:
            out.append(("uts", int(rng.integers(0, 2 ** 31)), tree_depth, 4.0))
            inits.append(None)
        else:
            out.append(x)
            inits.append(rng.integers(0, 1000, size=batch_instance_words(x, nsm)).astype(np.uint32))
    return out, inits


def _tree_counts(insts):
    """Each tree search's counts from the standalone kernel: a served result
    must equal it (alone == in the mix)."""
    return {k: uts_geo_run(x[1], x[2], x[3])[:3] for k, x in enumerate(insts) if x[0] == "uts"}


def _check(insts, inits, outs, comps, trees):
    for k, x in enumerate(insts):
        if comps[k]["status"] != 0:
            return False
        if x[0] == "uts":
            if serve_uts_counts(outs[k]) != trees[k]:
                return False
        elif not np.array_equal(outs[k], batch_expected(x, inits[k])):
            return False
    return True


def request_class(x) -> str:
    """Request class for per-class figures: tree search, relaxed-atomics kind, or SyncPrims."""
    if x[0] == "uts":
        return "tree_search"
    return "relaxed" if x[0] >= 60 else "syncprims"


def window_rates(arrival_s, latency_us, lo_q: float = 0.1, hi_q: float = 0.9):
    """(arrived, completed) requests per second inside the arrival window of the
    middle requests (between the lo_q and hi_q quantiles of the arrival times).
    A server that keeps up completes requests there as fast as they arrive,
    whatever the warm-up and the drain at the ends of a finite run; comparing
    with the arrivals realised in the same window, not with the Poisson rate
    parameter, keeps the arrival process's own sampling noise out of the ratio."""
    arr = np.asarray(arrival_s, dtype=np.float64)
    done = arr + np.asarray(latency_us, dtype=np.float64) * 1e-6
    a, b = np.quantile(arr, lo_q), np.quantile(arr, hi_q)
    if b <= a:
        return float("inf"), float("inf")
    arrived = np.count_nonzero((arr >= a) & (arr <= b)) / (b - a)
    completed = np.count_nonzero((done >= a) & (done <= b)) / (b - a)
    return float(arrived), float(completed)


def poisson_arrivals(rate: float, n: int, seed: int):
    rng = np.random.default_rng(seed)
    arr = np.cumsum(rng.exponential(1.0 / rate, size=n))
    return arr - arr[0]


def served_sweep(seed: int = 20260101, n: int = 256, iter_div: int = 50, slots: int = 64, gang: int = 8,
                 loads=(0.1, 0.3, 0.5, 0.7, 0.9), offline: bool = True, keep_up: float = 0.95, search_steps: int = 4):
    """The served-load figures.

    * burst: every request published at once (the drain rate of a full queue);
    * peak: the highest offered Poisson rate whose window throughput stays within
      `keep_up` of the arrivals on two independent arrival sequences, searched
      with the same open-loop driver (from the burst rate down by halves, then
      bisection);
    * loads: Poisson arrivals at each fraction of that peak: offered and achieved
      rates, p50/p99 latency, and slowdown -- each request's latency over its
      latency when served alone -- at p50/p99 overall and p99 per request class.
    Every served result is checked bit-exact against the closed form (tree
    searches against the standalone kernel's counts)."""
    insts, inits = make_requests(seed, n, iter_div)
    trees = _tree_counts(insts)
    classes = np.array([request_class(x) for x in insts])
    ops = sum(x[2] * x[3] for x in insts if x[0] != "uts")
    res = {"requests": n, "tree_searches": len(trees), "tree_nodes": int(sum(t[0] for t in trees.values())),
           "iter_div": iter_div, "slots": slots, "gang": gang, "sync_ops": ops,
           "classes": {c: int(np.count_nonzero(classes == c)) for c in sorted(set(classes))}, "loads": {}}
    words = sum(a.size for a in inits if a is not None)
    srv = Server(slots=slots, gang=gang, arena_bytes=max(1 << 30, words * 8), staging_bytes=max(1 << 30, words * 8),
                 idle_timeout_s=30.0)
    exact = True
    try:
        # each request alone: the denominator of its slowdown
        alone = np.zeros(n)
        for k in range(n):
            outs, comps, _ = srv.drive([insts[k]], [inits[k]], np.zeros(1))
            exact &= _check([insts[k]], [inits[k]], outs, comps, {0: trees[k]} if k in trees else {})
            alone[k] = comps[0]["latency_us"]
        res["alone_us"] = {"p50": float(np.percentile(alone, 50)), "p99": float(np.percentile(alone, 99)),
                           "max": float(alone.max())}
        outs, comps, wall = srv.drive(insts, inits, np.zeros(n))
        exact &= _check(insts, inits, outs, comps, trees)
        burst = n / wall
        res["burst"] = {"requests_per_s": burst, "sync_ops_per_s": ops / wall, "wall_s": wall}

        def run(rate, tag):
            arr = poisson_arrivals(rate, n, seed + 1 + tag)
            o, c, w = srv.drive(insts, inits, arr)
            ok = _check(insts, inits, o, c, trees)
            lat = np.array([x["latency_us"] for x in c])
            return ok, arr, lat, w

        # sustainable peak: the highest rate whose window throughput keeps up
        tried = []
        hi, lo = burst, None
        rate = burst
        for tag in range(12):
            # a 256-request run is short beside its longest requests, so one
            # arrival sequence can keep up by luck: a rate must keep up on two
            keeps = True
            for rep in range(2):
                ok, arr, lat, _ = run(rate, 100 + 2 * tag + rep)
                exact &= ok
                arrived, completed = window_rates(arr, lat)
                tried.append({"offered": rate, "window_arrived": arrived, "window_completed": completed})
                keeps = completed >= keep_up * arrived
                if not keeps:
                    break
            if keeps:
                lo = rate
                if rate >= hi:
                    break
            else:
                hi = rate
            if lo is None:
                rate = rate / 2.0
            elif tag + 1 > search_steps or hi - lo < 0.02 * lo:
                break
            else:
                rate = 0.5 * (lo + hi)
        peak = lo if lo is not None else rate
        res["peak"] = {"requests_per_s": peak, "sync_ops_per_s": ops / (n / peak), "keep_up": keep_up,
                       "search": tried,
                       "definition": "highest offered Poisson rate at which the completions inside the middle 80%% "
                                     "of the arrival window keep up with the arrivals there within %.0f%%, on "
                                     "two arrival sequences"
                                     % ((1 - keep_up) * 100)}
        for i, f in enumerate(loads):
            ok, arr, lat, wall = run(f * peak, i)
            exact &= ok
            slow = lat / alone
            arrived, completed = window_rates(arr, lat)
            row = {"offered_requests_per_s": f * peak, "arrived_requests_per_s": arrived,
                   "achieved_requests_per_s": completed,
                   "p50_us": float(np.percentile(lat, 50)), "p99_us": float(np.percentile(lat, 99)),
                   "mean_us": float(lat.mean()),
                   "slowdown_p50": float(np.percentile(slow, 50)), "slowdown_p99": float(np.percentile(slow, 99)),
                   "per_class": {}}
            row["achieved_over_arrived"] = completed / arrived
            for c in sorted(set(classes)):
                m = classes == c
                row["per_class"][c] = {"p99_us": float(np.percentile(lat[m], 99)),
                                       "slowdown_p99": float(np.percentile(slow[m], 99))}
            res["loads"]["%d%%" % round(f * 100)] = row
        srv.stop()
    finally:
        srv.close()
    if offline:  # the same SyncPrims and relaxed requests as one batch (tree searches excluded)
        keep = [k for k, x in enumerate(insts) if x[0] != "uts"]
        b = Batch([insts[k] for k in keep], mode="inc")
        for i, k in enumerate(keep):
            b.set_storage(i, inits[k])
        b.autotune()
        for i, k in enumerate(keep):
            b.set_storage(i, inits[k])
        r = b.run()
        for i, k in enumerate(keep):
            exact &= bool(np.array_equal(b.get_storage(i), batch_expected(insts[k], inits[k])))
        res["offline_batch"] = {"requests": len(keep), "requests_per_s": len(keep) / (r.elapsed_ms * 1e-3),
                                "sync_ops_per_s": ops / (r.elapsed_ms * 1e-3), "ms": r.elapsed_ms,
                                "plan": list(b.tuned_settings())}
        b.close()
    res["bit_exact"] = bool(exact)
    return res
