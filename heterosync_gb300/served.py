"""Served-load measurement: the persistent server kernel under open-loop
Poisson arrivals.

The request mix is the mixed-instance generator's (primitive uniform over the
28 SyncPrims and the four relaxed-atomics kinds, numTBs log-uniform in [4, 512], numLdSt in [1, 128],
numCSIters in [10, 5000] divided by `iter_div`).  The peak request rate is
measured first by publishing every request at once; each offered load is then
a Poisson arrival process at that fraction of the peak over the same requests.
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


def served_sweep(seed: int = 20260101, n: int = 256, iter_div: int = 50, slots: int = 64, gang: int = 8,
                 loads=(0.1, 0.3, 0.5, 0.7, 0.9), offline: bool = True):
    insts, inits = make_requests(seed, n, iter_div)
    trees = _tree_counts(insts)
    ops = sum(x[2] * x[3] for x in insts if x[0] != "uts")
    res = {"requests": n, "tree_searches": len(trees), "tree_nodes": int(sum(t[0] for t in trees.values())),
           "iter_div": iter_div, "slots": slots, "gang": gang, "sync_ops": ops, "loads": {}}
    words = sum(a.size for a in inits if a is not None)
    srv = Server(slots=slots, gang=gang, arena_bytes=max(1 << 30, words * 8), staging_bytes=max(1 << 30, words * 8),
                 idle_timeout_s=30.0)
    exact = True
    try:
        outs, comps, wall = srv.drive(insts, inits, np.zeros(n))
        exact &= _check(insts, inits, outs, comps, trees)
        peak = n / wall
        res["peak"] = {"requests_per_s": peak, "sync_ops_per_s": ops / wall, "wall_s": wall}
        rng = np.random.default_rng(seed + 1)
        for f in loads:
            arr = np.cumsum(rng.exponential(1.0 / (f * peak), size=n))
            arr -= arr[0]
            outs, comps, wall = srv.drive(insts, inits, arr)
            exact &= _check(insts, inits, outs, comps, trees)
            lat = np.array([c["latency_us"] for c in comps])
            svc = np.array([c["service_us"] for c in comps])
            res["loads"]["%d%%" % round(f * 100)] = {
                "offered_requests_per_s": f * peak, "achieved_requests_per_s": n / wall,
                "p50_us": float(np.percentile(lat, 50)), "p99_us": float(np.percentile(lat, 99)),
                "mean_us": float(lat.mean()), "service_p50_us": float(np.percentile(svc, 50))}
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
