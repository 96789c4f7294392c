"""Served-load measurement: the persistent server kernel under open-loop
Poisson arrivals.

The request mix is the mixed-instance generator's (primitive uniform over the
28 SyncPrims and the four relaxed-atomics kinds, numTBs log-uniform in [4, 512], numLdSt in [1, 128],
numCSIters in [10, 5000] divided by `iter_div`).  The peak request rate is
measured first by publishing every request at once; each offered load is then
a Poisson arrival process at that fraction of the peak over the same requests.
Latency runs from a request's due time to the host seeing its completion, so
time queued on the host counts.  Every output is checked bit-exact against the
closed form of the reference golden.
"""
from __future__ import annotations

import numpy as np

from . import Batch, Server, batch_expected, batch_generate, batch_instance_words, device_info


def make_requests(seed: int, n: int, iter_div: int):
    insts = batch_generate(seed=seed, n=n, iter_div=iter_div)
    nsm = device_info()["nsm"]
    rng = np.random.default_rng(seed)
    inits = [rng.integers(0, 1000, size=batch_instance_words(x, nsm)).astype(np.uint32) for x in insts]
    return insts, inits


def _check(insts, inits, outs, comps):
    for k, x in enumerate(insts):
        if comps[k]["status"] != 0:
            return False
        if not np.array_equal(outs[k], batch_expected(x, inits[k])):
            return False
    return True


def served_sweep(seed: int = 20260101, n: int = 256, iter_div: int = 50, slots: int = 64, gang: int = 8,
                 loads=(0.1, 0.3, 0.5, 0.7, 0.9), offline: bool = True):
    insts, inits = make_requests(seed, n, iter_div)
    ops = sum(G * I for (_, _, G, I) in insts)
    res = {"requests": n, "iter_div": iter_div, "slots": slots, "gang": gang, "sync_ops": ops, "loads": {}}
    words = sum(a.size for a in inits)
    srv = Server(slots=slots, gang=gang, arena_bytes=max(1 << 30, words * 8), staging_bytes=max(1 << 30, words * 8),
                 idle_timeout_s=30.0)
    exact = True
    try:
        outs, comps, wall = srv.drive(insts, inits, np.zeros(n))
        exact &= _check(insts, inits, outs, comps)
        peak = n / wall
        res["peak"] = {"requests_per_s": peak, "sync_ops_per_s": ops / wall, "wall_s": wall}
        rng = np.random.default_rng(seed + 1)
        for f in loads:
            arr = np.cumsum(rng.exponential(1.0 / (f * peak), size=n))
            arr -= arr[0]
            outs, comps, wall = srv.drive(insts, inits, arr)
            exact &= _check(insts, inits, outs, comps)
            lat = np.array([c["latency_us"] for c in comps])
            svc = np.array([c["service_us"] for c in comps])
            res["loads"]["%d%%" % round(f * 100)] = {
                "offered_requests_per_s": f * peak, "achieved_requests_per_s": n / wall,
                "p50_us": float(np.percentile(lat, 50)), "p99_us": float(np.percentile(lat, 99)),
                "mean_us": float(lat.mean()), "service_p50_us": float(np.percentile(svc, 50))}
        srv.stop()
    finally:
        srv.close()
    if offline:
        b = Batch(insts, mode="inc")
        for i, a in enumerate(inits):
            b.set_storage(i, a)
        b.autotune()
        for i, a in enumerate(inits):
            b.set_storage(i, a)
        r = b.run()
        for i, x in enumerate(insts):
            exact &= bool(np.array_equal(b.get_storage(i), batch_expected(x, inits[i])))
        res["offline_batch"] = {"requests_per_s": n / (r.elapsed_ms * 1e-3),
                                "sync_ops_per_s": ops / (r.elapsed_ms * 1e-3), "ms": r.elapsed_ms,
                                "plan": list(b.tuned_settings())}
        b.close()
    res["bit_exact"] = bool(exact)
    return res
