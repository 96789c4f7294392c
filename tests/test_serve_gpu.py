"""GPU: the served request loop.  SyncPrims requests admitted into the
persistent server kernel's slots as they arrive; every result is compared with
the closed form of the reference golden, alone (one request at a time) and in
a mix (many in flight, overlapping on the device), and the two must agree."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRIMS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]


def _expected(hs, inst, init):
    return hs.batch_expected(inst, init)


def _requests(hs, seed):
    insts = [(p, 3 + (p * 7) % 40, 2 + (p * 5) % 37, 2 + p % 5) for p in PRIMS]
    insts += hs.batch_generate(seed=seed, n=16, iter_div=400)
    rng = np.random.default_rng(seed)
    nsm = hs.device_info()["nsm"]
    inits = [rng.integers(0, 2 ** 32, size=hs.batch_instance_words(x, nsm), dtype=np.uint64).astype(np.uint32)
             for x in insts]
    return insts, inits


def _submit_all(srv, insts, inits):
    outs = {}
    for x, a in zip(insts, inits):
        while True:
            try:
                rid, out = srv.submit(x, a)
                outs[rid] = out
                break
            except Exception as e:  # ring or staging pool full: let completions drain
                if getattr(e, "status", None) != 3:
                    raise
                time.sleep(0.001)
    return outs


def test_alone_and_in_mix_agree(hs):
    insts, inits = _requests(hs, 101)
    srv = hs.Server(slots=8, gang=4, arena_bytes=256 << 20, staging_bytes=256 << 20, idle_timeout_s=20.0)
    try:
        alone = []
        for x, a in zip(insts, inits):
            rid, out = srv.submit(x, a)
            c = srv.wait(1)[0]
            assert c["id"] == rid and c["status"] == 0, (x, c)
            alone.append(out.copy())
        ids = list(_submit_all(srv, insts, inits).items())
        comps = {c["id"]: c for c in srv.wait(len(insts))}
        for k, (rid, out) in enumerate(ids):
            assert comps[rid]["status"] == 0, (insts[k], comps[rid])
            want = _expected(hs, insts[k], inits[k])
            assert np.array_equal(alone[k], want), ("alone", insts[k])
            assert np.array_equal(out, want), ("mix", insts[k])
        srv.stop()
    finally:
        srv.close()


def test_admission_waits_for_device_memory(hs):
    """An arena that holds only a few requests at a time: admission waits for
    pages, every request still completes exactly; one larger than the whole
    arena is rejected with HS_ENORES."""
    insts = [(4, 64, 96, 3), (10, 48, 200, 2), (1, 32, 152, 2), (22, 64, 64, 3)] * 4
    rng = np.random.default_rng(7)
    nsm = hs.device_info()["nsm"]
    inits = [rng.integers(0, 1000, size=hs.Server.request_words(*x, nsm=nsm)).astype(np.uint32) for x in insts]
    biggest = max(a.size for a in inits) * 4
    srv = hs.Server(slots=8, gang=2, arena_bytes=3 * biggest + (1 << 20), staging_bytes=256 << 20,
                    idle_timeout_s=20.0)
    try:
        ids = list(_submit_all(srv, insts, inits).items())
        big = (1, 128, 512, 1)  # a barrier instance: 512 chunks, about 67 MB
        big_init = np.zeros(hs.Server.request_words(*big, nsm=nsm), np.uint32)
        big_id, _ = srv.submit(big, big_init)
        comps = {c["id"]: c for c in srv.wait(len(insts) + 1)}
        assert comps[big_id]["status"] == 3
        for k, (rid, out) in enumerate(ids):
            assert comps[rid]["status"] == 0
            assert np.array_equal(out, _expected(hs, insts[k], inits[k])), insts[k]
        srv.stop()
    finally:
        srv.close()


def test_open_loop_drive(hs):
    insts, inits = _requests(hs, 202)
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(0.0005, size=len(insts)))
    srv = hs.Server(slots=16, gang=4, arena_bytes=512 << 20, staging_bytes=256 << 20, idle_timeout_s=20.0)
    try:
        outs, comps, wall = srv.drive(insts, inits, arrivals)
        srv.stop()
    finally:
        srv.close()
    assert wall > 0
    for k, x in enumerate(insts):
        assert comps[k]["status"] == 0 and comps[k]["latency_us"] > 0
        assert np.array_equal(outs[k], _expected(hs, x, inits[k])), x


def test_stop_drains_then_idle_exit(hs):
    insts, inits = _requests(hs, 303)
    srv = hs.Server(slots=4, gang=4, arena_bytes=256 << 20, staging_bytes=128 << 20, idle_timeout_s=20.0)
    try:
        ids = list(_submit_all(srv, insts[:12], inits[:12]).items())
        srv.stop()  # returns once every published request was admitted and the kernel exited
        comps = {c["id"]: c for c in srv.wait(len(ids), timeout_s=5.0)}
        for k, (rid, out) in enumerate(ids):
            assert comps[rid]["status"] == 0
            assert np.array_equal(out, _expected(hs, insts[k], inits[k]))
    finally:
        srv.close()
    # a server with no requests ends by itself after its idle limit
    srv = hs.Server(slots=2, gang=2, arena_bytes=16 << 20, staging_bytes=16 << 20, idle_timeout_s=0.2)
    try:
        time.sleep(0.6)
        srv.stop(timeout_s=5.0)
    finally:
        srv.close()


def test_tree_search_requests_alone_and_in_mix(hs, oracle):
    """Geometric SHA-1 UTS requests run on a slot's CTAs (work stealing over
    the slot's queues): counts exact against the oracle, the same alone and
    mixed with SyncPrims requests."""
    trees = [("uts", s, d, 4.0) for s, d in [(2, 6), (3, 7), (4, 8), (5, 9), (7, 5), (11, 8)]]
    insts, inits = _requests(hs, 404)
    srv = hs.Server(slots=8, gang=8, arena_bytes=512 << 20, staging_bytes=256 << 20, idle_timeout_s=20.0)
    try:
        alone = []
        for t in trees:
            rid, out = srv.submit(t)
            c = srv.wait(1)[0]
            assert c["status"] == 0
            alone.append(hs.serve_uts_counts(out))
        mixed = list(zip(trees + insts, [None] * len(trees) + inits))
        outs = {}
        for x, a in mixed:
            rid, out = srv.submit(x, a)
            outs[rid] = (x, a, out)
        comps = {c["id"]: c for c in srv.wait(len(mixed))}
        srv.stop()
    finally:
        srv.close()
    for t, got in zip(trees, alone):
        assert got == oracle.geo_count(t[1], t[2], t[3]), t
    k = 0
    for rid, (x, a, out) in outs.items():
        assert comps[rid]["status"] == 0
        if x[0] == "uts":
            assert hs.serve_uts_counts(out) == alone[k], x
            k += 1
        else:
            assert np.array_equal(out, _expected(hs, x, a)), x


def test_admission_passes_a_head_that_does_not_fit(hs):
    """A large request that cannot fit while another large one runs does not
    hold up small requests behind it: they are admitted past it (within the
    admission window, before the head has waited 20 ms) and finish first; the
    large one then runs once pages are free.  Every result is exact."""
    nsm = hs.device_info()["nsm"]
    long_run = (0, 40, 64, 3000)    # a tree barrier instance of ~2.7 MB, thousands of episodes
    blocked = (0, 40, 64, 2)        # the same size: no room while the first one runs
    smalls = [(7, 4, 4, 10), (4, 3, 6, 8), (20, 5, 8, 6), (10, 2, 4, 5)]
    insts = [long_run, blocked] + smalls
    rng = np.random.default_rng(11)
    inits = [rng.integers(0, 1000, size=hs.Server.request_words(*x, nsm=nsm)).astype(np.uint32) for x in insts]
    big = max(a.size for a in inits[:2]) * 4
    # room for one large request and every small one, not for two large ones
    arena = (big // (64 << 10) + 1 + 4 * 8) * (64 << 10)
    srv = hs.Server(slots=4, gang=4, arena_bytes=arena, staging_bytes=64 << 20, idle_timeout_s=20.0)
    try:
        rid0, out0 = srv.submit(insts[0], inits[0])
        time.sleep(0.002)  # the long request is admitted and holds its pages
        ids = [(rid0, out0)] + [srv.submit(x, a) for x, a in zip(insts[1:], inits[1:])]
        order = [c["id"] for c in srv.wait(len(insts))]
        for k, (rid, out) in enumerate(ids):
            assert np.array_equal(out, _expected(hs, insts[k], inits[k])), insts[k]
        pos = {rid: i for i, rid in enumerate(order)}
        small_ids = [rid for rid, _ in ids[2:]]
        assert max(pos[r] for r in small_ids) < pos[ids[1][0]], order  # the small ones went past the blocked one
        srv.stop()
    finally:
        srv.close()
