"""GPU: seeded random configurations across every primitive, thread count,
numLdSt, numTBs, data mode and form flag.  Each run must end bit-exact with
the golden's closed form (or, for a tree barrier whose TBs cannot all be
resident, be refused with HS_ENORES before launch).  This reaches the forms a
planner picks from the sizes -- group-CTA barriers on the register path and
with bulk-copy buffers, clusters, die cohorts, four-part bulk loads, graph
replay -- at shapes the targeted tests do not list."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_CASES = 400


def _cases(nsm):
    rng = np.random.default_rng(20261204)
    prims = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]
    out = []
    for i in range(N_CASES):
        prim = int(rng.choice(prims))
        T = int(rng.choice([32, 64, 128, 256]))
        L = int(rng.choice([1, 3, 10, 17, 31, 33, 50, 64, 65, 100, 127]))
        mult = int(rng.choice([1, 2, 3, 4]))
        G = int(rng.choice([mult * nsm, max(1, mult * nsm - int(rng.integers(1, 7))), int(rng.integers(1, 40))]))
        if 24 <= prim <= 31 and G > nsm and G % nsm:
            # per-SM semaphores with uneven groups: the writer of an SM whose
            # rotation wraps past numTBs writes the next SM's chunks under its
            # own semaphore (main.cu:667, 819), concurrently with that SM's
            # writer -- a race in the reference's own algorithm, so no golden
            G = (G // nsm) * nsm
        mode = str(rng.choice(["ref", "inc"]))
        flags = 0
        for f in ("RUN_NO_COHORT", "RUN_NO_CLUSTER", "RUN_NO_GROUP_CTA", "RUN_REGISTER_CS", "RUN_CLUSTER_CS",
                  "RUN_GRAPH"):
            if rng.random() < 0.15:
                flags |= {"RUN_NO_COHORT": 32, "RUN_NO_CLUSTER": 4, "RUN_NO_GROUP_CTA": 128, "RUN_REGISTER_CS": 8,
                          "RUN_CLUSTER_CS": 64, "RUN_GRAPH": 16}[f]
        out.append((i, prim, T, L, G, mode, flags))
    return out


def test_random_configurations(hs):
    nsm = hs.device_info()["nsm"]
    refused = 0
    for i, prim, T, L, G, mode, flags in _cases(nsm):
        iters = 3 if L > 64 else 6
        cfg = hs.RunConfig(prim=prim, num_ldst=L, num_tbs=G, num_iters=iters, threads=T, repeats=2, mode=mode,
                           flags=flags, timeout_ns=5_000_000_000)
        init = np.random.default_rng(1000 + i).integers(0, 1 << 31, size=hs.storage_words(cfg)).astype(np.uint32)
        st = init.copy()
        r = hs.run(cfg, st, check=False)
        case = (i, hs.prim_name(prim), T, L, G, mode, flags)
        if r.status == hs.HS_ENORES and prim <= 3:
            refused += 1  # a barrier too large to be resident: refused before launch
            continue
        assert r.status == 0, (case, r)
        assert np.array_equal(st, hs.expected_storage(cfg, init)), case
    assert refused < N_CASES // 4
