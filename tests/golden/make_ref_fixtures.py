"""Generate tests/golden/ref_syncprims.json: final storage of the reference's
OWN SyncPrims kernels (oracle/_ref, built from the unmodified reference sources)
for small configurations, recorded as SHA-256 digests plus leading words.

Run on a GPU machine:  python tests/golden/make_ref_fixtures.py OUT.json
The CPU test test_ref_fixtures_cpu.py recomputes the oracle golden for each
entry and compares digests, pinning the oracle to the reference itself.
Initial storage is the reference's storage[i] = i (as float).

    python tests/golden/make_ref_fixtures.py relaxed OUT.json
records the reference's own refCounter kernel (oracle/_ref/refcounter_sm100.cubin)
for the sizes of REFCOUNTER_CASES: digests of both final counter arrays (the
deterministic output) and whether each delete-flag array has a set entry (the
reference's own check, refCounter.cu:86-120; which entries are set depends on
the interleaving).
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

# (prim, threads, numLdSt, numTBs as "k*NSM+c" multiplier/offset, iters, repeats)
CASES = [
    (7, 32, 25, (0, 2), 1, 10), (4, 32, 25, (0, 2), 1, 10), (5, 32, 25, (0, 2), 1, 10),
    (6, 32, 25, (0, 2), 1, 10), (7, 256, 30, (0, 3), 1, 10), (4, 256, 12, (0, 1), 1, 10),
    (20, 32, 25, (1, 8), 1, 10), (21, 32, 25, (1, 8), 1, 10), (22, 32, 25, (1, 8), 1, 10),
    (23, 32, 25, (1, 8), 1, 10), (23, 256, 25, (1, 8), 1, 10),
    # the reference's semaphore kernels (8-15, 24-31) are no longer run: see oracle/ref_runner.cpp;
    # the committed fixture keeps the digests recorded for 8-15 before that
    # the reference's Uniq semaphore kernels (24-31) are not run: they livelocked on GB300
    (0, 32, 25, (1, 0), 2, 10), (1, 32, 45, (2, 0), 2, 10), (2, 32, 25, (1, 0), 2, 10),
    (3, 32, 45, (2, 0), 2, 10), (0, 256, 25, (2, 0), 2, 10), (1, 256, 45, (4, 0), 2, 10),
    (2, 256, 25, (4, 0), 2, 10), (3, 256, 45, (2, 0), 2, 10), (1, 32, 25, (0, 100), 2, 10),
]


# (numSharersPerGroup, numTBs, tbSize, numRepeats): the reference's own run
# arguments (refCounter/run) first, then other sharing and sizes
REFCOUNTER_CASES = [(32, 64, 32, 4), (1, 8, 256, 3), (4, 152, 128, 2), (2, 16, 64, 10), (8, 608, 256, 1)]


def main_relaxed(out):
    entries = []
    for sharers, tbs, tb_size, reps in REFCOUNTER_CASES:
        c0, c1, d0, d1, ms = oracle.ref_refcounter(sharers, tbs, tb_size, reps)
        entries.append({"num_sharers": sharers, "num_tbs": tbs, "tb_size": tb_size, "num_repeats": reps,
                        "counters": int(c0.size), "sha256_counters0": hashlib.sha256(c0.tobytes()).hexdigest(),
                        "sha256_counters1": hashlib.sha256(c1.tobytes()).hexdigest(),
                        "del0_any": bool(d0.any()), "del1_any": bool(d1.any()), "ref_ms": ms})
        print("refCounter", sharers, tbs, tb_size, reps, "ok %.3f ms" % ms, flush=True)
    with open(out, "w") as f:
        json.dump({"generator": "tests/golden/make_ref_fixtures.py relaxed",
                   "kernel": "refCounter_kernel (cuda/relaxedAtomics/uvm/refCounter), one launch",
                   "entries": entries}, f, indent=1)


def main(out):
    nsm, _ = oracle.ref_device()
    entries = []
    for prim, T, L, (mul, off), iters, reps in CASES:
        G = mul * nsm + off
        n = oracle.storage_words(prim, T, L, G, nsm)
        init = np.arange(n, dtype=np.float32).view(np.uint32)
        final, ms = oracle.ref_run(prim, T, L, G, iters, reps, init)
        entries.append({"prim": prim, "threads": T, "num_ldst": L, "num_tbs": G, "iters": iters,
                        "repeats": reps, "nsm": nsm, "words": int(n),
                        "sha256": hashlib.sha256(final.tobytes()).hexdigest(),
                        "head": [int(x) for x in final[:48]], "ref_ms": ms})
        print(prim, T, L, G, iters, reps, "ok %.3f ms" % ms, flush=True)
    with open(out, "w") as f:
        json.dump({"generator": "tests/golden/make_ref_fixtures.py", "init": "storage[i] = (float)i",
                   "entries": entries}, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "relaxed":
        main_relaxed(sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(__file__), "ref_relaxed.json"))
    else:
        main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(__file__), "ref_syncprims.json"))
