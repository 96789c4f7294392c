"""GPU: the relaxed-atomics microbenchmarks and UTS through the C ABI, checked
against their exact outputs (final counters, sequence numbers, output pattern,
node counts) and invariants, at the reference's own run-file arguments and
other sizes; and the drop-in programs' PASS lines."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "heterosync_gb300", "bin")


@pytest.mark.parametrize("args", [(32, 64, 32, 4), (1, 8, 256, 3), (4, 16, 64, 1), (64, 64, 128, 2)])
def test_refcounter(hs, args):
    sharers, tbs, tb, reps = args
    c0, c1, d0, d1, r = hs.refcounter(sharers, tbs, tb, reps)
    assert not c0.any() and not c1.any()          # every increment undone (refCounter.cu:86-98)
    groups = tbs // sharers
    per = (tbs * tb // sharers) // groups
    # every counter's last decrement saw 1: some sharing thread marked it deleted
    for dels in (d0, d1):
        seen = np.zeros(groups * per, dtype=bool)
        for b in range(tbs):
            for t in range(tb):
                if dels[b * tb + t]:
                    seen[(b % groups) * per + t] = True
        used = np.zeros(groups * per, dtype=bool)
        for b in range(tbs):
            used[(b % groups) * per: (b % groups) * per + tb] = True
        assert seen[used].all()


@pytest.mark.parametrize("args", [(112, 32), (8, 256), (152, 64)])
def test_splitcounter(hs, args):
    tbs, tb = args
    c, o, r = hs.splitcounter(tbs, tb)
    assert np.array_equal(c, np.ones_like(c))     # splitCounter.cu:54-60
    lanes = np.arange(tbs * tb) % 32
    assert not o[lanes < 16].any()                # writers do not write outArr
    per_half_warp = (tbs * tb // 2) // (tb // 2) * 16
    assert (o[lanes >= 16] <= per_half_warp).all()


@pytest.mark.parametrize("args", [(512, 128, 4), (64, 32, 2), (160, 64, 16), (48, 256, 3)])
def test_seqlocks(hs, args):
    tbs, tb, group = args
    seq, d0, d1, o, r = hs.seqlocks(tbs, tb, group)
    for k in range(tbs // group):
        writers = sum(1 for b in range(tbs) if b % 16 == 0 and b % group == k)
        assert seq[k] == 2 * 10 * writers         # each writer: +2 per iteration, NUM_ITERS = 10
    assert r.dev_error_bits == 0


def _rand_arr(n, seed=2018):
    import ctypes
    import ctypes.util
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(seed)
    return np.array([libc.rand() for _ in range(n)], dtype=np.float64).astype(np.float32) / np.float32(4294967295.0)


@pytest.mark.parametrize("args", [(160, 32, 16, 4, 0.33, 1), (152, 64, 8, 2, 0.0, 4), (64, 128, 16, 3, 1.0, 2)])
def test_flags(hs, args):
    tbs, tb, accs, reps, cutoff, iters = args
    rnd = _rand_arr(tbs * iters)
    o, dirty, r = hs.flags(tbs, tb, accs, reps, cutoff, iters, rnd)
    want = np.zeros(tbs * tb, np.uint32)
    if dirty:
        want[tb * (tbs - 1):] = reps * accs * accs    # flags.cu:134-159
    assert np.array_equal(o, want)
    if cutoff >= 1.0:
        assert dirty > 0
    if cutoff == 0.0:
        assert dirty == 0 or (rnd == 0).any()


@pytest.mark.parametrize("n,fert,blocks", [(8193, 90, 128), (1001, 60, 8), (65537, 80, 304), (4097, 50, 1)])
def test_uts_counts_exact(hs, oracle, n, fert, blocks):
    tree, leaves, leaf_sum, _ = oracle.uts_tree(n, fert, 200)
    cores = min(blocks, 15)
    fr, proc = oracle.uts_frontier(tree, cores)
    ptree, *_ = hs.uts_tree(n, fert, 200)
    r = hs.uts_run(ptree, fr, proc, blocks, 128)
    assert (r.nodes_processed, r.leaves_found, r.leaf_sum) == (n, leaves, leaf_sum)


@pytest.mark.parametrize("prog,args,ok", [
    ("refCounter", ["32", "64", "32", "4"], "TEST PASSED!"),
    ("splitCounter", ["112", "32"], "PASSED"),
    ("seqlocks", ["512", "128", "4", "0"], None),
    ("flags", ["160", "32", "16", "4", "0.33", "1", "1"], "Test PASSED!"),
    ("uts", ["1", "8192", "90", "32", "128"], "SUCCESS!"),
])
def test_dropin_programs(hs, prog, args, ok):
    r = subprocess.run([os.path.join(BIN, prog)] + args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = r.stdout + r.stderr
    if ok:
        assert ok in out
    assert "ERROR" not in out
