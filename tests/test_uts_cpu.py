"""CPU: the UTS tree generator, golden and initial frontier of the product
(host side of hs_uts_*) against the oracle's restatement (oracle/uts.c) and an
independent pure-Python restatement driving glibc's rand() (uts.cu:290-383)."""
import ctypes
import ctypes.util

import numpy as np
import pytest


def py_tree(num_nodes, fertility, seed):
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(seed)
    value = [0] * num_nodes
    child = [(0, 0)] * num_nodes
    undecided, leaves = [0], []
    nxt = 1
    while nxt != num_nodes:
        if not undecided:
            undecided, leaves = leaves, []
        cur = undecided[0]
        value[cur] = libc.rand() % 100
        if libc.rand() % 100 < fertility:
            child[cur] = (nxt, nxt + 1)
            undecided += [nxt, nxt + 1]
            nxt += 2
        else:
            child[cur] = (0, 0)
            leaves.insert(0, cur)
        undecided.pop(0)
    total = 0
    for n in undecided:
        child[n] = (0, 0)
        value[n] = 1
        total += 1
    total += sum(value[n] for n in leaves)
    return value, child, len(leaves) + len(undecided), total


@pytest.mark.parametrize("n,fert", [(101, 90), (1001, 60), (8193, 90), (4097, 30)])
def test_tree_matches_oracle_and_python(hs, oracle, n, fert):
    t1, l1, s1, r1 = hs.uts_tree(n, fert, 200)
    t2, l2, s2, r2 = oracle.uts_tree(n, fert, 200)
    assert t1.tobytes() == t2.tobytes()
    assert (l1, s1, r1) == (l2, s2, r2)
    value, child, lv, ls = py_tree(n, fert, 200)
    assert list(t1["value"]) == value
    assert list(zip(t1["child_a"], t1["child_b"])) == [tuple(c) for c in child]
    assert (l1, s1) == (lv, ls)
    # golden = leaves of the tree, by definition
    leaf = t1["child_a"] == 0
    assert int(leaf.sum()) == l1 and int(t1["value"][leaf].sum()) == s1


@pytest.mark.parametrize("cores", [1, 8, 15])
def test_frontier_matches_oracle(hs, oracle, cores):
    t, *_ = hs.uts_tree(8193, 90, 200)
    f1, p1 = hs.uts_frontier(t, cores)
    f2, p2 = oracle.uts_frontier(t, cores)
    assert np.array_equal(f1, f2) and p1 == p2
    assert len(f1) == cores * 16 and len(set(f1.tolist())) == len(f1)


def test_even_tree_size_rejected(hs):
    with pytest.raises(hs.HsError):
        hs.uts_tree(100, 90, 200)


def test_large_tree_builders_agree(hs, oracle):
    """A 262,145-node tree (5 MB of nodes, allocated where a pointer no longer
    fits 32 bits): the oracle's generator and the library's host builder give
    the same tree and the same golden counts."""
    import numpy as np
    tree, leaves, leaf_sum, restarts = oracle.uts_tree(262145, 70, 200)
    mine, l2, s2, r2 = hs.uts_tree(262145, 70, 200)
    assert (leaves, leaf_sum, restarts) == (l2, s2, r2)
    assert np.array_equal(tree["child_a"], mine["child_a"]) and np.array_equal(tree["value"], mine["value"])
    fr, proc = oracle.uts_frontier(tree, 15)
    assert len(fr) == 15 * 16 and proc > 0
