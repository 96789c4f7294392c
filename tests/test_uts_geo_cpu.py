"""Geometric SHA-1 UTS: the oracle's SHA-1 against Python's hashlib, its
tree walk against a hashlib restatement of the tree definition, and the
library's threshold table against the oracle's (no GPU)."""
import hashlib
import os

import numpy as np


def test_sha1_matches_hashlib(oracle):
    rng = np.random.default_rng(1)
    for n in (0, 1, 19, 20, 24, 55):
        for _ in range(50):
            m = bytes(rng.integers(0, 256, size=n, dtype=np.uint8))
            assert oracle.sha1(m) == hashlib.sha1(m).digest()


def test_node_states_follow_the_definition(oracle):
    for seed in (0, 1, 2, 0xFFFFFFFF):
        root = hashlib.sha1(b"\0" * 16 + seed.to_bytes(4, "big")).digest()
        assert oracle.geo_root(seed) == root
        for i in (0, 1, 7, 95):
            assert oracle.geo_child(root, i) == hashlib.sha1(root + i.to_bytes(4, "big")).digest()


def _count_with_hashlib(seed, limit, b):
    q = b / (1.0 + b)
    t, p = [], q
    for _ in range(128):
        t.append(min(int(p * 2147483648.0), 0xFFFFFFFF))
        p *= q

    def nchildren(s, d):
        if d >= limit:
            return 0
        r = int.from_bytes(s[16:20], "big") & 0x7FFFFFFF
        m = 0
        while m < len(t) and r < t[m]:
            m += 1
        return m

    root = hashlib.sha1(b"\0" * 16 + seed.to_bytes(4, "big")).digest()
    nodes, leaves, deepest = 0, 0, 0
    stack = [(root, 0)]
    while stack:
        s, d = stack.pop()
        nodes += 1
        deepest = max(deepest, d)
        m = nchildren(s, d)
        if m == 0:
            leaves += 1
        for i in range(m):
            stack.append((hashlib.sha1(s + i.to_bytes(4, "big")).digest(), d + 1))
    return nodes, leaves, deepest


def test_oracle_count_matches_hashlib_walk(oracle):
    for seed, limit, b in [(2, 5, 4.0), (3, 5, 4.0), (4, 6, 4.0), (5, 5, 4.0), (9, 4, 8.0), (11, 7, 2.0)]:
        assert oracle.geo_count(seed, limit, b) == _count_with_hashlib(seed, limit, b)


def test_library_table_matches_oracle(hs, oracle):
    for b in (1.0, 2.0, 4.0, 8.0, 0.5):
        lt, lnz = hs.uts_geo_table(b)
        ot, onz = oracle.geo_table(b)
        assert lnz == onz and np.array_equal(lt, ot)
    t, nz = hs.uts_geo_table(4.0)
    assert nz == 96 and t[0] == int(0.8 * 2 ** 31) and all(t[i] >= t[i + 1] for i in range(127))
