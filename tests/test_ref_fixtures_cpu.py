"""Pin the oracle to the reference itself: tests/golden/ref_syncprims.json holds
SHA-256 digests of the final storage produced by the reference's OWN kernels
(its unmodified sources built into oracle/_ref, run on a GB300 by
tests/golden/make_ref_fixtures.py).  The oracle golden must reproduce every
digest on the same inputs (storage[i] = (float)i)."""
import hashlib
import json
import os

import numpy as np
import pytest

FIX = os.path.join(os.path.dirname(__file__), "golden", "ref_syncprims.json")


def _entries():
    if not os.path.exists(FIX):
        return []
    with open(FIX) as f:
        return json.load(f)["entries"]


@pytest.mark.skipif(not os.path.exists(FIX), reason="reference fixtures not generated yet")
@pytest.mark.parametrize("e", _entries(), ids=lambda e: "p%d_T%d_L%d_G%d" % (e["prim"], e["threads"], e["num_ldst"],
                                                                            e["num_tbs"]))
def test_oracle_reproduces_reference_output(oracle, e):
    n = oracle.storage_words(e["prim"], e["threads"], e["num_ldst"], e["num_tbs"], e["nsm"])
    assert n == e["words"]
    init = np.arange(n, dtype=np.float32).view(np.uint32)
    out = oracle.golden(e["prim"], e["threads"], e["num_ldst"], e["num_tbs"], e["iters"], e["repeats"], e["nsm"],
                        False, init)
    assert [int(x) for x in out[:48]] == e["head"]
    assert hashlib.sha256(out.tobytes()).hexdigest() == e["sha256"]


@pytest.mark.skipif(not os.path.exists(FIX), reason="reference fixtures not generated yet")
def test_fixture_covers_every_reference_family():
    prims = {e["prim"] for e in _entries()}
    assert {0, 1, 2, 3, 4, 5, 6, 7, 20, 23} <= prims


def test_refcounter_known_answer_is_the_references_output():
    """tests/golden/ref_relaxed.json holds digests of the reference's own
    refCounter kernel's final counters (made on a GB300 by
    tests/golden/make_ref_fixtures.py relaxed): they equal the known answer the
    build's tests use -- every counter back at 0 -- and the reference set delete
    flags in every run."""
    import hashlib
    import json
    import os
    import numpy as np
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_relaxed.json")
    with open(path) as f:
        d = json.load(f)
    assert len(d["entries"]) >= 4
    for e in d["entries"]:
        zeros = hashlib.sha256(np.zeros(e["counters"], np.uint32).tobytes()).hexdigest()
        assert e["counters"] == e["num_tbs"] * e["tb_size"] // e["num_sharers"]
        assert e["sha256_counters0"] == zeros and e["sha256_counters1"] == zeros, e
        assert e["del0_any"] and e["del1_any"]
