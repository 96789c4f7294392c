"""GPU: HS_RUN_GRAPH, the repeats of a run captured as one CUDA graph and
replayed.  Final storage must equal the plain launches' (and the golden's
closed form) on every primitive family, on host and device storage, on the
legacy and a user stream, with thread-block clusters, and on a replay of the
cached graph; the sweep driver's graph mode must report exact points."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [("faMutex", 10, 1, 30), ("sleepMutex", 20, 2, 20), ("spinSemEBO10", 10, 2, 20),
         ("spinMutexUniq", 10, 2, 20), ("spinSemUniq2", 5, 1, 20), ("atomicTreeBarrUniq", 10, 1, 50),
         ("lfTreeBarrUniqLocalExch", 64, 2, 30), ("atomicTreeBarrUniqLocalExch", 100, 2, 20),
         ("PRspinSem10", 10, 1, 20), ("atomicTreeBarrUniqNaiveSRB", 10, 1, 20)]


def _init(hs, cfg, seed):
    return np.random.default_rng(seed).integers(0, 1000, size=hs.storage_words(cfg)).astype(np.uint32)


@pytest.mark.parametrize("prim,L,mult,iters", CASES)
def test_graph_equals_plain_launches(hs, prim, L, mult, iters):
    nsm = hs.device_info()["nsm"]
    plain = hs.RunConfig(prim, L, mult * nsm, iters, threads=256, repeats=4, mode="inc")
    graph = hs.RunConfig(prim, L, mult * nsm, iters, threads=256, repeats=4, mode="inc", flags=hs.RUN_GRAPH)
    init = _init(hs, plain, 5)
    want = hs.expected_storage(plain, init)
    a = init.copy()
    ra = hs.run(plain, a)
    for _ in range(2):  # captured, then replayed from the context's cache
        b = init.copy()
        rb = hs.run(graph, b)
        assert np.array_equal(b, want), prim
        assert rb.launches == 4 and rb.cluster == ra.cluster
    assert np.array_equal(a, want)


def test_graph_on_device_storage_and_user_stream(hs):
    torch = pytest.importorskip("torch")
    nsm = hs.device_info()["nsm"]
    cfg = hs.RunConfig("spinMutexEBO", 10, nsm, 40, threads=256, repeats=3, mode="inc", flags=hs.RUN_GRAPH)
    init = _init(hs, cfg, 9)
    want = hs.expected_storage(cfg, init)
    s = torch.cuda.Stream()
    for stream in (None, s.cuda_stream):
        t = torch.from_numpy(init.view(np.int32).copy()).cuda()
        torch.cuda.synchronize()
        hs.run(cfg, t, stream=stream)
        torch.cuda.synchronize()
        assert np.array_equal(t.cpu().numpy().view(np.uint32), want)


def test_graph_with_sync_each_is_rejected(hs):
    cfg = hs.RunConfig("faMutex", 10, 8, 10, flags=hs.RUN_GRAPH | hs.RUN_SYNC_EACH)
    with pytest.raises(hs.HsError) as e:
        hs.run(cfg, np.zeros(hs.storage_words(cfg), np.uint32))
    assert e.value.status == hs.HS_EINVAL


def test_sweep_driver_graph_mode(hs):
    nsm = hs.device_info()["nsm"]
    p = subprocess.run([sys.executable, "-m", "heterosync_gb300.cli", "sweep", "--graph", "--prims",
                        "faMutex spinSem10 atomicTreeBarrUniq spinMutexUniq", "--num-tbs", "%d,%d" % (nsm, 2 * nsm),
                        "--iters", "5", "--runs", "2"], capture_output=True, text=True, cwd=ROOT)
    assert p.returncode == 0, p.stderr
    rows = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(rows) == 8
    assert all(r["graph"] and r["bit_exact"] and r["average_ms"] > 0 for r in rows)
