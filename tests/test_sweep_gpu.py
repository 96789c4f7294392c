"""GPU: the results-script sweep driver and the drop-in program on the HIP
build's extra primitive names."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sweep_driver_parses_average(hs):
    nsm = hs.device_info()["nsm"]
    p = subprocess.run([sys.executable, "-m", "heterosync_gb300.cli", "sweep", "--prims",
                        "faMutex spinSem10 atomicTreeBarrUniq spinMutexUniq", "--num-tbs", "%d,%d" % (nsm, 2 * nsm),
                        "--iters", "5"], capture_output=True, text=True, cwd=ROOT)
    assert p.returncode == 0, p.stderr
    rows = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(rows) == 8
    assert all(r["average_ms"] is not None and r["average_ms"] > 0 for r in rows)


@pytest.mark.parametrize("name", ["PRspinSem10", "PRspinSemEBO1", "atomicTreeBarrUniqLocalExchSRB",
                                  "atomicTreeBarrUniqNaiveAllSRB"])
def test_program_runs_hip_names(hs, name):
    exe = os.path.join(ROOT, "heterosync_gb300", "bin", "allSyncPrims-1kernel")
    nsm = hs.device_info()["nsm"]
    p = subprocess.run([exe, name, "10", str(2 * nsm), "20"], capture_output=True, text=True)
    assert p.returncode == 0 and "PASSED" in p.stdout, p.stdout + p.stderr
