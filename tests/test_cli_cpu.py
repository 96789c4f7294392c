"""Command-line behaviour that needs no GPU: argument count and exit codes
(main.cu:1132-1172)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "heterosync_gb300", "bin", "allSyncPrims-1kernel")


def test_usage_on_wrong_argc(hs):
    r = subprocess.run([CLI, "faMutex", "10"], capture_output=True, text=True)
    assert r.returncode == 255
    assert "./allSyncPrims-1kernel <syncPrim> <numLdSt> <numTBs> <numCSIters>" in r.stderr
    assert "spinSemEBOUniq120" in r.stderr


def test_usage_lists_all_primitives(hs):
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 255
    for name in hs.PRIM_NAMES:
        assert "\t\t%s - " % name in r.stderr


def test_usage_lists_hip_extensions():
    import os
    import subprocess
    exe = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "heterosync_gb300", "bin",
                       "allSyncPrims-1kernel")
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode != 0 and "PRspinSem" in p.stderr and "NaiveAllSRB" in p.stderr
