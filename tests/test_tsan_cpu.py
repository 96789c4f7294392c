"""The host-thread code under the thread sanitizer: the cohort protocol model
(tests/cohort_model.cpp: the queue cohorts over test-and-set and ticket locks,
and the semaphore-writer cohorts) and
the std::thread twins that serve as the oracle's concurrent restatement and the
CPU baseline (oracle/twins.cpp, driven by tests/twins_tsan_main.cpp and checked
against the oracle golden).  A data race, or any result that differs, fails."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), "oracle")
ENV = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66")


def _tsan_build(out, sources, lang_flags):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    probe = subprocess.run([cxx, "-fsanitize=thread", "-x", "c++", "-", "-o", out + ".probe"],
                           input="int main(){return 0;}", capture_output=True, text=True)
    if probe.returncode != 0 or subprocess.run([out + ".probe"], capture_output=True).returncode != 0:
        pytest.skip("thread sanitizer unavailable")
    subprocess.run([cxx, "-fsanitize=thread", "-O1", "-g", "-pthread"] + lang_flags + sources + ["-o", out],
                   check=True)
    return out


def test_cohort_model_under_tsan(tmp_path):
    exe = _tsan_build(str(tmp_path / "cohort_tsan"), [os.path.join(HERE, "cohort_model.cpp")], ["-std=c++17"])
    for args in (["tas", "4", "3000", "2", "7", "5"], ["ticket", "4", "3000", "2", "7", "5"],
                 ["sem", "4", "2000", "2", "3", "1", "5"], ["sem", "3", "2000", "32", "2", "10", "7"]):
        p = subprocess.run([exe] + args, capture_output=True, text=True, timeout=300, env=ENV)
        assert p.returncode == 0 and p.stdout.startswith("ok"), (args, p.stdout, p.stderr[-3000:])


def test_twins_under_tsan(tmp_path):
    golden_o = str(tmp_path / "golden.o")
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not found")
    subprocess.run([gcc, "-fsanitize=thread", "-O1", "-g", "-std=c11", "-c", os.path.join(ORACLE, "golden.c"),
                    "-o", golden_o], check=True)
    exe = _tsan_build(str(tmp_path / "twins_tsan"),
                      [os.path.join(HERE, "twins_tsan_main.cpp"), os.path.join(ORACLE, "twins.cpp"), golden_o],
                      ["-std=c++17"])
    p = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=ENV)
    assert p.returncode == 0 and p.stdout.strip() == "ok", (p.stdout, p.stderr[-3000:])
