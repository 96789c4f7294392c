"""The cohort (die-aware) protocols, modelled on the host: std::threads stand
for TBs on two dies and run the device code's encodings (a die ticket queue,
its turn word carrying the pass count, over a global test-and-set word or a
global ticket;
semaphore writers as ticket cohorts over the packed semaphore word, with
readers beside them).  Small ticket wraps and pass limits drive the
wrap-around and global release branches.  Mutual exclusion must hold (for the
semaphore: no reader beside a writer, at most N readers), every critical
section must count, and every lock word must end free."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("cohort") / "cohort_model")
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", os.path.join(HERE, "cohort_model.cpp"), "-o", exe],
                   check=True)
    return exe


@pytest.mark.parametrize("kind", ["tas", "ticket"])
@pytest.mark.parametrize("threads,iters,max_pass,lwrap,gwrap", [
    (4, 20000, 63, (1 << 25) - 1, 1000000000),  # the device's constants
    (6, 20000, 2, 7, 5),                         # every other op crosses; tickets wrap constantly
    (8, 10000, 32, 3, 1),
    (3, 30000, 1, 6, 2),                         # max_pass 1: never passes, always the global lock
])
def test_cohort_protocol(model, kind, threads, iters, max_pass, lwrap, gwrap):
    # a local wrap must exceed the threads that can hold tickets at once, as on the device (2^25 - 1)
    if lwrap + 1 < (threads + 1) // 2 + 1:
        pytest.skip("wrap smaller than the waiters of one die")
    p = subprocess.run([model, kind, str(threads), str(iters), str(max_pass), str(lwrap), str(gwrap)],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0 and p.stdout.startswith("ok %d" % (threads * iters)), p.stdout + p.stderr


@pytest.mark.parametrize("writers,iters,max_pass,readers,n,lwrap", [
    (4, 20000, 63, 4, 1, (1 << 25) - 1),  # the device's pass limit and ticket wrap, semaphore of 1
    (6, 10000, 2, 3, 2, 7),               # frequent global posts, tickets wrap constantly
    (5, 10000, 1, 6, 10, 5),              # never passes
    (8, 5000, 32, 0, 120, 4),             # writers only (numTBs <= NUM_SM: every TB a writer)
])
def test_cohort_semaphore_writers(model, writers, iters, max_pass, readers, n, lwrap):
    p = subprocess.run([model, "sem", str(writers), str(iters), str(max_pass), str(readers), str(n), str(lwrap)],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0 and p.stdout.startswith("ok %d" % (writers * iters)), p.stdout + p.stderr
