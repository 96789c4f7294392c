"""The C-ABI library loads without a GPU and exports every function its
public headers declare; host-only entry points behave."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include", "hs")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.append(name)
    return names


def test_headers_declare_functions():
    names = declared_functions()
    assert "hs_run" in names and "cudaLocksInit" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(hs):
    out = subprocess.run(["nm", "-D", "--defined-only", hs.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_prim_name_table(hs):
    L = hs.lib()
    for name, pid in hs.PRIM_NAMES.items():
        assert L.hs_prim_id(name.encode()) == pid
        assert L.hs_prim_name(pid).decode() == name
    assert L.hs_prim_id(b"noSuchPrim") == -1
    assert len(hs.PRIM_NAMES) == 28


def test_labels_match_reference(hs):
    # main.cu:1352-1451, including the "002" the reference prints for spinSem120
    assert hs.prim_label("faMutex", 100) == "fetchadd_mutex_100"
    assert hs.prim_label("atomicTreeBarrUniqLocalExch", 7) == "atomic_tree_barrier_localExch_007"
    assert hs.prim_label("spinSem120", 10) == "spin_lock_sem_002_010"
    assert hs.prim_label("spinSemUniq120", 10) == "spin_lock_sem_uniq_002_010"
    assert hs.prim_label("spinSemEBO120", 10) == "ebo_sem_120_010"
    assert hs.prim_label("lfTreeBarrUniq", 1000) == "fbs_tree_barrier_1000"


def test_storage_words_and_validation(hs):
    cfg = hs.RunConfig(prim="faMutex", num_ldst=10, num_tbs=8, threads=32)
    assert hs.storage_words(cfg, 152) == 32 * 11
    cfg = hs.RunConfig(prim="spinSem10", num_ldst=10, num_tbs=296, threads=256)
    assert hs.storage_words(cfg, 148) == 2 * 256 * 11
    cfg = hs.RunConfig(prim="faMutexUniq", num_ldst=3, num_tbs=300, threads=32)
    assert hs.storage_words(cfg, 152) == 152 * 32 * 4
    for bad in (dict(threads=24), dict(threads=2048), dict(num_tbs=0), dict(num_ldst=0),
                dict(prim="spinSem1", mode="slice"), dict(backoff_max_ns=1000)):
        c = hs.RunConfig(**{**dict(prim="faMutex"), **bad})
        with pytest.raises(hs.HsError) as e:
            hs.storage_words(c, 152)
        assert e.value.status == 1


def test_status_strings(hs):
    L = hs.lib()
    assert L.hs_status_string(0) == b"ok"
    assert L.hs_status_string(2) == b"device wait timed out"
    assert L.hs_version() >= 1


def test_hip_extension_names_and_bases(hs):
    """The HIP build's extra primitives (main.hip.cpp:2056-2083) resolve by name,
    print the HIP labels and run as their CUDA base primitive."""
    L = hs.lib()
    for name, pid in hs.HIP_PRIM_NAMES.items():
        assert L.hs_prim_id(name.encode()) == pid
    assert hs.prim_base("PRspinSem10") == (10, 1)
    assert hs.prim_base("PRspinSemEBO120") == (15, 1)
    assert hs.prim_base("atomicTreeBarrUniqSRB") == (0, 2)
    assert hs.prim_base("atomicTreeBarrUniqLocalExchNaiveSRB") == (1, 3)
    assert hs.prim_base("atomicTreeBarrUniqLocalExchNaiveAllSRB") == (1, 4)
    assert hs.prim_base("faMutex") == (7, 0)
    assert hs.prim_label("PRspinSem120", 10) == "prior_spin_lock_sem_002_010"
    assert hs.prim_label("PRspinSemEBO2", 10) == "prior_ebo_sem_002_010"
    assert hs.prim_label("atomicTreeBarrUniqLocalExchNaiveAllSRB", 5) == "atomic_tree_barrier_localExch_NaiveAllSRB_005"


def test_hip_extension_storage_and_closed_form(hs):
    for name, base in [("PRspinSem2", "spinSem2"), ("atomicTreeBarrUniqNaiveSRB", "atomicTreeBarrUniq"),
                       ("atomicTreeBarrUniqLocalExchSRB", "atomicTreeBarrUniqLocalExch")]:
        a = hs.RunConfig(prim=name, num_ldst=7, num_tbs=24, num_iters=3, threads=64, repeats=2, mode="inc", nsm=8)
        b = hs.RunConfig(prim=base, num_ldst=7, num_tbs=24, num_iters=3, threads=64, repeats=2, mode="inc", nsm=8)
        assert hs.storage_words(a) == hs.storage_words(b)
        init = np.arange(hs.storage_words(a), dtype=np.uint32)
        assert np.array_equal(hs.expected_storage(a, init), hs.expected_storage(b, init))


def test_run_structs_match_the_header(hs, tmp_path):
    """The ctypes mirrors of hs_run_config and hs_run_result have the C layout
    (size and the offset of the last field), compiled from include/hs/hs.h."""
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if not cc:
        import pytest
        pytest.skip("gcc not found")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "hs/hs.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu\\n", sizeof(hs_run_config), '
                   'offsetof(hs_run_config, flags), sizeof(hs_run_result), offsetof(hs_run_result, tbs_per_cta));'
                   'return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I" + os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(hs._RunConfig), hs._RunConfig.flags.offset, ctypes.sizeof(hs._RunResult),
                   hs._RunResult.tbs_per_cta.offset]
