"""The reference's device and host API, run on the GPU: kernels written against
include/hs/hs_device_ref.cuh with the reference's own index math
(tests/ref_api_kernels.cu: cudaMutex*Lock/Unlock[Local], cudaSemaphore*Wait/
Post[Local], joinBarrier_helper, joinLFBarrier_helper, cudaBarrier[Atomic]Local)
on lock state from cudaLocksInit -> hs_lock_data_get -> cudaMutexCreate* /
cudaSemaphoreCreate*, exactly as a program written for heterosync's
cudaLocks.h would get it.  Every one of the 28 primitives' final storage must
equal the oracle's restatement of the reference golden (main.cu:1633-1788).

A wait that runs out ends the calling CTA (fail-fast) instead of letting it
enter its critical section without the lock: the timeout test holds a mutex
that nothing releases and checks that no critical section ran, that the failure
is recorded, and that the context still runs work afterwards."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

PRIMS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31]
SEM_COUNT = {0: 1, 1: 2, 2: 10, 3: 120}


@pytest.fixture(scope="module")
def api(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    out = str(tmp_path_factory.mktemp("refapi") / "libref_api.so")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode=arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
                    "-shared", "-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "ref_api_kernels.cu"),
                    "-o", out], check=True)
    L = ctypes.CDLL(out)
    L.ref_api_run.argtypes = [ctypes.c_int, ctypes.c_uint] + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 6
    L.ref_api_lock_marks.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    L.ref_api_status.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.ref_api_hold_mutex.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_int]
    return L


def _host_api(hs):
    L = hs.lib()
    L.cudaLocksInit.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_bool, ctypes.c_int]
    L.hs_lock_data_get.restype = ctypes.c_void_p
    for f in ("cudaMutexCreateSpin", "cudaMutexCreateEBO", "cudaMutexCreateFA", "cudaMutexCreateSleep"):
        getattr(L, f).argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_int]
    for f in ("cudaSemaphoreCreateSpin", "cudaSemaphoreCreateEBO"):
        getattr(L, f).argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_int, ctypes.c_uint, ctypes.c_int]
    return L


def _max_blocks(G, nsm):
    """The smallest MAX_BLOCKS >= numTBs whose lock-data stride, (MAX_BLOCKS +
    NUM_SM) / 16 * 16, exceeds it (cudaLocksInit refuses the others)."""
    mb = G
    while (mb + nsm) // 16 * 16 <= mb:
        mb += 1
    return mb


def _init_locks(hs, nsm, max_blocks):
    H = _host_api(hs)
    # the reference's own sizing: 8 mutexes and 24 semaphores per SM (main.cu:1277-1279)
    assert H.cudaLocksInit(max_blocks, 8 * nsm, 24 * nsm, False, nsm) == 0
    ld = H.hs_lock_data_get()
    assert ld
    return H, ld


def _handle(H, prim, nsm):
    h = ctypes.c_uint()
    if 4 <= prim <= 7 or 20 <= prim <= 23:
        create = ("cudaMutexCreateSpin", "cudaMutexCreateEBO", "cudaMutexCreateSleep", "cudaMutexCreateFA")[prim % 4]
        assert getattr(H, create)(ctypes.byref(h), 3) == 0
    elif 8 <= prim <= 15 or 24 <= prim <= 31:
        create = "cudaSemaphoreCreateEBO" if (12 <= prim <= 15 or prim >= 28) else "cudaSemaphoreCreateSpin"
        assert getattr(H, create)(ctypes.byref(h), prim % 8, SEM_COUNT[prim % 4], nsm) == 0
    return h.value


@pytest.mark.parametrize("prim", PRIMS)
@pytest.mark.parametrize("T,L,G,nsm,iters", [(64, 5, 8, 4, 4), (32, 3, 12, 4, 3)])
def test_reference_api_matches_golden(hs, api, prim, T, L, G, nsm, iters):
    torch = pytest.importorskip("torch")
    import oracle
    mb = _max_blocks(G, nsm)
    H, ld = _init_locks(hs, nsm, max_blocks=mb)
    handle = _handle(H, prim, nsm)
    n = oracle.storage_words(prim, T, L, G, nsm)
    init = np.random.default_rng(prim * 131 + T).integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    storage = torch.from_numpy(init.view(np.int32).copy()).cuda()
    per_sm = torch.zeros(nsm * mb * 2, dtype=torch.int32, device="cuda")  # main.cu:1281
    torch.cuda.synchronize()
    rc = api.ref_api_run(prim, handle, storage.data_ptr(), ld, per_sm.data_ptr(), T, L, G, iters, nsm, mb)
    st = np.zeros(2, dtype=np.uint32)
    api.ref_api_status(st.ctypes.data, 1)
    assert rc == 0 and st[0] == 0, (prim, rc, st)
    got = storage.cpu().numpy().view(np.uint32)
    want = oracle.golden(prim, T, L, G, iters, 1, nsm, False, init)
    assert np.array_equal(got, want), prim


def test_timed_out_lock_ends_the_cta(hs, api):
    """A spin mutex held by nobody who will release it: every TB's lock wait
    runs out (2 s without progress), the CTAs end without running their
    critical sections, the failure and its site are recorded, and the context
    keeps working."""
    torch = pytest.importorskip("torch")
    nsm, G = 4, 6
    H, ld = _init_locks(hs, nsm, max_blocks=_max_blocks(G, nsm))
    handle = _handle(H, 4, nsm)
    assert api.ref_api_hold_mutex(handle, ld, nsm) == 0
    marks = torch.zeros(G, dtype=torch.int32, device="cuda")
    api.ref_api_status(np.zeros(2, dtype=np.uint32).ctypes.data, 1)
    assert api.ref_api_lock_marks(handle, ld, marks.data_ptr(), G, nsm) == 0  # the launch completes
    st = np.zeros(2, dtype=np.uint32)
    api.ref_api_status(st.ctypes.data, 1)
    assert st[0] & 1 and st[1] == 1, st          # HS_DEV_TIMEOUT at HS_SITE_SPIN_LOCK
    assert int(marks.sum().item()) == 0          # no critical section ran without the lock
    # the context still runs work: a fresh lock state and a full faMutex run
    test_reference_api_matches_golden(hs, api, 7, 64, 5, 8, 4, 4)


def test_lock_data_sizes_with_no_room_are_refused(hs):
    """The reference's stride formula rounds down to 0 for 8 blocks on 4 SMs:
    cudaLocksInit refuses instead of handing out a zero-byte barrier buffer."""
    H = _host_api(hs)
    assert H.cudaLocksInit(8, 32, 96, False, 4) == 1  # cudaErrorInvalidValue
    assert H.cudaLocksInit(12, 32, 96, False, 4) == 0  # stride 16

