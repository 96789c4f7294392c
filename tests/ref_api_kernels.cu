// Test kernels written against the reference's device API (include/hs/hs_device_ref.cuh):
// the drop-in check that a program using heterosync's cudaLocks*.cu device
// functions, with the reference's lock-state arrays and index math, runs on
// this build's primitives and leaves the storage the reference's golden
// predicts.  Built by tests/test_ref_api_gpu.py (nvcc -shared) into a
// temporary directory; test code only.
//
// Index math per kernel family (heterosync cuda/syncPrims/uvm/main.cu):
//   mutexes (104-529)      global: every TB works on chunk 0 (tid = threadIdx.x);
//                          Uniq: chunk smID = blockIdx % NUM_SM
//   semaphores (533-836)   numSM = min(gridDim, NUM_SM); perSM_blockID =
//                          blockIdx / numSM; writer iff perSM_blockID ==
//                          smID % numTBs_perSM; writers shift every chunk their
//                          SM's TBs read, readers only load
//   tree barriers (104-315) chunk = current block ID, rotated by 1 each
//                          episode; LocalExch also works on the chunk
//                          numBlocksAtBarr ahead after a local barrier
// One difference: maxSemCount is read from word 3 of the semaphore (the
// initial count + 1, never written), not from the live count in word 0 as
// main.cu:542-543 does -- a CTA starting after a writer has taken the
// semaphore would read 0 there and wait forever.
#include <cuda_runtime.h>
#include <cstdint>

#define HS_REF_TIMEOUT_NS 2000000000ull  // 2 s without progress ends the CTA (the timeout test uses this)
#include "hs/hs_device_ref.cuh"
#include "hs/hs.h"

namespace {

constexpr int kWordsPerLine = 16;  // the reference's NUM_WORDS_PER_CACHELINE

// One critical section: the region of half-warp (tid / 16) shifts up by one line.
__device__ void shift_region(float* storage, int tid, int L) {
  const int base = (tid / kWordsPerLine) * (L + 1);
  const int off = threadIdx.x % kWordsPerLine;
  for (int n = L - 1; n >= 0; --n)
    storage[(base + n + 1) * kWordsPerLine + off] = storage[(base + n) * kWordsPerLine + off];
}

// A semaphore reader's loads (kept in shared memory so they are not elided).
__device__ void read_region(const float* storage, int tid, int L, volatile float* sink) {
  const int base = (tid / kWordsPerLine) * (L + 1);
  const int off = threadIdx.x % kWordsPerLine;
  for (int n = L - 1; n >= 0; --n) {
    sink[threadIdx.x] += storage[(base + n) * kWordsPerLine + off];
    __syncthreads();
  }
}

// kind: 0 spin, 1 EBO, 2 sleep (ring), 3 fetch-and-add
template <int KIND, bool UNIQ>
__global__ void k_api_mutex(cudaMutex_t mutex, float* storage, hs_lock_data* gpuLockData, int iters, int L,
                            int NUM_SM) {
  const int smID = blockIdx.x % NUM_SM;
  const int tid = UNIQ ? smID * blockDim.x + threadIdx.x : threadIdx.x;
  for (int i = 0; i < iters; ++i) {
    unsigned slot = 0;
    if (KIND == 0) {
      if (UNIQ) cudaMutexSpinLockLocal(mutex, smID, gpuLockData->mutexBufferHeads, NUM_SM);
      else cudaMutexSpinLock(mutex, gpuLockData->mutexBufferHeads, NUM_SM);
    } else if (KIND == 1) {
      if (UNIQ) cudaMutexEBOLockLocal(mutex, smID, gpuLockData->mutexBufferHeads, NUM_SM);
      else cudaMutexEBOLock(mutex, gpuLockData->mutexBufferHeads, NUM_SM);
    } else if (KIND == 2) {
      slot = UNIQ ? cudaMutexSleepLockLocal(mutex, smID, gpuLockData->mutexBuffers, gpuLockData->mutexBufferTails,
                                            gpuLockData->maxBufferSize, gpuLockData->arrayStride, NUM_SM)
                  : cudaMutexSleepLock(mutex, gpuLockData->mutexBuffers, gpuLockData->mutexBufferTails,
                                       gpuLockData->maxBufferSize, gpuLockData->arrayStride, NUM_SM);
    } else {
      if (UNIQ)
        cudaMutexFALockLocal(mutex, smID, gpuLockData->mutexBufferHeads, gpuLockData->mutexBufferTails, NUM_SM);
      else cudaMutexFALock(mutex, gpuLockData->mutexBufferHeads, gpuLockData->mutexBufferTails, NUM_SM);
    }
    shift_region(storage, tid, L);
    if (KIND == 0) {
      if (UNIQ) cudaMutexSpinUnlockLocal(mutex, smID, gpuLockData->mutexBufferHeads, NUM_SM);
      else cudaMutexSpinUnlock(mutex, gpuLockData->mutexBufferHeads, NUM_SM);
    } else if (KIND == 1) {
      if (UNIQ) cudaMutexEBOUnlockLocal(mutex, smID, gpuLockData->mutexBufferHeads, NUM_SM);
      else cudaMutexEBOUnlock(mutex, gpuLockData->mutexBufferHeads, NUM_SM);
    } else if (KIND == 2) {
      if (UNIQ)
        cudaMutexSleepUnlockLocal(mutex, smID, gpuLockData->mutexBuffers, slot, gpuLockData->maxBufferSize,
                                  gpuLockData->arrayStride, NUM_SM);
      else cudaMutexSleepUnlock(mutex, gpuLockData->mutexBuffers, slot, gpuLockData->maxBufferSize,
                                gpuLockData->arrayStride, NUM_SM);
    } else {
      if (UNIQ) cudaMutexFAUnlockLocal(mutex, smID, gpuLockData->mutexBufferTails, NUM_SM);
      else cudaMutexFAUnlock(mutex, gpuLockData->mutexBufferTails, NUM_SM);
    }
  }
}

template <bool EBO, bool UNIQ>
__global__ void k_api_sem(cudaSemaphore_t sem, float* storage, hs_lock_data* gpuLockData, int iters, int L,
                          int NUM_SM) {
  __shared__ volatile float sink[1024];
  const unsigned maxSemCount = gpuLockData->semaphoreBuffers[sem * 4 * NUM_SM + 3];
  const int numSM = (int)gridDim.x < NUM_SM ? (int)gridDim.x : NUM_SM;
  const int smID = blockIdx.x % (UNIQ ? numSM : NUM_SM);
  const int perTB = (gridDim.x + numSM - 1) / numSM;
  const int rank = blockIdx.x / numSM;
  const bool isWriter = rank == smID % perTB;
  sink[threadIdx.x] = 0.f;
  for (int i = 0; i < iters; ++i) {
    if (UNIQ) {
      if (EBO) cudaSemaphoreEBOWaitLocal(sem, smID, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
      else cudaSemaphoreSpinWaitLocal(sem, smID, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
    } else {
      if (EBO) cudaSemaphoreEBOWait(sem, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
      else cudaSemaphoreSpinWait(sem, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
    }
    if (isWriter) {
      int block = blockIdx.x;
      for (int j = 0; j < perTB; ++j) {  // every chunk the TBs of this SM read
        shift_region(storage, (UNIQ ? block : j) * blockDim.x + threadIdx.x, L);
        block = (block + numSM) % gridDim.x;
      }
    } else {
      read_region(storage, (UNIQ ? blockIdx.x : rank) * blockDim.x + threadIdx.x, L, sink);
    }
    if (UNIQ) {
      if (EBO) cudaSemaphoreEBOPostLocal(sem, smID, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
      else cudaSemaphoreSpinPostLocal(sem, smID, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
    } else {
      if (EBO) cudaSemaphoreEBOPost(sem, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
      else cudaSemaphoreSpinPost(sem, isWriter, maxSemCount, gpuLockData->semaphoreBuffers, NUM_SM);
    }
  }
}

template <bool LF, bool EXCH>
__global__ void k_api_barrier(float* storage, hs_lock_data* gpuLockData, unsigned* perSMBarrierBuffers, int iters,
                              int L, int NUM_SM, int MAX_BLOCKS) {
  const bool isMasterThread = threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0;
  const unsigned numBlocksAtBarr = gridDim.x < (unsigned)NUM_SM ? gridDim.x : (unsigned)NUM_SM;
  const int smID = blockIdx.x % numBlocksAtBarr;
  const int perSM_blockID = blockIdx.x / numBlocksAtBarr;
  const int numTBs_perSM = (gridDim.x + numBlocksAtBarr - 1) / numBlocksAtBarr;
  int block = blockIdx.x;
  for (int i = 0; i < iters; ++i) {
    shift_region(storage, block * blockDim.x + threadIdx.x, L);
    if (EXCH && numTBs_perSM > 1) {
      if (LF)
        cudaBarrierLocal(gpuLockData->barrierBuffers, numBlocksAtBarr, gpuLockData->arrayStride, perSMBarrierBuffers,
                         smID, numTBs_perSM, perSM_blockID, false, MAX_BLOCKS);
      else
        cudaBarrierAtomicLocal(perSMBarrierBuffers, smID, numTBs_perSM, isMasterThread, MAX_BLOCKS);
      block = (block + numBlocksAtBarr) % gridDim.x;
      shift_region(storage, block * blockDim.x + threadIdx.x, L);
    }
    if (LF)
      joinLFBarrier_helper(gpuLockData->barrierBuffers, perSMBarrierBuffers, numBlocksAtBarr, smID, perSM_blockID,
                           numTBs_perSM, gpuLockData->arrayStride, MAX_BLOCKS);
    else
      joinBarrier_helper(gpuLockData->barrierBuffers, perSMBarrierBuffers, numBlocksAtBarr, smID, perSM_blockID,
                         numTBs_perSM, isMasterThread, MAX_BLOCKS);
    block = (block + 1) % gridDim.x;
  }
}

// The timeout check: thread 0 of every TB marks its slot after the lock, so a
// slot left 0 shows a critical section that did not run.
__global__ void k_api_lock_marks(cudaMutex_t mutex, hs_lock_data* gpuLockData, unsigned* marks, int NUM_SM) {
  cudaMutexSpinLock(mutex, gpuLockData->mutexBufferHeads, NUM_SM);
  if (threadIdx.x == 0) marks[blockIdx.x] = 1u;
  cudaMutexSpinUnlock(mutex, gpuLockData->mutexBufferHeads, NUM_SM);
}

template <class K, class... A>
int launch(K k, int grid, int threads, A... a) {
  k<<<grid, threads>>>(a...);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}

}  // namespace

// Run reference syncPrim `prim` (ids 0-15, 20-31) with `handle` (the mutex or
// semaphore number) on `storage`; returns a cudaError_t value.
extern "C" int ref_api_run(int prim, unsigned handle, float* storage, hs_lock_data* ld, unsigned* perSM, int T, int L,
                           int G, int iters, int nsm, int max_blocks) {
  switch (prim) {
    case 0: return launch(k_api_barrier<false, false>, G, T, storage, ld, perSM, iters, L, nsm, max_blocks);
    case 1: return launch(k_api_barrier<false, true>, G, T, storage, ld, perSM, iters, L, nsm, max_blocks);
    case 2: return launch(k_api_barrier<true, false>, G, T, storage, ld, perSM, iters, L, nsm, max_blocks);
    case 3: return launch(k_api_barrier<true, true>, G, T, storage, ld, perSM, iters, L, nsm, max_blocks);
    case 4: return launch(k_api_mutex<0, false>, G, T, handle, storage, ld, iters, L, nsm);
    case 5: return launch(k_api_mutex<1, false>, G, T, handle, storage, ld, iters, L, nsm);
    case 6: return launch(k_api_mutex<2, false>, G, T, handle, storage, ld, iters, L, nsm);
    case 7: return launch(k_api_mutex<3, false>, G, T, handle, storage, ld, iters, L, nsm);
    case 20: return launch(k_api_mutex<0, true>, G, T, handle, storage, ld, iters, L, nsm);
    case 21: return launch(k_api_mutex<1, true>, G, T, handle, storage, ld, iters, L, nsm);
    case 22: return launch(k_api_mutex<2, true>, G, T, handle, storage, ld, iters, L, nsm);
    case 23: return launch(k_api_mutex<3, true>, G, T, handle, storage, ld, iters, L, nsm);
    default: break;
  }
  if (prim >= 8 && prim <= 11) return launch(k_api_sem<false, false>, G, T, handle, storage, ld, iters, L, nsm);
  if (prim >= 12 && prim <= 15) return launch(k_api_sem<true, false>, G, T, handle, storage, ld, iters, L, nsm);
  if (prim >= 24 && prim <= 27) return launch(k_api_sem<false, true>, G, T, handle, storage, ld, iters, L, nsm);
  if (prim >= 28 && prim <= 31) return launch(k_api_sem<true, true>, G, T, handle, storage, ld, iters, L, nsm);
  return (int)cudaErrorInvalidValue;
}

// G TBs take spin mutex `handle` once each and mark their slot in `marks`.
extern "C" int ref_api_lock_marks(unsigned handle, hs_lock_data* ld, unsigned* marks, int G, int nsm) {
  return launch(k_api_lock_marks, G, 64, handle, ld, marks, nsm);
}

// Take spin mutex `handle` from the host (its word set to 1), so that no TB's
// lock wait can end: the timeout test.
extern "C" int ref_api_hold_mutex(unsigned handle, hs_lock_data* ld, int nsm) {
  const unsigned one = 1u;
  return (int)cudaMemcpy(ld->mutexBufferHeads + handle * nsm, &one, sizeof(one), cudaMemcpyHostToDevice);
}

// The failure record of the reference-signature API in this file: reset, read.
extern "C" int ref_api_status(unsigned* out2, int reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out2, hs_ref_wait_status, sizeof(unsigned) * 2);
  if (e == cudaSuccess && reset) {
    const unsigned z[2] = {0u, 0u};
    e = cudaMemcpyToSymbol(hs_ref_wait_status, z, sizeof(z));
  }
  return (int)e;
}
