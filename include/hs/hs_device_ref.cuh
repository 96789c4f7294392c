// hs_device_ref.cuh -- the reference's device API, same names and parameters,
// implemented on the sm_103a primitives of hs_device.cuh.
//
// A kernel written against heterosync's cuda/syncPrims/uvm/cudaLocks*.cu device
// functions compiles unchanged against this header.  The lock-state arrays are
// the ones the caller passes (the fields of the cudaLockData_t returned by
// cudaLocksInit in hs.h), indexed exactly as the reference indexes them:
//   mutex m (global)       heads/tails[m * NUM_SM]
//   mutex m, SM s (Local)  heads/tails[m * NUM_SM + s]
//   ring of mutex m        mutexBuffers[(m * NUM_SM (+ s)) * arrayStride ...]
//   semaphore s, SM id     semaphoreBuffers[s * 4 * NUM_SM + id * 4 + {0..3}]
//   global barrier         barrierBuffers[0..2*arrayStride)
//   per-SM barrier         perSMBarrierBuffers[smID * MAX_BLOCKS * 2 ...]
//
// Differences that do not change results:
//  * waits are bounded and fail fast: a wait that sees no progress for
//    HS_REF_TIMEOUT_NS records the failure in hs_ref_wait_status (per
//    translation unit: word 0 the error bits, word 1 the wait site) and ends
//    the calling CTA -- every thread of the CTA executes PTX `exit` at the same
//    point, so no critical section runs without its lock and no thread is left
//    at a CTA barrier.  CTAs waiting on an ended one see the recorded status at
//    their next poll and end the same way, so the launch completes and the
//    context stays usable; the host reads the status after the launch
//    (cudaMemcpyFromSymbol of hs_ref_wait_status in the including file).  The
//    reference's functions have no error path (they spin forever instead);
//    TryWait still returns false without ending anything;
//  * the semaphore keeps its reader/writer admission rules but packs the
//    writer-waiting flag into bit 31 of word 0 (count), so wait and post are a
//    CAS and a red instead of a lock round trip (word 1, the reference's CAS
//    lock, and word 2 are unused; word 3 still holds the initial count+1);
//  * the barriers use generation-valued words instead of resetting counters
//    and flags.
#pragma once
#include "hs_device.cuh"

#ifndef HS_REF_MAX_BACKOFF
#define HS_REF_MAX_BACKOFF 1024u  // reference main.cu:7 (MAX_BACKOFF)
#endif
#ifndef HS_REF_TIMEOUT_NS
#define HS_REF_TIMEOUT_NS 10000000000ull
#endif

typedef unsigned int cudaMutex_t;      // reference cudaLocks.h:18
typedef unsigned int cudaSemaphore_t;  // reference cudaLocks.h:19

// Failure record for the reference-signature API (no error path exists there).
static __device__ unsigned hs_ref_wait_status[2];

__device__ __forceinline__ hs::HsEnv hs_ref_env() {
  return hs::HsEnv{hs_ref_wait_status, HS_REF_TIMEOUT_NS};
}
__device__ __forceinline__ bool hs_ref_failed() {
  return hs::ld_relaxed<hs::GPU>(hs_ref_wait_status) != 0u;
}
// End the calling CTA when a block-collective wait failed (ok is the same in
// every thread of the CTA).
__device__ __forceinline__ void hs_ref_end_if(bool failed) {
  if (failed) asm volatile("exit;" ::: "memory");
}

// --- spin mutex: cudaLocksMutexSpin.cu:13,38,53,81 --------------------------
__device__ __forceinline__ void cudaMutexSpinLock(const cudaMutex_t mutex, unsigned int* mutexBufferHeads,
                                                  const int NUM_SM) {
  hs_ref_end_if(!hs::spin_lock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM, hs_ref_env()));
}
__device__ __forceinline__ void cudaMutexSpinUnlock(const cudaMutex_t mutex, unsigned int* mutexBufferHeads,
                                                    const int NUM_SM) {
  hs::spin_unlock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM);
  __syncthreads();
}
__device__ __forceinline__ void cudaMutexSpinLockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                       unsigned int* mutexBufferHeads, const int NUM_SM) {
  hs_ref_end_if(!hs::spin_lock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM + smID, hs_ref_env()));
}
__device__ __forceinline__ void cudaMutexSpinUnlockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                         unsigned int* mutexBufferHeads, const int NUM_SM) {
  hs::spin_unlock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM + smID);
  __syncthreads();
}

// --- EBO mutex: cudaLocksMutexEBO.cu:13,59,73,121 ---------------------------
__device__ __forceinline__ void cudaMutexEBOLock(const cudaMutex_t mutex, unsigned int* mutexBufferHeads,
                                                 const int NUM_SM) {
  hs_ref_end_if(!hs::ebo_lock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM, 1u, HS_REF_MAX_BACKOFF, hs_ref_env()));
}
__device__ __forceinline__ void cudaMutexEBOUnlock(const cudaMutex_t mutex, unsigned int* mutexBufferHeads,
                                                   const int NUM_SM) {
  hs::spin_unlock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM);
  __syncthreads();
}
__device__ __forceinline__ void cudaMutexEBOLockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                      unsigned int* mutexBufferHeads, const int NUM_SM) {
  hs_ref_end_if(
      !hs::ebo_lock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM + smID, 1u, HS_REF_MAX_BACKOFF, hs_ref_env()));
}
__device__ __forceinline__ void cudaMutexEBOUnlockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                        unsigned int* mutexBufferHeads, const int NUM_SM) {
  hs::spin_unlock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM + smID);
  __syncthreads();
}

// --- fetch-and-add mutex: cudaLocksMutexFA.cu:13,53,72,115 ------------------
__device__ __forceinline__ void cudaMutexFALock(const cudaMutex_t mutex, unsigned int* mutexBufferHeads,
                                                unsigned int* mutexBufferTails, const int NUM_SM) {
  hs_ref_end_if(!hs::ticket_lock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM, mutexBufferTails + mutex * NUM_SM,
                                          1000000000u, 0u, 0u, hs_ref_env()));
}
__device__ __forceinline__ void cudaMutexFAUnlock(const cudaMutex_t mutex, unsigned int* mutexBufferTails,
                                                  const int NUM_SM) {
  hs::ticket_unlock<hs::GPU>(mutexBufferTails + mutex * NUM_SM, 1000000000u);
  __syncthreads();
}
__device__ __forceinline__ void cudaMutexFALockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                     unsigned int* mutexBufferHeads, unsigned int* mutexBufferTails,
                                                     const int NUM_SM) {
  hs_ref_end_if(!hs::ticket_lock<hs::GPU>(mutexBufferHeads + mutex * NUM_SM + smID,
                                          mutexBufferTails + mutex * NUM_SM + smID, 100000000u, 0u, 0u, hs_ref_env()));
}
__device__ __forceinline__ void cudaMutexFAUnlockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                       unsigned int* mutexBufferTails, const int NUM_SM) {
  hs::ticket_unlock<hs::GPU>(mutexBufferTails + mutex * NUM_SM + smID, 100000000u);
  __syncthreads();
}

// --- sleep (ring buffer) mutex: cudaLocksMutexSleep.cu:20,79,111,168 --------
__device__ __forceinline__ unsigned int cudaMutexSleepLock(const cudaMutex_t mutex, int* mutexBuffers,
                                                           unsigned int* mutexBufferTails, const int maxRingBufferSize,
                                                           const int arrayStride, const int NUM_SM) {
  __shared__ int s_slot;
  unsigned* ring = reinterpret_cast<unsigned*>(mutexBuffers) + (size_t)(mutex * NUM_SM) * arrayStride;
  int r = hs::queue_lock<hs::GPU>(mutexBufferTails + mutex * NUM_SM, ring, 1u, (unsigned)maxRingBufferSize, 0u,
                                  hs_ref_env(), &s_slot);
  hs_ref_end_if(r < 0);
  return (unsigned)r;
}
__device__ __forceinline__ void cudaMutexSleepUnlock(const cudaMutex_t mutex, int* mutexBuffers,
                                                     unsigned int myBufferLoc, const int maxRingBufferSize,
                                                     const int arrayStride, const int NUM_SM) {
  unsigned* ring = reinterpret_cast<unsigned*>(mutexBuffers) + (size_t)(mutex * NUM_SM) * arrayStride;
  hs::queue_unlock<hs::GPU>(ring, 1u, (unsigned)maxRingBufferSize, myBufferLoc);
  __syncthreads();
}
__device__ __forceinline__ unsigned int cudaMutexSleepLockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                                int* mutexBuffers, unsigned int* mutexBufferTails,
                                                                const int maxRingBufferSize, const int arrayStride,
                                                                const int NUM_SM) {
  __shared__ int s_slot;
  unsigned* ring = reinterpret_cast<unsigned*>(mutexBuffers) + (size_t)(mutex * NUM_SM + smID) * arrayStride;
  int r = hs::queue_lock<hs::GPU>(mutexBufferTails + mutex * NUM_SM + smID, ring, 1u, (unsigned)maxRingBufferSize,
                                  0u, hs_ref_env(), &s_slot);
  hs_ref_end_if(r < 0);
  return (unsigned)r;
}
__device__ __forceinline__ void cudaMutexSleepUnlockLocal(const cudaMutex_t mutex, const unsigned int smID,
                                                          int* mutexBuffers, unsigned int myBufferLoc,
                                                          const int maxRingBufferSize, const int arrayStride,
                                                          const int NUM_SM) {
  unsigned* ring = reinterpret_cast<unsigned*>(mutexBuffers) + (size_t)(mutex * NUM_SM + smID) * arrayStride;
  hs::queue_unlock<hs::GPU>(ring, 1u, (unsigned)maxRingBufferSize, myBufferLoc);
  __syncthreads();
}

// --- semaphores: cudaLocksSemaphoreSpin.cu:25,139,151,216,332,345 and
//     cudaLocksSemaphoreEBO.cu:23,139,185,244,363,402 ------------------------
__device__ __forceinline__ unsigned* hs_ref_sem_word(cudaSemaphore_t sem, unsigned smID, unsigned* buf, int NUM_SM) {
  return buf + (size_t)sem * 4 * NUM_SM + smID * 4;
}
__device__ __forceinline__ bool cudaSemaphoreSpinTryWait(const cudaSemaphore_t sem, const bool isWriter,
                                                         const unsigned int maxSemCount, unsigned int* semaphoreBuffers,
                                                         const int NUM_SM) {
  int ok = 0;
  if (hs::is_master()) ok = hs::sem_try_once<hs::GPU>(hs_ref_sem_word(sem, 0, semaphoreBuffers, NUM_SM), isWriter,
                                                      maxSemCount);
  return __syncthreads_or(ok) != 0;
}
__device__ __forceinline__ void cudaSemaphoreSpinWait(const cudaSemaphore_t sem, const bool isWriter,
                                                      const unsigned int maxSemCount, unsigned int* semaphoreBuffers,
                                                      const int NUM_SM) {
  hs_ref_end_if(!hs::sem_wait<hs::GPU>(hs_ref_sem_word(sem, 0, semaphoreBuffers, NUM_SM), isWriter, maxSemCount,
                                       false, false, 0u, 0u, hs_ref_env()));
}
__device__ __forceinline__ void cudaSemaphoreSpinPost(const cudaSemaphore_t sem, const bool isWriter,
                                                      const unsigned int maxSemCount, unsigned int* semaphoreBuffers,
                                                      const int NUM_SM) {
  hs::sem_post<hs::GPU>(hs_ref_sem_word(sem, 0, semaphoreBuffers, NUM_SM), isWriter, maxSemCount);
  __syncthreads();
}
__device__ __forceinline__ bool cudaSemaphoreSpinTryWaitLocal(const cudaSemaphore_t sem, const unsigned int smID,
                                                              const bool isWriter, const unsigned int maxSemCount,
                                                              unsigned int* semaphoreBuffers, const int NUM_SM) {
  int ok = 0;
  if (hs::is_master()) ok = hs::sem_try_once<hs::GPU>(hs_ref_sem_word(sem, smID, semaphoreBuffers, NUM_SM), isWriter,
                                                      maxSemCount);
  return __syncthreads_or(ok) != 0;
}
__device__ __forceinline__ void cudaSemaphoreSpinWaitLocal(const cudaSemaphore_t sem, const unsigned int smID,
                                                           const bool isWriter, const unsigned int maxSemCount,
                                                           unsigned int* semaphoreBuffers, const int NUM_SM) {
  hs_ref_end_if(!hs::sem_wait<hs::GPU>(hs_ref_sem_word(sem, smID, semaphoreBuffers, NUM_SM), isWriter, maxSemCount,
                                       false, false, 0u, 0u, hs_ref_env()));
}
__device__ __forceinline__ void cudaSemaphoreSpinPostLocal(const cudaSemaphore_t sem, const unsigned int smID,
                                                           const bool isWriter, const unsigned int maxSemCount,
                                                           unsigned int* semaphoreBuffers, const int NUM_SM) {
  hs::sem_post<hs::GPU>(hs_ref_sem_word(sem, smID, semaphoreBuffers, NUM_SM), isWriter, maxSemCount);
  __syncthreads();
}
__device__ __forceinline__ bool cudaSemaphoreEBOTryWait(const cudaSemaphore_t sem, const bool isWriter,
                                                        const unsigned int maxSemCount, unsigned int* semaphoreBuffers,
                                                        const int NUM_SM) {
  return cudaSemaphoreSpinTryWait(sem, isWriter, maxSemCount, semaphoreBuffers, NUM_SM);
}
__device__ __forceinline__ void cudaSemaphoreEBOWait(const cudaSemaphore_t sem, const bool isWriter,
                                                     const unsigned int maxSemCount, unsigned int* semaphoreBuffers,
                                                     const int NUM_SM) {
  hs_ref_end_if(!hs::sem_wait<hs::GPU>(hs_ref_sem_word(sem, 0, semaphoreBuffers, NUM_SM), isWriter, maxSemCount,
                                       true, true, 1u, HS_REF_MAX_BACKOFF, hs_ref_env()));
}
__device__ __forceinline__ void cudaSemaphoreEBOPost(const cudaSemaphore_t sem, const bool isWriter,
                                                     const unsigned int maxSemCount, unsigned int* semaphoreBuffers,
                                                     const int NUM_SM) {
  cudaSemaphoreSpinPost(sem, isWriter, maxSemCount, semaphoreBuffers, NUM_SM);
}
__device__ __forceinline__ bool cudaSemaphoreEBOTryWaitLocal(const cudaSemaphore_t sem, const unsigned int smID,
                                                             const bool isWriter, const unsigned int maxSemCount,
                                                             unsigned int* semaphoreBuffers, const int NUM_SM) {
  return cudaSemaphoreSpinTryWaitLocal(sem, smID, isWriter, maxSemCount, semaphoreBuffers, NUM_SM);
}
__device__ __forceinline__ void cudaSemaphoreEBOWaitLocal(const cudaSemaphore_t sem, const unsigned int smID,
                                                          const bool isWriter, const unsigned int maxSemCount,
                                                          unsigned int* semaphoreBuffers, const int NUM_SM) {
  hs_ref_end_if(!hs::sem_wait<hs::GPU>(hs_ref_sem_word(sem, smID, semaphoreBuffers, NUM_SM), isWriter, maxSemCount,
                                       true, false, 1u, HS_REF_MAX_BACKOFF, hs_ref_env()));
}
__device__ __forceinline__ void cudaSemaphoreEBOPostLocal(const cudaSemaphore_t sem, const unsigned int smID,
                                                          const bool isWriter, const unsigned int maxSemCount,
                                                          unsigned int* semaphoreBuffers, const int NUM_SM) {
  cudaSemaphoreSpinPostLocal(sem, smID, isWriter, maxSemCount, semaphoreBuffers, NUM_SM);
}

// --- atomic tree barrier: cudaLocksBarrierAtomic.cu:67,127,147 --------------
// barrierBuffers[0] = arrival counter, barrierBuffers[1] = generation.
// The per-SM group uses perSM[smID*MAX_BLOCKS + {0,1}] the same way.
__device__ __forceinline__ void hs_ref_counter_barrier(unsigned* cnt, unsigned n, const bool isMasterThread) {
  __syncthreads();
  bool ok = true;
  if (isMasterThread) {
    hs::HsEnv env = hs_ref_env();
    const unsigned gen = hs::ld_relaxed<hs::GPU>(cnt + 1);
    hs::counter_barrier<hs::GPU>(cnt, cnt + 1, n, gen, 0u, env, hs::HS_SITE_BAR_GLOBAL, [] { return true; }, &ok);
  }
  hs_ref_end_if(__syncthreads_or(!ok) != 0);
}
__device__ __forceinline__ void cudaBarrierAtomic(unsigned int* barrierBuffers, const unsigned int numBarr,
                                                  const bool isMasterThread) {
  hs_ref_counter_barrier(barrierBuffers, numBarr, isMasterThread);
}
__device__ __forceinline__ void cudaBarrierAtomicLocal(unsigned int* perSMBarrierBuffers, const unsigned int smID,
                                                       const unsigned int numTBs_thisSM, const bool isMasterThread,
                                                       const int MAX_BLOCKS) {
  hs_ref_counter_barrier(perSMBarrierBuffers + (size_t)smID * MAX_BLOCKS, numTBs_thisSM, isMasterThread);
}
__device__ __forceinline__ void joinBarrier_helper(unsigned int* barrierBuffers, unsigned int* perSMBarrierBuffers,
                                                   const unsigned int numBlocksAtBarr, const int smID,
                                                   const int perSM_blockID, const int numTBs_perSM,
                                                   const bool isMasterThread, const int MAX_BLOCKS) {
  if (numTBs_perSM > 1) {
    cudaBarrierAtomicLocal(perSMBarrierBuffers, smID, numTBs_perSM, isMasterThread, MAX_BLOCKS);
    if (perSM_blockID == 0) cudaBarrierAtomic(barrierBuffers, numBlocksAtBarr, isMasterThread);
    cudaBarrierAtomicLocal(perSMBarrierBuffers, smID, numTBs_perSM, isMasterThread, MAX_BLOCKS);
  } else {
    cudaBarrierAtomic(barrierBuffers, numBlocksAtBarr, isMasterThread);
  }
}

// --- lock-free barrier: cudaLocksBarrierFast.cu:182,226,295,315 -------------
// inVars[b] / outVars hold generations; outVars[0] is the release word.
__device__ __forceinline__ void hs_ref_flag_barrier(unsigned* inVars, unsigned* outVars, unsigned numBlocks,
                                                    unsigned myIdx, bool isMain) {
  hs::HsEnv env = hs_ref_env();
  __shared__ unsigned s_gen;
  __syncthreads();
  if (hs::is_master()) {
    s_gen = hs::ld_relaxed<hs::GPU>(outVars) + 1u;
    hs::st_release<hs::GPU>(inVars + myIdx, s_gen);
  }
  __syncthreads();
  const unsigned e = s_gen;
  bool ok = true;
  if (isMain) {
    ok = hs::scan_flags<hs::GPU>(inVars, numBlocks, e, 0u, env, hs::HS_SITE_BAR_SCAN);
    if (ok && hs::is_master()) hs::st_release<hs::GPU>(outVars, e);
  } else if (hs::is_master()) {
    ok = hs::wait_until([&] { return (int)(hs::ld_acquire<hs::GPU>(outVars) - e) >= 0; }, [] {}, env,
                        hs::HS_SITE_BAR_GO);
  }
  hs_ref_end_if(__syncthreads_or(!ok) != 0);
}
__device__ __forceinline__ void cudaBarrier(unsigned int* barrierBuffers, const int arrayStride,
                                            const unsigned int numBlocksAtBarr) {
  hs_ref_flag_barrier(barrierBuffers, barrierBuffers + arrayStride, numBlocksAtBarr, blockIdx.x, blockIdx.x == 0);
}
__device__ __forceinline__ void cudaBarrierLocal(unsigned int* barrierBuffers, const unsigned int numBlocksAtBarr,
                                                 const int arrayStride, unsigned int* perSMBarrierBuffers,
                                                 const unsigned int smID, const unsigned int numTBs_perSM,
                                                 const unsigned int perSM_blockID, const bool isLocalGlobalBarr,
                                                 const int MAX_BLOCKS) {
  unsigned* inVars = perSMBarrierBuffers + (size_t)MAX_BLOCKS * smID * 2;
  unsigned* outVars = inVars + MAX_BLOCKS;
  if (isLocalGlobalBarr) {
    // local arrival, then the main TB of this SM joins the global barrier, then local release
    hs::HsEnv env = hs_ref_env();
    __shared__ unsigned s_gen;
    __syncthreads();
    if (hs::is_master()) {
      s_gen = hs::ld_relaxed<hs::GPU>(outVars) + 1u;
      hs::st_release<hs::GPU>(inVars + perSM_blockID, s_gen);
    }
    __syncthreads();
    const unsigned e = s_gen;
    bool ok = true;
    if (perSM_blockID == 0) {
      hs_ref_end_if(!hs::scan_flags<hs::GPU>(inVars, numTBs_perSM, e, 0u, env, hs::HS_SITE_BAR_SCAN));
      cudaBarrier(barrierBuffers, arrayStride, numBlocksAtBarr);
      if (hs::is_master()) hs::st_release<hs::GPU>(outVars, e);
    } else if (hs::is_master()) {
      ok = hs::wait_until([&] { return (int)(hs::ld_acquire<hs::GPU>(outVars) - e) >= 0; }, [] {}, env,
                          hs::HS_SITE_BAR_GO);
    }
    hs_ref_end_if(__syncthreads_or(!ok) != 0);
  } else {
    hs_ref_flag_barrier(inVars, outVars, numTBs_perSM, perSM_blockID, perSM_blockID == 0);
  }
}
__device__ __forceinline__ void cudaBarrierLocalGlobal(unsigned int* barrierBuffers, const unsigned int numBlocksAtBarr,
                                                       const int arrayStride, unsigned int* perSMBarrierBuffers,
                                                       const unsigned int smID, const unsigned int numTBs_perSM,
                                                       const unsigned int perSM_blockID, const int MAX_BLOCKS) {
  cudaBarrierLocal(barrierBuffers, numBlocksAtBarr, arrayStride, perSMBarrierBuffers, smID, numTBs_perSM,
                   perSM_blockID, true, MAX_BLOCKS);
}
__device__ __forceinline__ void joinLFBarrier_helper(unsigned int* barrierBuffers, unsigned int* perSMBarrierBuffers,
                                                     const unsigned int numBlocksAtBarr, const int smID,
                                                     const int perSM_blockID, const int numTBs_perSM,
                                                     const int arrayStride, const int MAX_BLOCKS) {
  if (numTBs_perSM > 1)
    cudaBarrierLocalGlobal(barrierBuffers, numBlocksAtBarr, arrayStride, perSMBarrierBuffers, smID, numTBs_perSM,
                           perSM_blockID, MAX_BLOCKS);
  else
    cudaBarrier(barrierBuffers, arrayStride, numBlocksAtBarr);
}
