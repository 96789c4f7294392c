// hs_relaxed.cu -- the relaxed-atomics microbenchmarks (heterosync
// cuda/relaxedAtomics/uvm/{refCounter,splitCounter,seqlocks,flags}) for sm_103a.
//
// Each kernel keeps the reference's work per thread and its observable results
// (final counters, sequence numbers, output arrays) and maps the accesses onto
// scoped PTX: relaxed red/atom where the reference's atomic needs no ordering,
// ld.relaxed instead of atomicAdd(x, 0) for atomic loads, acquire/release
// instead of atomic + __threadfence.  Three reference constructs that are
// undefined behaviour on independent-thread-scheduling GPUs are replaced:
//  * splitCounter's reader reduction calls __syncthreads from half-warps
//    (splitCounter_kernel.cu:50-72, called from a divergent branch at 93-100):
//    here each reader half-warp reduces with shuffles;
//  * seqlocks' readers/writers keep seq0/seq1 in per-thread registers that only
//    thread 0 sets, then loop on them (seqlocks_kernel.cu:60-84, 148-173): here
//    thread 0's values are broadcast through shared memory;
//  * flags' workers index randArr past its end (flags_kernel.cu:105,129 vs
//    flags.cu:77): here the index wraps modulo the array length.
// Every wait is bounded (hs_device.cuh).
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/hs/hs_device.cuh"

namespace hs {

// ---------------------------------------------------------------------------
// RefCounter: refCounter_kernel.cu:4-55.  Per repeat: +1 on two shared counters,
// a shared-memory delay of 2*numRepeats barrier steps, then -1 on both
// (atomicDec semantics: wrap at 1e9) with acquire-release ordering; a thread
// whose decrement saw <= 1 marks the object deleted.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_refcounter(unsigned* c0, unsigned* c1, unsigned* del0, unsigned* del1,
                                                   unsigned numRepeats, unsigned numSharingGroups,
                                                   unsigned numCounters_perSharingGroup) {
  __shared__ volatile int dummyLocal[256];
  const unsigned myBaseLoc = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned myCounterLoc = (blockIdx.x % numSharingGroups) * numCounters_perSharingGroup + threadIdx.x;
  unsigned* a0 = c0 + myCounterLoc;
  unsigned* a1 = c1 + myCounterLoc;
  dummyLocal[threadIdx.x] = 0;
  __syncthreads();
  for (unsigned i = 0; i < numRepeats; ++i) {
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(a0) : "memory");
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(a1) : "memory");
    for (unsigned j = 0; j < numRepeats * 2; ++j) {
      dummyLocal[threadIdx.x] += j;
      __syncthreads();
    }
    unsigned o0, o1;
    asm volatile("atom.acq_rel.gpu.global.dec.u32 %0, [%1], 1000000000;" : "=r"(o0) : "l"(a0) : "memory");
    asm volatile("atom.acq_rel.gpu.global.dec.u32 %0, [%1], 1000000000;" : "=r"(o1) : "l"(a1) : "memory");
    if (o0 <= 1u) del0[myBaseLoc] = 1u;
    if (o1 <= 1u) del1[myBaseLoc] = 1u;
  }
}

// ---------------------------------------------------------------------------
// SplitCounter: splitCounter_kernel.cu:10-103.  Lower half-warps add INC_VAL to
// their own counter; upper half-warps read every counter (relaxed atomic loads,
// strided as the reference strides them) and write the approximate sum.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_splitcounter(unsigned* counters, unsigned* outArr) {
  const unsigned numCounters_perTB = blockDim.x >> 1;
  const unsigned warpID = threadIdx.x / 32;
  const unsigned lane = threadIdx.x % 32;
  const unsigned threadID = blockIdx.x * blockDim.x + threadIdx.x;
  if (lane < 16) {
    unsigned* p = counters + blockIdx.x * numCounters_perTB + warpID * 16 + (lane % 16);
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(p) : "memory");
  } else {
    const unsigned numCounters = gridDim.x * numCounters_perTB;
    const unsigned numAccsPerThr = numCounters / (blockDim.x >> 1);
    const unsigned myBaseLoc = numCounters_perTB * blockIdx.x + (numAccsPerThr * 16) * warpID + (lane % 16);
    unsigned cur = myBaseLoc % numCounters;
    unsigned sum = 0;
    for (unsigned i = 0; i < numAccsPerThr; ++i) {
      sum += ld_relaxed<GPU>(counters + cur);
      cur = (cur + numCounters_perTB) % numCounters;
    }
    // half-warp reduction (lanes 16..31), then every reader thread writes the
    // sum its half-warp saw (the reference writes the CTA-wide reduction of the
    // readers' partial sums; see SplitCounter notes in the oracle)
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFF0000u, sum, o);
    outArr[threadID] = sum;
  }
}

// ---------------------------------------------------------------------------
// Seqlocks: seqlocks_kernel.cu:17-232.  1/16 of TBs are writers (blockIdx%16==0):
// thread 0 moves the sequence word even->odd with a CAS (backoff 1,3,..,31),
// all threads write the data words, thread 0 publishes seq+2 with release.
// Readers retry until they saw the same even sequence number before and after
// reading the data.  REF data semantics: destructive reads (atomicExch(..., 0))
// and writes of the sequence number by thread 0 (0 by the other threads, as in
// the reference, whose other threads' seq0 is never set).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_seqlocks(unsigned* seqlock, int* data0, int* data1, int* outArr,
                                                  int groupSize, int iters, unsigned* status,
                                                  unsigned long long timeout_ns) {
  __shared__ unsigned s_seq0, s_seq1;
  const HsEnv env{status, timeout_ns};
  const unsigned threadID = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned dataLoc = threadIdx.x % 32;
  unsigned* sl = seqlock + (blockIdx.x % groupSize);
  const bool writer = (blockIdx.x % 16 == 0);
  for (int it = 0; it < iters; ++it) {
    if (writer) {
      int ok = 0;
      if (is_master()) {
        unsigned s0 = ld_relaxed<GPU>(sl);
        unsigned backoff = 1;
        ok = wait_until_p([&] {
                            if (s0 & 1u) return false;
                            const unsigned o = atom_cas_acquire<GPU>(sl, s0, s0 + 1u);
                            if (o == s0) return true;
                            s0 = o;
                            return false;
                          },
                          [&] { return s0; },
                          [&] {
                            backoff = ((backoff << 1) + 1u) & 31u;
                            sleep_ns(backoff);
                            s0 = ld_relaxed<GPU>(sl);
                          },
                          env, HS_SITE_RELAXED);
        s_seq0 = s0;
      }
      if (!__syncthreads_or(ok)) return;
      const int v = is_master() ? (int)s_seq0 : 0;
      atomicExch(data0 + dataLoc, v);
      atomicExch(data1 + dataLoc, v);
      __syncthreads();
      if (is_master()) st_release<GPU>(sl, s_seq0 + 2u);
    } else {
      int r1 = 0, r2 = 0;
      unsigned polls = 0;
      const unsigned long long t0 = globaltimer();
      for (;;) {
        if (is_master()) s_seq0 = ld_acquire<GPU>(sl);
        __syncthreads();
        r1 = atomicExch(data0 + dataLoc, 0);
        r2 = atomicExch(data1 + dataLoc, 0);
        __threadfence();
        if (is_master()) s_seq1 = ld_relaxed<GPU>(sl);
        __syncthreads();
        const unsigned a = s_seq0, b = s_seq1;
        __syncthreads();
        if (a == b && !(a & 1u)) break;
        if ((++polls & 15u) == 0u) {
          int bad = 0;
          if (is_master()) bad = ld_relaxed<GPU>(status) != 0u || globaltimer() - t0 > timeout_ns;
          if (__syncthreads_or(bad)) {
            if (is_master()) fail(env, HS_DEV_TIMEOUT, HS_SITE_RELAXED);
            return;
          }
        }
      }
      outArr[threadID] = r1 + r2;
    }
  }
}

// ---------------------------------------------------------------------------
// Flags: flags_kernel.cu:13-242.  The last TB is the main TB: it sums in shared
// memory, sets stop, joins a grid barrier and, if dirty, writes its sums.  The
// other TBs loop until stop is set (and at least numIters times), setting dirty
// when their random value is under the cutoff, then join the barrier.  The
// barrier is this build's generation-valued counter barrier over all TBs
// (the reference uses its lock-free tree barrier, which needs numTBs to be a
// multiple of NUM_SM -- the shipped run of 160 TBs does not finish on 152 SMs).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_flags(unsigned* stop, unsigned* dirty, unsigned* outArr, const float* randArr,
                                              unsigned randLen, unsigned* bar, int numAccsPerThr, int numRepeats,
                                              float cutoffVal, unsigned numIters, unsigned* status,
                                              unsigned long long timeout_ns) {
  __shared__ volatile unsigned mainSum[256];
  __shared__ volatile unsigned dataArr[256];
  __shared__ unsigned s_gen;
  const HsEnv env{status, timeout_ns};
  const bool isMain = (blockIdx.x == gridDim.x - 1);
  const unsigned myBaseLoc = blockIdx.x * blockDim.x + threadIdx.x;
  if (is_master()) s_gen = ld_relaxed<GPU>(bar + kLineWords);
  if (isMain) {
    mainSum[threadIdx.x] = 0;
    __syncthreads();
    for (int i = 0; i < numRepeats; ++i) {
      for (int j = 0; j < numAccsPerThr; ++j) mainSum[threadIdx.x] += (unsigned)numAccsPerThr;
      __syncthreads();
    }
    if (is_master()) red_release_add<GPU>(stop, 1u);
    __syncthreads();
  } else {
    dataArr[threadIdx.x] = threadIdx.x;
    unsigned randLoc = (blockIdx.x * blockDim.x) % randLen;
    unsigned iters = 0;
    const unsigned numDummy = (unsigned)numAccsPerThr / 4u;
    unsigned backoff = 2;
    const unsigned long long t0 = globaltimer();
    for (;;) {
      int stopSet = 0;
      if (is_master()) stopSet = ld_relaxed<GPU>(stop) != 0u;
      stopSet = __syncthreads_or(stopSet);
      if (stopSet && iters >= numIters) break;
      if (randArr[randLoc] <= cutoffVal) {
        for (unsigned i = 0; i < numDummy; ++i) dataArr[threadIdx.x] = dataArr[threadIdx.x] + 1u;
        __syncthreads();
        if (is_master()) asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(dirty) : "memory");
      } else {
        backoff = (backoff * 2u) & 255u;
        sleep_ns(backoff);
      }
      ++iters;
      randLoc = (randLoc + gridDim.x) % randLen;
      if ((iters & 63u) == 0u) {
        int bad = 0;
        if (is_master()) bad = ld_relaxed<GPU>(status) != 0u || globaltimer() - t0 > timeout_ns;
        if (__syncthreads_or(bad)) {
          if (is_master()) fail(env, HS_DEV_TIMEOUT, HS_SITE_RELAXED);
          return;
        }
      }
    }
  }
  // grid barrier: every TB must have stopped before the main TB reads dirty
  __syncthreads();
  int ok = 1;
  if (is_master()) {
    bool okb = true;
    counter_barrier<GPU>(bar, bar + kLineWords, gridDim.x, s_gen, 0u, env, HS_SITE_BAR_GLOBAL, [] { return true; },
                         &okb);
    ok = okb;
  }
  if (__syncthreads_or(!ok)) return;
  if (isMain) {
    __shared__ int isDirty;
    if (is_master()) isDirty = ld_acquire<GPU>(dirty) != 0u;
    __syncthreads();
    if (isDirty) outArr[myBaseLoc] = mainSum[threadIdx.x];
  }
}

cudaError_t launch_refcounter(unsigned* c0, unsigned* c1, unsigned* del0, unsigned* del1, int numTBs, int tbSize,
                              unsigned numRepeats, unsigned groups, unsigned perGroup, cudaStream_t st) {
  k_refcounter<<<numTBs, tbSize, 0, st>>>(c0, c1, del0, del1, numRepeats, groups, perGroup);
  return cudaGetLastError();
}
cudaError_t launch_splitcounter(unsigned* counters, unsigned* outArr, int numTBs, int tbSize, cudaStream_t st) {
  k_splitcounter<<<numTBs, tbSize, 0, st>>>(counters, outArr);
  return cudaGetLastError();
}
cudaError_t launch_seqlocks(unsigned* seq, int* d0, int* d1, int* out, int numTBs, int tbSize, int groupSize, int iters,
                            unsigned* status, unsigned long long timeout_ns, cudaStream_t st) {
  k_seqlocks<<<numTBs, tbSize, 0, st>>>(seq, d0, d1, out, groupSize, iters, status, timeout_ns);
  return cudaGetLastError();
}
cudaError_t launch_flags(unsigned* stop, unsigned* dirty, unsigned* outArr, const float* randArr, unsigned randLen,
                         unsigned* bar, int numTBs, int tbSize, int numAccsPerThr, int numRepeats, float cutoff,
                         unsigned numIters, unsigned* status, unsigned long long timeout_ns, cudaStream_t st) {
  k_flags<<<numTBs, tbSize, 0, st>>>(stop, dirty, outArr, randArr, randLen, bar, numAccsPerThr, numRepeats, cutoff,
                                     numIters, status, timeout_ns);
  return cudaGetLastError();
}
cudaError_t occupancy_flags(int tbSize, int* per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_flags, tbSize, 0);
}

}  // namespace hs
