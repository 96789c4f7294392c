// hs_cohort.cu -- die topology for the cohort (die-aware) global mutexes.
//
// A GB300's 152 SMs sit on two dies, and every L2 line is homed on one of
// them: an atomic from an SM to a line homed on its own die takes ~150 ns,
// one that crosses the dies ~330 ns.  Two measurements, made once per context:
//  1. every SM in turn times a chain of dependent atomics to one reference
//     line; the SMs split into the near half (die 0: the line's home) and the
//     far half (die 1);
//  2. one die-0 SM times each candidate lock line of the cohort pool; near
//     lines are homed on die 0, far ones on die 1.
// The cohort locks then give each die three lines homed on it.  If either
// split is not clean (a single-die part), the cohort locks stay off.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "hs_internal.h"
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

void hs_note_launches(unsigned n);

namespace hs {

constexpr unsigned long long kCalTimeoutNs = 2000000000ull;

__device__ __forceinline__ unsigned cal_smid() {
  unsigned s;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(s));
  return s;
}

__device__ __forceinline__ float atomic_chain_ns(unsigned* line, int n, unsigned zmask) {
  unsigned z = 0;
  const unsigned long long t0 = globaltimer();
  for (int i = 0; i < n; ++i) {
    unsigned old;
    asm volatile("atom.relaxed.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(line + z) : "memory");
    z = old & zmask;  // zmask is 0 at run time: each atomic waits for the previous one
  }
  return (float)(globaltimer() - t0) / (float)n;
}

// One CTA per SM (cooperative launch, shared memory sized for one per SM).
// CTAs take turns so that no two time the line at once.
__global__ void k_cal_sms(unsigned* turn, unsigned* line, float* rtt_by_sm, unsigned* err, unsigned zmask) {
  extern __shared__ unsigned char cal_pad[];
  if (threadIdx.x != 0) return;
  cal_pad[0] = 0;
  const unsigned k = blockIdx.x;
  const unsigned long long t0 = globaltimer();
  for (unsigned spin = 0; ld_acquire<GPU>(turn) != k; ++spin) {
    if ((spin & 255u) == 255u && (ld_relaxed<GPU>(err) != 0u || globaltimer() - t0 > kCalTimeoutNs)) {
      atomicOr(err, 1u);
      return;
    }
  }
  rtt_by_sm[cal_smid() & 255u] = atomic_chain_ns(line, 32, zmask);
  st_release<GPU>(turn, k + 1u);
}

// The CTA that lands on SM `target` times each candidate line.
__global__ void k_cal_lines(unsigned* lines, int nlines, unsigned target, float* rtt, unsigned* found,
                            unsigned zmask) {
  extern __shared__ unsigned char cal_pad[];
  if (threadIdx.x != 0) return;
  cal_pad[0] = 0;
  if (cal_smid() != target) return;
  for (int j = 0; j < nlines; ++j) rtt[j] = atomic_chain_ns(lines + (size_t)j * kLineWords, 16, zmask);
  *found = 1u;
}

}  // namespace hs

using namespace hs;

// Calibrates the pool (device memory: kCohortMapWords words of die map, then
// `ncand` candidate lines).  On success writes the die map into the pool and
// returns in sel[die][i] the candidate indices of three lines homed on each
// die; returns false when the part shows no clean two-die split.
bool hs::hs_cohort_calibrate(int device, unsigned* pool, int ncand, int sel[2][3]) {
  int nsm = 0, coop = 0, smem_sm = 0, smem_blk = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
  cudaDeviceGetAttribute(&smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (!coop || nsm < 2 || nsm > 256) return false;
  const int smem = smem_sm / 2 + 1024;  // one CTA per SM
  if (smem > smem_blk) return false;
  if (cudaFuncSetAttribute(k_cal_sms, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_cal_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  unsigned* lines = pool + kCohortMapWords;
  unsigned *scratch = nullptr;  // [0] turn, [32] err, [64] found, [96..] reference line
  float* rtt = nullptr;         // 256 by SM, then ncand by line
  if (cudaMalloc(&scratch, 256 * 4) != cudaSuccess || cudaMalloc(&rtt, (256 + (size_t)ncand) * 4) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(scratch);
    return false;
  }
  cudaMemset(scratch, 0, 256 * 4);
  cudaMemset(rtt, 0, (256 + (size_t)ncand) * 4);
  cudaMemset(lines, 0, (size_t)ncand * kLineWords * 4);
  unsigned* turn = scratch;
  unsigned* err = scratch + 32;
  unsigned* found = scratch + 64;
  unsigned* ref = lines;  // candidate 0 is the reference line
  unsigned zmask = 0;
  bool ok = false;
  std::vector<float> by_sm(256, 0.f), by_line(ncand, 0.f);
  do {
    void* a1[] = {&turn, &ref, &rtt, &err, &zmask};
    if (cudaLaunchCooperativeKernel((const void*)k_cal_sms, dim3((unsigned)nsm), dim3(32), a1, (size_t)smem, 0) !=
            cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
      break;
    hs_note_launches(1);
    unsigned herr = 0;
    cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(by_sm.data(), rtt, 256 * 4, cudaMemcpyDeviceToHost);
    if (herr) break;
    float lo = 1e30f, hi = 0.f;
    int present = 0;
    for (int s = 0; s < 256; ++s)
      if (by_sm[s] > 0.f) {
        lo = std::min(lo, by_sm[s]);
        hi = std::max(hi, by_sm[s]);
        ++present;
      }
    if (present < nsm || !(hi > 1.5f * lo)) break;  // no two-die split
    const float th = 0.5f * (lo + hi);
    unsigned char map[256];
    std::memset(map, 0, sizeof(map));
    int target = -1, near_n = 0, far_n = 0, ambiguous = 0;
    for (int s = 0; s < 256; ++s) {
      if (by_sm[s] <= 0.f) continue;
      const bool near = by_sm[s] < th;
      map[s] = near ? 0 : 1;
      (near ? near_n : far_n)++;
      if (near && target < 0) target = s;
      if (std::fabs(by_sm[s] - th) < 0.25f * (hi - lo)) ++ambiguous;
    }
    if (near_n < 1 || far_n < 1 || ambiguous || target < 0) break;
    // the candidate lines as seen from a die-0 SM
    unsigned tgt = (unsigned)target;
    float* rl = rtt + 256;
    void* a2[] = {&lines, &ncand, &tgt, &rl, &found, &zmask};
    if (cudaLaunchCooperativeKernel((const void*)k_cal_lines, dim3((unsigned)nsm), dim3(32), a2, (size_t)smem, 0) !=
            cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
      break;
    hs_note_launches(1);
    unsigned hf = 0;
    cudaMemcpy(&hf, found, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(by_line.data(), rl, (size_t)ncand * 4, cudaMemcpyDeviceToHost);
    if (!hf) break;
    float llo = 1e30f, lhi = 0.f;
    for (int j = 0; j < ncand; ++j) {
      llo = std::min(llo, by_line[j]);
      lhi = std::max(lhi, by_line[j]);
    }
    if (!(lhi > 1.5f * llo)) break;
    const float lth = 0.5f * (llo + lhi);
    int n0 = 0, n1 = 0;
    for (int j = 1; j < ncand && (n0 < 3 || n1 < 3); ++j) {  // candidate 0 was hammered by every SM: skip it
      const float v = by_line[j];
      if (v < lth - 0.2f * (lhi - llo) && n0 < 3) sel[0][n0++] = j;
      else if (v > lth + 0.2f * (lhi - llo) && n1 < 3) sel[1][n1++] = j;
    }
    if (n0 < 3 || n1 < 3) break;
    unsigned words[kCohortMapWords];
    std::memcpy(words, map, sizeof(map));
    cudaMemcpy(pool, words, sizeof(words), cudaMemcpyHostToDevice);
    ok = true;
  } while (false);
  cudaGetLastError();
  cudaFree(scratch);
  cudaFree(rtt);
  cudaMemset(lines, 0, (size_t)ncand * kLineWords * 4);
  return ok;
}
