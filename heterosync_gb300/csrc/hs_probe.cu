// hs_probe.cu -- roofline probes measured on the local GPU.
//
// Lock hand-off latencies (hs_probe_latency): the floor under a serialised
// lock's op is a chain of such latencies (the release seen by the next
// holder, its atomic, its critical section's load and the store ack before
// its own release), so these set the sync-ops bound for the lock kernels.
//
// L2 atomic rate: every thread issues red.relaxed.gpu.global.add.u32 to its own
// word, words 128 bytes apart, so no two atomics contend for a line: the
// aggregate rate is the chip's contention-free L2 atomic throughput, the
// denominator of the sync-ops roofline.
//
// L2 bandwidth: a copy between two buffers that together fit in L2, with
// loads and stores that bypass L1 (ld/st .cg), repeated in one launch: the
// chip's L2-resident copy rate, the denominator for critical sections and
// exchanges whose data stays in L2.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

namespace hs {

__global__ void __launch_bounds__(1024) k_probe_red(unsigned* words, int iters, unsigned stride_words) {
  unsigned* p = words + ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * stride_words;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(p) : "memory");
}

// Same-address atomics from one lane per CTA: the rate a single contended lock
// word can sustain (the ceiling for centralised locks).
__global__ void k_probe_same(unsigned* word, int iters) {
  if (threadIdx.x == 0)
    for (int i = 0; i < iters; ++i) asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(word) : "memory");
}

// L2-resident copy: grid-stride, four 16-byte loads in flight per thread, L1 bypassed.
__global__ void __launch_bounds__(512) k_probe_copy(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                    size_t n, int reps) {
  const size_t step = (size_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * step < n; i += 4 * step) {
      const uint4 a = __ldcg(src + i), b = __ldcg(src + i + step), c = __ldcg(src + i + 2 * step),
                  d = __ldcg(src + i + 3 * step);
      __stcg(dst + i, a);
      __stcg(dst + i + step, b);
      __stcg(dst + i + 2 * step, c);
      __stcg(dst + i + 3 * step, d);
    }
    for (; i < n; i += step) __stcg(dst + i, __ldcg(src + i));
  }
}

constexpr unsigned long long kLatTimeoutNs = 2000000000ull;

// Bounded poll until *f == want; false (and err set) on timeout or another side's error.
__device__ bool lat_wait(const unsigned* f, unsigned want, unsigned* err, unsigned long long t_start) {
  for (unsigned spin = 0;; ++spin) {
    if (ld_acquire<GPU>(f) == want) return true;
    if ((spin & 255u) == 255u) {
      if (ld_relaxed<GPU>(err) != 0u) return false;
      if (globaltimer() - t_start > kLatTimeoutNs) {
        atomicOr(err, 1u);
        return false;
      }
    }
  }
}

// One thread per CTA works; grid = one CTA per SM (cooperative launch: all co-resident).
__global__ void k_probe_latency(unsigned* flags, unsigned long long* ns, unsigned* chase, unsigned* lines,
                                int rounds, int chain, unsigned zmask, unsigned* err) {
  if (threadIdx.x != 0) return;
  const unsigned long long t_start = globaltimer();
  const unsigned k = blockIdx.x;
  if (k != 0) {  // partner k: answer CTA 0's rounds when its turn comes
    unsigned* f = flags + (size_t)k * 32;
    for (int i = 0; i < rounds; ++i) {
      if (!lat_wait(f, 2u * i + 1u, err, t_start)) return;
      st_release<GPU>(f, 2u * i + 2u);
    }
    return;
  }
  for (unsigned p = 1; p < gridDim.x; ++p) {
    unsigned* f = flags + (size_t)p * 32;
    const unsigned long long t0 = globaltimer();
    for (int i = 0; i < rounds; ++i) {
      st_release<GPU>(f, 2u * i + 1u);
      if (!lat_wait(f, 2u * i + 2u, err, t_start)) return;
    }
    ns[p] = globaltimer() - t0;
  }
  // dependent atomics: the next line's index depends on the returned value
  // (zmask is 0 at run time, unknown to the compiler)
  unsigned z = 0;
  unsigned long long t0 = globaltimer();
  for (int i = 0; i < chain; ++i) {
    unsigned old;
    asm volatile("atom.relaxed.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(lines + (size_t)((i * 37) & 63) * 32 + z) : "memory");
    z = old & zmask;
  }
  ns[gridDim.x] = globaltimer() - t0;
  // dependent L2 loads around the linked cycle
  unsigned idx = 0;
  t0 = globaltimer();
  for (int i = 0; i < chain; ++i) idx = ld_relaxed<GPU>(chase + idx);
  ns[gridDim.x + 1] = globaltimer() - t0;
  ns[gridDim.x + 2] = idx;  // keeps the chain live
}

}  // namespace hs

void hs_note_launches(unsigned n);

extern "C" int hs_probe_latency(int rounds, hs_latency_result* r) {
  if (rounds <= 0 || rounds > (1 << 20) || !r) return HS_EINVAL;
  std::memset(r, 0, sizeof(*r));
  int dev = 0, nsm = 0, coop = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop || nsm < 2) {
    cudaGetLastError();
    return HS_ENODEV;
  }
  constexpr unsigned kCycle = 4096;  // 128-byte lines: 512 KiB, L2-resident
  const int chain = 4096;
  std::vector<unsigned> cyc(kCycle * 32, 0u), order(kCycle);
  std::iota(order.begin(), order.end(), 0u);
  std::shuffle(order.begin() + 1, order.end(), std::mt19937(12345));
  for (unsigned i = 0; i < kCycle; ++i) cyc[order[i] * 32] = order[(i + 1) % kCycle] * 32;
  unsigned *flags = nullptr, *chase = nullptr, *lines = nullptr, *err = nullptr;
  unsigned long long* ns = nullptr;
  if (cudaMalloc(&flags, (size_t)nsm * 32 * 4) != cudaSuccess || cudaMalloc(&chase, cyc.size() * 4) != cudaSuccess ||
      cudaMalloc(&lines, 64 * 32 * 4) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess ||
      cudaMalloc(&ns, (size_t)(nsm + 3) * 8) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(flags); cudaFree(chase); cudaFree(lines); cudaFree(err); cudaFree(ns);
    return HS_ENORES;
  }
  cudaMemcpy(chase, cyc.data(), cyc.size() * 4, cudaMemcpyHostToDevice);
  cudaMemset(lines, 0, 64 * 32 * 4);
  cudaError_t e = cudaSuccess;
  std::vector<unsigned long long> h(nsm + 3, 0ull);
  unsigned herr = 0;
  for (int pass = 0; pass < 2 && e == cudaSuccess && herr == 0; ++pass) {  // pass 0 warms lines and code
    cudaMemset(flags, 0, (size_t)nsm * 32 * 4);
    cudaMemset(err, 0, 4);
    cudaMemset(ns, 0, (size_t)(nsm + 3) * 8);
    int rr = pass ? rounds : 8, ch = pass ? chain : (int)kCycle;
    unsigned zmask = 0;
    void* args[] = {&flags, &ns, &chase, &lines, &rr, &ch, &zmask, &err};
    e = cudaLaunchCooperativeKernel((const void*)hs::k_probe_latency, dim3((unsigned)nsm), dim3(32), args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    hs_note_launches(1);
    if (e == cudaSuccess) {
      cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
      cudaMemcpy(h.data(), ns, h.size() * 8, cudaMemcpyDeviceToHost);
    }
  }
  cudaFree(flags); cudaFree(chase); cudaFree(lines); cudaFree(err); cudaFree(ns);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return HS_ECUDA;
  }
  r->dev_error_bits = herr;
  if (herr) return HS_ETIMEDOUT;
  std::vector<double> ho;
  for (int p = 1; p < nsm; ++p) ho.push_back((double)h[p] / (2.0 * rounds));
  std::sort(ho.begin(), ho.end());
  r->partners = (int)ho.size();
  r->handoff_ns_min = ho.front();
  r->handoff_ns_max = ho.back();
  r->handoff_ns_median = ho[ho.size() / 2];
  r->atomic_rtt_ns = (double)h[nsm] / chain;
  r->load_rtt_ns = (double)h[nsm + 1] / chain;
  return HS_OK;
}

extern "C" int hs_probe_l2_atomics(int blocks, int threads, int iters, int same_address, double* atomics_per_s) {
  if (blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0 || !atomics_per_s) return HS_EINVAL;
  const size_t stride = 32;  // 128-byte spacing
  const size_t n = same_address ? 32 : (size_t)blocks * threads * stride;
  unsigned* w = nullptr;
  if (cudaMalloc(&w, n * 4) != cudaSuccess) { cudaGetLastError(); return HS_ENORES; }
  cudaMemset(w, 0, n * 4);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto launch = [&]() {
    if (same_address) hs::k_probe_same<<<blocks, 32>>>(w, iters);
    else hs::k_probe_red<<<blocks, threads>>>(w, iters, (unsigned)stride);
  };
  launch();  // warm-up
  cudaEventRecord(a);
  launch();
  cudaEventRecord(b);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  hs_note_launches(2);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(w);
  if (e != cudaSuccess) return HS_ECUDA;
  const double total = same_address ? (double)blocks * iters : (double)blocks * threads * iters;
  *atomics_per_s = total / (ms * 1e-3);
  return HS_OK;
}

extern "C" int hs_probe_l2_bandwidth(size_t bytes, int reps, double* copy_gbs) {
  if (bytes < (1u << 20) || reps <= 0 || reps > 10000 || !copy_gbs) return HS_EINVAL;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) {
    cudaGetLastError();
    return HS_ENODEV;
  }
  const size_t n = bytes / 2 / sizeof(uint4);  // vectors per buffer
  uint4 *src = nullptr, *dst = nullptr;
  if (cudaMalloc(&src, n * sizeof(uint4)) != cudaSuccess || cudaMalloc(&dst, n * sizeof(uint4)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(src);
    return HS_ENORES;
  }
  cudaMemset(src, 1, n * sizeof(uint4));
  cudaMemset(dst, 0, n * sizeof(uint4));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const unsigned grid = (unsigned)nsm * 4u;
  hs::k_probe_copy<<<grid, 512>>>(src, dst, n, 2);  // warm-up: both buffers into L2
  cudaEventRecord(a);
  hs::k_probe_copy<<<grid, 512>>>(src, dst, n, reps);
  cudaEventRecord(b);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  hs_note_launches(2);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(src);
  cudaFree(dst);
  if (e != cudaSuccess) return HS_ECUDA;
  *copy_gbs = 2.0 * (double)n * sizeof(uint4) * reps / (ms * 1e-3) * 1e-9;  // bytes read + written
  return HS_OK;
}
