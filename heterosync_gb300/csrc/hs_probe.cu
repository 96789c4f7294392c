// hs_probe.cu -- roofline probes measured on the local GPU.
//
// L2 atomic rate: every thread issues red.relaxed.gpu.global.add.u32 to its own
// word, words 128 bytes apart, so no two atomics contend for a line: the
// aggregate rate is the chip's contention-free L2 atomic throughput, the
// denominator of the sync-ops roofline.
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/hs/hs.h"

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

}  // namespace hs

void hs_note_launches(unsigned n);

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
