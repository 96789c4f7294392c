// hs_relaxed_api.cu -- C ABI for the relaxed-atomics microbenchmarks.
// Host arrays in and out (the reference keeps these arrays in managed memory,
// e.g. refCounter.cu:43-50); copies happen inside the call, the kernel alone is
// timed with CUDA events.
#include <cuda_runtime.h>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

namespace hs {
cudaError_t launch_refcounter(unsigned*, unsigned*, unsigned*, unsigned*, int, int, unsigned, unsigned, unsigned,
                              cudaStream_t);
cudaError_t launch_splitcounter(unsigned*, unsigned*, int, int, cudaStream_t);
cudaError_t launch_seqlocks(unsigned*, int*, int*, int*, int, int, int, int, unsigned*, unsigned long long,
                            cudaStream_t);
cudaError_t launch_flags(unsigned*, unsigned*, unsigned*, const float*, unsigned, unsigned*, int, int, int, int, float,
                         unsigned, unsigned*, unsigned long long, cudaStream_t);
cudaError_t occupancy_flags(int tbSize, int* per_sm);
}  // namespace hs
void hs_note_launches(unsigned n);

namespace {
thread_local std::string g_rerr;

struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, n * sizeof(T) + 16);
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

struct Timer {
  cudaEvent_t a{}, b{};
  Timer() { cudaEventCreate(&a); cudaEventCreate(&b); }
  ~Timer() { cudaEventDestroy(a); cudaEventDestroy(b); }
  float ms() {
    float m = 0.f;
    cudaEventElapsedTime(&m, a, b);
    return m;
  }
};

int fail_cuda(const char* what, cudaError_t e) {
  g_rerr = std::string(what) + ": " + cudaGetErrorString(e);
  return HS_ECUDA;
}

int status_of(unsigned* d_status, hs_relaxed_result* r) {
  unsigned h[2] = {0, 0};
  cudaMemcpy(h, d_status, sizeof(h), cudaMemcpyDeviceToHost);
  r->dev_error_bits = h[0];
  r->dev_error_site = h[1];
  if (h[0] & hs::HS_DEV_TIMEOUT) { g_rerr = "device wait timed out"; return HS_ETIMEDOUT; }
  return HS_OK;
}
}  // namespace

extern "C" const char* hs_relaxed_last_error(void) { return g_rerr.c_str(); }

// refCounter.cu:5-155
extern "C" int hs_refcounter(int numSharersPerGroup, int numTBs, int tbSize, int numRepeats, unsigned* counters0,
                             unsigned* counters1, unsigned* del0, unsigned* del1, hs_relaxed_result* r) {
  std::memset(r, 0, sizeof(*r));
  if (numSharersPerGroup <= 0 || numTBs <= 0 || tbSize <= 0 || tbSize > 256 || numRepeats < 0 ||
      numSharersPerGroup > numTBs) {
    g_rerr = "need 0 < numSharersPerGroup <= numTBs and 0 < tbSize <= 256";
    return HS_EINVAL;
  }
  const unsigned numThrs = (unsigned)tbSize * numTBs;
  const unsigned numCounters = numThrs / numSharersPerGroup;
  const unsigned groups = numTBs / numSharersPerGroup;
  const unsigned perGroup = numCounters / groups;
  if (perGroup < (unsigned)tbSize) { g_rerr = "counters per group below tbSize"; return HS_EINVAL; }
  DevBufs B;
  unsigned *c0 = B.alloc<unsigned>(numCounters), *c1 = B.alloc<unsigned>(numCounters);
  unsigned *d0 = B.alloc<unsigned>(numThrs), *d1 = B.alloc<unsigned>(numThrs);
  if (!c0 || !c1 || !d0 || !d1) { g_rerr = "cudaMalloc"; return HS_ENORES; }
  cudaMemcpy(c0, counters0, numCounters * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(c1, counters1, numCounters * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d0, del0, numThrs * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d1, del1, numThrs * 4, cudaMemcpyHostToDevice);
  Timer t;
  cudaEventRecord(t.a);
  cudaError_t e = hs::launch_refcounter(c0, c1, d0, d1, numTBs, tbSize, (unsigned)numRepeats, groups, perGroup, 0);
  cudaEventRecord(t.b);
  if (e != cudaSuccess) return fail_cuda("refCounter launch", e);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail_cuda("refCounter", e);
  hs_note_launches(1);
  r->elapsed_ms = t.ms();
  r->ops = (unsigned long long)numThrs * numRepeats * 4ull;
  cudaMemcpy(counters0, c0, numCounters * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(counters1, c1, numCounters * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(del0, d0, numThrs * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(del1, d1, numThrs * 4, cudaMemcpyDeviceToHost);
  return HS_OK;
}

// splitCounter.cu:5-98
extern "C" int hs_splitcounter(int numTBs, int tbSize, unsigned* counters, unsigned* outArr, hs_relaxed_result* r) {
  std::memset(r, 0, sizeof(*r));
  if (numTBs <= 0 || tbSize < 32 || tbSize > 256 || (tbSize % 32) != 0) {
    g_rerr = "need numTBs > 0 and tbSize a multiple of 32 in [32, 256]";
    return HS_EINVAL;
  }
  const unsigned numThrs = (unsigned)numTBs * tbSize;
  DevBufs B;
  unsigned *c = B.alloc<unsigned>(numThrs / 2), *o = B.alloc<unsigned>(numThrs);
  if (!c || !o) { g_rerr = "cudaMalloc"; return HS_ENORES; }
  cudaMemcpy(c, counters, numThrs / 2 * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(o, outArr, numThrs * 4, cudaMemcpyHostToDevice);
  Timer t;
  cudaEventRecord(t.a);
  cudaError_t e = hs::launch_splitcounter(c, o, numTBs, tbSize, 0);
  cudaEventRecord(t.b);
  if (e != cudaSuccess) return fail_cuda("splitCounter launch", e);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail_cuda("splitCounter", e);
  hs_note_launches(1);
  r->elapsed_ms = t.ms();
  r->ops = numThrs;
  cudaMemcpy(counters, c, numThrs / 2 * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(outArr, o, numThrs * 4, cudaMemcpyDeviceToHost);
  return HS_OK;
}

// seqlocks.cu:5-111 (NUM_ITERS = 10, seqlocks_kernel.cu:3)
extern "C" int hs_seqlocks(int numTBs, int tbSize, int groupSize, int useTFs, unsigned* seqlock, int* data0,
                           int* data1, int* outArr, unsigned long long timeout_ns, hs_relaxed_result* r) {
  (void)useTFs;  // scoped acquire/release already orders what the reference's extra fences order
  std::memset(r, 0, sizeof(*r));
  if (numTBs <= 0 || tbSize <= 0 || tbSize > 1024 || groupSize <= 0) { g_rerr = "bad sizes"; return HS_EINVAL; }
  const int numSeq = numTBs / groupSize > groupSize ? numTBs / groupSize : groupSize;
  const unsigned numThrs = (unsigned)numTBs * tbSize;
  DevBufs B;
  unsigned* s = B.alloc<unsigned>(numSeq);
  int *d0 = B.alloc<int>(32), *d1 = B.alloc<int>(32), *o = B.alloc<int>(numThrs);
  unsigned* st = B.alloc<unsigned>(64);
  if (!s || !d0 || !d1 || !o || !st) { g_rerr = "cudaMalloc"; return HS_ENORES; }
  cudaMemcpy(s, seqlock, (size_t)(numTBs / groupSize) * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d0, data0, 32 * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d1, data1, 32 * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(o, outArr, numThrs * 4, cudaMemcpyHostToDevice);
  Timer t;
  cudaEventRecord(t.a);
  cudaError_t e = hs::launch_seqlocks(s, d0, d1, o, numTBs, tbSize, groupSize, 10, st,
                                      timeout_ns ? timeout_ns : 10000000000ull, 0);
  cudaEventRecord(t.b);
  if (e != cudaSuccess) return fail_cuda("seqlocks launch", e);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail_cuda("seqlocks", e);
  hs_note_launches(1);
  r->elapsed_ms = t.ms();
  r->ops = (unsigned long long)numTBs * 10ull;
  cudaMemcpy(seqlock, s, (size_t)(numTBs / groupSize) * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(data0, d0, 32 * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(data1, d1, 32 * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(outArr, o, numThrs * 4, cudaMemcpyDeviceToHost);
  return status_of(st, r);
}

// flags.cu:19-176
extern "C" int hs_flags(int numTBs, int tbSize, int numAccsPerThr, int numRepeats, float cutoffVal, int numIters,
                        const float* randArr, int randLen, unsigned* outArr, unsigned* dirty_out,
                        unsigned long long timeout_ns, hs_relaxed_result* r) {
  std::memset(r, 0, sizeof(*r));
  if (numTBs <= 0 || tbSize <= 0 || tbSize > 256 || randLen <= 0 || !(cutoffVal >= 0.f && cutoffVal <= 1.f)) {
    g_rerr = "need numTBs > 0, 0 < tbSize <= 256, randLen > 0 and cutoff in [0, 1]";
    return HS_EINVAL;
  }
  int per_sm = 0, nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  hs::occupancy_flags(tbSize, &per_sm);
  if ((long long)per_sm * nsm < numTBs) { g_rerr = "flags TBs cannot all be co-resident"; return HS_ENORES; }
  const unsigned numThrs = (unsigned)numTBs * tbSize;
  DevBufs B;
  unsigned *stop = B.alloc<unsigned>(32), *dirty = B.alloc<unsigned>(32), *o = B.alloc<unsigned>(numThrs);
  unsigned *bar = B.alloc<unsigned>(64), *st = B.alloc<unsigned>(64);
  float* ra = B.alloc<float>((size_t)randLen);
  if (!stop || !dirty || !o || !bar || !st || !ra) { g_rerr = "cudaMalloc"; return HS_ENORES; }
  cudaMemcpy(o, outArr, numThrs * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(ra, randArr, (size_t)randLen * 4, cudaMemcpyHostToDevice);
  Timer t;
  cudaEventRecord(t.a);
  cudaError_t e = hs::launch_flags(stop, dirty, o, ra, (unsigned)randLen, bar, numTBs, tbSize, numAccsPerThr,
                                   numRepeats, cutoffVal, (unsigned)numIters, st,
                                   timeout_ns ? timeout_ns : 10000000000ull, 0);
  cudaEventRecord(t.b);
  if (e != cudaSuccess) return fail_cuda("flags launch", e);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail_cuda("flags", e);
  hs_note_launches(1);
  r->elapsed_ms = t.ms();
  r->ops = numTBs;
  cudaMemcpy(outArr, o, numThrs * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(dirty_out, dirty, 4, cudaMemcpyDeviceToHost);
  return status_of(st, r);
}
