// hs_uts_geo.cu -- geometric UTS (SHA-1 splittable node generator) with
// work stealing across per-CTA lock-free queues.
//
// Tree (the published Unbalanced Tree Search geometric shape; the reference
// repository's UTS, cuda/uts/uvm/uts.cu, has only its rand() binary tree):
//   root state    = SHA-1(16 zero bytes || seed, big-endian)
//   child i state = SHA-1(parent state || i, big-endian)
//   r             = last state word & 0x7fffffff
//   children      = 0 at depth >= depth_limit, else #{k >= 1 : r < T[k-1]},
//                   T[k-1] = floor(2^31 q^k), q = b / (1 + b), q^k by k - 1
//                   multiplications in IEEE double (geometric, mean b).
// A state is kept as the five SHA-1 chaining words, which are also the first
// five message words of a child's hash, so hashing needs no byte shuffling.
//
// Traversal: every thread walks its own subtree depth-first with a stack of
// frames (a node's state and the range of its children still to visit) in
// registers and local memory, hashing in registers.  Work moves through one
// bounded lock-free queue per CTA (a multi-producer multi-consumer ring with
// per-cell sequence numbers): while some thread is idle, a busy thread gives
// away the upper half of the children left in its oldest frame (the largest
// subtrees); an idle thread takes from its own CTA's queue first and then
// steals from other CTAs' queues.  Termination: one counter holds the queued
// items plus the busy threads; a push adds one before the item is visible, a
// thread whose stack empties subtracts one, so the counter reaches zero only
// when no work exists anywhere.
#include <cuda_runtime.h>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/hs/hs.h"
#include "hs_uts_geo.cuh"

void hs_note_launches(unsigned n);

namespace hs {

__global__ void __launch_bounds__(256) k_uts_geo(GeoArgs a) { uts_geo_walk(a, blockIdx.x); }

}  // namespace hs

using namespace hs;

namespace {
thread_local std::string g_gerr;
}

extern "C" const char* hs_uts_geo_last_error(void) { return g_gerr.c_str(); }

// T[k-1] = floor(2^31 q^k), q = b / (1 + b), q^k by repeated multiplication.
extern "C" int hs_uts_geo_table(double b, uint32_t* t, int n) {
  if (!t || n <= 0 || !(b > 0.0)) return HS_EINVAL;
  const double q = b / (1.0 + b);
  double p = q;
  int nz = 0;
  for (int k = 0; k < n; ++k) {
    const double v = p * 2147483648.0;
    t[k] = v >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)v;
    if (t[k]) nz = k + 1;
    p *= q;
  }
  return nz;
}

extern "C" int hs_uts_geo_run(unsigned seed, int depth_limit, double branching, int blocks, int threads,
                              unsigned long long timeout_ns, hs_uts_geo_result* r) {
  if (!r) return HS_EINVAL;
  std::memset(r, 0, sizeof(*r));
  if (depth_limit < 0 || depth_limit > kGeoMaxDepth || !(branching > 0.0) || blocks <= 0 || threads <= 0 ||
      threads > 256 || (threads % 32)) {
    g_gerr = "need 0 <= depth_limit <= 30, branching > 0, blocks > 0, threads a multiple of 32 up to 256";
    return HS_EINVAL;
  }
  uint32_t table[kGeoTable];
  const int nt = hs_uts_geo_table(branching, table, kGeoTable);
  const int nq = blocks;
  const size_t qcells = (size_t)nq * kGeoQueueCap;
  unsigned *d_seq = nullptr, *d_pos = nullptr, *d_ctl = nullptr, *d_table = nullptr;
  GeoItem* d_items = nullptr;
  if (cudaMalloc(&d_seq, qcells * 4) != cudaSuccess || cudaMalloc(&d_items, qcells * sizeof(GeoItem)) != cudaSuccess ||
      cudaMalloc(&d_pos, (size_t)nq * 64 * 4) != cudaSuccess || cudaMalloc(&d_ctl, 256 * 4) != cudaSuccess ||
      cudaMalloc(&d_table, sizeof(table)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d_seq); cudaFree(d_items); cudaFree(d_pos); cudaFree(d_ctl); cudaFree(d_table);
    g_gerr = "cudaMalloc";
    return HS_ENORES;
  }
  // cell i of every queue starts with sequence number i (empty, writable)
  std::vector<unsigned> seq0(qcells);
  for (size_t i = 0; i < qcells; ++i) seq0[i] = (unsigned)(i % kGeoQueueCap);
  cudaMemcpy(d_seq, seq0.data(), qcells * 4, cudaMemcpyHostToDevice);
  cudaMemset(d_pos, 0, (size_t)nq * 64 * 4);
  cudaMemset(d_ctl, 0, 256 * 4);
  const unsigned one = 1u;
  cudaMemcpy(d_ctl + 32, &one, 4, cudaMemcpyHostToDevice);  // work = 1: the root's thread
  cudaMemcpy(d_table, table, sizeof(table), cudaMemcpyHostToDevice);
  GeoArgs a;
  a.qseq = d_seq;
  a.qitem = d_items;
  a.qpos = d_pos;
  a.status = d_ctl;
  a.work = d_ctl + 32;
  a.idle = d_ctl + 64;
  a.out = reinterpret_cast<unsigned long long*>(d_ctl + 128);
  a.table = d_table;
  a.nt = nt;
  a.limit = depth_limit;
  a.nq = nq;
  a.seed = seed;
  a.timeout_ns = timeout_ns ? timeout_ns : 10000000000ull;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  k_uts_geo<<<blocks, threads>>>(a);
  cudaEventRecord(e1);
  cudaError_t e = cudaDeviceSynchronize();
  hs_note_launches(1);
  unsigned ctl[256] = {0};
  float ms = 0.f;
  if (e == cudaSuccess) {
    cudaEventElapsedTime(&ms, e0, e1);
    cudaMemcpy(ctl, d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_seq); cudaFree(d_items); cudaFree(d_pos); cudaFree(d_ctl); cudaFree(d_table);
  if (e != cudaSuccess) {
    g_gerr = cudaGetErrorString(e);
    return HS_ECUDA;
  }
  const unsigned long long* o = reinterpret_cast<const unsigned long long*>(ctl + 128);
  r->nodes = o[0];
  r->leaves = o[8];
  r->max_depth = (unsigned)o[16];
  r->elapsed_ms = ms;
  r->dev_error_bits = ctl[0];
  if (ctl[0]) {
    g_gerr = "device wait timed out";
    return HS_ETIMEDOUT;
  }
  return HS_OK;
}
