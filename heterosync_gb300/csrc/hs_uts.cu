// hs_uts.cu -- UTS (unbalanced tree search) on sm_103a: heterosync
// cuda/uts/uvm/uts.cu.
//
// Tree and initial frontier: built on the host exactly as the reference builds
// them (uts.cu:290-383: srand(200), rand()%100 values, fertility test, BFS
// order, leftovers become leaves of value 1; frontier of cores_used*16 nodes by
// expanding from the root), so the final counts match the reference's golden.
//
// Traversal: the reference runs 15 lock-protected local stacks plus a global
// stack with lane-0 locking (uts.cu:91-242).  Here every node the GPU must
// process passes once through one lock-free ticket queue in global memory:
// pop = atom.add on the head ticket, then a bounded acquire-wait until the slot
// is filled; push = atom.add on the tail ticket, then a release store of
// node+1 into the reserved slots.  Each GPU-processed node enters the queue
// exactly once, so the number of slots is known (numNodes - nodes the host
// expanded) and a thread whose ticket is past it is done.  A filled slot is
// always processed without waiting, so the slots keep filling until the end:
// no deadlock, and no lock at all.
#include <cuda_runtime.h>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <string>
#include <vector>
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

void hs_note_launches(unsigned n);

namespace hs {

__global__ void __launch_bounds__(256) k_uts(hs_uts_node* nodes, unsigned* q, unsigned* ctl, unsigned total_slots,
                                            unsigned* status, unsigned long long timeout_ns) {
  // ctl: [0] head ticket, [32] tail ticket, [64] nodes_processed, [96] leaves_found, [128] leaf_sum
  unsigned* head = ctl;
  unsigned* tail = ctl + 32;
  const HsEnv env{status, timeout_ns};
  for (;;) {
    const unsigned slot = atomicAdd(head, 1u);
    if (slot >= total_slots) break;
    unsigned v = 0;
    const bool ok = wait_until_p([&] { v = ld_acquire<GPU>(q + slot); return v != 0u; },
                                 [&] { return ld_relaxed<GPU>(tail); }, [] { sleep_ns(64); }, env, HS_SITE_UTS);
    if (!ok) break;
    const int n = (int)(v - 1u);
    hs_uts_node& nd = nodes[n];
    const int a = nd.child_a, b = nd.child_b;
    nd.value += nd.to_add;
    if (a == 0) {
      asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" :: "l"(ctl + 128), "r"(nd.value) : "memory");
      asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(ctl + 96) : "memory");
    } else {
      nodes[a].depth = nd.depth + 1;
      nodes[b].depth = nd.depth + 1;
      nodes[a].to_add = 0;
      nodes[b].to_add = 0;
      const unsigned s = atomicAdd(tail, 2u);
      st_release<GPU>(q + s, (unsigned)a + 1u);
      st_release<GPU>(q + s + 1, (unsigned)b + 1u);
    }
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(ctl + 64) : "memory");
  }
}

}  // namespace hs

namespace {
thread_local std::string g_uerr;
}

extern "C" const char* hs_uts_last_error(void) { return g_uerr.c_str(); }

// uts.cu:290-339 (tree) with the golden leaf count and sum.
extern "C" int hs_uts_tree_build(int num_nodes, int fertility, unsigned seed, hs_uts_node* tree, unsigned* leaves,
                                 unsigned* leaf_sum, unsigned* restarts) {
  if (num_nodes <= 0 || !tree || (num_nodes % 2) == 0) {
    g_uerr = "num_nodes must be positive and odd (children come in pairs; uts.cu:580)";
    return HS_EINVAL;
  }
  std::memset(tree, 0, sizeof(hs_uts_node) * (size_t)num_nodes);
  srand(seed);
  std::deque<int> undecided;
  std::vector<int> leaf_nodes;  // kept in the reference's order (new leaves go to the front)
  undecided.push_back(0);
  int next = 1;
  unsigned restart_count = 0;
  while (next != num_nodes) {
    if (undecided.empty()) {
      undecided.assign(leaf_nodes.begin(), leaf_nodes.end());
      leaf_nodes.clear();
      ++restart_count;
    }
    const int cur = undecided.front();
    tree[cur].value = (unsigned)(rand() % 100);
    tree[cur].depth = 0;
    tree[cur].to_add = 0;
    if ((rand() % 100) < fertility) {
      tree[cur].child_a = next;
      undecided.push_back(next++);
      tree[cur].child_b = next;
      undecided.push_back(next++);
    } else {
      tree[cur].child_a = 0;
      tree[cur].child_b = 0;
      leaf_nodes.insert(leaf_nodes.begin(), cur);
    }
    undecided.pop_front();
  }
  unsigned sum = 0;
  for (int n : undecided) {
    tree[n].child_a = tree[n].child_b = 0;
    tree[n].value = 1;
    tree[n].depth = 0;
    tree[n].to_add = 0;
    sum += 1;
  }
  for (int n : leaf_nodes) sum += tree[n].value;
  if (leaves) *leaves = (unsigned)(leaf_nodes.size() + undecided.size());
  if (leaf_sum) *leaf_sum = sum;
  if (restarts) *restarts = restart_count;
  return HS_OK;
}

// uts.cu:341-383: expand from the root until the frontier holds cores_used*16
// nodes (leaves cycle to the back).  Returns the frontier in the order the
// reference deals it out and the number of internal nodes expanded on the host.
extern "C" int hs_uts_frontier(const hs_uts_node* tree, int num_nodes, int cores_used, int* frontier, int* count,
                               unsigned* host_processed) {
  const int want = cores_used * 16;
  std::deque<int> init;
  init.push_back(0);
  unsigned processed = 0;
  size_t guard = 0;
  while ((int)init.size() < want) {
    if (init.empty() || ++guard > (size_t)num_nodes * 4 + 1024) {
      g_uerr = "not enough nodes to fill the initial frontier";
      return HS_EINVAL;
    }
    const int n = init.front();
    init.pop_front();
    if (tree[n].child_a > 0) {
      init.push_back(tree[n].child_a);
      init.push_back(tree[n].child_b);
      ++processed;
    } else {
      init.push_back(n);
    }
  }
  int i = 0;
  for (int n : init) frontier[i++] = n;
  *count = i;
  *host_processed = processed;
  return HS_OK;
}

extern "C" int hs_uts_run(const hs_uts_node* tree, int num_nodes, const int* frontier, int n_frontier,
                          unsigned host_processed, int blocks, int threads, unsigned long long timeout_ns,
                          hs_uts_result* out) {
  std::memset(out, 0, sizeof(*out));
  if (num_nodes <= 0 || n_frontier <= 0 || blocks <= 0 || threads <= 0 || threads > 256) {
    g_uerr = "bad sizes";
    return HS_EINVAL;
  }
  const unsigned total = (unsigned)num_nodes - host_processed;
  hs_uts_node* d_tree = nullptr;
  unsigned *q = nullptr, *ctl = nullptr, *st = nullptr;
  const size_t qwords = (size_t)total + 64;
  if (cudaMalloc(&d_tree, sizeof(hs_uts_node) * (size_t)num_nodes) != cudaSuccess ||
      cudaMalloc(&q, qwords * 4) != cudaSuccess || cudaMalloc(&ctl, 256 * 4) != cudaSuccess ||
      cudaMalloc(&st, 64 * 4) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d_tree); cudaFree(q); cudaFree(ctl); cudaFree(st);
    g_uerr = "cudaMalloc";
    return HS_ENORES;
  }
  cudaMemcpy(d_tree, tree, sizeof(hs_uts_node) * (size_t)num_nodes, cudaMemcpyHostToDevice);
  std::vector<unsigned> hq((size_t)n_frontier);
  for (int i = 0; i < n_frontier; ++i) hq[i] = (unsigned)frontier[i] + 1u;
  cudaMemset(q, 0, qwords * 4);
  cudaMemcpy(q, hq.data(), hq.size() * 4, cudaMemcpyHostToDevice);
  unsigned hctl[256] = {0};
  hctl[32] = (unsigned)n_frontier;  // tail
  hctl[64] = host_processed;         // nodes_processed starts at the host's count (uts.cu:362)
  cudaMemcpy(ctl, hctl, sizeof(hctl), cudaMemcpyHostToDevice);
  cudaMemset(st, 0, 64 * 4);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a);
  hs::k_uts<<<blocks, threads>>>(d_tree, q, ctl, total, st, timeout_ns ? timeout_ns : 10000000000ull);
  cudaEventRecord(b);
  cudaError_t e = cudaDeviceSynchronize();
  hs_note_launches(1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  unsigned hst[2] = {0, 0};
  if (e == cudaSuccess) {
    cudaMemcpy(hctl, ctl, sizeof(hctl), cudaMemcpyDeviceToHost);
    cudaMemcpy(hst, st, sizeof(hst), cudaMemcpyDeviceToHost);
  }
  cudaFree(d_tree); cudaFree(q); cudaFree(ctl); cudaFree(st);
  if (e != cudaSuccess) { g_uerr = cudaGetErrorString(e); return HS_ECUDA; }
  out->nodes_processed = hctl[64];
  out->leaves_found = hctl[96];
  out->leaf_sum = hctl[128];
  out->elapsed_ms = ms;
  out->dev_error_bits = hst[0];
  if (hst[0]) { g_uerr = "device wait timed out"; return HS_ETIMEDOUT; }
  return HS_OK;
}
