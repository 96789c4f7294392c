// hs_uts.cu -- UTS (unbalanced tree search) on sm_103a: heterosync
// cuda/uts/uvm/uts.cu.
//
// Tree and initial frontier: built on the host exactly as the reference builds
// them (uts.cu:290-383: srand(200), rand()%100 values, fertility test, BFS
// order, leftovers become leaves of value 1; frontier of cores_used*16 nodes by
// expanding from the root), so the final counts match the reference's golden.
//
// Traversal: the reference runs 15 lock-protected local stacks plus a global
// stack with lane-0 locking (uts.cu:91-242).  Here every CTA owns two deques:
//  * a shared-memory deque (a ring of node ids): each step the CTA takes its
//    newest nodes, one per thread, processes them and appends their children
//    behind them (a block-wide scan gives each child its place), so a CTA works
//    depth-first on what it owns, with no global traffic at all;
//  * a global lock-free deque for stealing, with a single producer (its owner)
//    and many consumers: work beyond two steps' worth spills into it oldest
//    first (the roots of the largest remaining subtrees), published by a
//    release store of `bottom`; a CTA with no local work takes from its own
//    deque first and otherwise steals the oldest half of another CTA's,
//    reading the items before a CAS on `top` claims them (top only grows, so
//    no ABA; the owner writes a slot again only once top has passed it).
// A global count of processed nodes against the known total ends the run, and
// every wait is bounded.
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

constexpr int kUtsPool = 2048;  // shared-memory deque per CTA (node ids), a power of two

// One CTA's stealing deque: top (consumers) and bottom (the owner) on their own lines.
struct __align__(128) UtsDeque {
  unsigned long long top;
  unsigned pad0[30];
  unsigned long long bottom;
  unsigned pad1[30];
};

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long cas_acqrel64(unsigned long long* p, unsigned long long c,
                                                           unsigned long long v) {
  unsigned long long o;
  asm volatile("atom.acq_rel.gpu.cas.b64 %0, [%1], %2, %3;" : "=l"(o) : "l"(p), "l"(c), "l"(v) : "memory");
  return o;
}

// Exclusive block scan of one small count per thread (blockDim a multiple of 32, <= 1024).
__device__ __forceinline__ int block_scan(int x, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int v = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) s_warp[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int i = 0; i < nw; ++i) {
      const int t = s_warp[i];
      s_warp[i] = acc;
      acc += t;
    }
    s_warp[32] = acc;
  }
  __syncthreads();
  *total = s_warp[32];
  return s_warp[w] + v - x;
}

__global__ void __launch_bounds__(256) k_uts(hs_uts_node* nodes, unsigned* items, UtsDeque* dq, unsigned cap,
                                            const unsigned* frontier, int n_front, unsigned* ctl, unsigned total,
                                            unsigned* status, unsigned long long timeout_ns) {
  // ctl: [64] nodes processed (starts at the host's count), [96] leaves found,
  // [128] leaf sum, [160] nodes processed on the GPU (the end test)
  __shared__ unsigned s_pool[kUtsPool];
  __shared__ unsigned s_stage[256];
  __shared__ int s_warp[33];
  __shared__ int s_lo, s_hi, s_k, s_v, s_cmd;
  __shared__ unsigned long long s_t, s_bot;
  const HsEnv env{status, timeout_ns};
  const int T = (int)blockDim.x, tid = (int)threadIdx.x, c = (int)blockIdx.x, ncta = (int)gridDim.x;
  constexpr int M = kUtsPool - 1;
  const unsigned long long mask = cap - 1u;
  unsigned* done_ctr = ctl + 160;
  // the frontier is dealt round-robin: entry i to CTA i % ncta
  const int mine = n_front > c ? (n_front - c + ncta - 1) / ncta : 0;
  for (int j = tid; j < mine; j += T) s_pool[j] = frontier[c + j * ncta];
  if (tid == 0) {
    s_lo = 0;
    s_hi = mine;
    s_bot = 0;
  }
  __syncthreads();
  unsigned leaves = 0, lsum = 0;
  unsigned long long t0 = 0;
  unsigned last = 0;
  bool failed = false;
  for (;;) {
    const int n = s_hi - s_lo;
    if (n == 0) {
      // refill: the first deque (own first, then the others in turn) with work
      if (tid == 0) s_v = ncta;
      __syncthreads();
      for (int j = tid; j < ncta; j += T) {
        const int v = (c + j) % ncta;
        const long long avail = (long long)(ld_relaxed64(&dq[v].bottom) - ld_relaxed64(&dq[v].top));
        if (avail > 0) atomicMin(&s_v, j);
      }
      __syncthreads();
      if (s_v < ncta) {
        const int v = (c + s_v) % ncta;
        if (tid == 0) {
          const unsigned long long t = ld_acquire64(&dq[v].top);
          const unsigned long long b = ld_acquire64(&dq[v].bottom);
          const long long avail = (long long)(b - t);
          int k = 0;
          if (avail > 0) k = v == c ? (int)min(avail, (long long)T) : (int)min((long long)T, max(1ll, avail / 2));
          s_k = k;
          s_t = t;
        }
        __syncthreads();
        const int k = s_k;
        if (k > 0) {
          const unsigned* src = items + (size_t)v * cap;
          if (tid < k) s_stage[tid] = src[(s_t + (unsigned long long)tid) & mask];
          __syncthreads();  // every item is read before the claim
          if (tid == 0) s_cmd = cas_acqrel64(&dq[v].top, s_t, s_t + (unsigned long long)k) == s_t;
          __syncthreads();
          if (s_cmd) {
            if (tid < k) s_pool[(s_hi + tid) & M] = s_stage[tid];
            __syncthreads();
            if (tid == 0) s_hi += k;
            t0 = 0;
          }
        }
        __syncthreads();
        continue;
      }
      // nothing anywhere: finished, or work is in flight in other CTAs
      if (tid == 0) {
        const unsigned d = ld_acquire<GPU>(done_ctr);
        s_cmd = d >= total ? 1 : 0;
        if (!s_cmd) {
          const unsigned long long now = globaltimer();
          if (!t0 || d != last) {
            t0 = now;
            last = d;
          } else if (now - t0 > env.timeout_ns) {
            fail(env, HS_DEV_TIMEOUT, HS_SITE_UTS);
            s_cmd = 2;
          }
          if (!s_cmd && ld_relaxed<GPU>(env.status) != 0u) s_cmd = 2;
          if (!s_cmd) sleep_ns(128);
        }
      }
      __syncthreads();
      if (s_cmd) {
        failed = s_cmd == 2;
        break;
      }
      continue;
    }
    // one step: the newest k nodes, their children appended in their place
    const int k = min(min(n, T), kUtsPool - n);
    const int base = s_hi - k;
    int node = tid < k ? (int)s_pool[(base + tid) & M] : -1;
    int ch = 0, a = 0, b = 0;
    if (node >= 0) {
      hs_uts_node& nd = nodes[node];
      a = nd.child_a;
      b = nd.child_b;
      const unsigned val = nd.value + nd.to_add;
      nd.value = val;
      if (a == 0) {
        ++leaves;
        lsum += val;
      } else {
        const unsigned dep = nd.depth + 1u;
        nodes[a].depth = dep;
        nodes[b].depth = dep;
        nodes[a].to_add = 0u;
        nodes[b].to_add = 0u;
        ch = 2;
      }
    }
    int made = 0;
    const int off = block_scan(ch, s_warp, &made);  // its barriers also order the reads above
    if (ch) {
      s_pool[(base + off) & M] = (unsigned)a;
      s_pool[(base + off + 1) & M] = (unsigned)b;
    }
    __syncthreads();
    if (tid == 0) {
      s_hi = base + made;
      if (k) {
        asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" :: "l"(ctl + 64), "r"((unsigned)k) : "memory");
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(done_ctr), "r"((unsigned)k) : "memory");
      }
    }
    __syncthreads();
    // spill what is beyond two steps' worth, oldest first, to this CTA's stealing deque
    const int have = s_hi - s_lo;
    if (have > 2 * T) {
      if (tid == 0) {
        const unsigned long long t = ld_acquire64(&dq[c].top);
        const long long space = (long long)cap - (long long)(s_bot - t);
        s_k = (int)min((long long)(have - 2 * T), max(0ll, space));
      }
      __syncthreads();
      const int m = s_k;
      if (m > 0) {
        unsigned* dst = items + (size_t)c * cap;
        for (int i = tid; i < m; i += T) dst[(s_bot + (unsigned long long)i) & mask] = s_pool[(s_lo + i) & M];
        __syncthreads();  // every item is written before the release of bottom
        if (tid == 0) {
          s_bot += (unsigned long long)m;
          st_release64(&dq[c].bottom, s_bot);
          s_lo += m;
        }
      }
      __syncthreads();
    }
  }
  (void)failed;
  // leaf count and sum of the CTA
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    leaves += __shfl_xor_sync(0xFFFFFFFFu, leaves, o);
    lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, o);
  }
  if ((tid & 31) == 0 && leaves) {
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" :: "l"(ctl + 96), "r"(leaves) : "memory");
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" :: "l"(ctl + 128), "r"(lsum) : "memory");
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
  if (num_nodes <= 0 || n_frontier <= 0 || blocks <= 0 || threads < 32 || threads > 256 || threads % 32 ||
      (long long)n_frontier > (long long)blocks * hs::kUtsPool || host_processed > (unsigned)num_nodes) {
    g_uerr = "bad sizes (threads a multiple of 32 up to 256, frontier within the CTAs' deques)";
    return HS_EINVAL;
  }
  const unsigned total = (unsigned)num_nodes - host_processed;
  // a stealing deque per CTA, large enough that no CTA's can fill while others
  // are empty: twice a fair share plus slack, a power of two
  unsigned cap = 4096;
  while (cap < 2ull * total / (unsigned)blocks + 4096ull) cap <<= 1;
  hs_uts_node* d_tree = nullptr;
  unsigned *items = nullptr, *ctl = nullptr, *st = nullptr, *fr = nullptr;
  hs::UtsDeque* dq = nullptr;
  if (cudaMalloc(&d_tree, sizeof(hs_uts_node) * (size_t)num_nodes) != cudaSuccess ||
      cudaMalloc(&items, (size_t)cap * blocks * 4) != cudaSuccess ||
      cudaMalloc(&dq, sizeof(hs::UtsDeque) * (size_t)blocks) != cudaSuccess ||
      cudaMalloc(&fr, (size_t)n_frontier * 4) != cudaSuccess || cudaMalloc(&ctl, 256 * 4) != cudaSuccess ||
      cudaMalloc(&st, 64 * 4) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d_tree); cudaFree(items); cudaFree(dq); cudaFree(fr); cudaFree(ctl); cudaFree(st);
    g_uerr = "cudaMalloc";
    return HS_ENORES;
  }
  cudaMemcpy(d_tree, tree, sizeof(hs_uts_node) * (size_t)num_nodes, cudaMemcpyHostToDevice);
  std::vector<unsigned> hf((size_t)n_frontier);
  for (int i = 0; i < n_frontier; ++i) hf[i] = (unsigned)frontier[i];
  cudaMemcpy(fr, hf.data(), hf.size() * 4, cudaMemcpyHostToDevice);
  cudaMemset(dq, 0, sizeof(hs::UtsDeque) * (size_t)blocks);
  unsigned hctl[256] = {0};
  hctl[64] = host_processed;  // nodes_processed starts at the host's count (uts.cu:362)
  cudaMemcpy(ctl, hctl, sizeof(hctl), cudaMemcpyHostToDevice);
  cudaMemset(st, 0, 64 * 4);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a);
  hs::k_uts<<<blocks, threads>>>(d_tree, items, dq, cap, fr, n_frontier, ctl, total, st,
                                 timeout_ns ? timeout_ns : 10000000000ull);
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
  cudaFree(d_tree); cudaFree(items); cudaFree(dq); cudaFree(fr); cudaFree(ctl); cudaFree(st);
  if (e != cudaSuccess) { g_uerr = cudaGetErrorString(e); return HS_ECUDA; }
  out->nodes_processed = hctl[64];
  out->leaves_found = hctl[96];
  out->leaf_sum = hctl[128];
  out->elapsed_ms = ms;
  out->dev_error_bits = hst[0];
  if (hst[0]) { g_uerr = "device wait timed out"; return HS_ETIMEDOUT; }
  return HS_OK;
}
