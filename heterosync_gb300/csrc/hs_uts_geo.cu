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
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include "../../include/hs/hs.h"
#include "hs_uts_geo.cuh"

void hs_note_launches(unsigned n);

namespace hs {

__global__ void __launch_bounds__(256) k_uts_geo(GeoArgs a) { uts_geo_walk(a, blockIdx.x); }
__global__ void __launch_bounds__(256) k_uts_geo_coop(GeoArgs a) { uts_geo_walk<true>(a, blockIdx.x); }

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

// ---------------------------------------------------------------------------
// Cooperative CPU+GPU walk: the host side.  Host walkers run the same
// depth-first walk as a GPU thread, hashing with the same generator, and share
// work among themselves through one locked deque (host threads are few).  The
// bridge layout and the count rules are described with GeoBridge.
// ---------------------------------------------------------------------------
namespace {

inline unsigned h_load(const unsigned* p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }
inline unsigned h_load_relaxed(const unsigned* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
inline void h_store(unsigned* p, unsigned v) { __atomic_store_n(p, v, __ATOMIC_RELEASE); }
inline unsigned h_add(unsigned* p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_ACQ_REL); }

// Host consumer of the GPU->host ring.
bool host_g2h_pop(const GeoBridge& b, GeoItem& it) {
  unsigned* deq = b.ctl + 128;
  unsigned pos = h_load_relaxed(deq);
  for (int tries = 0; tries < 64; ++tries) {
    const unsigned c = pos & (kBridgeCap - 1);
    const int dif = (int)(h_load(b.g2h_seq + c) - (pos + 1u));
    if (dif == 0) {
      if (__atomic_compare_exchange_n(deq, &pos, pos + 1u, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
        const unsigned* src = reinterpret_cast<const unsigned*>(b.g2h_item + c);
        unsigned* dst = reinterpret_cast<unsigned*>(&it);
        for (int k = 0; k < 8; ++k) dst[k] = h_load_relaxed(src + k);
        h_store(b.g2h_seq + c, pos + kBridgeCap);
        return true;
      }
      continue;  // pos holds the current position
    }
    if (dif < 0) return false;  // empty
    pos = h_load_relaxed(deq);
  }
  return false;
}

// Host producer of the host->GPU ring.
bool host_h2g_push(const GeoBridge& b, const GeoItem& it) {
  unsigned* enq = b.ctl + 160;
  unsigned pos = h_load_relaxed(enq);
  for (int tries = 0; tries < 64; ++tries) {
    const unsigned c = pos & (kBridgeCap - 1);
    const int dif = (int)(h_load(b.h2g_seq + c) - pos);
    if (dif == 0) {
      if (__atomic_compare_exchange_n(enq, &pos, pos + 1u, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
        unsigned* dst = reinterpret_cast<unsigned*>(b.h2g_item + c);
        const unsigned* src = reinterpret_cast<const unsigned*>(&it);
        for (int k = 0; k < 8; ++k) __atomic_store_n(dst + k, src[k], __ATOMIC_RELAXED);
        h_store(b.h2g_seq + c, pos + 1u);
        return true;
      }
      continue;
    }
    if (dif < 0) return false;  // full
    pos = h_load_relaxed(enq);
  }
  return false;
}

struct HostWalk {
  GeoBridge br;
  const unsigned* table;
  int nt, limit;
  unsigned seed;
  unsigned long long timeout_ns;
  std::atomic<unsigned> work{0};  // the host side's count: queued host items plus busy walkers
  std::mutex qm;
  std::deque<GeoItem> q;
  std::atomic<unsigned> queued{0};
  std::atomic<unsigned long long> nodes{0}, leaves{0}, to_host{0}, to_gpu{0};
  std::atomic<unsigned> deepest{0};
  std::atomic<int> timed_out{0};
};

GeoItem take_upper_half(GeoFrame& f, unsigned depth) {
  const int left = f.end - f.next;
  GeoItem it;
  for (int k = 0; k < 5; ++k) it.s[k] = f.s[k];
  it.depth = depth;
  it.first = (unsigned)(f.next + left / 2);
  it.end = (unsigned)f.end;
  return it;
}

}  // namespace

namespace {

// One host walker; `root` walks from the tree's root (host-only runs).
void host_walker(HostWalk& h, bool root) {
  unsigned* G = h.br.ctl;
  GeoFrame st[kGeoMaxDepth + 1];
  int sp = 0;
  unsigned base = 0, deepest = 0, batches = 0;
  unsigned long long nodes = 0, leaves = 0;
  bool busy = false;
  auto finish_side = [&]() {  // this walker's stack emptied
    if (h.work.fetch_sub(1u, std::memory_order_acq_rel) == 1u) h_add(G, 0xFFFFFFFFu);
  };
  if (root) {
    unsigned r[5];
    geo_root(h.seed, r);
    nodes = 1;
    const int m = geo_nchildren(r, 0, h.limit, h.table, h.nt);
    if (m == 0) {
      leaves = 1;
      finish_side();
    } else {
      for (int k = 0; k < 5; ++k) st[0].s[k] = r[k];
      st[0].next = 0;
      st[0].end = m;
      sp = 1;
      busy = true;
    }
  }
  bool counted_idle = false;
  auto t0 = std::chrono::steady_clock::now();
  unsigned long long last_sig = ~0ull;
  unsigned spins = 0;
  for (;;) {
    if (busy) {
      for (int step = 0; step < 64 && sp > 0; ++step) {
        GeoFrame& f = st[sp - 1];
        if (f.next == f.end) {
          --sp;
          continue;
        }
        unsigned c[5];
        geo_child(f.s, (unsigned)f.next, c);
        f.next += 1;
        const unsigned d = base + (unsigned)sp;
        ++nodes;
        if (d > deepest) deepest = d;
        const int m = geo_nchildren(c, (int)d, h.limit, h.table, h.nt);
        if (m == 0) {
          ++leaves;
        } else {
          GeoFrame& g = st[sp];
          for (int k = 0; k < 5; ++k) g.s[k] = c[k];
          g.next = 0;
          g.end = m;
          ++sp;
        }
      }
      if (sp == 0) {
        busy = false;
        finish_side();
        continue;
      }
      if ((++batches & 15u) == 0u) h_add(h.br.ctl + 224, 1u);  // heartbeat every 1024 nodes
      int f = 0;
      while (f < sp && st[f].end - st[f].next < 2) ++f;
      if (f == sp) continue;
      if (h_load_relaxed(h.br.ctl + 64) != 0u) {
        // GPU threads are idle: give them the upper half of the oldest frame
        const GeoItem it = take_upper_half(st[f], base + (unsigned)f);
        h_add(G, 1u);
        if (host_h2g_push(h.br, it)) {
          st[f].end = (int)it.first;
          __atomic_store_n(h.br.ctl + 64, 0u, __ATOMIC_RELAXED);
          h.to_gpu.fetch_add(1u, std::memory_order_relaxed);
        } else {
          h_add(G, 0xFFFFFFFFu);
        }
      } else if (h.queued.load(std::memory_order_relaxed) < h_load_relaxed(h.br.ctl + 32)) {
        const GeoItem it = take_upper_half(st[f], base + (unsigned)f);
        h.work.fetch_add(1u, std::memory_order_acq_rel);
        {
          std::lock_guard<std::mutex> g(h.qm);
          h.q.push_back(it);
          h.queued.store((unsigned)h.q.size(), std::memory_order_relaxed);
        }
        st[f].end = (int)it.first;
      }
      continue;
    }
    // idle: the host deque, then the GPU->host ring
    GeoItem it;
    bool got = false;
    {
      std::lock_guard<std::mutex> g(h.qm);
      if (!h.q.empty()) {
        it = h.q.front();
        h.q.pop_front();
        h.queued.store((unsigned)h.q.size(), std::memory_order_relaxed);
        got = true;
      }
    }
    if (!got && host_g2h_pop(h.br, it)) {
      got = true;
      h.to_host.fetch_add(1u, std::memory_order_relaxed);
      // the item's share of the global count becomes this side's, unless the side was active already
      if (h.work.fetch_add(1u, std::memory_order_acq_rel) != 0u) h_add(G, 0xFFFFFFFFu);
    }
    if (got) {
      if (counted_idle) {
        h_add(h.br.ctl + 32, 0xFFFFFFFFu);
        counted_idle = false;
      }
      for (int k = 0; k < 5; ++k) st[0].s[k] = it.s[k];
      st[0].next = (int)it.first;
      st[0].end = (int)it.end;
      base = it.depth;
      sp = 1;
      busy = true;
      last_sig = ~0ull;
      continue;
    }
    if (!counted_idle) {
      h_add(h.br.ctl + 32, 1u);
      counted_idle = true;
    }
    const unsigned g = h_load(G);
    if (g == 0u || h_load_relaxed(h.br.ctl + 96) != 0u) break;
    // bounded: the global count, this side's count or a heartbeat must move within the time limit
    const unsigned long long sig = ((unsigned long long)g << 32) ^ h.work.load(std::memory_order_relaxed) ^
                                   ((unsigned long long)h_load_relaxed(h.br.ctl + 192) << 12) ^
                                   ((unsigned long long)h_load_relaxed(h.br.ctl + 224) << 40);
    const auto now = std::chrono::steady_clock::now();
    if (sig != last_sig) {
      last_sig = sig;
      t0 = now;
    } else if ((unsigned long long)std::chrono::duration_cast<std::chrono::nanoseconds>(now - t0).count() >
               h.timeout_ns) {
      h.timed_out.store(1);
      __atomic_store_n(h.br.ctl + 96, 1u, __ATOMIC_RELEASE);
      break;
    }
    if (++spins & 63u) std::this_thread::yield();
    else std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  if (counted_idle) h_add(h.br.ctl + 32, 0xFFFFFFFFu);
  h.nodes.fetch_add(nodes);
  h.leaves.fetch_add(leaves);
  unsigned cur = h.deepest.load();
  while (deepest > cur && !h.deepest.compare_exchange_weak(cur, deepest)) {
  }
}

}  // namespace

extern "C" int hs_uts_geo_coop_run(unsigned seed, int depth_limit, double branching, int blocks, int threads,
                                   int host_threads, unsigned long long timeout_ns, hs_uts_coop_result* r) {
  if (!r) return HS_EINVAL;
  std::memset(r, 0, sizeof(*r));
  if (host_threads < 0) host_threads = std::max(1, (int)std::thread::hardware_concurrency() - 1);
  if (depth_limit < 0 || depth_limit > kGeoMaxDepth || !(branching > 0.0) || blocks < 0 || host_threads > 1024 ||
      blocks + host_threads == 0 || (blocks > 0 && (threads <= 0 || threads > 256 || (threads % 32)))) {
    g_gerr = "need 0 <= depth_limit <= 30, branching > 0, blocks >= 0, 0 <= host_threads <= 1024, a walker on "
             "some side, threads a multiple of 32 up to 256";
    return HS_EINVAL;
  }
  if (blocks > 0 && host_threads > 0) {
    int dev = 0, native = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&native, cudaDevAttrHostNativeAtomicSupported, dev) != cudaSuccess || !native) {
      cudaGetLastError();
      g_gerr = "the host link has no native atomics (cudaDevAttrHostNativeAtomicSupported is 0)";
      return HS_EINVAL;
    }
  }
  if (!timeout_ns) timeout_ns = 10000000000ull;
  uint32_t table[kGeoTable];
  const int nt = hs_uts_geo_table(branching, table, kGeoTable);

  // bridge: ctl (256 words), two rings of sequence numbers, two rings of items
  const size_t words = 256 + 2 * (size_t)kBridgeCap + 2 * (size_t)kBridgeCap * 8;
  std::vector<unsigned> host_only;
  unsigned* hb = nullptr;
  unsigned* hb_dev = nullptr;
  if (blocks > 0) {
    if (cudaHostAlloc((void**)&hb, words * 4, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&hb_dev, hb, 0) != cudaSuccess) {
      cudaGetLastError();
      if (hb) cudaFreeHost(hb);
      g_gerr = "cudaHostAlloc (mapped)";
      return HS_ENORES;
    }
  } else {
    host_only.assign(words, 0u);
    hb = host_only.data();
  }
  std::memset(hb, 0, words * 4);
  auto carve = [&](unsigned* p) {
    GeoBridge b;
    b.ctl = p;
    b.g2h_seq = p + 256;
    b.h2g_seq = p + 256 + kBridgeCap;
    b.g2h_item = reinterpret_cast<GeoItem*>(p + 256 + 2 * kBridgeCap);
    b.h2g_item = reinterpret_cast<GeoItem*>(p + 256 + 2 * kBridgeCap + 8 * kBridgeCap);
    b.dev = nullptr;
    return b;
  };
  HostWalk h;
  h.br = carve(hb);
  for (unsigned i = 0; i < kBridgeCap; ++i) h.br.g2h_seq[i] = h.br.h2g_seq[i] = i;
  h.br.ctl[0] = 1u;  // one active side: the one holding the root
  h.table = table;
  h.nt = nt;
  h.limit = depth_limit;
  h.seed = seed;
  h.timeout_ns = timeout_ns;
  if (blocks == 0) h.work.store(1u);  // host walker 0 holds the root
  std::atomic_thread_fence(std::memory_order_seq_cst);

  // device side (as hs_uts_geo_run, plus the bridge's device words)
  unsigned *d_seq = nullptr, *d_pos = nullptr, *d_ctl = nullptr, *d_table = nullptr, *d_bdev = nullptr;
  GeoItem* d_items = nullptr;
  auto release = [&]() {
    if (blocks > 0) {
      cudaFree(d_seq); cudaFree(d_items); cudaFree(d_pos); cudaFree(d_ctl); cudaFree(d_table); cudaFree(d_bdev);
      cudaFreeHost(hb);
    }
  };
  auto t_start = std::chrono::steady_clock::now();
  if (blocks > 0) {
    const size_t qcells = (size_t)blocks * kGeoQueueCap;
    if (cudaMalloc(&d_seq, qcells * 4) != cudaSuccess || cudaMalloc(&d_items, qcells * sizeof(GeoItem)) != cudaSuccess ||
        cudaMalloc(&d_pos, (size_t)blocks * 64 * 4) != cudaSuccess || cudaMalloc(&d_ctl, 256 * 4) != cudaSuccess ||
        cudaMalloc(&d_table, sizeof(table)) != cudaSuccess || cudaMalloc(&d_bdev, 128 * 4) != cudaSuccess) {
      cudaGetLastError();
      release();
      g_gerr = "cudaMalloc";
      return HS_ENORES;
    }
    std::vector<unsigned> seq0(qcells);
    for (size_t i = 0; i < qcells; ++i) seq0[i] = (unsigned)(i % kGeoQueueCap);
    cudaMemcpy(d_seq, seq0.data(), qcells * 4, cudaMemcpyHostToDevice);
    cudaMemset(d_pos, 0, (size_t)blocks * 64 * 4);
    cudaMemset(d_ctl, 0, 256 * 4);
    cudaMemset(d_bdev, 0, 128 * 4);
    const unsigned one = 1u;
    cudaMemcpy(d_ctl + 32, &one, 4, cudaMemcpyHostToDevice);  // the GPU's count: the root's thread
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
    a.nq = blocks;
    a.seed = seed;
    a.timeout_ns = timeout_ns;
    a.br = carve(hb_dev);
    a.br.dev = d_bdev;
    t_start = std::chrono::steady_clock::now();
    k_uts_geo_coop<<<blocks, threads>>>(a);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
      cudaDeviceSynchronize();
      release();
      g_gerr = cudaGetErrorString(le);
      return HS_ECUDA;
    }
    hs_note_launches(1);
  }
  std::vector<std::thread> pool;
  for (int i = 0; i < host_threads; ++i) {
    try {
      pool.emplace_back(host_walker, std::ref(h), blocks == 0 && i == 0);
    } catch (...) {
      break;  // fewer walkers: the others (and the GPU) balance the load
    }
  }
  const int ran = (int)pool.size();
  if (ran == 0 && blocks == 0) {  // walker 0 would have held the root: nothing ran
    g_gerr = "could not start a host thread";
    return HS_ENORES;
  }
  for (auto& t : pool) t.join();
  cudaError_t e = cudaSuccess;
  unsigned ctl[256] = {0};
  if (blocks > 0) {
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) cudaMemcpy(ctl, d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
  }
  const auto t_end = std::chrono::steady_clock::now();
  const unsigned g_end = h_load(h.br.ctl);
  release();
  if (e != cudaSuccess) {
    g_gerr = cudaGetErrorString(e);
    return HS_ECUDA;
  }
  const unsigned long long* o = reinterpret_cast<const unsigned long long*>(ctl + 128);
  r->gpu_nodes = o[0];
  r->host_nodes = h.nodes.load();
  r->nodes = r->gpu_nodes + r->host_nodes;
  r->leaves = o[8] + h.leaves.load();
  r->max_depth = std::max((unsigned)o[16], h.deepest.load());
  r->to_host = h.to_host.load();
  r->to_gpu = h.to_gpu.load();
  r->host_threads = ran;
  r->elapsed_ms = (float)std::chrono::duration<double, std::milli>(t_end - t_start).count();
  r->dev_error_bits = ctl[0];
  if (ctl[0] || h.timed_out.load() || g_end != 0u) {
    g_gerr = ctl[0] ? "device wait timed out" : h.timed_out.load() ? "host walker timed out"
                                                                    : "walk ended with work outstanding";
    return HS_ETIMEDOUT;
  }
  return HS_OK;
}
