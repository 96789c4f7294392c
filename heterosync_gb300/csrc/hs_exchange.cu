// hs_exchange.cu -- tree barrier with local exchange on thread-block clusters.
//
// The reference's LocalExch tree barriers (heterosync cuda/syncPrims/uvm/
// main.cu:153-211 atomic, 213-270 lock-free) alternate a data phase with a
// two-level barrier: a per-SM local barrier, the SM leaders' global barrier,
// and the local barrier again (joinBarrier_helper, cudaLocksBarrierAtomic.cu:
// 147-172; joinLFBarrier_helper, cudaLocksBarrierFast.cu:315-330), and in the
// exchange phase each TB works on data another TB produced.  On sm_103a the
// local level is a thread-block cluster: its barrier is the hardware cluster
// barrier and its data moves through distributed shared memory.
//
// Workload: n CTAs (n a multiple of the cluster size cl), each owning a buffer
// of `elems` 32-bit words kept in shared memory.  One episode rotates every
// buffer to the next CTA, b -> (b + 1) mod n, and ends with one tree barrier:
//   - within a cluster, rank r pushes its buffer into rank r+1's spare buffer
//     with one bulk copy shared::cta -> shared::cluster that completes on the
//     receiver's mbarrier;
//   - the cluster's last rank stores its buffer to an L2 staging slot with a
//     bulk store, for rank 0 of the next cluster;
//   - barrier: cluster barrier (local), the cluster leaders' global stage
//     (a generation counter: atomic tree; per-cluster flags scanned by one
//     master CTA: lock-free tree), cluster barrier (local release);
//   - rank 0 loads its new buffer from the staging slot with a bulk load.
// Staging slots alternate between two sets by episode parity, so a slot is
// rewritten only after the barrier that follows its read.  With cl = 1 every
// edge goes through L2 (the flat form the cluster form is compared against).
//
// The words are only moved, never interpreted, so the final buffers are the
// initial ones rotated by `episodes` (a bit-exact permutation).
#include <cuda_runtime.h>
#include <cstring>
#include <random>
#include <string>
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

void hs_note_launches(unsigned n);

namespace hs {

constexpr int kExchThreads = 256;

struct ExchDesc {
  const unsigned* in;     // n * elems
  unsigned* out;          // n * elems
  unsigned* staging;      // 2 * (n / cl) * elems
  unsigned* ctr;          // global counter (atomic tree), one line
  unsigned* flags;        // n / cl lines (lock-free tree) + the go line at the end
  unsigned* status;       // error bits, wait site
  int n, elems, episodes, lf;
  unsigned long long timeout_ns;
};

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned mapa_shared(unsigned addr, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}

__device__ __forceinline__ void mbar_expect(unsigned mbar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_load(unsigned dst_smem, const void* src, unsigned bytes, unsigned mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(dst_smem), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

__device__ __forceinline__ void bulk_store(void* dst, unsigned src_smem, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
               :: "l"(dst), "r"(src_smem), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

__device__ __forceinline__ bool mbar_wait(unsigned mbar, unsigned phase, const HsEnv& env) {
  return wait_until([&] {
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
    return done != 0;
  }, [] {}, env, HS_SITE_EXCH);
}

// Global stage of episode e among the ncl cluster leaders (rank-0 CTAs).
// Atomic tree: one release add per leader on a generation counter, then an
// acquire poll until it reaches (e + 1) * ncl (no resets: the count only grows).
// Lock-free tree: each leader release-stores e + 1 into its own flag line; the
// master CTA (cluster 0) scans all flags with its threads and release-stores
// e + 1 into the go line that the other leaders poll.
__device__ __forceinline__ bool exch_global(const ExchDesc& x, int cid, int ncl, unsigned e, const HsEnv& env) {
  const unsigned gen = e + 1u;
  if (!x.lf) {
    int ok = 1;
    if (is_master()) {
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" :: "l"(x.ctr) : "memory");
      const unsigned target = gen * (unsigned)ncl;
      ok = wait_until_p([&] { return (int)(ld_acquire<GPU>(x.ctr) - target) >= 0; },
                        [&] { return ld_relaxed<GPU>(x.ctr); }, [] {}, env, HS_SITE_BAR_GLOBAL);
    }
    return ok;
  }
  unsigned* go = x.flags + (size_t)ncl * kLineWords;
  if (is_master()) st_release<GPU>(x.flags + (size_t)cid * kLineWords, gen);
  if (cid == 0) {
    int ok = 1;
    for (int c = threadIdx.x; c < ncl && ok; c += blockDim.x)
      ok = wait_until([&] { return (int)(ld_acquire<GPU>(x.flags + (size_t)c * kLineWords) - gen) >= 0; }, [] {},
                      env, HS_SITE_BAR_SCAN);
    ok = __syncthreads_and(ok);
    if (is_master() && ok) st_release<GPU>(go, gen);
    return ok != 0;
  }
  int ok = 1;
  if (is_master())
    ok = wait_until([&] { return (int)(ld_acquire<GPU>(go) - gen) >= 0; }, [] {}, env, HS_SITE_BAR_GO);
  return ok;
}

__global__ void __launch_bounds__(kExchThreads) k_exchange(ExchDesc x) {
  extern __shared__ __align__(128) unsigned char exch_smem[];
  __shared__ __align__(8) unsigned long long s_mbar;
  const HsEnv env{x.status, x.timeout_ns};
  const int b = blockIdx.x;
  const int cl = (int)cluster_nctarank(), cr = (int)cluster_ctarank();
  const int ncl = x.n / cl, cid = b / cl;
  const unsigned bytes = (unsigned)x.elems * 4u;
  const unsigned buf0 = smem_addr(exch_smem), mbar = smem_addr(&s_mbar);
  if (is_master()) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // Thread 0 issues every copy and owns the mbarrier phase; `live` drops after
  // its first failed wait so that it issues and awaits nothing more.  Episode
  // e's incoming buffer completes mbarrier phase e + 1 (phase 0 is the initial
  // load).  (Receiving the cluster edge on a flag of its own, beside the global
  // stage, measured slower than letting the barrier carry the signal.)
  bool live = true;
  if (is_master()) {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    mbar_expect(mbar, bytes);
    bulk_load(buf0, x.in + (size_t)b * x.elems, bytes, mbar);
    live = mbar_wait(mbar, 0u, env);
  }
  cluster_sync_all();  // every mbarrier initialised before any peer completes on it
  for (int e = 0; e < x.episodes; ++e) {
    const unsigned cur = buf0 + (unsigned)(e & 1) * bytes, nxt = buf0 + (unsigned)((e + 1) & 1) * bytes;
    const unsigned parity = (unsigned)(e + 1) & 1u;
    unsigned* slot = x.staging + (size_t)(e & 1) * ncl * x.elems;
    if (is_master() && live) {
      mbar_expect(mbar, bytes);  // this episode's incoming buffer
      if (cr + 1 < cl) {
        asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     :: "r"(mapa_shared(nxt, (unsigned)cr + 1u)), "r"(cur), "r"(bytes),
                        "r"(mapa_shared(mbar, (unsigned)cr + 1u)) : "memory");
      } else {
        bulk_store(slot + (size_t)((cid + 1) % ncl) * x.elems, cur, bytes);
      }
      if (cr > 0) live = mbar_wait(mbar, parity, env);
    }
    cluster_sync_all();  // local stage: the cluster's pushes have landed, its edge store is done
    if (cr == 0) {
      const bool ok = exch_global(x, cid, ncl, (unsigned)e, env);
      if (is_master()) live = live && ok;
    }
    cluster_sync_all();  // local release
    if (cr == 0 && is_master() && live) {
      asm volatile("fence.proxy.async.global;" ::: "memory");
      bulk_load(nxt, slot + (size_t)cid * x.elems, bytes, mbar);
      live = mbar_wait(mbar, parity, env);
    }
  }
  if (is_master() && live) bulk_store(x.out + (size_t)b * x.elems, buf0 + (unsigned)(x.episodes & 1) * bytes, bytes);
  // A CTA that gave up may still receive a peer's push: let copies in flight
  // land before any CTA of the cluster exits.
  cluster_sync_all();
  if (ld_relaxed<GPU>(x.status) != 0u) __nanosleep(1000000);
  cluster_sync_all();
}

}  // namespace hs

using namespace hs;

namespace {
thread_local std::string g_xerr;
}

extern "C" const char* hs_exchange_last_error(void) { return g_xerr.c_str(); }

// Initial buffers: word i = bits of the fp32 value (int32)(r >> 40) * 2^-23 - 1
// for the i-th draw r of std::mt19937_64(seed): uniform in [-1, 1), exact.
extern "C" int hs_exchange_fill(unsigned long long seed, size_t words, uint32_t* out) {
  if (!out) return HS_EINVAL;
  std::mt19937_64 rng(seed);
  for (size_t i = 0; i < words; ++i) {
    const float f = (float)(int32_t)(rng() >> 40) * (1.0f / 8388608.0f) - 1.0f;
    std::memcpy(out + i, &f, 4);
  }
  return HS_OK;
}

extern "C" int hs_exchange_run(const uint32_t* host_in, uint32_t* host_out, int n, int elems, int cluster, int lf,
                               int episodes, unsigned long long timeout_ns, hs_exchange_result* r) {
  if (!r) return HS_EINVAL;
  std::memset(r, 0, sizeof(*r));
  if (!host_in || !host_out || n <= 0 || episodes < 0 || elems <= 0 || (elems % 4) != 0 ||
      elems * 8 > 200 * 1024 || (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8) || (n % cluster)) {
    g_xerr = "need n a multiple of the cluster size (1, 2, 4, 8), elems a positive multiple of 4 with "
             "2 * elems * 4 bytes <= 200 KB, episodes >= 0";
    return HS_EINVAL;
  }
  const int ncl = n / cluster;
  const size_t words = (size_t)n * elems;
  const size_t smem = (size_t)elems * 8;
  if (cudaFuncSetAttribute((const void*)k_exchange, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    g_xerr = "shared memory attribute";
    return HS_ECUDA;
  }
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3((unsigned)n);
  lc.blockDim = dim3((unsigned)kExchThreads);
  lc.dynamicSmemBytes = smem;
  lc.attrs = attr;
  lc.numAttrs = 1;
  int fit = 0;
  if (cudaOccupancyMaxActiveClusters(&fit, (const void*)k_exchange, &lc) != cudaSuccess) {
    cudaGetLastError();
    g_xerr = "cluster occupancy query failed";
    return HS_ECUDA;
  }
  if (fit < ncl) {  // every CTA waits on every other: all must be resident
    g_xerr = std::to_string(ncl) + " clusters of " + std::to_string(cluster) + " needed, " + std::to_string(fit) +
             " can be resident";
    return HS_ENORES;
  }
  unsigned *d_in = nullptr, *d_out = nullptr, *d_stage = nullptr, *d_sync = nullptr;
  const size_t sync_words = 64 + (size_t)(ncl + 1) * kLineWords;
  if (cudaMalloc(&d_in, words * 4) != cudaSuccess || cudaMalloc(&d_out, words * 4) != cudaSuccess ||
      cudaMalloc(&d_stage, (size_t)2 * ncl * elems * 4) != cudaSuccess ||
      cudaMalloc(&d_sync, sync_words * 4) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d_in); cudaFree(d_out); cudaFree(d_stage); cudaFree(d_sync);
    g_xerr = "cudaMalloc";
    return HS_ENORES;
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaMemcpy(d_in, host_in, words * 4, cudaMemcpyHostToDevice);
  cudaMemset(d_sync, 0, sync_words * 4);
  ExchDesc x;
  x.in = d_in;
  x.out = d_out;
  x.staging = d_stage;
  x.status = d_sync;
  x.ctr = d_sync + 32;
  x.flags = d_sync + 64;
  x.n = n;
  x.elems = elems;
  x.episodes = episodes;
  x.lf = lf ? 1 : 0;
  x.timeout_ns = timeout_ns ? timeout_ns : 10000000000ull;
  void* args[] = {&x};
  cudaEventRecord(a);
  cudaError_t e = cudaLaunchKernelExC(&lc, (const void*)k_exchange, args);
  cudaEventRecord(b);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  hs_note_launches(1);
  unsigned st[2] = {0, 0};
  if (e == cudaSuccess) {
    cudaEventElapsedTime(&r->elapsed_ms, a, b);
    cudaMemcpy(host_out, d_out, words * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(st, d_sync, sizeof(st), cudaMemcpyDeviceToHost);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d_in); cudaFree(d_out); cudaFree(d_stage); cudaFree(d_sync);
  if (e != cudaSuccess) {
    g_xerr = cudaGetErrorString(e);
    return HS_ECUDA;
  }
  r->dev_error_bits = st[0];
  r->wait_site = st[1];
  r->clusters = ncl;
  const double s = r->elapsed_ms * 1e-3;
  r->episodes_per_s = s > 0 ? episodes / s : 0.0;
  r->exchange_gbs = s > 0 ? 2.0 * (double)words * 4.0 * episodes / s * 1e-9 : 0.0;
  if (st[0]) {
    g_xerr = "device wait timed out";
    return HS_ETIMEDOUT;
  }
  return HS_OK;
}
