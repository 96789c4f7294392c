// hs_batch.cu -- many SyncPrims instances in one persistent launch.
//
// An instance is one run of one primitive (numTBs logical TBs, numLdSt,
// numCSIters) with its own storage and lock state.  The batch kernel gives
// instance i a gang of c_i co-resident CTAs and executes its numTBs logical TBs
// on them: logical TB b runs on gang CTA b mod c_i, and a CTA works through its
// logical TBs one operation at a time (iteration-major).  Synchronisation is the
// instance's own: each operation acquires and releases the instance's lock or
// semaphore; barrier instances join a counter barrier among the gang's CTAs
// after every data phase.  Nothing waits on a logical TB that is not running
// (a CTA takes a ticket, slot or semaphore only for the operation it is doing),
// so any gang sizes are deadlock-free; barrier gangs are co-resident because
// the whole grid is.
//
// The final storage of every instance equals the standalone run's (the same
// critical sections touch the same chunks the same number of times), which the
// tests check against the closed form of the reference golden.
//
// The launch (lock-state reset plus the persistent kernel) is captured once in
// a CUDA graph and replayed.  hs_batch_run_serial() is the comparison point:
// one standalone launch per instance on the same stream.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include "hs_exec.cuh"
#include "../../include/hs/hs.h"

void hs_note_launches(unsigned n);
int hs_layout_for(const hs_run_config* c, int nsm, hs::Layout* out);

namespace hs {
using KernelFn = void (*)(RunDesc);
KernelFn syncprim_plan(int prim, int mode, int threads, int num_ldst, size_t* smem_bytes, bool bulk = true);
cudaError_t prepare_smem(KernelFn fn, size_t smem_bytes);
cudaError_t launch_ring_init(unsigned* ring, unsigned slots_per_group, unsigned groups, cudaStream_t st);
cudaError_t launch_fill_lines(unsigned* base, size_t n, size_t stride, unsigned value, cudaStream_t st);

struct BatchInst {
  RunDesc d;
  int first_cta;  // first CTA of the gang
  int gang;       // CTAs in the gang
  int ecl;        // CTAs per executor: 1, or the cluster size (gang aligned to clusters)
  int index;      // instance number
};

// Staging bytes per CTA for the bulk-copy critical section (default).
constexpr unsigned kBatchBufSmall = 40u * 1024u;

template <int MODE>
__global__ void __launch_bounds__(256, 4) k_batch(const BatchInst* insts, int n_inst) {
  __shared__ int s_slot;
  __shared__ int s_inst;
  __shared__ int s_ok[9];  // [0] grant, [1 + rank] share succeeded
  __shared__ unsigned s_gen;
  __shared__ unsigned long long s_mbar;
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  TmaCtx tma;
  tma_init(tma, &s_mbar, dyn_smem);
  tma.cap = dyn_smem_bytes();
  const int cta = blockIdx.x;
  const int cl = (int)cluster_nctarank();
  const int cr = (int)cluster_ctarank();
  if (is_master()) {  // gang lookup: binary search over first_cta
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (insts[mid].first_cta <= cta) lo = mid;
      else hi = mid - 1;
    }
    s_inst = lo;
    s_gen = ld_relaxed<GPU>(insts[lo].d.locks + (size_t)(insts[lo].d.l_glob + 1) * kLineWords);
  }
  __syncthreads();
  const BatchInst& bi = insts[s_inst];
  const RunDesc d = bi.d;
  const int rank = cta - bi.first_cta, c = bi.gang;
  const HsEnv env{d.status, d.timeout_ns};
  if (rank >= 0 && rank < c) {
    if (is_relaxed_prim(d.prim)) {
      bool ok = true;
      for (int j = 0; j < d.iters && ok; ++j)
        for (int b = rank; b < d.num_tbs && ok; b += c) ok = relaxed_op(d, b, j, env);
    } else if (is_mutex_prim(d.prim) || is_sem_prim(d.prim)) {
      // one executor per ecl CTAs (a whole cluster, or one CTA); executor x
      // runs the logical TBs congruent to x
      const int ecl = bi.ecl, er = ecl == 1 ? 0 : cr;
      const int execs = c / ecl, x = rank / ecl;
      const bool mtx = is_mutex_prim(d.prim);
      bool ok = true;
      for (int j = 0; j < d.iters && ok; ++j)
        for (int b = x; b < d.num_tbs && ok; b += execs)
          ok = mtx ? cl_mutex_op<MODE>(d, b, er, ecl, &s_slot, s_ok, tma, env)
                   : cl_sem_op<MODE>(d, b, er, ecl, s_ok, tma, env);
    } else {
      batch_barrier<MODE>(d, rank, c, s_gen, tma, env);
    }
  }
  // no CTA of a cluster may exit while another rank can still read its shared memory
  cl_barrier(cl);
}

// One standalone launch of a relaxed-atomics instance: CTA b is logical TB b.
__global__ void __launch_bounds__(256) k_relaxed_inst(RunDesc d) {
  const HsEnv env{d.status, d.timeout_ns};
  for (int j = 0; j < d.iters; ++j)
    if (!relaxed_op(d, (int)blockIdx.x, j, env)) return;
}

}  // namespace hs

using namespace hs;

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct hs_batch {
  int n = 0, nsm = 0, threads = 256, mode = HS_MODE_INC;
  std::vector<hs_batch_instance> inst;
  std::vector<hs_run_config> cfg;
  std::vector<size_t> words;
  std::vector<Layout> lay;
  std::vector<BatchInst> host_desc;  // by instance
  std::vector<BatchInst> dev_order;  // by first CTA (the device copy)
  unsigned* storage = nullptr;   // all instances' storage, 256-byte aligned slices
  std::vector<size_t> st_off;    // word offsets
  unsigned* state = nullptr;     // all lock state, rings, sinks, status
  size_t state_words = 0;
  BatchInst* d_desc = nullptr;
  int grid = 0, v = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned graph_kernels = 0;
  unsigned stage = kBatchBufSmall;  // staging bytes per CTA
  int cl = 1, serial_execs = 0;
  unsigned bo_min = 1, bo_max = 1024;  // EBO bounds of the batched launch (the per-launch form keeps 1..1024)
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace {
thread_local std::string g_berr;
size_t round64(size_t w) { return (w + 63) / 64 * 64; }
bool is_barrier_p(int p) { return p >= 0 && p <= 3; }
bool is_usem_p(int p) { return p >= 24 && p <= 31; }
}  // namespace

extern "C" const char* hs_batch_last_error(void) { return g_berr.c_str(); }

static bool relaxed_kind(int p) { return p >= HS_BATCH_REFCOUNTER && p <= HS_BATCH_FLAGS; }

// Storage words of one instance (SyncPrims: the reference's storage; the
// relaxed kinds: their counters, payload and data words).
extern "C" int hs_batch_instance_words(const hs_batch_instance* x, int nsm, size_t* words) {
  if (!x || !words || nsm <= 0 || x->num_tbs <= 0 || x->num_iters <= 0 || x->num_ldst <= 0) return HS_EINVAL;
  switch (x->prim) {
    case HS_BATCH_REFCOUNTER: *words = 2 * (size_t)x->num_ldst; return HS_OK;
    case HS_BATCH_SPLITCOUNTER: *words = 2 * (size_t)nsm; return HS_OK;
    case HS_BATCH_SEQLOCK: *words = 9; return HS_OK;
    case HS_BATCH_FLAGS: *words = (size_t)x->num_ldst + 1; return HS_OK;
    default: break;
  }
  hs_run_config c;
  hs_run_config_default(&c);
  c.prim = x->prim;
  c.num_ldst = x->num_ldst;
  c.num_tbs = x->num_tbs;
  c.num_iters = x->num_iters;
  c.threads = 256;
  c.repeats = 1;
  c.mode = HS_MODE_INC;
  return hs_storage_words(&c, nsm, words);
}

static unsigned long long seq_pattern_host(unsigned seq, int i) {
  return (unsigned long long)seq * 0x9E3779B97F4A7C15ull + (unsigned long long)i;
}

// Final storage of one instance after one run at 256 threads per TB, from its
// initial storage (the closed forms of the operations in hs_exec.cuh).
extern "C" int hs_batch_expected_storage(const hs_batch_instance* x, int nsm, int mode, const uint32_t* init,
                                         uint32_t* out, size_t words) {
  size_t need = 0;
  int s = hs_batch_instance_words(x, nsm, &need);
  if (s) return s;
  if (!init || !out || words < need) return HS_EINVAL;
  const int T = 256, L = x->num_ldst, G = x->num_tbs, I = x->num_iters;
  std::memcpy(out, init, need * 4);
  switch (x->prim) {
    case HS_BATCH_REFCOUNTER: {
      // total[k] += #{(b, j, t) : (b + j + t) mod L == k}
      std::vector<unsigned long long> bj(L, 0), tt(L, 0);
      for (long long v = 0; v <= (long long)G - 1 + I - 1; ++v) {
        const long long lo_b = std::max(0LL, v - (I - 1)), hi_b = std::min((long long)G - 1, v);
        if (hi_b >= lo_b) bj[v % L] += (unsigned long long)(hi_b - lo_b + 1);
      }
      for (int t = 0; t < T; ++t) tt[t % L] += 1;
      for (int k = 0; k < L; ++k) {
        unsigned long long n = 0;
        for (int r = 0; r < L; ++r) n += bj[r] * tt[((k - r) % L + L) % L];
        out[L + k] = init[L + k] + (uint32_t)n;
      }
      return HS_OK;
    }
    case HS_BATCH_SPLITCOUNTER: {
      for (int sm = 0; sm < nsm; ++sm) {
        const unsigned long long tbs = (unsigned long long)(G / nsm + (sm < G % nsm ? 1 : 0));
        unsigned long long v = (unsigned long long)init[2 * sm] | ((unsigned long long)init[2 * sm + 1] << 32);
        v += tbs * (unsigned long long)I * (unsigned long long)T * (unsigned long long)L;
        out[2 * sm] = (uint32_t)v;
        out[2 * sm + 1] = (uint32_t)(v >> 32);
      }
      return HS_OK;
    }
    case HS_BATCH_SEQLOCK: {
      const unsigned writers = (unsigned)((G + 3) / 4);
      const unsigned seq = 2u * writers * (unsigned)I;
      for (int i = 0; i < 4; ++i) {
        const unsigned long long p = seq_pattern_host(seq, i);
        out[2 * i] = (uint32_t)p;
        out[2 * i + 1] = (uint32_t)(p >> 32);
      }
      return HS_OK;  // torn-read count (word 8) unchanged
    }
    case HS_BATCH_FLAGS:
      for (int k = 0; k < L; ++k) out[k] = (uint32_t)I;
      return HS_OK;  // violation count (word L) unchanged
    default: {
      hs_run_config c;
      hs_run_config_default(&c);
      c.prim = x->prim;
      c.num_ldst = L;
      c.num_tbs = G;
      c.num_iters = I;
      c.threads = T;
      c.repeats = 1;
      c.mode = mode;
      return hs_expected_storage(&c, nsm, init, out, words);
    }
  }
}

// The mixed batch: instances drawn from std::mt19937_64(seed) in the order
// primitive, numTBs, numLdSt, numCSIters; u = (draw >> 11) * 2^-53.
// primitive uniform over the 28 SyncPrims and the four relaxed-atomics kinds
// (RefCounter, SplitCounter, Seqlock, Flags), numTBs = round(exp(U(ln 4, ln 512))),
// numLdSt = 1 + floor(128 u), numCSIters = 10 + floor(4991 u) divided by
// iter_div (>= 1).  Barrier and per-SM-semaphore instances with numTBs above
// NUM_SM are rounded to a multiple of NUM_SM (the reference defines those only
// for whole SM groups: README.txt:80, main.cu:1775-1786).
extern "C" int hs_batch_generate(unsigned long long seed, int n, int nsm, int iter_div, hs_batch_instance* out) {
  static const int prims[32] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15,
                                20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31,
                                HS_BATCH_REFCOUNTER, HS_BATCH_SPLITCOUNTER, HS_BATCH_SEQLOCK, HS_BATCH_FLAGS};
  if (n <= 0 || nsm <= 0 || !out) return HS_EINVAL;
  if (iter_div < 1) iter_div = 1;
  std::mt19937_64 rng(seed);
  auto u = [&] { return (double)(rng() >> 11) * (1.0 / 9007199254740992.0); };
  for (int i = 0; i < n; ++i) {
    hs_batch_instance& x = out[i];
    x.prim = prims[std::min(31, (int)(u() * 32.0))];
    int G = (int)std::lround(std::exp(std::log(4.0) + u() * (std::log(512.0) - std::log(4.0))));
    if ((is_barrier_p(x.prim) || is_usem_p(x.prim)) && G > nsm) G = std::max(1, (int)std::lround((double)G / nsm)) * nsm;
    x.num_tbs = G;
    x.num_ldst = 1 + std::min(127, (int)(u() * 128.0));
    x.num_iters = std::max(1, (10 + std::min(4990, (int)(u() * 4991.0))) / iter_div);
  }
  return HS_OK;
}

extern "C" int hs_batch_create(const hs_batch_instance* inst, int n, int threads, int mode, hs_batch** out) {
  if (!inst || n <= 0 || !out || threads != 256 || (mode != HS_MODE_INC && mode != HS_MODE_REF)) {
    g_berr = "need instances, 256 threads per TB and HS_MODE_INC or HS_MODE_REF";
    return HS_EINVAL;
  }
  hs_batch* B = new hs_batch();
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, dev);
  B->n = n;
  B->threads = threads;
  B->mode = mode;
  B->inst.assign(inst, inst + n);
  size_t st_total = 0, state_total = 0;
  std::vector<size_t> state_off;
  for (int i = 0; i < n; ++i) {
    hs_run_config c;
    hs_run_config_default(&c);
    c.prim = inst[i].prim;
    c.num_ldst = inst[i].num_ldst;
    c.num_tbs = inst[i].num_tbs;
    c.num_iters = inst[i].num_iters;
    c.threads = threads;
    c.repeats = 1;
    c.mode = mode;
    size_t w = 0;
    Layout L;
    if (relaxed_kind(c.prim)) {
      int s = hs_batch_instance_words(&inst[i], B->nsm, &w);
      if (s) { g_berr = "bad relaxed-atomics instance"; delete B; return s; }
      std::memset(&L, 0, sizeof(L));
      L.l_glob = 0;
      L.l_grp = 4;  // line 4: seqlock sequence / flags word
      L.groups = 1;
      L.lines = 8;
    } else {
      int s = hs_storage_words(&c, B->nsm, &w);
      if (s) { g_berr = hs_last_error(); delete B; return s; }
      hs_layout_for(&c, B->nsm, &L);
    }
    B->cfg.push_back(c);
    B->words.push_back(w);
    B->lay.push_back(L);
    B->st_off.push_back(st_total);
    st_total += round64(w);
    state_off.push_back(state_total);
    state_total += 64 + round64((size_t)L.lines * kLineWords) + round64(L.ring_words) + round64((size_t)c.num_tbs);
  }
  if (cudaMalloc(&B->storage, st_total * 4 + 256) != cudaSuccess ||
      cudaMalloc(&B->state, state_total * 4 + 256) != cudaSuccess ||
      cudaMalloc(&B->d_desc, sizeof(BatchInst) * n) != cudaSuccess) {
    cudaGetLastError();
    g_berr = "cudaMalloc";
    hs_batch_destroy(B);
    return HS_ENORES;
  }
  cudaMemset(B->storage, 0, st_total * 4);
  B->state_words = state_total;
  for (int i = 0; i < n; ++i) {
    const Layout& L = B->lay[i];
    const hs_run_config& c = B->cfg[i];
    RunDesc d;
    std::memset(&d, 0, sizeof(d));
    unsigned* base = B->state + state_off[i];
    d.status = base;
    d.locks = base + 64;
    d.ring = d.locks + round64((size_t)L.lines * kLineWords);
    d.sink = d.ring + round64(L.ring_words);
    d.data = B->storage + B->st_off[i];
    d.prim = c.prim;
    d.mode = c.mode;
    d.T = c.threads;
    d.L = c.num_ldst;
    d.num_tbs = c.num_tbs;
    d.iters = c.num_iters;
    d.nsm = B->nsm;
    d.sem_max = relaxed_kind(c.prim) ? 1u : (unsigned)hs_prim_sem_count(c.prim) + 1u;
    d.bo_min = 1;
    d.bo_max = 1024;
    d.bo_unit = 0;
    d.ring_max = (unsigned)c.num_tbs;
    d.timeout_ns = 10000000000ull;
    d.skip_tb = -1;
    d.cluster = 1;
    d.l_glob = L.l_glob;
    d.l_gflag = L.l_gflag;
    d.l_grp = L.l_grp;
    d.l_lflag = L.l_lflag;
    d.lflag_lines = L.lflag_lines;
    BatchInst bi;
    bi.d = d;
    bi.first_cta = 0;
    bi.gang = 1;
    bi.ecl = 1;
    bi.index = i;
    B->host_desc.push_back(bi);
  }
  cudaEventCreate(&B->e0);
  cudaEventCreate(&B->e1);
  *out = B;
  return HS_OK;
}

extern "C" int hs_batch_destroy(hs_batch* B) {
  if (!B) return HS_EINVAL;
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  cudaFree(B->storage);
  cudaFree(B->state);
  cudaFree(B->d_desc);
  if (B->e0) cudaEventDestroy(B->e0);
  if (B->e1) cudaEventDestroy(B->e1);
  delete B;
  return HS_OK;
}

extern "C" int hs_batch_set_storage(hs_batch* B, int i, const uint32_t* host) {
  if (!B || i < 0 || i >= B->n) return HS_EINVAL;
  return cudaMemcpy(B->storage + B->st_off[i], host, B->words[i] * 4, cudaMemcpyHostToDevice) == cudaSuccess
             ? HS_OK : HS_ECUDA;
}
extern "C" int hs_batch_get_storage(hs_batch* B, int i, uint32_t* host) {
  if (!B || i < 0 || i >= B->n) return HS_EINVAL;
  return cudaMemcpy(host, B->storage + B->st_off[i], B->words[i] * 4, cudaMemcpyDeviceToHost) == cudaSuccess
             ? HS_OK : HS_ECUDA;
}
extern "C" size_t hs_batch_storage_words(hs_batch* B, int i) {
  return (!B || i < 0 || i >= B->n) ? 0 : B->words[i];
}

// Lock-state reset of every instance (semaphore counts, ring slots).
static int reset_state(hs_batch* B, cudaStream_t st, unsigned* launches) {
  if (cudaMemsetAsync(B->state, 0, B->state_words * 4, st) != cudaSuccess) return HS_ECUDA;
  for (int i = 0; i < B->n; ++i) {
    const RunDesc& d = B->host_desc[i].d;
    if (d.sem_max > 1u) {
      if (launch_fill_lines(d.locks + (size_t)B->lay[i].l_grp * kLineWords, (size_t)B->lay[i].groups,
                            (size_t)4 * kLineWords, d.sem_max, st) != cudaSuccess)
        return HS_ECUDA;
      ++*launches;
    }
    if (d.prim == 6 || d.prim == 22) {
      if (launch_ring_init(d.ring, d.ring_max + 1u, d.prim == 22 ? (unsigned)B->nsm : 1u, st) != cudaSuccess)
        return HS_ECUDA;
      ++*launches;
    }
  }
  return HS_OK;
}

static int read_statuses(hs_batch* B, hs_batch_result* r) {
  for (int i = 0; i < B->n; ++i) {
    unsigned h[2] = {0, 0};
    cudaMemcpy(h, B->host_desc[i].d.status, sizeof(h), cudaMemcpyDeviceToHost);
    if (h[0]) {
      r->dev_error_bits = h[0];
      r->failed_instance = i;
      g_berr = "instance " + std::to_string(i) + " device wait timed out";
      return HS_ETIMEDOUT;
    }
  }
  return HS_OK;
}

static unsigned long long total_ops(const hs_batch* B) {
  unsigned long long o = 0;
  for (const auto& c : B->cfg) o += (unsigned long long)c.num_tbs * c.num_iters;
  return o;
}

// Gang plan.  cl: thread-block cluster size of the launch; serial_execs:
// executors of the heaviest instance whose operations serialise on one lock or
// semaphore (global mutexes and semaphores; 0 = ceil(numTBs / v) for each);
// v: logical TBs per executor for the other instances (per-SM locks and
// semaphores, barriers).  Returns HS_ENORES if the gangs cannot be co-resident.
static bool serialized_prim(int p) { return p >= 4 && p <= 15; }
static double cs_work(const hs_run_config& c) { return (double)c.num_tbs * c.num_iters * (c.num_ldst + 1); }
// Below this many loads/stores per thread the two cluster barriers of an
// operation cost more than splitting its critical section saves.
constexpr int kClusterMinLdSt = 33;

extern "C" int hs_batch_plan_ex(hs_batch* B, int cl, int serial_execs, int v, int* grid_out, int* capacity_out) {
  if (!B || v <= 0 || cl < 1 || cl > 8 || (cl & (cl - 1))) return HS_EINVAL;
  auto fn = B->mode == HS_MODE_INC ? k_batch<M_INC> : k_batch<M_REF>;
  if (B->stage > 48u * 1024u &&
      cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B->stage) != cudaSuccess)
    return HS_ECUDA;
  int cap = 0;
  if (cl == 1) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, B->threads, B->stage) != cudaSuccess)
      return HS_ECUDA;
    cap = per_sm * B->nsm;
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(cl * 64));
    cfg.blockDim = dim3((unsigned)B->threads);
    cfg.dynamicSmemBytes = B->stage;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, (const void*)fn, &cfg) != cudaSuccess) {
      cudaGetLastError();
      return HS_ECUDA;
    }
    cap = clusters * cl;
  }
  // Serialised instances share serial_execs executors in proportion to their
  // critical-section work numTBs * numCSIters * (numLdSt + 1) (the heaviest
  // gets serial_execs); those with numLdSt >= kClusterMinLdSt execute as whole
  // clusters.  Cluster-executed gangs are placed first (aligned), one-CTA
  // executors after them, packed.
  double wmax = 0.0;
  for (int i = 0; i < B->n; ++i)
    if (serialized_prim(B->cfg[i].prim)) wmax = std::max(wmax, cs_work(B->cfg[i]));
  std::vector<int> execs(B->n), ecl(B->n);
  for (int i = 0; i < B->n; ++i) {
    const hs_run_config& c = B->cfg[i];
    const int G = c.num_tbs;
    int e = (G + v - 1) / v;
    ecl[i] = 1;
    if (serialized_prim(c.prim)) {
      if (serial_execs > 0) e = (int)std::lround(serial_execs * cs_work(c) / wmax);
      if (cl > 1 && c.num_ldst >= kClusterMinLdSt) ecl[i] = cl;
    }
    execs[i] = std::max(1, std::min(G, e));
  }
  int grid = 0;
  for (int pass = 0; pass < 2; ++pass)
    for (int i = 0; i < B->n; ++i) {
      if ((ecl[i] > 1) != (pass == 0)) continue;
      B->host_desc[i].first_cta = grid;
      B->host_desc[i].gang = execs[i] * ecl[i];
      B->host_desc[i].ecl = ecl[i];
      grid += execs[i] * ecl[i];
    }
  grid = (grid + cl - 1) / cl * cl;  // the tail's idle CTAs complete the last cluster
  if (capacity_out) *capacity_out = cap;
  if (grid_out) *grid_out = grid;
  if (grid > cap) {
    g_berr = "gangs need " + std::to_string(grid) + " co-resident CTAs, capacity " + std::to_string(cap);
    return HS_ENORES;
  }
  if (B->exec) { cudaGraphExecDestroy(B->exec); B->exec = nullptr; }
  if (B->graph) { cudaGraphDestroy(B->graph); B->graph = nullptr; }
  B->grid = grid;
  B->v = v;
  B->cl = cl;
  B->serial_execs = serial_execs;
  B->dev_order = B->host_desc;
  for (auto& x : B->dev_order) {
    x.d.bo_min = B->bo_min;
    x.d.bo_max = B->bo_max;
  }
  std::sort(B->dev_order.begin(), B->dev_order.end(),
            [](const BatchInst& x, const BatchInst& y) { return x.first_cta < y.first_cta; });
  if (cudaMemcpy(B->d_desc, B->dev_order.data(), sizeof(BatchInst) * B->n, cudaMemcpyHostToDevice) != cudaSuccess)
    return HS_ECUDA;
  return HS_OK;
}

// Gangs of ceil(numTBs / v) CTAs, no clusters.
extern "C" int hs_batch_plan(hs_batch* B, int v, int* grid_out, int* capacity_out) {
  return hs_batch_plan_ex(B, 1, 0, v, grid_out, capacity_out);
}

// Capture (once per plan) and replay: lock-state reset + the persistent kernel.
extern "C" int hs_batch_run(hs_batch* B, void* stream, hs_batch_result* r) {
  std::memset(r, 0, sizeof(*r));
  r->failed_instance = -1;
  if (!B || !B->grid) { g_berr = "call hs_batch_plan first"; return HS_EINVAL; }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned launches = 0;
  if (!B->exec) {
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return HS_ECUDA;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return HS_ECUDA;
    unsigned n_init = 0;
    int s = reset_state(B, cap, &n_init);
    const BatchInst* dd = B->d_desc;
    int ni = B->n;
    void* args[] = {&dd, &ni};
    const void* fn = B->mode == HS_MODE_INC ? (const void*)k_batch<M_INC> : (const void*)k_batch<M_REF>;
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)B->cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.gridDim = dim3((unsigned)B->grid);
    lc.blockDim = dim3((unsigned)B->threads);
    lc.dynamicSmemBytes = B->stage;
    lc.stream = cap;
    lc.attrs = attr;
    lc.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelExC(&lc, fn, args);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (s || e != cudaSuccess || e2 != cudaSuccess) {
      g_berr = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
      if (g) cudaGraphDestroy(g);
      return HS_ECUDA;
    }
    B->graph = g;
    B->graph_kernels = n_init + 1u;
    if (cudaGraphInstantiate(&B->exec, g, 0) != cudaSuccess) { g_berr = "graph instantiate"; return HS_ECUDA; }
  }
  launches = B->graph_kernels;
  cudaEventRecord(B->e0, st);
  if (cudaGraphLaunch(B->exec, st) != cudaSuccess) return HS_ECUDA;
  cudaEventRecord(B->e1, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) { g_berr = "batch kernel failed"; return HS_ECUDA; }
  hs_note_launches(launches);
  cudaEventElapsedTime(&r->elapsed_ms, B->e0, B->e1);
  r->launches = launches;
  r->ops = total_ops(B);
  r->grid = B->grid;
  r->tbs_per_cta = B->v;
  return read_statuses(B, r);
}

// The comparison point: one standalone launch per instance, same stream.
extern "C" int hs_batch_run_serial(hs_batch* B, void* stream, hs_batch_result* r) {
  std::memset(r, 0, sizeof(*r));
  r->failed_instance = -1;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned launches = 0;
  if (reset_state(B, st, &launches)) return HS_ECUDA;
  std::vector<KernelFn> fns(B->n);
  std::vector<size_t> smem(B->n);
  for (int i = 0; i < B->n; ++i) {
    if (relaxed_kind(B->cfg[i].prim)) {
      fns[i] = k_relaxed_inst;
      smem[i] = 0;
      continue;
    }
    fns[i] = syncprim_plan(B->cfg[i].prim, B->cfg[i].mode, B->threads, B->cfg[i].num_ldst, &smem[i]);
    if (!fns[i] || prepare_smem(fns[i], smem[i]) != cudaSuccess) { g_berr = "no kernel"; return HS_EINVAL; }
  }
  cudaEventRecord(B->e0, st);
  for (int i = 0; i < B->n; ++i) {
    RunDesc d = B->host_desc[i].d;
    void* args[] = {&d};
    if (cudaLaunchKernel((const void*)fns[i], dim3(B->cfg[i].num_tbs), dim3(B->threads), args, smem[i], st) !=
        cudaSuccess)
      return HS_ECUDA;
    ++launches;
  }
  cudaEventRecord(B->e1, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) { g_berr = "serial launches failed"; return HS_ECUDA; }
  hs_note_launches(launches);
  cudaEventElapsedTime(&r->elapsed_ms, B->e0, B->e1);
  r->launches = launches;
  r->ops = total_ops(B);
  return read_statuses(B, r);
}

// Staging bytes per CTA for the bulk-copy critical section (0: the largest
// instance chunk, i.e. whole-chunk copies).  Invalidates the plan.
extern "C" int hs_batch_set_stage(hs_batch* B, unsigned bytes) {
  if (!B) return HS_EINVAL;
  size_t mx = 1024;
  for (const auto& c : B->cfg) mx = std::max(mx, (size_t)c.threads * (c.num_ldst + 1) * 4);
  if (bytes == 0) bytes = (unsigned)mx;
  bytes = (bytes + 127u) / 128u * 128u;
  if (bytes > kTmaMaxBytes) { g_berr = "staging buffer above the shared-memory limit"; return HS_EINVAL; }
  B->stage = bytes;
  B->grid = 0;
  if (B->exec) { cudaGraphExecDestroy(B->exec); B->exec = nullptr; }
  if (B->graph) { cudaGraphDestroy(B->graph); B->graph = nullptr; }
  return HS_OK;
}
extern "C" unsigned hs_batch_get_stage(hs_batch* B) { return B ? B->stage : 0u; }

// Autotuner: for staging sizes 40 and 56 KB (four or three CTAs per SM),
// cluster sizes 1, 2, 4, 8 and 8 to 32 executors for the heaviest serialised
// instance, take the smallest v (1, 2, 4, ...) whose gangs fit, time one replay
// on a copy of the initial storage and keep the fastest plan; then, for that
// plan, the exponential-backoff bounds: start (I_min) 1, 8 or 64 ns and cap
// (I_max) 1024, 256 or 32 ns.  The executor CTA stays one logical TB of 256
// threads: its critical sections split their work by the TB's own threads.
extern "C" int hs_batch_autotune(hs_batch* B, void* stream, int* best_v, float* best_ms) {
  if (!B) return HS_EINVAL;
  std::vector<std::vector<uint32_t>> saved(B->n);
  for (int i = 0; i < B->n; ++i) {
    saved[i].resize(B->words[i]);
    hs_batch_get_storage(B, i, saved[i].data());
  }
  int max_g = 1;
  for (const auto& c : B->cfg) max_g = std::max(max_g, c.num_tbs);
  float best_t = 1e30f;
  int bcl = 0, bse = 0, bv = 0;
  unsigned bstage = B->stage, bbo = B->bo_max;
  auto trial = [&]() -> float {
    hs_batch_result r;
    const int s = hs_batch_run(B, stream, &r);
    for (int i = 0; i < B->n; ++i) hs_batch_set_storage(B, i, saved[i].data());
    return s == HS_OK ? r.elapsed_ms : 1e30f;
  };
  // staging size (four or three CTAs per SM), cluster size, executors of the
  // heaviest serialised instance; smallest v that fits
  for (unsigned stage : {40u * 1024u, 56u * 1024u}) {
    if (hs_batch_set_stage(B, stage) != HS_OK) continue;
    for (int cl : {1, 2, 4, 8}) {
      for (int se : {8, 16, 32}) {
        int v = 1;
        while (v <= max_g && hs_batch_plan_ex(B, cl, se, v, nullptr, nullptr) != HS_OK) v *= 2;
        if (v > max_g) continue;
        const float t = trial();
        if (t < best_t) { best_t = t; bcl = cl; bse = se; bv = v; bstage = stage; }
      }
    }
  }
  if (!bcl) { g_berr = "no plan fits"; return HS_ENORES; }
  // exponential-backoff start and cap for the winner (the default 1 / 1024 was timed above)
  hs_batch_set_stage(B, bstage);
  const unsigned timed_min = B->bo_min, timed_max = B->bo_max;  // the bounds the plans above ran with
  unsigned bmin = timed_min;
  for (unsigned cap : {1024u, 256u, 32u}) {
    for (unsigned lo : {1u, 8u, 64u}) {
      if (lo >= cap || (lo == timed_min && cap == timed_max)) continue;
      if (hs_batch_set_backoff(B, lo, cap) != HS_OK) continue;
      if (hs_batch_plan_ex(B, bcl, bse, bv, nullptr, nullptr) != HS_OK) continue;
      const float t = trial();
      if (t < best_t) { best_t = t; bbo = cap; bmin = lo; }
    }
  }
  hs_batch_set_backoff(B, bmin, bbo);
  hs_batch_plan_ex(B, bcl, bse, bv, nullptr, nullptr);
  if (best_v) *best_v = bv;
  if (best_ms) *best_ms = best_t;
  return HS_OK;
}

// Exponential-backoff bounds of the batched launch (EBO mutexes and
// semaphores; bo_max a power of two).  Invalidates the plan.
extern "C" int hs_batch_set_backoff(hs_batch* B, unsigned bo_min, unsigned bo_max) {
  if (!B || bo_min == 0 || bo_max < 2 || (bo_max & (bo_max - 1))) return HS_EINVAL;
  B->bo_min = bo_min;
  B->bo_max = bo_max;
  B->grid = 0;
  if (B->exec) { cudaGraphExecDestroy(B->exec); B->exec = nullptr; }
  if (B->graph) { cudaGraphDestroy(B->graph); B->graph = nullptr; }
  return HS_OK;
}
extern "C" int hs_batch_get_backoff(hs_batch* B, unsigned* bo_min, unsigned* bo_max) {
  if (!B) return HS_EINVAL;
  if (bo_min) *bo_min = B->bo_min;
  if (bo_max) *bo_max = B->bo_max;
  return HS_OK;
}

extern "C" int hs_batch_get_plan(hs_batch* B, int* cl, int* serial_execs, int* v, int* grid) {
  if (!B) return HS_EINVAL;
  if (cl) *cl = B->cl;
  if (serial_execs) *serial_execs = B->serial_execs;
  if (v) *v = B->v;
  if (grid) *grid = B->grid;
  return HS_OK;
}
