// hs_api.cu -- host runtime behind include/hs/hs.h: name table, storage sizing,
// lock-state allocation and initialisation, launches, timing, status readback,
// and the reference's host API (cudaLocksInit & co.).
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "hs_internal.h"
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

namespace hs {
using KernelFn = void (*)(RunDesc);
KernelFn syncprim_plan(int prim, int mode, int threads, int num_ldst, size_t* smem_bytes, bool bulk = true);
cudaError_t prepare_smem(KernelFn fn, size_t smem_bytes);
size_t barrier_tile_bytes(int threads, int num_ldst, int num_tbs, int phys_nsm, size_t base);
KernelFn prim_cluster_kernel(int mode);
KernelFn barrier_group_kernel(int prim, int mode);
KernelFn barrier_group_tma_kernel(int prim, int mode);
cudaError_t launch_ring_init(unsigned* ring, unsigned slots_per_group, unsigned groups, cudaStream_t st);
cudaError_t launch_fill_lines(unsigned* base, size_t n, size_t stride, unsigned value, cudaStream_t st);
}  // namespace hs

using namespace hs;

static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};

void hs_note_launches(unsigned n) { g_launches += n; }

static int set_cuda_err(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return HS_ECUDA;
}
#define HS_CK(call)                                   \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return set_cuda_err(e_, #call); \
  } while (0)

extern "C" int hs_version(void) { return 1; }
extern "C" const char* hs_last_error(void) { return g_err.c_str(); }
extern "C" const char* hs_status_string(int s) {
  switch (s) {
    case HS_OK: return "ok";
    case HS_EINVAL: return "invalid argument";
    case HS_ETIMEDOUT: return "device wait timed out";
    case HS_ENORES: return "not enough resources (co-residency or memory)";
    case HS_ECUDA: return "CUDA error";
    case HS_ENODEV: return "no CUDA device";
    case HS_EMISMATCH: return "results differ from expected";
    default: return "unknown status";
  }
}
extern "C" unsigned long long hs_launch_count(void) { return g_launches.load(); }

extern "C" int hs_device_info(int device, int* nsm, int* cc_major, int* cc_minor, int* max_tpb) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    g_err = "no CUDA device";
    return HS_ENODEV;
  }
  if (device < 0 || device >= n) return HS_EINVAL;
  cudaDeviceProp p;
  HS_CK(cudaGetDeviceProperties(&p, device));
  if (nsm) *nsm = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  if (max_tpb) *max_tpb = p.maxThreadsPerBlock;
  return HS_OK;
}

// ---------------------------------------------------------------------------
// Names and labels: main.cu:1224-1256 (names), 1352-1451 (labels, including the
// reference's "002" printed for the 120-count spin semaphores).
// ---------------------------------------------------------------------------
struct PrimInfo {
  int id;
  const char* name;
  const char* label;  // printf format; semaphores take (count, iters)
  int label_count;    // semaphore count printed in the label
  int sem_count;
};
static const PrimInfo kPrims[] = {
    {0, "atomicTreeBarrUniq", "atomic_tree_barrier_%03d", 0, 0},
    {1, "atomicTreeBarrUniqLocalExch", "atomic_tree_barrier_localExch_%03d", 0, 0},
    {2, "lfTreeBarrUniq", "fbs_tree_barrier_%03d", 0, 0},
    {3, "lfTreeBarrUniqLocalExch", "fbs_tree_barrier_localExch_%03d", 0, 0},
    {4, "spinMutex", "spin_lock_mutex_%03d", 0, 0},
    {5, "spinMutexEBO", "ebo_mutex_%03d", 0, 0},
    {6, "sleepMutex", "sleeping_mutex_%03d", 0, 0},
    {7, "faMutex", "fetchadd_mutex_%03d", 0, 0},
    {8, "spinSem1", "spin_lock_sem_%03d_%03d", 1, 1},
    {9, "spinSem2", "spin_lock_sem_%03d_%03d", 2, 2},
    {10, "spinSem10", "spin_lock_sem_%03d_%03d", 10, 10},
    {11, "spinSem120", "spin_lock_sem_%03d_%03d", 2, 120},
    {12, "spinSemEBO1", "ebo_sem_%03d_%03d", 1, 1},
    {13, "spinSemEBO2", "ebo_sem_%03d_%03d", 2, 2},
    {14, "spinSemEBO10", "ebo_sem_%03d_%03d", 10, 10},
    {15, "spinSemEBO120", "ebo_sem_%03d_%03d", 120, 120},
    {20, "spinMutexUniq", "spin_lock_mutex_uniq_%03d", 0, 0},
    {21, "spinMutexEBOUniq", "ebo_mutex_uniq_%03d", 0, 0},
    {22, "sleepMutexUniq", "sleeping_mutex_uniq_%03d", 0, 0},
    {23, "faMutexUniq", "fetchadd_mutex_uniq_%03d", 0, 0},
    {24, "spinSemUniq1", "spin_lock_sem_uniq_%03d_%03d", 1, 1},
    {25, "spinSemUniq2", "spin_lock_sem_uniq_%03d_%03d", 2, 2},
    {26, "spinSemUniq10", "spin_lock_sem_uniq_%03d_%03d", 10, 10},
    {27, "spinSemUniq120", "spin_lock_sem_uniq_%03d_%03d", 2, 120},
    {28, "spinSemEBOUniq1", "ebo_sem_uniq_%03d_%03d", 1, 1},
    {29, "spinSemEBOUniq2", "ebo_sem_uniq_%03d_%03d", 2, 2},
    {30, "spinSemEBOUniq10", "ebo_sem_uniq_%03d_%03d", 10, 10},
    {31, "spinSemEBOUniq120", "ebo_sem_uniq_%03d_%03d", 120, 120},
    // HIP build only (hip/syncPrims/uvm/main.hip.cpp:2056-2083 names, 2240-2338 labels)
    {16, "PRspinSem1", "prior_spin_lock_sem_%03d_%03d", 1, 1},
    {17, "PRspinSem2", "prior_spin_lock_sem_%03d_%03d", 2, 2},
    {18, "PRspinSem10", "prior_spin_lock_sem_%03d_%03d", 10, 10},
    {19, "PRspinSem120", "prior_spin_lock_sem_%03d_%03d", 2, 120},
    {32, "PRspinSemEBO1", "prior_ebo_sem_%03d_%03d", 1, 1},
    {33, "PRspinSemEBO2", "prior_ebo_sem_%03d_%03d", 2, 2},
    {34, "PRspinSemEBO10", "prior_ebo_sem_%03d_%03d", 10, 10},
    {35, "PRspinSemEBO120", "prior_ebo_sem_%03d_%03d", 120, 120},
    {37, "atomicTreeBarrUniqSRB", "atomic_tree_barrier_SRB_%03d", 0, 0},
    {38, "atomicTreeBarrUniqLocalExchSRB", "atomic_tree_barrier_localExch_SRB_%03d", 0, 0},
    {39, "atomicTreeBarrUniqNaiveSRB", "atomic_tree_barrier_NaiveSRB_%03d", 0, 0},
    {40, "atomicTreeBarrUniqLocalExchNaiveSRB", "atomic_tree_barrier_localExch_NaiveSRB_%03d", 0, 0},
    {41, "atomicTreeBarrUniqNaiveAllSRB", "atomic_tree_barrier_NaiveAllSRB_%03d", 0, 0},
    {42, "atomicTreeBarrUniqLocalExchNaiveAllSRB", "atomic_tree_barrier_localExch_NaiveAllSRB_%03d", 0, 0},
};

// The CUDA primitive a HIP-extension id runs, and its variant.
static int canon_prim(int prim, int* variant) {
  *variant = PV_NONE;
  if (prim >= 16 && prim <= 19) { *variant = PV_PRIORITY; return prim - 8; }   // -> spinSem*
  if (prim >= 32 && prim <= 35) { *variant = PV_PRIORITY; return prim - 20; }  // -> spinSemEBO*
  if (prim >= 37 && prim <= 42) {
    static const int v[6] = {PV_SRB, PV_SRB, PV_NAIVE, PV_NAIVE, PV_NAIVE_ALL, PV_NAIVE_ALL};
    *variant = v[prim - 37];
    return (prim - 37) % 2;  // -> atomicTreeBarrUniq(LocalExch)
  }
  return prim;
}

// A copy of the configuration with the primitive replaced by its CUDA base.
static const hs_run_config* canon(const hs_run_config* c, hs_run_config* tmp, int* variant) {
  if (!c) return c;
  *tmp = *c;
  tmp->prim = canon_prim(c->prim, variant);
  return tmp;
}
extern "C" int hs_prim_base(int prim, int* variant) {
  int v = 0;
  const int b = canon_prim(prim, &v);
  if (variant) *variant = v;
  return b;
}
static const PrimInfo* find_prim(int id) {
  for (const auto& p : kPrims)
    if (p.id == id) return &p;
  return nullptr;
}
extern "C" int hs_prim_id(const char* name) {
  if (!name) return -1;
  for (const auto& p : kPrims)
    if (std::strcmp(p.name, name) == 0) return p.id;
  return -1;
}
extern "C" const char* hs_prim_name(int prim) {
  const PrimInfo* p = find_prim(prim);
  return p ? p->name : nullptr;
}
extern "C" int hs_prim_label(int prim, int iters, char* buf, int n) {
  const PrimInfo* p = find_prim(prim);
  if (!p) return -1;
  if (p->label_count) return std::snprintf(buf, n, p->label, p->label_count, iters);
  return std::snprintf(buf, n, p->label, iters);
}
extern "C" int hs_prim_sem_count(int prim) {
  const PrimInfo* p = find_prim(prim);
  return p ? p->sem_count : 0;
}

static bool is_barrier(int prim) { return prim >= 0 && prim <= 3; }
static bool is_gmutex(int prim) { return prim >= 4 && prim <= 7; }
static bool is_gsem(int prim) { return prim >= 8 && prim <= 15; }
static bool is_umutex(int prim) { return prim >= 20 && prim <= 23; }
static bool is_usem(int prim) { return prim >= 24 && prim <= 31; }

// numLocsMult: main.cu:1283-1301.
static long long locs_mult(int prim, int num_tbs, int nsm) {
  if (is_barrier(prim) || is_usem(prim)) return num_tbs;
  if (is_gmutex(prim)) return 1;
  if (is_gsem(prim)) return ceil_div(num_tbs, nsm);
  if (is_umutex(prim)) return std::min(num_tbs, nsm);
  return -1;
}

static int device_nsm(int nsm_cfg) {
  if (nsm_cfg > 0) return nsm_cfg;
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return -1; }
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) { cudaGetLastError(); return -1; }
  return n;
}

static int validate(const hs_run_config* c, int nsm) {
  if (!c) { g_err = "null config"; return HS_EINVAL; }
  if (!find_prim(c->prim)) { g_err = "unknown primitive id"; return HS_EINVAL; }
  if (c->num_ldst <= 0 || c->num_tbs <= 0 || c->num_iters < 0 || c->repeats < 0) {
    g_err = "numLdSt and numTBs must be positive, numCSIters and repeats non-negative";
    return HS_EINVAL;
  }
  if (c->threads < 16 || c->threads > 1024 || (c->threads % 16) != 0) {
    g_err = "threads per TB must be a multiple of 16 in [16, 1024]";
    return HS_EINVAL;
  }
  if (nsm <= 0) { g_err = "NUM_SM must be positive"; return HS_EINVAL; }
  if (c->mode == HS_MODE_SLICE && !(is_gmutex(c->prim) || is_umutex(c->prim))) {
    g_err = "HS_MODE_SLICE is defined for the mutex primitives only";
    return HS_EINVAL;
  }
  if (c->mode < 0 || c->mode > 2) { g_err = "unknown mode"; return HS_EINVAL; }
  if (c->backoff_max_ns && (c->backoff_max_ns & (c->backoff_max_ns - 1))) {
    g_err = "backoff_max_ns must be a power of two";
    return HS_EINVAL;
  }
  return HS_OK;
}

extern "C" int hs_storage_words(const hs_run_config* c0, int nsm, size_t* words) {
  hs_run_config tmp;
  int variant = 0;
  const hs_run_config* c = canon(c0, &tmp, &variant);
  nsm = device_nsm(nsm > 0 ? nsm : (c ? c->nsm : 0));
  int v = validate(c, nsm);
  if (v) return v;
  if (c->mode == HS_MODE_SLICE) *words = (size_t)c->num_tbs * c->num_ldst;
  else *words = (size_t)locs_mult(c->prim, c->num_tbs, nsm) * c->threads * (c->num_ldst + 1);
  return HS_OK;
}

extern "C" void hs_run_config_default(hs_run_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->prim = 7;
  c->num_ldst = 10;
  c->num_tbs = 8;
  c->num_iters = 100;
  c->threads = 32;
  c->repeats = 10;
  c->mode = HS_MODE_REF;
  c->nsm = 0;
  c->backoff_min_ns = 1;
  c->backoff_max_ns = 1024;
  c->backoff_unit_ns = 0;
  c->timeout_ns = 0;
  c->skip_tb = -1;
  c->flags = 0;
}

// ---------------------------------------------------------------------------
// Closed form of the reference golden (main.cu:1633-1788): the golden applies,
// per repeat and iteration, one line shift to a set of chunks; the only thing
// that matters is how many shifts each chunk receives.  Region line n after s
// shifts holds the initial line max(n - s, 0).
// ---------------------------------------------------------------------------
static void shift_counts(const hs_run_config* c, int nsm, std::vector<unsigned long long>& cnt) {
  const long long nchunks = locs_mult(c->prim, c->num_tbs, nsm);
  cnt.assign((size_t)nchunks, 0ull);
  const unsigned long long RI = (unsigned long long)c->repeats * (unsigned long long)c->num_iters;
  const int G = c->num_tbs;
  if (is_barrier(c->prim)) {
    const int nb = std::min(G, nsm);
    const int k = ceil_div(G, nsm);  // numTBs_perSM as main.cu:1219 computes it
    (void)nb;
    const bool exch = (c->prim == 1 || c->prim == 3) && k > 1;
    for (auto& x : cnt) x = RI * (exch ? 2ull : 1ull);
  } else if (is_gmutex(c->prim)) {
    cnt[0] = RI * (unsigned long long)G;
  } else if (is_gsem(c->prim)) {
    const int numSM = std::min(G, nsm);
    const int k = ceil_div(G, numSM);
    unsigned long long writers = 0;
    for (int tb = 0; tb < G; ++tb)
      if (tb / numSM == (tb % numSM) % k) ++writers;
    for (auto& x : cnt) x = RI * writers;
  } else if (is_umutex(c->prim)) {
    for (int b = 0; b < G; ++b) cnt[(size_t)(b % nsm)] += RI;
  } else {
    for (auto& x : cnt) x = RI;
  }
}

extern "C" int hs_expected_storage(const hs_run_config* c0, int nsm, const uint32_t* init, uint32_t* out,
                                   size_t words) {
  hs_run_config tmp;
  int variant = 0;
  const hs_run_config* c = canon(c0, &tmp, &variant);
  nsm = device_nsm(nsm > 0 ? nsm : (c ? c->nsm : 0));
  int v = validate(c, nsm);
  if (v) return v;
  size_t need = 0;
  hs_storage_words(c, nsm, &need);
  if (words < need || !init || !out) { g_err = "storage too small"; return HS_EINVAL; }
  const int L = c->num_ldst;
  if (c->mode == HS_MODE_SLICE) {
    const uint32_t add = (uint32_t)((unsigned long long)c->repeats * c->num_iters);
    for (size_t i = 0; i < need; ++i) out[i] = init[i] + add;
    return HS_OK;
  }
  std::vector<unsigned long long> cnt;
  shift_counts(c, nsm, cnt);
  const size_t cw = (size_t)c->threads * (L + 1);
  const int regions = c->threads / 16;
  for (size_t ch = 0; ch < cnt.size(); ++ch) {
    const unsigned long long s = cnt[ch];
    for (int h = 0; h < regions; ++h) {
      const size_t base = ch * cw + (size_t)h * 16 * (L + 1);
      for (int n = 0; n <= L; ++n) {
        for (int o = 0; o < 16; ++o) {
          const size_t at = base + (size_t)n * 16 + o;
          if (c->mode == HS_MODE_REF) {
            const long long src = (unsigned long long)n > s ? (long long)(n - (long long)s) : 0;
            out[at] = init[base + (size_t)src * 16 + o];
          } else {
            out[at] = n == 0 ? init[at] : init[at] + (uint32_t)s;
          }
        }
      }
    }
  }
  return HS_OK;
}

// ---------------------------------------------------------------------------
// Context: cached device buffers for lock state, rings, status, staging.
// ---------------------------------------------------------------------------
struct hs_ctx {
  int device = 0;
  int nsm = 0;
  int max_tpb = 1024;
  void* locks = nullptr;
  size_t locks_cap = 0;
  void* ring = nullptr;
  size_t ring_cap = 0;
  unsigned* status = nullptr;
  void* sink = nullptr;
  size_t sink_cap = 0;
  void* staging = nullptr;
  size_t staging_cap = 0;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // launch, H2D, D2H pairs
  // HS_RUN_GRAPH: the last captured repeats and what they were captured for
  cudaStream_t gstream = nullptr;  // capture stream when the caller passes the legacy default stream
  cudaGraphExec_t gexec = nullptr;
  std::vector<unsigned char> gkey;
  // cohort mutexes: die map and per-die lock lines (hs_cohort.cu); state 0 not
  // yet calibrated, 1 ready, -1 unavailable on this part
  unsigned* coh_pool = nullptr;
  int coh_state = 0;
  unsigned* coh_lines[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

// The cohort pool, calibrated on first use; false if the part has no two-die split.
static bool cohort_ready(hs_ctx* ctx) {
  if (ctx->coh_state == 0) {
    ctx->coh_state = -1;
    const size_t words = kCohortMapWords + (size_t)kCohortCandidates * kLineWords;
    if (cudaMalloc(&ctx->coh_pool, words * 4) != cudaSuccess) {
      cudaGetLastError();
      ctx->coh_pool = nullptr;
      return false;
    }
    cudaMemset(ctx->coh_pool, 0, words * 4);
    int sel[2][3];
    if (hs_cohort_calibrate(ctx->device, ctx->coh_pool, kCohortCandidates, sel)) {
      for (int dd = 0; dd < 2; ++dd)
        for (int i = 0; i < 3; ++i)
          ctx->coh_lines[3 * dd + i] = ctx->coh_pool + kCohortMapWords + (size_t)sel[dd][i] * kLineWords;
      ctx->coh_state = 1;
    }
  }
  return ctx->coh_state == 1;
}

static int ensure(void** p, size_t* cap, size_t bytes) {
  if (*cap >= bytes) return HS_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    g_err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return HS_ENORES;
  }
  *cap = bytes;
  return HS_OK;
}

extern "C" int hs_ctx_create(int device, hs_ctx** out) {
  if (!out) return HS_EINVAL;
  int nsm = 0, tpb = 0;
  int s = hs_device_info(device, &nsm, nullptr, nullptr, &tpb);
  if (s) return s;
  HS_CK(cudaSetDevice(device));
  hs_ctx* c = new hs_ctx();
  c->device = device;
  c->nsm = nsm;
  c->max_tpb = tpb;
  cudaError_t e = cudaMalloc(&c->status, 256);
  if (e != cudaSuccess) { delete c; return set_cuda_err(e, "cudaMalloc(status)"); }
  for (auto& ev : c->ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) { delete c; return set_cuda_err(e, "cudaEventCreate"); }
  }
  *out = c;
  return HS_OK;
}

extern "C" int hs_ctx_destroy(hs_ctx* c) {
  if (!c) return HS_EINVAL;
  cudaFree(c->locks);
  cudaFree(c->ring);
  cudaFree(c->status);
  cudaFree(c->sink);
  cudaFree(c->staging);
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->gstream) cudaStreamDestroy(c->gstream);
  cudaFree(c->coh_pool);
  delete c;
  return HS_OK;
}

static Layout make_layout(const hs_run_config* c, int nsm) {
  Layout L{};
  const int G = c->num_tbs;
  const int nb = std::min(G, nsm);
  L.groups = std::max(nsm, 1);
  const int kmax = ceil_div(G, nb) + 1;
  L.l_glob = 0;
  L.l_gflag = 4;
  const int gf_lines = ceil_div(L.groups, kLineWords);
  L.l_grp = L.l_gflag + gf_lines;
  L.l_lflag = L.l_grp + 4 * L.groups;
  L.lflag_lines = ceil_div(kmax, kLineWords);
  L.lines = L.l_lflag + L.groups * L.lflag_lines;
  const int ring_groups = is_umutex(c->prim) ? nsm : 1;
  L.ring_words = (size_t)ring_groups * ((size_t)G + 1) * kRingStride;
  return L;
}

// Prepare descriptor + lock state for a run (shared with the batch path).
int hs_prepare_run(hs_ctx* ctx, const hs_run_config* c, int nsm, void* dev_storage, cudaStream_t st, RunDesc* d,
                   bool init_state) {
  const Layout lay = make_layout(c, nsm);
  int s;
  if ((s = ensure(&ctx->locks, &ctx->locks_cap, (size_t)lay.lines * kLineWords * 4))) return s;
  if ((s = ensure(&ctx->ring, &ctx->ring_cap, lay.ring_words * 4))) return s;
  if ((s = ensure(&ctx->sink, &ctx->sink_cap, (size_t)c->num_tbs * 4 + 256))) return s;
  std::memset(d, 0, sizeof(*d));
  d->data = static_cast<unsigned*>(dev_storage);
  d->locks = static_cast<unsigned*>(ctx->locks);
  d->ring = static_cast<unsigned*>(ctx->ring);
  d->status = ctx->status;
  d->sink = static_cast<unsigned*>(ctx->sink);
  d->prim = c->prim;
  d->mode = c->mode;
  d->T = c->threads;
  d->L = c->num_ldst;
  d->num_tbs = c->num_tbs;
  d->iters = c->num_iters;
  d->nsm = nsm;
  d->sem_max = (unsigned)hs_prim_sem_count(c->prim) + 1u;
  d->bo_min = c->backoff_min_ns ? c->backoff_min_ns : 1u;
  d->bo_max = c->backoff_max_ns ? c->backoff_max_ns : 1024u;
  d->bo_unit = c->backoff_unit_ns;
  d->ring_max = (unsigned)c->num_tbs;
  d->timeout_ns = c->timeout_ns ? c->timeout_ns : 10000000000ull;
  d->skip_tb = c->skip_tb;
  d->cluster = 1;
  d->l_glob = lay.l_glob;
  d->l_gflag = lay.l_gflag;
  d->l_grp = lay.l_grp;
  d->l_lflag = lay.l_lflag;
  d->lflag_lines = lay.lflag_lines;
  HS_CK(cudaMemsetAsync(ctx->status, 0, 256, st));
  if (init_state) {
    HS_CK(cudaMemsetAsync(ctx->locks, 0, (size_t)lay.lines * kLineWords * 4, st));
    if (hs_prim_sem_count(c->prim)) {
      HS_CK(launch_fill_lines(d->locks + (size_t)lay.l_grp * kLineWords, (size_t)lay.groups,
                              (size_t)4 * kLineWords, d->sem_max, st));
      hs_note_launches(1);
    }
    if (c->prim == 6 || c->prim == 22) {
      const unsigned groups = c->prim == 22 ? (unsigned)nsm : 1u;
      HS_CK(launch_ring_init(d->ring, d->ring_max + 1u, groups, st));
      hs_note_launches(1);
    }
  }
  return HS_OK;
}

static int read_status(hs_ctx* ctx, cudaStream_t st, hs_run_result* r) {
  unsigned h[2] = {0, 0};
  HS_CK(cudaMemcpyAsync(h, ctx->status, sizeof(h), cudaMemcpyDeviceToHost, st));
  HS_CK(cudaStreamSynchronize(st));
  r->dev_error_bits = h[0];
  r->dev_error_site = h[1];
  if (h[0] & HS_DEV_TIMEOUT) {
    g_err = "device wait timed out at site " + std::to_string(h[1]);
    return HS_ETIMEDOUT;
  }
  if (h[0]) {
    g_err = "device error bits " + std::to_string(h[0]);
    return HS_EMISMATCH;
  }
  return HS_OK;
}

extern "C" int hs_run(hs_ctx* ctx, const hs_run_config* c0, void* storage, int on_device, void* stream,
                      hs_run_result* r) {
  if (!ctx || !c0 || !storage || !r) { g_err = "null argument"; return HS_EINVAL; }
  hs_run_config tmp;
  int variant = 0;
  const hs_run_config* c = canon(c0, &tmp, &variant);
  std::memset(r, 0, sizeof(*r));
  const int nsm = c->nsm > 0 ? c->nsm : ctx->nsm;
  int s = validate(c, nsm);
  if (s) return r->status = s;
  if (c->threads > ctx->max_tpb) { g_err = "threads per TB above the device limit"; return r->status = HS_EINVAL; }
  if ((c->flags & HS_RUN_GRAPH) && (c->flags & HS_RUN_SYNC_EACH)) {
    g_err = "HS_RUN_GRAPH replays the repeats as one graph: no host synchronisation between them";
    return r->status = HS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  HS_CK(cudaSetDevice(ctx->device));
  size_t words = 0;
  hs_storage_words(c, nsm, &words);
  const size_t bytes = words * 4;

  size_t smem = 0;
  KernelFn fn = syncprim_plan(c->prim, c->mode, c->threads, c->num_ldst, &smem, !(c->flags & HS_RUN_REGISTER_CS));
  if (!fn) { g_err = "no kernel for this primitive/mode"; return r->status = HS_EINVAL; }
  // bulk-copy tiles of a barrier: the shared memory its co-resident TBs leave free
  if (is_barrier(c->prim)) smem = barrier_tile_bytes(c->threads, c->num_ldst, c->num_tbs, ctx->nsm, smem);
  HS_CK(prepare_smem(fn, smem));
  // Tree barriers whose logical-SM groups are all the same size (numTBs a
  // multiple of NUM_SM, 2 to 8 per group) run each group as one thread-block
  // cluster: the local stage becomes the hardware cluster barrier.
  int cluster = 1;
  // Uniq mutexes and semaphores with whole groups of 2, 4 or 8 TBs per logical
  // SM run each group as one cluster (lock word in distributed shared memory).
  if ((is_umutex(c->prim) || is_usem(c->prim)) && !(c->flags & HS_RUN_NO_CLUSTER) && c->num_tbs % nsm == 0 &&
      (c->num_tbs / nsm == 2 || c->num_tbs / nsm == 4 || c->num_tbs / nsm == 8)) {
    const int m = c->num_tbs / nsm;
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)m;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.gridDim = dim3((unsigned)c->num_tbs);
    lc.blockDim = dim3((unsigned)c->threads);
    lc.dynamicSmemBytes = smem;
    lc.attrs = attr;
    lc.numAttrs = 1;
    int fit = 0;
    // groups never wait on one another, but a second wave of clusters doubles
    // the time: clusters only when every group's cluster is resident at once
    if (cudaOccupancyMaxActiveClusters(&fit, (const void*)fn, &lc) == cudaSuccess && fit >= nsm) cluster = m;
    cudaGetLastError();
  }
  // Tree barriers whose whole logical-SM groups fit one CTA (m * threads <=
  // 1024) run each group as one CTA on the register path: the local stage is
  // the CTA barrier.  Measured (1000 episodes, 256 threads, us per episode):
  // lfTreeBarrUniqLocalExch at 608 TBs, numLdSt 10: 5.17 against 8.01 flat;
  // at 304 TBs 3.79 against 5.89 on clusters of 2; at numLdSt 64 it still
  // beats the bulk-copy tiles (304 TBs: 6.34 against 7.10 for
  // lfTreeBarrUniq), at numLdSt 100 the tiles win (608 TBs: 12.89 against
  // 14.22), so up to numLdSt 64.  Every group CTA must be resident at once.
  int block = c->threads, tbs_per_cta = 1;
  if (is_barrier(c->prim) && c->mode != HS_MODE_SLICE && c->num_ldst <= 64 &&
      !(c->flags & (HS_RUN_NO_CLUSTER | HS_RUN_NO_GROUP_CTA)) && c->skip_tb < 0 && variant != PV_NAIVE &&
      variant != PV_NAIVE_ALL) {
    const int nb = c->num_tbs < nsm ? c->num_tbs : nsm;
    const int m = c->num_tbs / nb;
    KernelFn gfn = barrier_group_kernel(c->prim, c->mode);
    int per_sm = 0;
    if (gfn && m >= 2 && c->num_tbs % nb == 0 && m * c->threads <= 1024 && m * c->threads <= ctx->max_tpb &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gfn, m * c->threads, 0) == cudaSuccess &&
        (long long)per_sm * ctx->nsm >= nb) {
      fn = gfn;
      smem = 0;
      block = m * c->threads;
      tbs_per_cta = m;
    }
    cudaGetLastError();
  }
  // Above numLdSt 64 the same group CTA gives each member its own bulk-copy
  // buffer (k_barrier_grp_tma): the members' copies stay in flight side by side,
  // as with one CTA per TB, while the local stage stays the CTA barrier.
  // Measured at numLdSt 100 (us per episode): lfTreeBarrUniq at 304 TBs 7.12
  // against 8.68 with one CTA per TB, at 608 TBs 11.54 against 12.83.
  unsigned tile_cap = 0;
  if (is_barrier(c->prim) && c->mode != HS_MODE_SLICE && c->num_ldst > 64 &&
      !(c->flags & (HS_RUN_NO_CLUSTER | HS_RUN_NO_GROUP_CTA | HS_RUN_REGISTER_CS)) && c->skip_tb < 0 &&
      variant != PV_NAIVE && variant != PV_NAIVE_ALL && tbs_per_cta == 1 && c->threads % 32 == 0) {
    const int nb = c->num_tbs < nsm ? c->num_tbs : nsm;
    const int m = c->num_tbs / nb;
    KernelFn gfn = barrier_group_tma_kernel(c->prim, c->mode);
    const size_t region = (size_t)64 * (c->num_ldst + 1);
    const size_t chunk = region * (size_t)(c->threads / 16);
    const size_t cap = m >= 1 ? std::min(chunk, (size_t)(216 * 1024) / (size_t)m / region * region) : 0;
    int per_sm = 0;
    if (gfn && m >= 2 && m <= 15 && c->num_tbs % nb == 0 && m * c->threads <= 1024 &&
        m * c->threads <= ctx->max_tpb && cap >= region &&
        cudaFuncSetAttribute((const void*)gfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(m * cap)) ==
            cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gfn, m * c->threads, m * cap) == cudaSuccess &&
        (long long)per_sm * ctx->nsm >= nb) {
      fn = gfn;
      smem = m * cap;
      tile_cap = (unsigned)cap;
      block = m * c->threads;
      tbs_per_cta = m;
    }
    cudaGetLastError();
  }
  if (is_barrier(c->prim) && tbs_per_cta == 1) {
    const int nb = c->num_tbs < nsm ? c->num_tbs : nsm;
    const int m = c->num_tbs / nb;
    if (!(c->flags & HS_RUN_NO_CLUSTER) && c->skip_tb < 0 && c->num_tbs % nb == 0 && (m == 2 || m == 4 || m == 8) &&
        variant != PV_NAIVE && variant != PV_NAIVE_ALL) {
      cudaLaunchConfig_t lc = {};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)m;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      lc.gridDim = dim3((unsigned)c->num_tbs);
      lc.blockDim = dim3((unsigned)c->threads);
      lc.dynamicSmemBytes = smem;
      lc.attrs = attr;
      lc.numAttrs = 1;
      int fit = 0;
      if (cudaOccupancyMaxActiveClusters(&fit, (const void*)fn, &lc) == cudaSuccess && fit >= nb) cluster = m;
      cudaGetLastError();
    }
    if (cluster == 1) {
      int per_sm = 0;
      HS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, c->threads, smem));
      if ((long long)per_sm * ctx->nsm < c->num_tbs) {
        g_err = "barrier TBs cannot all be co-resident (" + std::to_string(per_sm) + " per SM x " +
                std::to_string(ctx->nsm) + " SMs < " + std::to_string(c->num_tbs) + ")";
        return r->status = HS_ENORES;
      }
    }
  }

  // Global mutexes and semaphores with a bulk-copy critical section: one
  // cluster of m CTAs per logical TB, the critical section split over its SMs
  // (m = 8, or fewer when the TB has fewer half-warp regions).  Measured at
  // numLdSt 100 (reference mode, us per op, cluster against flat): faster
  // only where a semaphore writer moves 4 or more chunks (spinSem1 at 608 TBs
  // 4.72 against 5.40); slower for mutexes (faMutex 4.34 against 3.26) and
  // smaller writers, so by default only there.
  int grid = tbs_per_cta > 1 ? c->num_tbs / tbs_per_cta : c->num_tbs;
  const bool sem_prim = c->prim >= 8 && c->prim <= 15;
  const int sem_numSM = c->num_tbs < nsm ? c->num_tbs : nsm;
  const int sem_k = sem_prim ? (c->num_tbs + sem_numSM - 1) / sem_numSM : 1;  // chunks a semaphore writer owns
  if (c->prim >= 4 && c->prim <= 15 && c->mode != HS_MODE_SLICE && c->num_ldst > 32 && c->threads <= 256 &&
      !(c->flags & (HS_RUN_NO_CLUSTER | HS_RUN_REGISTER_CS)) && ((c->flags & HS_RUN_CLUSTER_CS) || sem_k >= 4)) {
    const int R = c->threads / 16;
    int m = 8;
    while (m > R) m >>= 1;
    KernelFn cfn = prim_cluster_kernel(c->mode);
    if (m >= 2 && cfn) {
      const int k = sem_k;
      const size_t region = (size_t)64 * (c->num_ldst + 1);
      size_t stage = (size_t)k * ((R + m - 1) / m) * region;      // a rank's share of every chunk: one tile
      stage = std::min(stage, (size_t)(200 * 1024) / region * region);
      cudaLaunchConfig_t lc = {};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)m;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      lc.gridDim = dim3((unsigned)(c->num_tbs * m));
      lc.blockDim = dim3((unsigned)c->threads);
      lc.dynamicSmemBytes = stage;
      lc.attrs = attr;
      lc.numAttrs = 1;
      int fit = 0;
      if (stage >= region && prepare_smem(cfn, stage) == cudaSuccess &&
          cudaOccupancyMaxActiveClusters(&fit, (const void*)cfn, &lc) == cudaSuccess && fit >= 1) {
        fn = cfn;
        smem = stage;
        cluster = m;
        grid = c->num_tbs * m;
      }
      cudaGetLastError();
    }
  }

  void* dev = storage;
  if (!on_device) {
    if ((s = ensure(&ctx->staging, &ctx->staging_cap, bytes + 16))) return r->status = s;
    dev = ctx->staging;
    HS_CK(cudaEventRecord(ctx->ev[2], st));
    HS_CK(cudaMemcpyAsync(dev, storage, bytes, cudaMemcpyHostToDevice, st));
    HS_CK(cudaEventRecord(ctx->ev[3], st));
  }
  RunDesc d;
  if ((s = hs_prepare_run(ctx, c, nsm, dev, st, &d, !(c->flags & HS_RUN_KEEP_STATE)))) return r->status = s;

  d.cluster = cluster;
  d.variant = variant;
  d.grp = tbs_per_cta;
  d.tile_cap = tile_cap;
  r->cluster = cluster;
  r->tbs_per_cta = tbs_per_cta;
  // global spin, EBO and ticket mutexes, or global semaphore (its writers), with
  // more than one TB: the die-aware cohort form.  The ring ("sleep") mutex is a
  // queue lock already; in front of it a die queue measured no faster at
  // numLdSt 10 and 3% slower at 100, so it stays plain.
  if (c->prim >= 4 && c->prim <= 15 && c->prim != 6 && c->num_tbs > 1 && grid == c->num_tbs &&
      !(c->flags & HS_RUN_NO_COHORT) && cohort_ready(ctx)) {
    d.cohort = 1;
    d.die_map = reinterpret_cast<const unsigned char*>(ctx->coh_pool);
    for (int i = 0; i < 6; ++i) {
      d.coh[i] = ctx->coh_lines[i];
      if (!(c->flags & HS_RUN_KEEP_STATE)) HS_CK(cudaMemsetAsync(d.coh[i], 0, kLineWords * 4, st));
    }
    r->cohort = 1;
  }
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3((unsigned)grid);
  lc.blockDim = dim3((unsigned)block);
  lc.dynamicSmemBytes = smem;
  lc.stream = st;
  lc.attrs = attr;
  lc.numAttrs = cluster > 1 ? 1 : 0;
  cudaStream_t lst = st;  // the stream the repeats run on
  if ((c->flags & HS_RUN_GRAPH) && c->repeats > 0) {
    // A capture cannot run on the legacy default stream: use a blocking stream
    // of the context, which orders itself with the legacy stream's work.
    if (!st) {
      if (!ctx->gstream) HS_CK(cudaStreamCreate(&ctx->gstream));
      lst = ctx->gstream;
    }
    std::vector<unsigned char> key(sizeof(RunDesc) + sizeof(lc.gridDim) + sizeof(lc.blockDim) + 4 * sizeof(size_t));
    size_t o = 0;
    auto put = [&](const void* p, size_t n) { std::memcpy(key.data() + o, p, n); o += n; };
    const size_t extra[4] = {(size_t)fn, smem, (size_t)cluster, (size_t)c->repeats};
    put(&d, sizeof(RunDesc));
    put(&lc.gridDim, sizeof(lc.gridDim));
    put(&lc.blockDim, sizeof(lc.blockDim));
    put(extra, sizeof(extra));
    if (!ctx->gexec || key != ctx->gkey) {
      if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
      ctx->gexec = nullptr;
      ctx->gkey.clear();
      HS_CK(cudaStreamBeginCapture(lst, cudaStreamCaptureModeThreadLocal));
      lc.stream = lst;
      cudaError_t ce = cudaSuccess;
      for (int rep = 0; rep < c->repeats && ce == cudaSuccess; ++rep) {
        void* args[] = {&d};
        ce = cudaLaunchKernelExC(&lc, (const void*)fn, args);
      }
      cudaGraph_t g = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(lst, &g);
      if (ce == cudaSuccess && ee == cudaSuccess) ce = cudaGraphInstantiate(&ctx->gexec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (ce != cudaSuccess || ee != cudaSuccess) {
        cudaGetLastError();
        ctx->gexec = nullptr;
        g_err = std::string("graph capture: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ee);
        return r->status = HS_ECUDA;
      }
      ctx->gkey = key;
    }
    HS_CK(cudaEventRecord(ctx->ev[0], lst));
    HS_CK(cudaGraphLaunch(ctx->gexec, lst));
    r->launches += (unsigned)c->repeats;
    HS_CK(cudaEventRecord(ctx->ev[1], lst));
  } else {
    HS_CK(cudaEventRecord(ctx->ev[0], st));
    for (int rep = 0; rep < c->repeats; ++rep) {
      void* args[] = {&d};
      HS_CK(cudaLaunchKernelExC(&lc, (const void*)fn, args));
      r->launches++;
      if (c->flags & HS_RUN_SYNC_EACH) HS_CK(cudaStreamSynchronize(st));
    }
    HS_CK(cudaEventRecord(ctx->ev[1], st));
  }
  hs_note_launches(r->launches);
  if (!on_device) {
    HS_CK(cudaEventRecord(ctx->ev[4], st));
    HS_CK(cudaMemcpyAsync(storage, dev, bytes, cudaMemcpyDeviceToHost, st));
    HS_CK(cudaEventRecord(ctx->ev[5], st));
  }
  if (lst != st) HS_CK(cudaStreamSynchronize(lst));
  HS_CK(cudaStreamSynchronize(st));
  HS_CK(cudaEventElapsedTime(&r->elapsed_ms, ctx->ev[0], ctx->ev[1]));
  if (!on_device) {
    HS_CK(cudaEventElapsedTime(&r->h2d_ms, ctx->ev[2], ctx->ev[3]));
    HS_CK(cudaEventElapsedTime(&r->d2h_ms, ctx->ev[4], ctx->ev[5]));
  }
  r->avg_ms = c->repeats ? r->elapsed_ms / c->repeats : 0.f;
  r->ops = (unsigned long long)c->num_tbs * c->num_iters * c->repeats;
  s = read_status(ctx, st, r);
  return r->status = s;
}

// ---------------------------------------------------------------------------
// The reference's host API: cudaLocks.cu:3-95 and the Create functions.
// ---------------------------------------------------------------------------
static hs_lock_data* g_lock = nullptr;
static float g_lock_copy_ms = 0.f;

extern "C" hs_lock_data* hs_lock_data_get(void) { return g_lock; }
extern "C" float hs_locks_init_copy_ms(void) { return g_lock_copy_ms; }

extern "C" int cudaLocksInit(const int maxBlocksPerKernel, const int numMutexes, const int numSemaphores,
                             const bool pageAlign, const int NUM_SM) {
  (void)pageAlign;
  if (maxBlocksPerKernel <= 0 || numMutexes <= 0 || numSemaphores <= 0 || NUM_SM <= 0)
    return (int)cudaErrorInitializationError;  // cudaLocks.cu:13-15
  // The reference's stride (cudaLocks.cu:19) must leave room for a ring of
  // maxBlocksPerKernel + 1 slots and for the barrier's in/out flags; with few
  // SMs it can round down to maxBlocksPerKernel or below (even to 0, a
  // zero-byte barrier buffer).  Such sizes are refused here.
  if ((maxBlocksPerKernel + NUM_SM) / 16 * 16 <= maxBlocksPerKernel) return (int)cudaErrorInvalidValue;
  if (g_lock) cudaLocksDestroy();
  hs_lock_data* L = nullptr;
  cudaError_t e = cudaMallocHost(&L, sizeof(hs_lock_data));
  if (e != cudaSuccess) return (int)e;
  std::memset(L, 0, sizeof(*L));
  L->maxBufferSize = maxBlocksPerKernel;
  L->arrayStride = (maxBlocksPerKernel + NUM_SM) / 16 * 16;  // cudaLocks.cu:19
  L->mutexCount = numMutexes;
  L->semaphoreCount = numSemaphores;
  const size_t stride = (size_t)L->arrayStride;
  if ((e = cudaMalloc(&L->barrierBuffers, 4 * stride * 2)) != cudaSuccess) return (int)e;
  if ((e = cudaMalloc(&L->mutexBuffers, 4 * stride * numMutexes)) != cudaSuccess) return (int)e;
  if ((e = cudaMalloc(&L->mutexBufferHeads, 4 * (size_t)numMutexes)) != cudaSuccess) return (int)e;
  if ((e = cudaMalloc(&L->mutexBufferTails, 4 * (size_t)numMutexes)) != cudaSuccess) return (int)e;
  if ((e = cudaMalloc(&L->semaphoreBuffers, 4 * 4 * (size_t)numSemaphores)) != cudaSuccess) return (int)e;
  cudaMemset(L->barrierBuffers, 0, 4 * stride * 2);
  cudaMemset(L->mutexBufferHeads, 0, 4 * (size_t)numMutexes);
  cudaMemset(L->mutexBufferTails, 0, 4 * (size_t)numMutexes);
  cudaMemset(L->semaphoreBuffers, 0, 4 * 4 * (size_t)numSemaphores);
  // rings: first slot of every ring 1, the rest -1 (cudaLocks.cu:58-65)
  std::vector<int> ring(stride * numMutexes, -1);
  for (size_t i = 0; i < ring.size(); i += stride) ring[i] = 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;  // the copy is timed, as cudaLocks.cu:66-74 times it
  if ((e = cudaEventCreate(&e0)) != cudaSuccess) return (int)e;
  if ((e = cudaEventCreate(&e1)) != cudaSuccess) { cudaEventDestroy(e0); return (int)e; }
  cudaEventRecord(e0, 0);
  e = cudaMemcpy(L->mutexBuffers, ring.data(), ring.size() * 4, cudaMemcpyHostToDevice);
  cudaEventRecord(e1, 0);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&g_lock_copy_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return (int)e;
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return (int)e;
  g_lock = L;
  return 0;
}

extern "C" int cudaLocksDestroy(void) {
  if (!g_lock) return (int)cudaErrorInitializationError;
  cudaFree(g_lock->barrierBuffers);
  cudaFree(g_lock->mutexBuffers);
  cudaFree(g_lock->mutexBufferHeads);
  cudaFree(g_lock->mutexBufferTails);
  cudaFree(g_lock->semaphoreBuffers);
  cudaFreeHost(g_lock);
  g_lock = nullptr;
  return 0;
}

extern "C" int cudaMutexCreateSpin(unsigned int* const h, const int n) { *h = (unsigned)n; return 0; }
extern "C" int cudaMutexCreateEBO(unsigned int* const h, const int n) { *h = (unsigned)n; return 0; }
extern "C" int cudaMutexCreateFA(unsigned int* const h, const int n) { *h = (unsigned)n; return 0; }
extern "C" int cudaMutexCreateSleep(unsigned int* const h, const int n) { *h = (unsigned)n; return 0; }

// Initial words for every SM copy: {count+1, 0, 0, count+1} (cudaLocksSemaphoreSpin.cu:12-22),
// written with one copy instead of 4*NUM_SM.
static int sem_create(unsigned int* const h, const int sem, const unsigned count, const int NUM_SM) {
  if (!g_lock) return (int)cudaErrorInitializationError;
  if (sem < 0 || (long long)(sem + 1) * NUM_SM > g_lock->semaphoreCount) return (int)cudaErrorInvalidValue;
  *h = (unsigned)sem;
  std::vector<unsigned> w((size_t)4 * NUM_SM);
  for (int id = 0; id < NUM_SM; ++id) {
    w[4 * id + 0] = count + 1;
    w[4 * id + 1] = 0;
    w[4 * id + 2] = 0;
    w[4 * id + 3] = count + 1;
  }
  return (int)cudaMemcpy(g_lock->semaphoreBuffers + (size_t)sem * 4 * NUM_SM, w.data(), w.size() * 4,
                         cudaMemcpyHostToDevice);
}
extern "C" int cudaSemaphoreCreateSpin(unsigned int* const h, const int s, const unsigned int count, const int nsm) {
  return sem_create(h, s, count, nsm);
}
extern "C" int cudaSemaphoreCreateEBO(unsigned int* const h, const int s, const unsigned int count, const int nsm) {
  return sem_create(h, s, count, nsm);
}

// Lock-state layout of a run, for entry points that place the state in memory
// they do not allocate here.
int hs_layout_for(const hs_run_config* c0, int nsm, hs::Layout* out) {
  hs_run_config tmp;
  int variant = 0;
  const hs_run_config* c = canon(c0, &tmp, &variant);
  *out = make_layout(c, nsm);
  return HS_OK;
}
