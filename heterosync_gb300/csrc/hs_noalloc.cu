// hs_noalloc.cu -- hs_run_noalloc(): the SyncPrims run for callers that cannot
// allocate device memory.
//
// hs_run() allocates its lock state, ring slots, status words and reader sink
// with cudaMalloc the first time a size is seen.  Some callers cannot allow
// that: host frameworks that own every byte of device memory through their own
// pool and forbid side allocations, processes that run under a device-memory
// budget fixed at start-up, and latency-critical loops where cudaMalloc's
// implicit device-wide synchronisation would stall work on other streams.
// This entry point uses instead one
// file-scope device array of fixed size, HS_NOALLOC_SCRATCH_BYTES, which the
// module holds on every GPU that loads the library until the process exits.
// The caller passes the storage (inputs and outputs) already in device memory.
//
// Rules of use:
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture begins;
//  * every call shares the one array and leaves its contents behind; each call
//    clears what must start at zero itself, but calls whose work overlaps on
//    the GPU (different streams, no ordering) race on it and must not be made;
//  * a run whose lock state does not fit is rejected with HS_EINVAL before
//    anything is launched.
#include <cuda_runtime.h>
#include <chrono>
#include <cstring>
#include <mutex>
#include <cstdio>
#include "hs_internal.h"
#include "../../include/hs/hs.h"
#include "../../include/hs/hs_device.cuh"

namespace hs {
using KernelFn = void (*)(RunDesc);
KernelFn syncprim_plan(int prim, int mode, int threads, int num_ldst, size_t* smem_bytes, bool bulk = true);
cudaError_t prepare_smem(KernelFn fn, size_t smem_bytes);
size_t barrier_tile_bytes(int threads, int num_ldst, int num_tbs, int phys_nsm, size_t base);
cudaError_t launch_ring_init(unsigned* ring, unsigned slots_per_group, unsigned groups, cudaStream_t st);
cudaError_t launch_fill_lines(unsigned* base, size_t n, size_t stride, unsigned value, cudaStream_t st);
}  // namespace hs
int hs_layout_for(const hs_run_config* c, int nsm, hs::Layout* out);
void hs_note_launches(unsigned n);

// The scratch array (device memory owned by this module, never allocated at run time).
static __device__ __align__(256) unsigned hs_noalloc_scratch[HS_NOALLOC_SCRATCH_BYTES / 4];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned* g_addr[kMaxDevices] = {};
thread_local char g_noalloc_err[256];  // fixed buffer: the error path allocates nothing either

void set_err(const char* msg) { std::snprintf(g_noalloc_err, sizeof(g_noalloc_err), "%s", msg); }

// A failed CUDA call: its text goes to the error buffer, and a non-sticky error
// is cleared from the runtime so it cannot surface in an unrelated later call.
int cuda_err(cudaError_t e, const char* what) {
  std::snprintf(g_noalloc_err, sizeof(g_noalloc_err), "%s: %s", what, cudaGetErrorString(e));
  cudaGetLastError();
  return HS_ECUDA;
}
#define NA_CK(call)                                          \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return r->status = cuda_err(e_, #call); \
  } while (0)

// Device address of the scratch array on the current device (looked up once per device).
int scratch_address(unsigned** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_err(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) { set_err("device index beyond the scratch table"); return HS_EINVAL; }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, hs_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      return cuda_err(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    }
    g_addr[dev] = static_cast<unsigned*>(p);
  }
  *out = g_addr[dev];
  return HS_OK;
}

size_t round64(size_t w) { return (w + 63) / 64 * 64; }  // 256-byte granules
}  // namespace

extern "C" const char* hs_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int hs_prim_base(int prim, int* variant);

extern "C" int hs_run_noalloc(const hs_run_config* c0, void* storage, void* stream, hs_run_result* r) {
  using namespace hs;
  if (!c0 || !storage || !r) { set_err("null argument"); return HS_EINVAL; }
  hs_run_config cc = *c0;  // a HIP-extension id runs its CUDA base primitive (variant below)
  int variant = 0;
  cc.prim = hs_prim_base(c0->prim, &variant);
  const hs_run_config* c = &cc;
  std::memset(r, 0, sizeof(*r));
  r->cluster = 1;
  // Runs here are always the flat, single-CTA-per-TB form with the plain (not
  // die-aware) locks and fresh lock state: the flags that ask for that, or for
  // host synchronisation after each launch, are honoured; the others would need
  // state or launches this entry point does not have and are refused.
  const int kHonoured = HS_RUN_SYNC_EACH | HS_RUN_NO_CLUSTER | HS_RUN_REGISTER_CS | HS_RUN_NO_COHORT;
  if (c->flags & ~kHonoured) {
    set_err("hs_run_noalloc takes only HS_RUN_SYNC_EACH, HS_RUN_NO_CLUSTER, HS_RUN_REGISTER_CS and "
            "HS_RUN_NO_COHORT (no kept state, graphs or cluster critical sections)");
    return r->status = HS_EINVAL;
  }
  int dev = 0, dev_sms = 0;
  NA_CK(cudaGetDevice(&dev));
  NA_CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev));
  const int nsm = c->nsm > 0 ? c->nsm : dev_sms;
  size_t words = 0;
  int s = hs_storage_words(c, nsm, &words);
  if (s) { set_err(hs_last_error()); return r->status = s; }
  size_t smem = 0;
  KernelFn fn = syncprim_plan(c->prim, c->mode, c->threads, c->num_ldst, &smem, !(c->flags & HS_RUN_REGISTER_CS));
  if (!fn) { set_err("no kernel for this primitive/mode"); return r->status = HS_EINVAL; }
  const bool barrier = c->prim >= 0 && c->prim <= 3;
  // a barrier's bulk-copy tiles: the same size hs_run() gives them
  if (barrier) smem = barrier_tile_bytes(c->threads, c->num_ldst, c->num_tbs, dev_sms, smem);
  NA_CK(prepare_smem(fn, smem));

  Layout lay;
  std::memset(&lay, 0, sizeof(lay));
  if ((s = hs_layout_for(c, nsm, &lay))) { set_err("no lock-state layout for this run"); return r->status = s; }
  const size_t w_status = 64;
  const size_t w_locks = round64((size_t)lay.lines * kLineWords);
  const size_t w_ring = round64(lay.ring_words);
  const size_t w_sink = round64((size_t)c->num_tbs);
  const size_t need = w_status + w_locks + w_ring + w_sink;
  if (need * 4 > HS_NOALLOC_SCRATCH_BYTES) {
    std::snprintf(g_noalloc_err, sizeof(g_noalloc_err),
                  "lock state needs %zu bytes; hs_run_noalloc holds at most %zu bytes (use hs_run)", need * 4,
                  (size_t)HS_NOALLOC_SCRATCH_BYTES);
    return r->status = HS_EINVAL;
  }
  int max_tpb = 0;
  NA_CK(cudaDeviceGetAttribute(&max_tpb, cudaDevAttrMaxThreadsPerBlock, dev));
  if (c->threads > max_tpb) { set_err("threads per TB above the device limit"); return r->status = HS_EINVAL; }
  if (barrier) {  // every TB of a barrier must be resident at once, with the shared memory it launches with
    int per_sm = 0;
    NA_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, c->threads, smem));
    if ((long long)per_sm * dev_sms < c->num_tbs) {
      std::snprintf(g_noalloc_err, sizeof(g_noalloc_err),
                    "barrier TBs cannot all be co-resident (%d per SM x %d SMs < %d)", per_sm, dev_sms, c->num_tbs);
      return r->status = HS_ENORES;
    }
  }
  unsigned* base = nullptr;
  if ((s = scratch_address(&base))) return r->status = s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  RunDesc d;
  std::memset(&d, 0, sizeof(d));
  d.status = base;
  d.locks = base + w_status;
  d.ring = d.locks + w_locks;
  d.sink = d.ring + w_ring;
  d.data = static_cast<unsigned*>(storage);
  d.prim = c->prim;
  d.variant = variant;
  d.mode = c->mode;
  d.T = c->threads;
  d.L = c->num_ldst;
  d.num_tbs = c->num_tbs;
  d.iters = c->num_iters;
  d.nsm = nsm;
  d.sem_max = (unsigned)hs_prim_sem_count(c->prim) + 1u;
  d.bo_min = c->backoff_min_ns ? c->backoff_min_ns : 1u;
  d.bo_max = c->backoff_max_ns ? c->backoff_max_ns : 1024u;
  d.bo_unit = c->backoff_unit_ns;
  d.ring_max = (unsigned)c->num_tbs;
  d.timeout_ns = c->timeout_ns ? c->timeout_ns : 10000000000ull;
  d.skip_tb = c->skip_tb;
  d.cluster = 1;
  d.l_glob = lay.l_glob;
  d.l_gflag = lay.l_gflag;
  d.l_grp = lay.l_grp;
  d.l_lflag = lay.l_lflag;
  d.lflag_lines = lay.lflag_lines;

  const auto t0 = std::chrono::steady_clock::now();
  // clear what must start at zero: status and lock state (the array keeps the last call's contents)
  NA_CK(cudaMemsetAsync(d.status, 0, w_status * 4, st));
  NA_CK(cudaMemsetAsync(d.locks, 0, w_locks * 4, st));
  unsigned extra = 0;
  if (hs_prim_sem_count(c->prim)) {
    NA_CK(launch_fill_lines(d.locks + (size_t)lay.l_grp * kLineWords, (size_t)lay.groups, (size_t)4 * kLineWords,
                            d.sem_max, st));
    ++extra;
  }
  if (c->prim == 6 || c->prim == 22) {
    NA_CK(launch_ring_init(d.ring, d.ring_max + 1u, c->prim == 22 ? (unsigned)nsm : 1u, st));
    ++extra;
  }
  for (int rep = 0; rep < c->repeats; ++rep) {
    void* args[] = {&d};
    NA_CK(cudaLaunchKernel((const void*)fn, dim3(c->num_tbs), dim3(c->threads), args, smem, st));
    r->launches++;
    if (c->flags & HS_RUN_SYNC_EACH) NA_CK(cudaStreamSynchronize(st));
  }
  hs_note_launches(r->launches + extra);
  unsigned h[2] = {0, 0};
  NA_CK(cudaMemcpyAsync(h, d.status, sizeof(h), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  r->elapsed_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  r->avg_ms = c->repeats ? r->elapsed_ms / c->repeats : 0.f;
  r->ops = (unsigned long long)c->num_tbs * c->num_iters * c->repeats;
  r->dev_error_bits = h[0];
  r->dev_error_site = h[1];
  if (h[0] & HS_DEV_TIMEOUT) {
    std::snprintf(g_noalloc_err, sizeof(g_noalloc_err), "device wait timed out at site %u", h[1]);
    return r->status = HS_ETIMEDOUT;
  }
  if (h[0]) {
    std::snprintf(g_noalloc_err, sizeof(g_noalloc_err), "device error bits %u", h[0]);
    return r->status = HS_EMISMATCH;
  }
  g_noalloc_err[0] = '\0';
  return r->status = HS_OK;
}
