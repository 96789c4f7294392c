// hs_serve.cu -- a device-resident request loop that serves SyncPrims
// instances as they arrive (continuous batching).
//
// One persistent kernel holds `slots` slots of `gang` co-resident CTAs.  The
// host publishes requests into a submission ring in mapped pinned memory and
// never launches anything while the server runs.  Each slot loops:
//   1. admission (the slot's rank-0 CTA): under the server's ticket lock
//      (the project's fetch-and-add mutex, ticket_lock in hs_device.cuh) it
//      takes the oldest pending request if the device arena has room for its
//      storage and lock state -- admission is gated by free device memory, in
//      arrival order; while the oldest does not fit, a later one (within 32
//      entries) that fits may go first, until the oldest has waited 20 ms --
//      then it waits for running requests to release pages and nothing
//      passes it;
//   2. the slot's CTAs copy the request's storage in from the pinned staging
//      pool and lay out its lock state (zeroed words, semaphore counts, ring
//      slots) in the request's pages;
//   3. they execute the instance as the batched kernel does (hs_exec.cuh): each
//      CTA is an executor of the logical TBs congruent to its rank;
//   4. they copy the final storage back to the staging pool, publish a
//      completion record (release at system scope) and free the pages.
// Slots run different requests at the same time, so requests that arrive while
// others run are admitted as soon as a slot and pages are free, and their work
// overlaps on the device.  A request's result depends only on its own storage
// and lock state, so it is the same alone and in any mix (tests check both
// against the closed form of the reference golden).
//
// Every wait is bounded: admission gives up after an idle limit with no
// request (the kernel then exits), slot barriers after a slot limit.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include "hs_exec.cuh"
#include "hs_uts_geo.cuh"
#include "../../include/hs/hs.h"

void hs_note_launches(unsigned n);
int hs_layout_for(const hs_run_config* c, int nsm, hs::Layout* out);

namespace hs {

constexpr unsigned kServeQ = 4096;  // submission ring entries
constexpr unsigned kServeC = 4096;  // completion ring entries
constexpr int kServeThreads = 256;
constexpr unsigned kServeStage = 40u * 1024u;  // bulk-copy staging per CTA
constexpr unsigned long long kPageBytes = 64ull * 1024ull;
constexpr unsigned kTicketWrap = 1000000000u;

// One submitted request (host writes, device reads).  The pointer fields of d
// hold byte offsets from the start of the request's pages.
struct ServeDesc {
  RunDesc d;
  unsigned long long id;
  unsigned long long stage_off;    // byte offset of the storage words in the staging pool
  unsigned long long words;        // storage words (copied in, and out at the end)
  unsigned long long state_words;  // lock-state words at the start of the pages
  unsigned long long pages;        // arena pages needed
  unsigned groups;                 // semaphore groups whose count word starts at sem_max
  unsigned ring_groups;            // ring-mutex groups to initialise
};

// One completion (device writes, host reads); seq is written last.
struct ServeComp {
  unsigned long long id;
  unsigned long long t_admit, t_start, t_end;  // %globaltimer, ns
  unsigned status_bits, wait_site;
  unsigned long long seq;  // completion index + 1
};

struct ServeHostCtl {  // mapped host memory; the host writes
  unsigned long long tail;   // requests published
  unsigned long long stop;   // nonzero: exit once the ring is drained
  unsigned long long abort;  // nonzero: exit now (server waits give up)
};

struct ServeRec {  // one live page allocation
  unsigned long long start, pages;
  unsigned long long done;
};

struct ServeCtl {  // device memory
  unsigned lock[2 * kLineWords];  // ticket lock: [0] ticket, [kLineWords] turn
  unsigned long long qhead;       // next request to admit
  unsigned long long comp_next;   // completion slots handed out
  unsigned long long a_head, a_tail;      // arena ring allocator (pages)
  unsigned long long rec_head, rec_tail;  // live allocations, oldest first
  unsigned status[2];
  unsigned long long wait_req, wait_t0;   // the head request that did not fit (+1; 0: none) and since when
  unsigned char taken[kServeQ];           // ring entries past qhead already admitted out of order
};

// Admission past a head request that does not fit: a later request within
// kBypassWindow entries that fits is admitted first, but only while the head
// has waited less than kBypassAgeNs -- after that nothing passes it, running
// requests free their pages, and the head goes in: no request starves.
constexpr unsigned kBypassWindow = 32;
constexpr unsigned long long kBypassAgeNs = 20000000ull;

enum : int { CMD_IDLE = 0, CMD_RUN = 1, CMD_STOP = 2, CMD_REJECT = 3, CMD_WAIT = 4 };

// Tree-search requests: the walk's state image (copied in and out as the
// request's storage) and its queue items (lock-state pages, zeroed).
//   word 0 work, 32 idle, 64.. counts (u64 at byte offsets 0, 64, 128),
//   160 seed, 161 depth limit, 162 table length, 163 queues,
//   192 thresholds (128), 320 queue positions (64 per queue), then the
//   queues' cell sequence numbers (kGeoQueueCap per queue).
constexpr int kPrimUtsGeo = 50;
constexpr int kUtsQueues = 8;
constexpr size_t kUtsImageWords = 320 + (size_t)kUtsQueues * 64 + (size_t)kUtsQueues * kGeoQueueCap;

__device__ __forceinline__ void serve_uts_geo(const RunDesc& d, unsigned rank) {
  unsigned* base = d.data;
  GeoArgs g;
  g.work = base;
  g.idle = base + 32;
  g.out = reinterpret_cast<unsigned long long*>(base + 64);
  g.seed = base[160];
  g.limit = (int)base[161];
  g.nt = (int)base[162];
  g.nq = (int)base[163];
  g.table = base + 192;
  g.qpos = base + 320;
  g.qseq = base + 320 + (size_t)g.nq * 64;
  g.qitem = reinterpret_cast<GeoItem*>(d.ring);
  g.status = d.status;
  g.timeout_ns = d.timeout_ns;
  uts_geo_walk(g, rank);
}

struct __align__(128) SlotBox {  // per slot; written by its rank-0 CTA before a slot barrier
  RunDesc d;                     // absolute pointers
  unsigned long long req, rec, page, stage_off, words, state_words, id, t_admit;
  unsigned groups, ring_groups;
  int cmd, pad;
  unsigned bar[2 * kLineWords];  // slot barrier: [0] count, [kLineWords] generation
};

struct ServeArgs {
  ServeCtl* ctl;
  ServeRec* recs;
  unsigned n_recs;
  SlotBox* boxes;
  const ServeHostCtl* hctl;  // device views of mapped host memory
  const ServeDesc* ring;
  ServeComp* comp;
  unsigned char* staging;
  unsigned char* arena;
  unsigned long long pages;
  int gang;
  unsigned long long idle_ns, slot_ns;
};

__device__ __forceinline__ unsigned long long ld_acquire_sys64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_sys64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.sys.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

// Arena ring allocator (thread 0, under the server lock).  Allocations are
// contiguous page runs handed out in admission order; a run is returned when
// it and every older run are done.  Returns the first page or -1.
__device__ long long arena_alloc(const ServeArgs& a, unsigned long long need, unsigned long long* rec) {
  ServeCtl* c = a.ctl;
  if (c->rec_head - c->rec_tail >= a.n_recs) return -1;
  const unsigned long long P = a.pages;
  unsigned long long h = c->a_head, t = c->a_tail;
  long long start = -1;
  if (c->rec_head == c->rec_tail) {
    h = t = 0;
    if (need <= P) start = 0;
  } else if (h > t) {  // live [t, h): free [h, P) and [0, t)
    if (P - h >= need) start = (long long)h;
    else if (t >= need) start = 0;
  } else {  // live [t, P) and [0, h): free [h, t)
    if (t - h >= need) start = (long long)h;
  }
  if (start < 0) return -1;
  const unsigned long long r = c->rec_head % a.n_recs;
  a.recs[r].start = (unsigned long long)start;
  a.recs[r].pages = need;
  a.recs[r].done = 0;
  *rec = c->rec_head;
  c->rec_head += 1;
  c->a_head = (unsigned long long)start + need;
  c->a_tail = t;
  return start;
}

__device__ void arena_free(const ServeArgs& a, unsigned long long rec) {
  ServeCtl* c = a.ctl;
  a.recs[rec % a.n_recs].done = 1;
  while (c->rec_tail < c->rec_head && a.recs[c->rec_tail % a.n_recs].done) c->rec_tail += 1;
  if (c->rec_tail == c->rec_head) c->a_head = c->a_tail = 0;
  else c->a_tail = a.recs[c->rec_tail % a.n_recs].start;
}

// Counter barrier among the slot's CTAs (generation-valued, no resets).  Its
// wait also gives up when the host raises the abort word.
__device__ __forceinline__ bool slot_barrier(SlotBox* box, int gang, unsigned& gen, const HsEnv& env,
                                             const ServeHostCtl* hctl) {
  __syncthreads();  // every thread's stores (state, storage) precede the master's release
  int ok = 1;
  if (is_master()) {
    unsigned* count = box->bar;
    unsigned* genw = box->bar + kLineWords;
    const unsigned old = atom_add_acqrel<GPU>(count, 1u);
    if (old == (unsigned)gang - 1u) {
      st_relaxed<GPU>(count, 0u);
      st_release<GPU>(genw, gen + 1u);
    } else {
      const unsigned long long t0 = globaltimer();
      for (unsigned i = 1;; ++i) {
        if (ld_acquire<GPU>(genw) != gen) break;
        sleep_ns(256);
        if ((i & 63u) == 0u) {
          if (ld_relaxed<GPU>(env.status) != 0u || ld_relaxed_sys64(&hctl->abort) != 0ull) {
            ok = 0;
            break;
          }
          if (globaltimer() - t0 > env.timeout_ns) {
            fail(env, HS_DEV_TIMEOUT, HS_SITE_SERVE);
            ok = 0;
            break;
          }
        }
      }
    }
  }
  gen += 1u;
  return __syncthreads_or(!ok) == 0;
}

// Admission by the slot's rank-0 CTA (all its threads).  Returns the command
// for the slot; on CMD_RUN / CMD_REJECT the box holds the request.
__device__ int serve_admit(const ServeArgs& a, SlotBox* box, const HsEnv& env) {
  __shared__ int s_cmd;
  unsigned long long t_idle = globaltimer(), t_wait = 0;
  unsigned nap = 256;
  for (;;) {
    // peek without the lock: anything to admit, or a stop to honour?
    if (is_master()) {
      const unsigned long long tail = ld_acquire_sys64(&a.hctl->tail);
      const unsigned long long head = *reinterpret_cast<volatile unsigned long long*>(&a.ctl->qhead);
      s_cmd = head < tail ? CMD_RUN : (ld_relaxed_sys64(&a.hctl->stop) ? CMD_STOP : CMD_IDLE);
      if (ld_relaxed<GPU>(env.status) != 0u || ld_relaxed_sys64(&a.hctl->abort) != 0ull) s_cmd = CMD_STOP;
    }
    __syncthreads();
    int cmd = s_cmd;
    __syncthreads();
    if (cmd == CMD_RUN) {
      if (!ticket_lock<GPU>(a.ctl->lock, a.ctl->lock + kLineWords, kTicketWrap, 0u, 0u, env)) return CMD_STOP;
      if (is_master()) {
        ServeCtl* c = a.ctl;
        unsigned long long head = c->qhead;
        const unsigned long long tail = ld_acquire_sys64(&a.hctl->tail);
        while (head < tail && c->taken[head % kServeQ]) {  // skip entries admitted out of order
          c->taken[head % kServeQ] = 0;
          ++head;
        }
        c->qhead = head;
        // request k: run it if the arena has room, reject it if it never fits
        auto take = [&](unsigned long long k) {
          const ServeDesc* q = a.ring + (k % kServeQ);
          const unsigned long long need = ld_relaxed_sys64(&q->pages);
          unsigned long long rec = 0;
          int rr = CMD_WAIT;
          if (need == 0 || need > a.pages) {
            rr = CMD_REJECT;
          } else {
            const long long page = arena_alloc(a, need, &rec);
            if (page >= 0) {
              rr = CMD_RUN;
              box->rec = rec;
              box->page = (unsigned long long)page;
            }
          }
          if (rr != CMD_WAIT) box->req = k;
          return rr;
        };
        int r = CMD_IDLE;
        if (head < tail) {
          r = take(head);
          if (r != CMD_WAIT) {
            c->qhead = head + 1;
          } else {
            const unsigned long long now = globaltimer();
            if (c->wait_req != head + 1) {
              c->wait_req = head + 1;
              c->wait_t0 = now;
            }
            if (now - c->wait_t0 < kBypassAgeNs) {
              for (unsigned long long k = head + 1; k < tail && k < head + kBypassWindow; ++k) {
                if (c->taken[k % kServeQ]) continue;
                const int rk = take(k);
                if (rk != CMD_WAIT) {
                  c->taken[k % kServeQ] = 1;
                  r = rk;
                  break;
                }
              }
            }
          }
        }
        s_cmd = r;
      }
      ticket_unlock<GPU>(a.ctl->lock + kLineWords, kTicketWrap);
      __syncthreads();
      cmd = s_cmd;
      __syncthreads();
    }
    if (cmd == CMD_RUN || cmd == CMD_REJECT || cmd == CMD_STOP) return cmd;
    const unsigned long long now = globaltimer();
    if (cmd == CMD_WAIT) {  // requests are pending: running ones will free pages
      t_idle = now;
      if (!t_wait) t_wait = now;
      if (now - t_wait > a.slot_ns) {
        if (is_master()) fail(env, HS_DEV_TIMEOUT, HS_SITE_SERVE);
        return CMD_STOP;
      }
    } else {
      t_wait = 0;
      if (now - t_idle > a.idle_ns) return CMD_STOP;
    }
    if (is_master()) sleep_ns(nap);
    nap = nap < 2048u ? nap * 2u : 2048u;
    __syncthreads();
  }
}

// Copy n words between device memory and the mapped staging pool (both 256-byte
// aligned): 16-byte accesses, four in flight per thread, scalar tail.
__device__ __forceinline__ void copy_words(unsigned* dst, const unsigned* src, size_t n, size_t t, size_t stride) {
  const size_t n4 = n / 4;
  uint4* d4 = reinterpret_cast<uint4*>(dst);
  const uint4* s4 = reinterpret_cast<const uint4*>(src);
  size_t i = t;
  for (; i + 3 * stride < n4; i += 4 * stride) {
    const uint4 a = s4[i], b = s4[i + stride], c = s4[i + 2 * stride], e = s4[i + 3 * stride];
    d4[i] = a;
    d4[i + stride] = b;
    d4[i + 2 * stride] = c;
    d4[i + 3 * stride] = e;
  }
  for (; i < n4; i += stride) d4[i] = s4[i];
  for (size_t w = n4 * 4 + t; w < n; w += stride) dst[w] = src[w];
}

// The value word w of a request's lock state starts with.
__device__ __forceinline__ unsigned state_init_value(const RunDesc& d, const unsigned* base, size_t w, unsigned groups,
                                                     unsigned ring_groups) {
  const size_t locks = (size_t)(d.locks - base), ring = (size_t)(d.ring - base), sink = (size_t)(d.sink - base);
  if (w >= locks && w < ring) {
    const size_t x = w - locks;
    const size_t line = x / kLineWords, off = x % kLineWords;
    if (groups && off == 0 && line >= (size_t)d.l_grp && (line - d.l_grp) % 4 == 0 && (line - d.l_grp) / 4 < groups)
      return d.sem_max;
  } else if (w >= ring && w < sink && ring_groups) {
    const size_t x = w - ring;
    const size_t per = (size_t)d.ring_max + 1u;
    if (x % kRingStride == 0 && x / kRingStride < per * ring_groups)
      return ((x / kRingStride) % per == 0) ? 1u : 0xFFFFFFFFu;
  }
  return 0u;
}

// CL: the slot is a thread-block cluster of `gang` CTAs.  Its slot barriers are
// then the hardware cluster barrier (every CTA's work between two of them is
// bounded, and every CTA leaves the loop at the same barrier, on the command
// its rank 0 published), and a serialised instance (global mutex or
// semaphore) with numLdSt >= 33 runs as one cluster-wide executor that splits
// each critical section over the slot's SMs.
template <int MODE, bool CL>
__global__ void __launch_bounds__(kServeThreads, 4) k_serve(ServeArgs a) {
  __shared__ int s_slot;
  __shared__ int s_ok[9];
  __shared__ unsigned long long s_mbar;
  extern __shared__ __align__(128) unsigned char serve_smem[];
  TmaCtx tma;
  tma_init(tma, &s_mbar, serve_smem);
  tma.cap = dyn_smem_bytes();
  const int slot = blockIdx.x / a.gang, rank = blockIdx.x % a.gang;
  SlotBox* box = a.boxes + slot;
  const HsEnv senv{a.ctl->status, a.slot_ns};
  unsigned gen = 0;
  auto sbar = [&]() -> bool {
    if constexpr (CL) {
      cluster_sync_all();
      return true;
    } else {
      return slot_barrier(box, a.gang, gen, senv, a.hctl);
    }
  };
  const unsigned tid = threadIdx.x, nthr = blockDim.x;
  const size_t gtid = (size_t)rank * nthr + tid, gstride = (size_t)a.gang * nthr;
  for (;;) {
    if (rank == 0) {
      const int cmd = serve_admit(a, box, senv);
      if (cmd == CMD_RUN || cmd == CMD_REJECT) {
        const ServeDesc* q = a.ring + (box->req % kServeQ);
        // copy the descriptor (64-bit words, system scope) into the box
        constexpr int kW = (int)(sizeof(ServeDesc) / 8);
        __shared__ unsigned long long s_desc[kW];
        for (int i = tid; i < kW; i += nthr)
          s_desc[i] = ld_relaxed_sys64(reinterpret_cast<const unsigned long long*>(q) + i);
        __syncthreads();
        if (is_master()) {
          const ServeDesc* sd = reinterpret_cast<const ServeDesc*>(s_desc);
          RunDesc d = sd->d;
          if (cmd == CMD_RUN) {
            unsigned char* base = a.arena + box->page * kPageBytes;
            d.data = reinterpret_cast<unsigned*>(base + reinterpret_cast<size_t>(d.data));
            d.locks = reinterpret_cast<unsigned*>(base + reinterpret_cast<size_t>(d.locks));
            d.ring = reinterpret_cast<unsigned*>(base + reinterpret_cast<size_t>(d.ring));
            d.status = reinterpret_cast<unsigned*>(base + reinterpret_cast<size_t>(d.status));
            d.sink = reinterpret_cast<unsigned*>(base + reinterpret_cast<size_t>(d.sink));
          }
          box->d = d;
          box->id = sd->id;
          box->stage_off = sd->stage_off;
          box->words = sd->words;
          box->state_words = sd->state_words;
          box->groups = sd->groups;
          box->ring_groups = sd->ring_groups;
          box->t_admit = globaltimer();
        }
      }
      if (is_master()) box->cmd = cmd;
    }
    if (!sbar()) break;
    // the box was rewritten for this request: read it at gpu scope (no stale
    // L1 line from an earlier request) and share it through shared memory
    constexpr int kBW = (int)(offsetof(SlotBox, bar) / 8);
    __shared__ unsigned long long s_box[kBW];
    for (int i = tid; i < kBW; i += nthr) {
      unsigned long long v;
      asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v)
                   : "l"(reinterpret_cast<const unsigned long long*>(box) + i) : "memory");
      s_box[i] = v;
    }
    __syncthreads();
    const SlotBox& sb = *reinterpret_cast<const SlotBox*>(s_box);
    const int cmd = sb.cmd;
    if (cmd == CMD_STOP) break;
    const RunDesc d = sb.d;
    const unsigned long long id = sb.id, stage_off = sb.stage_off, words = sb.words;
    const unsigned long long t_admit = sb.t_admit, rec = sb.rec;
    unsigned long long t_start = 0;
    if (cmd == CMD_RUN) {
      // storage in from the staging pool; lock state laid out
      copy_words(d.data, reinterpret_cast<const unsigned*>(a.staging + stage_off), words, gtid, gstride);
      unsigned* base = d.status;
      const size_t sw = sb.state_words;
      const unsigned groups = sb.groups, rgroups = sb.ring_groups;
      for (size_t w = gtid; w < sw; w += gstride) base[w] = state_init_value(d, base, w, groups, rgroups);
      if (!sbar()) break;
      t_start = globaltimer();
      const HsEnv env{d.status, d.timeout_ns};
      if (d.prim == kPrimUtsGeo) {
        serve_uts_geo(d, (unsigned)rank);
      } else if (is_relaxed_prim(d.prim)) {
        bool ok = true;
        for (int j = 0; j < d.iters && ok; ++j)
          for (int b = rank; b < d.num_tbs && ok; b += a.gang) ok = relaxed_op(d, b, j, env);
      } else if (is_mutex_prim(d.prim) || is_sem_prim(d.prim)) {
        const bool mtx = is_mutex_prim(d.prim);
        const bool whole = CL && d.prim >= 4 && d.prim <= 15 && d.L >= 33;
        const int ecl = whole ? a.gang : 1, er = whole ? rank : 0;
        const int execs = a.gang / ecl, x = rank / ecl;
        bool ok = true;
        for (int j = 0; j < d.iters && ok; ++j)
          for (int b = x; b < d.num_tbs && ok; b += execs)
            ok = mtx ? cl_mutex_op<MODE>(d, b, er, ecl, &s_slot, s_ok, tma, env)
                     : cl_sem_op<MODE>(d, b, er, ecl, s_ok, tma, env);
      } else {
        batch_barrier<MODE>(d, rank, a.gang, 0u, tma, env);
      }
      if (!sbar()) break;
      copy_words(reinterpret_cast<unsigned*>(a.staging + stage_off), d.data, words, gtid, gstride);
      __syncthreads();
      if (is_master()) __threadfence_system();
      if (!sbar()) break;
    }
    if (rank == 0) {
      if (is_master()) {
        const unsigned long long k = atomicAdd(&a.ctl->comp_next, 1ull);
        ServeComp* r = a.comp + (k % kServeC);
        r->id = id;
        r->t_admit = t_admit;
        r->t_start = t_start;
        r->t_end = globaltimer();
        if (cmd == CMD_RUN) {
          r->status_bits = ld_relaxed<GPU>(d.status);
          r->wait_site = ld_relaxed<GPU>(d.status + 1);
        } else {
          r->status_bits = HS_DEV_BADARG;
          r->wait_site = 0;
        }
        __threadfence_system();
        st_release_sys64(&r->seq, k + 1ull);
      }
      if (cmd == CMD_RUN) {
        if (ticket_lock<GPU>(a.ctl->lock, a.ctl->lock + kLineWords, kTicketWrap, 0u, 0u, senv)) {
          if (is_master()) arena_free(a, rec);
          ticket_unlock<GPU>(a.ctl->lock + kLineWords, kTicketWrap);
        } else if (!CL) {
          break;  // the server status is set: the next admission stops every slot
        }
      }
    }
  }
}

}  // namespace hs

using namespace hs;

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {
thread_local std::string g_serr;
size_t r64(size_t w) { return (w + 63) / 64 * 64; }
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

struct hs_server {
  int slots = 0, gang = 0, nsm = 0, mode = HS_MODE_INC;
  unsigned long long pages = 0;
  cudaStream_t stream = nullptr;
  unsigned char* hblock = nullptr;  // mapped pinned host memory
  unsigned char* dblock = nullptr;  // its device view
  size_t hbytes = 0, staging_off = 0, staging_bytes = 0;
  ServeHostCtl* hctl = nullptr;
  ServeDesc* ring = nullptr;
  ServeComp* comp = nullptr;
  unsigned char* dev = nullptr;  // ServeCtl + recs + boxes
  unsigned char* arena = nullptr;
  std::mutex mu;
  unsigned long long next_id = 1, submitted = 0, polled = 0;
  std::map<size_t, size_t> free_stage;  // offset -> bytes
  struct Pending {
    size_t off, bytes;
    uint32_t* out;
    size_t words;
    double t_submit;
    unsigned ring_slot;
  };
  std::vector<char> ring_busy = std::vector<char>(kServeQ, 0);  // entry's request not yet polled
  std::unordered_map<unsigned long long, Pending> pending;
  bool running = false;
};

extern "C" const char* hs_serve_last_error(void) { return g_serr.c_str(); }

static int stage_alloc(hs_server* S, size_t bytes, size_t* off) {
  bytes = (bytes + 255) / 256 * 256;
  for (auto it = S->free_stage.begin(); it != S->free_stage.end(); ++it) {
    if (it->second >= bytes) {
      *off = it->first;
      const size_t rest = it->second - bytes, at = it->first + bytes;
      S->free_stage.erase(it);
      if (rest) S->free_stage[at] = rest;
      return HS_OK;
    }
  }
  return HS_ENORES;
}

static void stage_free(hs_server* S, size_t off, size_t bytes) {
  bytes = (bytes + 255) / 256 * 256;
  auto it = S->free_stage.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != S->free_stage.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    S->free_stage.erase(nx);
  }
  if (it != S->free_stage.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      S->free_stage.erase(it);
    }
  }
}

static void serve_free(hs_server* S) {
  if (S->stream) cudaStreamDestroy(S->stream);
  if (S->hblock) cudaFreeHost(S->hblock);
  cudaFree(S->dev);
  cudaFree(S->arena);
  delete S;
}

extern "C" int hs_serve_start(int slots, int gang, unsigned long long arena_bytes, unsigned long long staging_bytes,
                              double idle_timeout_s, hs_server** out) {
  if (!out || slots <= 0 || gang <= 0 || arena_bytes < kPageBytes || staging_bytes < 4096 || idle_timeout_s <= 0) {
    g_serr = "need slots > 0, gang > 0, arena >= 64 KiB, staging >= 4 KiB, idle timeout > 0";
    return HS_EINVAL;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  hs_server* S = new hs_server();
  S->slots = slots;
  S->gang = gang;
  cudaDeviceGetAttribute(&S->nsm, cudaDevAttrMultiProcessorCount, dev);
  // slots of 2, 4 or 8 CTAs run as thread-block clusters
  const bool cl = gang == 2 || gang == 4 || gang == 8;
  const void* fn = cl ? (const void*)k_serve<M_INC, true> : (const void*)k_serve<M_INC, false>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kServeStage) != cudaSuccess) {
    g_serr = "shared memory attribute";
    delete S;
    return HS_ECUDA;
  }
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl ? (unsigned)gang : 1u;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3((unsigned)(slots * gang));
  lc.blockDim = dim3((unsigned)kServeThreads);
  lc.dynamicSmemBytes = kServeStage;
  lc.attrs = attr;
  lc.numAttrs = cl ? 1 : 0;
  long long capacity = 0;
  if (cl) {
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, fn, &lc) != cudaSuccess) {
      cudaGetLastError();
      g_serr = "cluster occupancy query failed";
      delete S;
      return HS_ECUDA;
    }
    capacity = (long long)clusters * gang;
  } else {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kServeThreads, kServeStage);
    capacity = (long long)per_sm * S->nsm;
  }
  if ((long long)slots * gang > capacity) {
    g_serr = std::to_string(slots * gang) + " server CTAs cannot all be resident (" + std::to_string(capacity) + ")";
    delete S;
    return HS_ENORES;
  }
  S->pages = arena_bytes / kPageBytes;
  const size_t ring_off = 256, comp_off = ring_off + sizeof(ServeDesc) * kServeQ;
  S->staging_off = (comp_off + sizeof(ServeComp) * kServeC + 4095) / 4096 * 4096;
  S->staging_bytes = (size_t)staging_bytes;
  S->hbytes = S->staging_off + S->staging_bytes;
  const unsigned n_recs = (unsigned)(2 * slots + 2);
  const size_t recs_off = (sizeof(ServeCtl) + 255) / 256 * 256;
  const size_t boxes_off = recs_off + (sizeof(ServeRec) * n_recs + 255) / 256 * 256;
  const size_t dev_bytes = boxes_off + sizeof(SlotBox) * slots;
  if (cudaHostAlloc(&S->hblock, S->hbytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&S->dblock, S->hblock, 0) != cudaSuccess ||
      cudaMalloc(&S->dev, dev_bytes) != cudaSuccess || cudaMalloc(&S->arena, S->pages * kPageBytes) != cudaSuccess ||
      cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    g_serr = "allocation failed";
    serve_free(S);
    return HS_ENORES;
  }
  std::memset(S->hblock, 0, S->staging_off);
  S->hctl = reinterpret_cast<ServeHostCtl*>(S->hblock);
  S->ring = reinterpret_cast<ServeDesc*>(S->hblock + ring_off);
  S->comp = reinterpret_cast<ServeComp*>(S->hblock + comp_off);
  S->free_stage[0] = S->staging_bytes;
  if (cudaMemset(S->dev, 0, dev_bytes) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
    g_serr = "device init failed";
    serve_free(S);
    return HS_ECUDA;
  }
  ServeArgs a;
  a.ctl = reinterpret_cast<ServeCtl*>(S->dev);
  a.recs = reinterpret_cast<ServeRec*>(S->dev + recs_off);
  a.n_recs = n_recs;
  a.boxes = reinterpret_cast<SlotBox*>(S->dev + boxes_off);
  a.hctl = reinterpret_cast<const ServeHostCtl*>(S->dblock);
  a.ring = reinterpret_cast<const ServeDesc*>(S->dblock + ring_off);
  a.comp = reinterpret_cast<ServeComp*>(S->dblock + comp_off);
  a.staging = S->dblock + S->staging_off;
  a.arena = S->arena;
  a.pages = S->pages;
  a.gang = gang;
  a.idle_ns = (unsigned long long)(idle_timeout_s * 1e9);
  a.slot_ns = a.idle_ns + 120000000000ull;  // a slot waits for its own CTAs (admission, then one instance)
  void* args[] = {&a};
  lc.stream = S->stream;
  if (cudaLaunchKernelExC(&lc, fn, args) != cudaSuccess) {
    g_serr = "server launch failed";
    serve_free(S);
    return HS_ECUDA;
  }
  hs_note_launches(1);
  S->running = true;
  *out = S;
  return HS_OK;
}

// Storage words of a request (input = output = the instance's shared data).
extern "C" int hs_serve_request_words(const hs_serve_request* r, int nsm, size_t* words) {
  if (r && words && r->kind == HS_REQ_UTS_GEO) {
    *words = kUtsImageWords;
    return HS_OK;
  }
  if (!r || !words || r->kind != HS_REQ_SYNCPRIM) return HS_EINVAL;
  const hs_batch_instance x{r->prim, r->num_ldst, r->num_tbs, r->num_iters};
  return hs_batch_instance_words(&x, nsm, words);
}

extern "C" int hs_serve_uts_geo_counts(const uint32_t* w, size_t words, unsigned long long* nodes,
                                       unsigned long long* leaves, unsigned* deepest) {
  if (!w || words < kUtsImageWords) return HS_EINVAL;
  auto u64 = [&](size_t at) { return (unsigned long long)w[at] | ((unsigned long long)w[at + 1] << 32); };
  if (nodes) *nodes = u64(64);
  if (leaves) *leaves = u64(80);
  if (deepest) *deepest = (unsigned)u64(96);
  return HS_OK;
}

static int submit_uts_geo(hs_server* S, const hs_serve_request* r, uint32_t* output, unsigned long long* id_out);

extern "C" int hs_serve_submit(hs_server* S, const hs_serve_request* r, const uint32_t* input, uint32_t* output,
                               unsigned long long* id_out) {
  if (S && r && output && r->kind == HS_REQ_UTS_GEO) return submit_uts_geo(S, r, output, id_out);
  if (!S || !r || !input || !output || r->kind != HS_REQ_SYNCPRIM) {
    g_serr = "need a server, a SyncPrims or tree-search request, input and output";
    return HS_EINVAL;
  }
  hs_run_config c;
  hs_run_config_default(&c);
  c.prim = r->prim;
  c.num_ldst = r->num_ldst;
  c.num_tbs = r->num_tbs;
  c.num_iters = r->num_iters;
  c.threads = 256;
  c.repeats = 1;
  c.mode = HS_MODE_INC;
  size_t words = 0;
  Layout L;
  const bool relaxed = r->prim >= HS_BATCH_REFCOUNTER && r->prim <= HS_BATCH_FLAGS;
  if (relaxed) {  // counters / payload / data words; line 4 holds the sequence or flag word
    const hs_batch_instance x{r->prim, r->num_ldst, r->num_tbs, r->num_iters};
    if (hs_batch_instance_words(&x, S->nsm, &words) != HS_OK) {
      g_serr = "bad relaxed-atomics request";
      return HS_EINVAL;
    }
    std::memset(&L, 0, sizeof(L));
    L.l_grp = 4;
    L.groups = 1;
    L.lines = 8;
  } else {
    int s = hs_storage_words(&c, S->nsm, &words);
    if (s) {
      g_serr = hs_last_error();
      return s;
    }
    hs_layout_for(&c, S->nsm, &L);
  }
  // pages: status (64 words) | lock lines | ring | sink | data
  const size_t locks = 64, ring = locks + r64((size_t)L.lines * kLineWords), sink = ring + r64(L.ring_words);
  const size_t state_words = sink + r64((size_t)c.num_tbs);
  const size_t total = (state_words + r64(words)) * 4;
  const double t_submit = now_s();
  std::lock_guard<std::mutex> g(S->mu);
  if (!S->running) {
    g_serr = "server stopped";
    return HS_EINVAL;
  }
  const unsigned slot = (unsigned)(S->submitted % kServeQ);
  if (S->submitted - S->polled >= std::min(kServeQ, kServeC) - 1 || S->ring_busy[slot]) {
    g_serr = "too many requests in flight";
    return HS_ENORES;
  }
  size_t off = 0;
  if (stage_alloc(S, words * 4, &off) != HS_OK) {
    g_serr = "staging pool full";
    return HS_ENORES;
  }
  std::memcpy(S->hblock + S->staging_off + off, input, words * 4);
  const unsigned long long id = S->next_id++;
  ServeDesc q;
  std::memset(&q, 0, sizeof(q));
  RunDesc& d = q.d;
  d.status = reinterpret_cast<unsigned*>((size_t)0);
  d.locks = reinterpret_cast<unsigned*>(locks * 4);
  d.ring = reinterpret_cast<unsigned*>(ring * 4);
  d.sink = reinterpret_cast<unsigned*>(sink * 4);
  d.data = reinterpret_cast<unsigned*>(state_words * 4);
  d.prim = c.prim;
  d.mode = HS_MODE_INC;
  d.T = 256;
  d.L = c.num_ldst;
  d.num_tbs = c.num_tbs;
  d.iters = c.num_iters;
  d.nsm = S->nsm;
  d.sem_max = relaxed ? 1u : (unsigned)hs_prim_sem_count(c.prim) + 1u;
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
  q.id = id;
  q.stage_off = off;
  q.words = words;
  q.state_words = state_words;
  q.pages = (total + kPageBytes - 1) / kPageBytes;
  q.groups = d.sem_max > 1u ? (unsigned)L.groups : 0u;
  q.ring_groups = (c.prim == 6 || c.prim == 22) ? (c.prim == 22 ? (unsigned)S->nsm : 1u) : 0u;
  std::memcpy(&S->ring[slot], &q, sizeof(q));
  S->ring_busy[slot] = 1;
  S->pending[id] = hs_server::Pending{off, words * 4, output, words, t_submit, slot};
  S->submitted += 1;
  std::atomic_thread_fence(std::memory_order_release);
  __atomic_store_n(&S->hctl->tail, S->submitted, __ATOMIC_RELEASE);
  if (id_out) *id_out = id;
  return HS_OK;
}

// Publish a ready descriptor whose storage image (words) is `image`.
static int publish(hs_server* S, ServeDesc& q, const uint32_t* image, size_t words, uint32_t* output, double t_submit,
                   unsigned long long* id_out) {
  std::lock_guard<std::mutex> g(S->mu);
  if (!S->running) {
    g_serr = "server stopped";
    return HS_EINVAL;
  }
  const unsigned slot = (unsigned)(S->submitted % kServeQ);
  if (S->submitted - S->polled >= std::min(kServeQ, kServeC) - 1 || S->ring_busy[slot]) {
    g_serr = "too many requests in flight";
    return HS_ENORES;
  }
  size_t off = 0;
  if (stage_alloc(S, words * 4, &off) != HS_OK) {
    g_serr = "staging pool full";
    return HS_ENORES;
  }
  std::memcpy(S->hblock + S->staging_off + off, image, words * 4);
  const unsigned long long id = S->next_id++;
  q.id = id;
  q.stage_off = off;
  q.words = words;
  std::memcpy(&S->ring[slot], &q, sizeof(q));
  S->ring_busy[slot] = 1;
  S->pending[id] = hs_server::Pending{off, words * 4, output, words, t_submit, slot};
  S->submitted += 1;
  std::atomic_thread_fence(std::memory_order_release);
  __atomic_store_n(&S->hctl->tail, S->submitted, __ATOMIC_RELEASE);
  if (id_out) *id_out = id;
  return HS_OK;
}

static int submit_uts_geo(hs_server* S, const hs_serve_request* r, uint32_t* output, unsigned long long* id_out) {
  if (r->depth_limit < 0 || r->depth_limit > kGeoMaxDepth || !(r->branching > 0.0)) {
    g_serr = "tree search needs 0 <= depth_limit <= 30 and branching > 0";
    return HS_EINVAL;
  }
  const double t_submit = now_s();
  std::vector<uint32_t> img(kUtsImageWords, 0u);
  img[0] = 1u;  // work: the root's thread
  img[160] = r->seed;
  img[161] = (uint32_t)r->depth_limit;
  img[162] = (uint32_t)hs_uts_geo_table(r->branching, img.data() + 192, kGeoTable);
  img[163] = (uint32_t)kUtsQueues;
  for (int qn = 0; qn < kUtsQueues; ++qn)
    for (unsigned i = 0; i < kGeoQueueCap; ++i) img[320 + kUtsQueues * 64 + qn * kGeoQueueCap + i] = i;
  // pages: status (64 words) | queue items (lock state, zeroed) | sink | image
  const size_t items = 64, sink = items + r64((size_t)kUtsQueues * kGeoQueueCap * (sizeof(GeoItem) / 4));
  const size_t state_words = sink + 64;
  ServeDesc q;
  std::memset(&q, 0, sizeof(q));
  RunDesc& d = q.d;
  d.status = reinterpret_cast<unsigned*>((size_t)0);
  d.locks = reinterpret_cast<unsigned*>(items * 4);
  d.ring = reinterpret_cast<unsigned*>(items * 4);
  d.sink = reinterpret_cast<unsigned*>(sink * 4);
  d.data = reinterpret_cast<unsigned*>(state_words * 4);
  d.prim = kPrimUtsGeo;
  d.mode = HS_MODE_INC;
  d.T = 256;
  d.num_tbs = 1;
  d.iters = 1;
  d.nsm = S->nsm;
  d.sem_max = 1;
  d.timeout_ns = 10000000000ull;
  d.skip_tb = -1;
  d.cluster = 1;
  q.state_words = state_words;
  q.pages = ((state_words + r64(kUtsImageWords)) * 4 + kPageBytes - 1) / kPageBytes;
  q.groups = 0;
  q.ring_groups = 0;
  return publish(S, q, img.data(), kUtsImageWords, output, t_submit, id_out);
}

static int poll_locked(hs_server* S, hs_serve_completion* out, int max, int* n) {
  int k = 0;
  while (k < max) {
    ServeComp* r = &S->comp[S->polled % kServeC];
    if (__atomic_load_n(&r->seq, __ATOMIC_ACQUIRE) != S->polled + 1) break;
    const double t = now_s();
    hs_serve_completion& c = out[k];
    std::memset(&c, 0, sizeof(c));
    c.id = r->id;
    c.dev_error_bits = r->status_bits;
    c.wait_site = r->wait_site;
    c.service_us = r->t_start ? (double)(r->t_end - r->t_start) * 1e-3 : 0.0;
    c.admit_to_end_us = (double)(r->t_end - r->t_admit) * 1e-3;
    auto it = S->pending.find(r->id);
    if (it != S->pending.end()) {
      const hs_server::Pending& p = it->second;
      c.latency_us = (t - p.t_submit) * 1e6;
      if (r->status_bits == 0u) {
        std::memcpy(p.out, S->hblock + S->staging_off + p.off, p.words * 4);
        c.status = HS_OK;
      } else {
        c.status = (r->status_bits & HS_DEV_BADARG) ? HS_ENORES : HS_ETIMEDOUT;
      }
      stage_free(S, p.off, p.bytes);
      S->ring_busy[p.ring_slot] = 0;
      S->pending.erase(it);
    }
    S->polled += 1;
    ++k;
  }
  *n = k;
  return HS_OK;
}

extern "C" int hs_serve_poll(hs_server* S, hs_serve_completion* out, int max, int* n) {
  if (!S || !out || !n || max < 0) return HS_EINVAL;
  std::lock_guard<std::mutex> g(S->mu);
  return poll_locked(S, out, max, n);
}

extern "C" int hs_serve_pending(hs_server* S, unsigned long long* in_flight) {
  if (!S || !in_flight) return HS_EINVAL;
  std::lock_guard<std::mutex> g(S->mu);
  *in_flight = S->submitted - S->polled;
  return HS_OK;
}

// Drain and stop: the kernel exits once every published request is admitted;
// completions not yet polled stay readable until hs_serve_destroy.
extern "C" int hs_serve_stop(hs_server* S, double timeout_s) {
  if (!S) return HS_EINVAL;
  if (!S->running) return HS_OK;
  __atomic_store_n(&S->hctl->stop, 1ull, __ATOMIC_RELEASE);
  double t0 = now_s();
  cudaError_t e = cudaErrorNotReady;
  bool aborted = false;
  while ((e = cudaStreamQuery(S->stream)) == cudaErrorNotReady) {
    if (now_s() - t0 > timeout_s) {
      if (aborted) {
        g_serr = "server did not stop in time";
        return HS_ETIMEDOUT;  // still running: its memory stays allocated
      }
      // not drained in time: make every server wait give up (a running
      // instance still ends within its own wait limit)
      __atomic_store_n(&S->hctl->abort, 1ull, __ATOMIC_RELEASE);
      aborted = true;
      t0 = now_s();
      timeout_s = 60.0;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  S->running = false;
  if (e != cudaSuccess) {
    g_serr = cudaGetErrorString(e);
    return HS_ECUDA;
  }
  unsigned st[2] = {0, 0};
  cudaMemcpy(st, reinterpret_cast<ServeCtl*>(S->dev)->status, sizeof(st), cudaMemcpyDeviceToHost);
  if (st[0] || aborted) {
    g_serr = aborted ? "server aborted before its ring drained" : "server wait timed out";
    return HS_ETIMEDOUT;
  }
  return HS_OK;
}

extern "C" int hs_serve_destroy(hs_server* S) {
  if (!S) return HS_EINVAL;
  if (S->running) {
    const int s = hs_serve_stop(S, 120.0);
    if (s == HS_ETIMEDOUT && S->running) return s;  // still running: freeing its memory is not safe
  }
  serve_free(S);
  return HS_OK;
}

// Open-loop driver: request i is due at arrival_s[i] seconds after the start;
// one host thread publishes requests when due (retrying while the ring or the
// staging pool is full), another polls completions.  Latency is measured from
// the due time, so time spent queued on the host counts.
extern "C" int hs_serve_drive(hs_server* S, const hs_serve_request* reqs, int n, const uint32_t* const* inputs,
                              uint32_t* const* outputs, const double* arrival_s, double timeout_s,
                              hs_serve_completion* comps, double* wall_s) {
  if (!S || !reqs || n <= 0 || !inputs || !outputs || !arrival_s || !comps) return HS_EINVAL;
  std::vector<unsigned long long> ids(n, 0);
  std::vector<double> due(n);
  std::unordered_map<unsigned long long, int> index;
  std::mutex imu;
  std::atomic<int> submit_err{HS_OK};
  const double t0 = now_s();
  for (int i = 0; i < n; ++i) due[i] = t0 + arrival_s[i];
  std::thread pub([&] {
    for (int i = 0; i < n; ++i) {
      while (now_s() < due[i]) {
      }
      for (;;) {
        unsigned long long id = 0;
        const int s = hs_serve_submit(S, &reqs[i], inputs[i], outputs[i], &id);
        if (s == HS_OK) {
          std::lock_guard<std::mutex> g(imu);
          ids[i] = id;
          index[id] = i;
          break;
        }
        if (s != HS_ENORES || now_s() - t0 > timeout_s) {
          submit_err = s ? s : HS_ETIMEDOUT;
          return;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
    }
  });
  int done = 0, status = HS_OK;
  std::vector<hs_serve_completion> buf(256);
  while (done < n) {
    int k = 0;
    hs_serve_poll(S, buf.data(), (int)buf.size(), &k);
    const double t = now_s();
    for (int j = 0; j < k; ++j) {
      int i = -1;
      {
        std::lock_guard<std::mutex> g(imu);
        auto it = index.find(buf[j].id);
        if (it != index.end()) i = it->second;
      }
      if (i < 0) continue;
      comps[i] = buf[j];
      comps[i].latency_us = (t - due[i]) * 1e6;
      ++done;
    }
    if (k == 0) {
      if (submit_err.load() != HS_OK || now_s() - t0 > timeout_s) {
        status = submit_err.load() != HS_OK ? submit_err.load() : HS_ETIMEDOUT;
        break;
      }
      std::this_thread::yield();
    }
  }
  pub.join();
  if (wall_s) *wall_s = now_s() - t0;
  if (status != HS_OK) g_serr = "driver stopped early";
  return status;
}
