// hs_syncprims.cu -- the SyncPrims kernels (mutexes, semaphores, tree barriers)
// for sm_103a.
//
// Each kernel executes numCSIters iterations per TB of the reference kernel of
// the same name (heterosync cuda/syncPrims/uvm/main.cu:104-836): acquire,
// critical section on the shared data, release -- or, for barriers, data
// access then barrier.  Which TB touches which data, and when, follows the
// reference exactly, so the final shared data equals the reference's golden.
//
// What is different is how each step maps onto the GPU:
//  * the critical section moves whole 16-byte vectors: all loads of a pass are
//    issued before any store (one L2 round trip instead of numLdSt dependent
//    load->store round trips), separated by one CTA barrier;
//  * lock words are padded to their own 128-byte line;
//  * one lane polls with ld.acquire and broadcasts with one bar.red;
//  * releases are single st.release / red.release operations;
//  * barrier state is generation-valued (no resets) and groups may be uneven;
//  * every wait is bounded (see hs_device.cuh).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdlib>
#include "hs_exec.cuh"

namespace hs {

// ---------------------------------------------------------------------------
// Mutex kernels: main.cu:317-529.  Global variants: one lock, every TB works on
// chunk 0.  Uniq variants: lock and chunk per logical SM (blockIdx % NUM_SM).
// ---------------------------------------------------------------------------
// One TB's iterations of a mutex kernel, at scope S (GPU: lock words in L2;
// CLUSTER: lock words in the shared memory of the group's cluster rank 0).
template <int S, int KIND, int MODE, int V, bool TMA>
__device__ __forceinline__ void mutex_loop(const RunDesc& d, int g, int r, int m, int G, unsigned* w0, unsigned* w1,
                                           unsigned* w2, unsigned* ring, unsigned ring_max, unsigned wrap,
                                           int* s_slot, TmaCtx& tma, const HsEnv& env) {
  if constexpr (S == GPU && KIND != MK_SLEEP) {
    if (d.cohort) {  // global mutex as a cohort of per-die ticket queues (hs_device.cuh)
      unsigned sm;
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      const int die = d.die_map[sm & 255u] & 1;
      unsigned* const* c = d.coh + 3 * die;
      unsigned my = 0, pc = 0, aux = 0;  // meaningful in the master thread
      for (int j = 0; j < d.iters; ++j) {
        bool ok;
        if constexpr (KIND == MK_FA) {
          ok = cohort_ticket_lock(c[0], c[1], w0, w1, wrap, d.bo_unit, d.bo_max, env, my, pc, aux);
        } else {
          ok = cohort_queue_lock(
              c[0], c[1],
              [&] {
                unsigned b = d.bo_min;
                return wait_until(
                    [&] { return ld_relaxed<GPU>(w0) == 0u && atom_cas_acquire<GPU>(w0, 0u, 1u) == 0u; },
                    [&] {
                      if constexpr (KIND == MK_EBO) {
                        sleep_ns(b);
                        b = ebo_next(b, d.bo_max);
                      }
                    },
                    env, KIND == MK_EBO ? HS_SITE_EBO_LOCK : HS_SITE_SPIN_LOCK);
              },
              env, KIND == MK_EBO ? HS_SITE_EBO_LOCK : HS_SITE_SPIN_LOCK, my, pc, aux);
        }
        if (!ok) break;
        if constexpr (MODE == M_SLICE) cs_slice(d.data, g + ((r + j) % m) * G, d.L);
        else if constexpr (TMA) ok = cs_chunk_tma<MODE>(d, g, tma, env);
        else cs_chunk<MODE, V>(d, g);
        if constexpr (KIND == MK_FA) {
          cohort_ticket_unlock(c[1], w1, wrap, my, pc, aux);
        } else {
          cohort_queue_unlock(c[1], [&] { st_release<GPU>(w0, 0u); }, my, pc, aux);
        }
        if (!ok) break;
      }
      return;
    }
  }
  for (int j = 0; j < d.iters; ++j) {
    bool ok;
    int slot = 0;
    if constexpr (KIND == MK_SPIN) ok = spin_lock<S>(w0, env);
    else if constexpr (KIND == MK_EBO) ok = ebo_lock<S>(w0, d.bo_min, d.bo_max, env);
    else if constexpr (KIND == MK_FA) ok = ticket_lock<S>(w0, w1, wrap, d.bo_unit, d.bo_max, env);
    else {
      slot = queue_lock<S>(w2, ring, kRingStride, ring_max, d.bo_unit, env, s_slot);
      ok = slot >= 0;
    }
    if (!ok) break;

    if constexpr (MODE == M_SLICE) cs_slice(d.data, g + ((r + j) % m) * G, d.L);
    else if constexpr (TMA) ok = cs_chunk_tma<MODE>(d, g, tma, env);
    else cs_chunk<MODE, V>(d, g);

    if constexpr (KIND == MK_SPIN || KIND == MK_EBO) spin_unlock<S>(w0);
    else if constexpr (KIND == MK_FA) ticket_unlock<S>(w1, wrap);
    else queue_unlock<S>(ring, kRingStride, ring_max, (unsigned)slot);
    if (!ok) break;  // a bounded copy wait gave up (status already recorded)
  }
}

// ---------------------------------------------------------------------------
// Mutex kernels: main.cu:317-529.  Global variants: one lock, every TB works on
// chunk 0.  Uniq variants: lock and chunk per logical SM (blockIdx % NUM_SM).
// Uniq with d.cluster = m > 1 (numTBs = m * NUM_SM): each logical SM's group is
// one thread-block cluster -- physical CTA p runs logical TB g + r*NUM_SM with
// g = p / m, r = p % m -- and its lock lives in rank 0's shared memory, taken
// and released with cluster-scope atomics on distributed shared memory.
// ---------------------------------------------------------------------------
template <int KIND, bool UNIQ, int MODE, int V, bool TMA = false>
__global__ void __launch_bounds__(TMA ? 256 : Bounds<V>::kThreads) k_mutex(RunDesc d) {
  __shared__ int s_slot;
  __shared__ unsigned long long s_mbar[kTmaParts];
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  TmaCtx tma;
  if constexpr (TMA) tma_init(tma, s_mbar, dyn_smem, kTmaParts);
  const unsigned wrap = UNIQ ? 100000000u : 1000000000u;  // cudaLocksMutexFA.cu:24,83
  const HsEnv env{d.status, d.timeout_ns};
  if constexpr (UNIQ) {
    if (d.cluster > 1) {
      __shared__ unsigned s_cl_lock[3 * kLineWords];
      __shared__ unsigned s_cl_ring[9 * kRingStride];
      const int mc = d.cluster;
      const int g = (int)blockIdx.x / mc, r = (int)blockIdx.x % mc;
      if (r == 0) {  // the group's lock state, fresh for this launch (ring slot 0 holds the token)
        for (int i = threadIdx.x; i < 3 * kLineWords; i += blockDim.x) s_cl_lock[i] = 0u;
        for (int i = threadIdx.x; i < 9 * kRingStride; i += blockDim.x)
          s_cl_ring[i] = (i % kRingStride) ? 0u : (i == 0 ? 1u : 0xFFFFFFFFu);
      }
      cluster_sync_all();
      unsigned* lock0 = map_shared_rank(s_cl_lock, 0u);
      mutex_loop<CLUSTER, KIND, MODE, V, TMA>(d, g, r, mc, d.nsm, lock0, lock0 + kLineWords, lock0 + 2 * kLineWords,
                                              map_shared_rank(s_cl_ring, 0u), (unsigned)mc, wrap, &s_slot, tma,
                                              env);
      cluster_sync_all();  // rank 0's lock words stay valid until every rank is done
      return;
    }
  }
  const int b = blockIdx.x;
  const int g = UNIQ ? (b % d.nsm) : 0;
  // SLICE mode bookkeeping: group members b = g + r*G, r = 0..m-1.
  const int G = UNIQ ? d.nsm : 1;
  const int r = b / G;
  const int m = (d.num_tbs - g + G - 1) / G;
  mutex_loop<GPU, KIND, MODE, V, TMA>(d, g, r, m, G, group_line(d, g, 0), group_line(d, g, 1), group_line(d, g, 2),
                                      d.ring + (size_t)g * (d.ring_max + 1) * kRingStride, d.ring_max, wrap, &s_slot,
                                      tma, env);
}

// One TB's iterations of a semaphore kernel, at scope S.  A global semaphore
// with d.cohort set runs its writers as die cohorts (cohort_sem_writer_wait).
template <int S, bool EBO, bool UNIQ, int MODE, int V, bool TMA>
__device__ __forceinline__ void sem_loop(const RunDesc& d, int b, int numSM, int k, bool writer, unsigned* st,
                                         int rchunk, TmaCtx& tma, const HsEnv& env) {
  const int Gd = d.num_tbs;
  unsigned* const* local = nullptr;  // the writer's die cohort lines (cohort runs only)
  if constexpr (S == GPU && !UNIQ) {
    if (d.cohort && writer) {
      unsigned sm;
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      local = d.coh + 3 * (d.die_map[sm & 255u] & 1);
    }
  }
  for (int i = 0; i < d.iters; ++i) {
    unsigned my = 0, pc = 0, snap = 0;  // cohort state (master thread)
    const bool got = local ? cohort_sem_writer_wait(local[0], local[1], st, d.sem_max, EBO, d.bo_min, d.bo_max, env,
                                                    my, pc, snap)
                           : sem_wait<S>(st, writer, d.sem_max, EBO, !UNIQ, d.bo_min, d.bo_max, env);
    if (!got) break;
    bool ok = true;
    if (writer) {
      int cur = UNIQ ? b : 0;
      for (int j = 0; j < k && ok; ++j) {
        if constexpr (TMA) ok = cs_chunk_tma<MODE>(d, cur, tma, env);
        else cs_chunk<MODE, V>(d, cur);
        cur = UNIQ ? (cur + numSM) % Gd : cur + 1;
      }
    } else {
      if constexpr (TMA) ok = cs_read_tma(d, rchunk, tma, env, d.sink + b);
      else cs_read(d.data + (size_t)rchunk * chunk_words(d.T, d.L), d.T, d.L, d.sink + b);
    }
    if (local) cohort_sem_writer_post(local[1], st, d.sem_max, my, pc, snap);
    else sem_post<S>(st, writer, d.sem_max);
    if (!ok) break;
  }
}

// ---------------------------------------------------------------------------
// Semaphore kernels: main.cu:533-836.  One writer TB per logical SM
// (perSM_blockID == smID % numTBs_perSM); the rest are readers.  Uniq with
// d.cluster = m > 1: as the Uniq mutexes, the group's semaphore word lives in
// its cluster rank 0's shared memory.
// ---------------------------------------------------------------------------
template <bool EBO, bool UNIQ, int MODE, int V, bool TMA = false>
__global__ void __launch_bounds__(TMA ? 256 : Bounds<V>::kThreads) k_sem(RunDesc d) {
  __shared__ unsigned long long s_mbar[kTmaParts];
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  TmaCtx tma;
  if constexpr (TMA) tma_init(tma, s_mbar, dyn_smem, kTmaParts);
  const HsEnv env{d.status, d.timeout_ns};
  const int Gd = d.num_tbs;
  const int numSM = Gd < d.nsm ? Gd : d.nsm;
  if constexpr (UNIQ) {
    if (d.cluster > 1) {
      __shared__ unsigned s_cl_sem[kLineWords];
      const int mc = d.cluster;
      const int smID = (int)blockIdx.x / mc, p = (int)blockIdx.x % mc;
      const int b = smID + p * numSM;
      if (p == 0 && threadIdx.x == 0) s_cl_sem[0] = d.sem_max;
      cluster_sync_all();
      sem_loop<CLUSTER, EBO, UNIQ, MODE, V, TMA>(d, b, numSM, mc, p == smID % mc, map_shared_rank(s_cl_sem, 0u), b,
                                                 tma, env);
      cluster_sync_all();
      return;
    }
  }
  const int b = blockIdx.x;
  const int smID = b % numSM;
  const int k = ceil_div(Gd, numSM);
  const int p = b / numSM;
  const bool writer = (p == smID % k);
  sem_loop<GPU, EBO, UNIQ, MODE, V, TMA>(d, b, numSM, k, writer, group_line(d, UNIQ ? smID : 0, 0), UNIQ ? b : p,
                                         tma, env);
}

// ---------------------------------------------------------------------------
// Tree barriers: main.cu:104-315.  Logical SM group g = b % nb (nb = min(numTBs,
// NUM_SM)), member index r = b / nb, m_g members (uneven groups allowed).
//
// Atomic tree (LF == false): per-group counter barrier whose last arriver runs
// the global counter barrier among the nb groups, then publishes the group
// generation.  Lock-free tree (LF == true): members publish generation flags,
// the group's first member scans them and joins a flag barrier among group
// leaders scanned by group 0's leader, which publishes the global release word.
// ---------------------------------------------------------------------------
struct BarState {
  unsigned lgen;  // group generation (local stage)
  unsigned ggen;  // global generation
};

template <bool LF>
__device__ __forceinline__ bool local_only_barrier(const RunDesc& d, int g, int r, int m, BarState& s,
                                                   const HsEnv& env) {
  unsigned* lcount = group_line(d, g, 0);
  unsigned* lgen = group_line(d, g, 1);
  unsigned* lgo = group_line(d, g, 2);
  unsigned* lflags = d.locks + (size_t)(d.l_lflag + g * d.lflag_lines) * kLineWords;
  __syncthreads();  // every thread's critical-section stores precede the master's release
  int ok = 1;
  if constexpr (!LF) {
    if (is_master()) {
      bool okb = true;
      counter_barrier<GPU>(lcount, lgen, (unsigned)m, s.lgen, d.bo_unit, env, HS_SITE_BAR_LOCAL,
                           [] { return true; }, &okb);
      ok = okb;
    }
    s.lgen += 1u;
    return __syncthreads_or(!ok) == 0;  // non-masters keep ok == 1
  } else {
    // every member publishes its flag and scans the group's flags itself: one
    // hop, no leader release (the flags share one line)
    (void)lgo;
    const unsigned e = s.lgen + 1u;
    if (is_master()) st_release<GPU>(lflags + r, e);
    ok = scan_flags<GPU>(lflags, (unsigned)m, e, d.bo_unit, env, HS_SITE_BAR_SCAN);
    s.lgen = e;
    return ok != 0;
  }
}

template <bool LF>
__device__ __forceinline__ bool tree_barrier(const RunDesc& d, int g, int r, int m, int nb, BarState& s,
                                             const HsEnv& env) {
  unsigned* gcount = d.locks + (size_t)(d.l_glob + 0) * kLineWords;
  unsigned* ggenw = d.locks + (size_t)(d.l_glob + 1) * kLineWords;
  unsigned* ggo = d.locks + (size_t)(d.l_glob + 2) * kLineWords;
  unsigned* gflags = d.locks + (size_t)d.l_gflag * kLineWords;
  __syncthreads();  // every thread's critical-section stores precede the master's release
  int ok = 1;
  if constexpr (!LF) {
    if (m == 1) {  // no local stage
      if (is_master()) {
        bool okb = true;
        counter_barrier<GPU>(gcount, ggenw, (unsigned)nb, s.ggen, d.bo_unit, env, HS_SITE_BAR_GLOBAL,
                             [] { return true; }, &okb);
        ok = okb;
      }
    } else if (is_master()) {
      unsigned* lcount = group_line(d, g, 0);
      unsigned* lgen = group_line(d, g, 1);
      bool okb = true;
      const unsigned gg = s.ggen;
      counter_barrier<GPU>(lcount, lgen, (unsigned)m, s.lgen, d.bo_unit, env, HS_SITE_BAR_LOCAL,
                           [&] {
                             bool ok2 = true;
                             counter_barrier<GPU>(gcount, ggenw, (unsigned)nb, gg, d.bo_unit, env,
                                                  HS_SITE_BAR_GLOBAL, [] { return true; }, &ok2);
                             return ok2;
                           },
                           &okb);
      ok = okb;
    }
    if (m != 1) s.lgen += 1u;
    s.ggen += 1u;
    return __syncthreads_or(!ok) == 0;
  } else {
    // Members publish their flag and wait for the global release word
    // directly; the leader scans its group's flags, publishes the group's
    // flag, and group 0's leader scans those and releases.  The global release
    // implies every group's arrival, so members need no local release hop.
    const unsigned e = s.lgen + 1u;
    const unsigned E = s.ggen + 1u;
    unsigned* lflags = d.locks + (size_t)(d.l_lflag + g * d.lflag_lines) * kLineWords;
    if (r != 0) {
      if (is_master()) {
        st_release<GPU>(lflags + r, e);
        ok = wait_until([&] { return (int)(ld_acquire<GPU>(ggo) - E) >= 0; }, [&] { sleep_ns(d.bo_unit); }, env,
                        HS_SITE_BAR_GO);
      }
      ok = __syncthreads_or(!ok) == 0;
    } else {
      if (m > 1) {
        if (is_master()) st_release<GPU>(lflags, e);
        ok = scan_flags<GPU>(lflags + 1, (unsigned)(m - 1), e, d.bo_unit, env, HS_SITE_BAR_SCAN);
      }
      if (ok && is_master()) st_release<GPU>(gflags + g, E);
      if (g == 0) {
        if (ok) ok = scan_flags<GPU>(gflags, (unsigned)nb, E, d.bo_unit, env, HS_SITE_BAR_SCAN);
        if (ok && is_master()) st_release<GPU>(ggo, E);
      } else if (is_master() && ok) {
        ok = wait_until([&] { return (int)(ld_acquire<GPU>(ggo) - E) >= 0; }, [&] { sleep_ns(d.bo_unit); }, env,
                        HS_SITE_BAR_GO);
      }
      ok = __syncthreads_or(!ok) == 0;
    }
    if (m > 1) s.lgen = e;
    s.ggen = E;
    return ok != 0;
  }
}

__device__ __forceinline__ unsigned dyn_smem_bytes_b() {
  unsigned r;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

// The HIP build's naive sense-reversing barriers (hip/syncPrims/uvm/
// main.hip.cpp:238-302, 434-530): no local stage; every TB (PV_NAIVE) or every
// thread (PV_NAIVE_ALL) joins one global counter barrier.
__device__ __forceinline__ bool flat_barrier(const RunDesc& d, BarState& s, const HsEnv& env, bool all_threads) {
  unsigned* gcount = d.locks + (size_t)(d.l_glob + 0) * kLineWords;
  unsigned* ggenw = d.locks + (size_t)(d.l_glob + 1) * kLineWords;
  __syncthreads();  // every thread's critical-section stores precede the arrival
  int ok = 1;
  if (all_threads || is_master()) {
    bool okb = true;
    const unsigned n = all_threads ? (unsigned)d.num_tbs * blockDim.x : (unsigned)d.num_tbs;
    counter_barrier<GPU>(gcount, ggenw, n, s.ggen, d.bo_unit, env, HS_SITE_BAR_GLOBAL, [] { return true; }, &okb);
    ok = okb;
  }
  s.ggen += 1u;
  return __syncthreads_or(!ok) == 0;
}

// Tree barrier with the local stage on a thread-block cluster: the group's
// members are the cluster's CTAs.  Local arrival and local release are the
// hardware cluster barrier; between them the leader (rank 0) runs the global
// stage among the nb group leaders (generation counter, or flags scanned by
// group 0's leader and one release word).  The leader's outcome goes to its
// members through the group's spare line, written before the release barrier
// and read after it, so every CTA of the cluster continues or stops together.
template <bool LF>
__device__ __forceinline__ bool cluster_tree_barrier(const RunDesc& d, int g, int r, int nb, BarState& s,
                                                     const HsEnv& env) {
  cluster_sync_all();  // local arrival: every member's stores are released at cluster scope
  if (r == 0) {
    unsigned* gcount = d.locks + (size_t)(d.l_glob + 0) * kLineWords;
    unsigned* ggenw = d.locks + (size_t)(d.l_glob + 1) * kLineWords;
    unsigned* ggo = d.locks + (size_t)(d.l_glob + 2) * kLineWords;
    unsigned* gflags = d.locks + (size_t)d.l_gflag * kLineWords;
    int ok = 1;
    if constexpr (!LF) {
      if (is_master()) {
        bool okb = true;
        counter_barrier<GPU>(gcount, ggenw, (unsigned)nb, s.ggen, d.bo_unit, env, HS_SITE_BAR_GLOBAL,
                             [] { return true; }, &okb);
        ok = okb;
      }
      ok = __syncthreads_or(!ok) == 0;
    } else {
      const unsigned E = s.ggen + 1u;
      if (is_master()) st_release<GPU>(gflags + g, E);
      if (g == 0) {
        ok = scan_flags<GPU>(gflags, (unsigned)nb, E, d.bo_unit, env, HS_SITE_BAR_SCAN);
        if (ok && is_master()) st_release<GPU>(ggo, E);
      } else {
        if (is_master())
          ok = wait_until([&] { return (int)(ld_acquire<GPU>(ggo) - E) >= 0; }, [&] { sleep_ns(d.bo_unit); }, env,
                          HS_SITE_BAR_GO);
        ok = __syncthreads_or(!ok) == 0;
      }
    }
    if (is_master()) st_relaxed<GPU>(group_line(d, g, 3), ok ? 0u : 1u);
  }
  cluster_sync_all();  // local release
  s.ggen += 1u;
  return ld_relaxed<GPU>(group_line(d, g, 3)) == 0u;
}

// Barrier TBs must all be co-resident, so the kernel is held to 64 registers
// (four 256-thread TBs, 1024 threads, per SM).  With d.cluster = m > 1 the
// launch has clusters of m CTAs and numTBs = m * nb: physical CTA p runs
// logical TB g + r * nb with g = p / m, r = p % m, so each logical-SM group is
// one cluster (which physical CTA runs which logical TB does not change the
// result: the data a TB touches depends only on its logical index).
template <bool LF, bool EXCH, int MODE, int V, bool TMA = false>
__global__ void __launch_bounds__(TMA ? 256 : Bounds<V>::kThreads, TMA ? 4 : 1024 / Bounds<V>::kThreads)
    k_barrier(RunDesc d) {
  // TMA: the critical section is staged through the launch's dynamic shared
  // memory a tile of regions at a time (bulk copies); a bulk-copy wait that
  // runs out records the failure in the status word, which every barrier
  // wait sees, so all CTAs leave at the same barrier.
  extern __shared__ __align__(128) unsigned char bar_smem[];
  __shared__ unsigned long long s_bar_mbar;
  TmaCtx tma;
  if constexpr (TMA) {
    tma_init(tma, &s_bar_mbar, bar_smem);
    tma.cap = dyn_smem_bytes_b();
  }
  const int Gd = d.num_tbs;
  const int nb = Gd < d.nsm ? Gd : d.nsm;
  const bool clustered = d.cluster > 1;
  const bool naive = !LF && (d.variant == PV_NAIVE || d.variant == PV_NAIVE_ALL);
  const int g = clustered ? (int)blockIdx.x / d.cluster : (int)blockIdx.x % nb;
  const int r = clustered ? (int)blockIdx.x % d.cluster : (int)blockIdx.x / nb;
  const int b = g + r * nb;
  const int m = (Gd - g + nb - 1) / nb;
  const int kmax = ceil_div(Gd, nb);
  const HsEnv env{d.status, d.timeout_ns};

  // Generations at kernel start (state persists across launches).
  __shared__ BarState s_init;
  if (is_master()) {
    // LF: a member's own flag holds the group generation it last published
    s_init.lgen = LF ? ld_relaxed<GPU>(d.locks + (size_t)(d.l_lflag + g * d.lflag_lines) * kLineWords + r)
                     : ld_relaxed<GPU>(group_line(d, g, 1));
    s_init.ggen = LF ? ld_relaxed<GPU>(d.locks + (size_t)(d.l_glob + 2) * kLineWords)
                     : ld_relaxed<GPU>(d.locks + (size_t)(d.l_glob + 1) * kLineWords);
  }
  __syncthreads();
  BarState s = s_init;

  int cur = b;
  const int phases = (EXCH && kmax > 1) ? 2 : 1;
  for (int i = 0; i < d.iters; ++i) {
    // phase 0: own chunk; phase 1 (local exchange): local barrier, then the chunk
    // numBlocksAtBarr TBs ahead (one call site keeps one inlined copy of the CS)
    for (int ph = 0; ph < phases; ++ph) {
      if (ph == 1) {
        if (naive) {  // no local stage: the naive barriers join the global one here
          if (!flat_barrier(d, s, env, d.variant == PV_NAIVE_ALL)) return;
        } else if (clustered) {
          cluster_sync_all();
        } else if (!local_only_barrier<LF>(d, g, r, m, s, env)) {
          return;
        }
        cur = (cur + nb) % Gd;
      }
      if constexpr (TMA) cs_chunk_tma_tiled<MODE>(d, cur, tma, tma.cap, env);
      else cs_chunk<MODE, V>(d, cur);
      if (b == d.skip_tb) return;  // fault injection: this TB never arrives (never in cluster mode)
    }
    if (naive) {
      if (!flat_barrier(d, s, env, d.variant == PV_NAIVE_ALL)) return;
    } else if (clustered ? !cluster_tree_barrier<LF>(d, g, r, nb, s, env) : !tree_barrier<LF>(d, g, r, m, nb, s, env)) {
      return;
    }
    cur = (cur + 1) % Gd;
  }
}

// Tree barrier with each logical-SM group in ONE CTA: d.grp = m logical TBs of
// T threads share a CTA of m * T threads, physical CTA g hosting group g
// (logical TB g + r * nb runs on threads [r * T, (r + 1) * T)).  The local
// stage is then the CTA barrier itself (bar.sync: no L2 round trip and no
// release fence, where a GPU-scope fence costs 135-320 ns and a flag hand-off
// 460 ns relaxed, 810 ns with st.release on this part); a group's members run
// their critical sections side by side, every sub-block passing through the
// same CTA barriers inside them; the local exchange only touches chunks of the
// same group (TB b's partner b + nb is its next member), so CTA-scope ordering
// covers it.  The global stage is the one the one-TB-per-SM tree runs among the
// nb group leaders (a counter barrier, or flags scanned by group 0 and one
// release word).  Register path only; m * T <= 1024, every group whole.
template <bool LF, bool EXCH, int MODE, int V>
__global__ void __launch_bounds__(1024, 1) k_barrier_grp(RunDesc d) {
  const int T = d.T;
  const int nb = (int)gridDim.x;
  const int Gd = d.num_tbs;
  const int g = (int)blockIdx.x;
  const int r = (int)threadIdx.x / T;
  const int tid = (int)threadIdx.x - r * T;
  const HsEnv env{d.status, d.timeout_ns};
  __shared__ BarState s_init;
  if (is_master()) {
    s_init.lgen = 0u;
    s_init.ggen = LF ? ld_relaxed<GPU>(d.locks + (size_t)(d.l_glob + 2) * kLineWords)
                     : ld_relaxed<GPU>(d.locks + (size_t)(d.l_glob + 1) * kLineWords);
  }
  __syncthreads();
  BarState s = s_init;
  const int phases = EXCH ? 2 : 1;
  int cur = g + r * nb;
  for (int i = 0; i < d.iters; ++i) {
    for (int ph = 0; ph < phases; ++ph) {
      if (ph == 1) {
        __syncthreads();  // the local barrier: every member's critical section is done
        cur = (cur + nb) % Gd;
      }
      cs_chunk<MODE, V>(d, cur, tid);
    }
    if (!tree_barrier<LF>(d, g, 0, 1, nb, s, env)) return;
    cur = (cur + 1) % Gd;
  }
}

// The group-CTA tree barrier with bulk-copy critical sections (numLdSt > 64,
// where the register path of k_barrier_grp loses to bulk copies).  Member r
// (threads [r*T, (r+1)*T)) works on its chunks exactly as in k_barrier_grp,
// through its own d.tile_cap-byte buffer and mbarrier, synchronising on named
// barrier r + 1 inside its critical section; the local stage is still the CTA
// barrier.  At most 15 members (named barriers 1..15), T a multiple of 32.
template <bool LF, bool EXCH, int MODE>
__global__ void __launch_bounds__(1024, 1) k_barrier_grp_tma(RunDesc d) {
  __shared__ unsigned long long s_mbar[15];
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  const int T = d.T;
  const int nb = (int)gridDim.x;
  const int Gd = d.num_tbs;
  const int g = (int)blockIdx.x;
  const int r = (int)threadIdx.x / T;
  const int tid = (int)threadIdx.x - r * T;
  const HsEnv env{d.status, d.timeout_ns};
  TmaCtx tma;
  tma.buf = dyn_smem + (size_t)r * d.tile_cap;
  tma.mbar = smem_addr(s_mbar + r);
  tma.phase = 0u;
  tma.cap = d.tile_cap;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(tma.mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ BarState s_init;
  if (is_master()) {
    s_init.lgen = 0u;
    s_init.ggen = LF ? ld_relaxed<GPU>(d.locks + (size_t)(d.l_glob + 2) * kLineWords)
                     : ld_relaxed<GPU>(d.locks + (size_t)(d.l_glob + 1) * kLineWords);
  }
  __syncthreads();
  BarState s = s_init;
  const int phases = EXCH ? 2 : 1;
  int cur = g + r * nb;
  for (int i = 0; i < d.iters; ++i) {
    for (int ph = 0; ph < phases; ++ph) {
      if (ph == 1) cur = (cur + nb) % Gd;
      const bool ok = cs_chunk_tma_sub<MODE>(d, cur, tma, d.tile_cap, env, r + 1, tid);
      // every member reaches this CTA barrier (a member whose copy wait gave up
      // returned from its critical section whole); between the phases it is
      // also the local barrier: every member's stores are complete
      if (__syncthreads_or(!ok)) return;
    }
    if (!tree_barrier<LF>(d, g, 0, 1, nb, s, env)) return;
    cur = (cur + 1) % Gd;
  }
}

// ---------------------------------------------------------------------------
// Ring initialisation: slot 0 of every group's ring = 1, the rest = -1
// (cudaLocks.cu:58-65).
// ---------------------------------------------------------------------------
__global__ void k_ring_init(unsigned* ring, unsigned slots_per_group, unsigned groups) {
  const size_t n = (size_t)slots_per_group * groups;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    ring[i * kRingStride] = (i % slots_per_group == 0) ? 1u : 0xFFFFFFFFu;
}

// ---------------------------------------------------------------------------
// Host-side dispatch.
// ---------------------------------------------------------------------------
using KernelFn = void (*)(RunDesc);

// The group-CTA tree barrier kernel of a barrier primitive (REF and INC modes).
KernelFn barrier_group_kernel(int prim, int mode) {
  if (mode == M_REF) {
    switch (prim) {
      case P_ATOMIC_TREE: return k_barrier_grp<false, false, M_REF, 8>;
      case P_ATOMIC_TREE_EXCH: return k_barrier_grp<false, true, M_REF, 8>;
      case P_LF_TREE: return k_barrier_grp<true, false, M_REF, 8>;
      case P_LF_TREE_EXCH: return k_barrier_grp<true, true, M_REF, 8>;
      default: return nullptr;
    }
  }
  if (mode == M_INC) {
    switch (prim) {
      case P_ATOMIC_TREE: return k_barrier_grp<false, false, M_INC, 8>;
      case P_ATOMIC_TREE_EXCH: return k_barrier_grp<false, true, M_INC, 8>;
      case P_LF_TREE: return k_barrier_grp<true, false, M_INC, 8>;
      case P_LF_TREE_EXCH: return k_barrier_grp<true, true, M_INC, 8>;
      default: return nullptr;
    }
  }
  return nullptr;
}

// The same with bulk-copy critical sections (two staging buffers of
// d.tile_cap bytes in dynamic shared memory).
KernelFn barrier_group_tma_kernel(int prim, int mode) {
  if (mode == M_REF) {
    switch (prim) {
      case P_ATOMIC_TREE: return k_barrier_grp_tma<false, false, M_REF>;
      case P_ATOMIC_TREE_EXCH: return k_barrier_grp_tma<false, true, M_REF>;
      case P_LF_TREE: return k_barrier_grp_tma<true, false, M_REF>;
      case P_LF_TREE_EXCH: return k_barrier_grp_tma<true, true, M_REF>;
      default: return nullptr;
    }
  }
  if (mode == M_INC) {
    switch (prim) {
      case P_ATOMIC_TREE: return k_barrier_grp_tma<false, false, M_INC>;
      case P_ATOMIC_TREE_EXCH: return k_barrier_grp_tma<false, true, M_INC>;
      case P_LF_TREE: return k_barrier_grp_tma<true, false, M_INC>;
      case P_LF_TREE_EXCH: return k_barrier_grp_tma<true, true, M_INC>;
      default: return nullptr;
    }
  }
  return nullptr;
}

template <int MODE, int V, bool TMA>
static KernelFn pick(int prim) {
  if constexpr (MODE != M_SLICE) {
    switch (prim) {
      case P_ATOMIC_TREE: return k_barrier<false, false, MODE, V, TMA>;
      case P_ATOMIC_TREE_EXCH: return k_barrier<false, true, MODE, V, TMA>;
      case P_LF_TREE: return k_barrier<true, false, MODE, V, TMA>;
      case P_LF_TREE_EXCH: return k_barrier<true, true, MODE, V, TMA>;
      default: break;
    }
    if (prim >= P_SPIN_SEM1 && prim <= P_SPIN_SEM120) return k_sem<false, false, MODE, V, TMA>;
    if (prim >= P_EBO_SEM1 && prim <= P_EBO_SEM120) return k_sem<true, false, MODE, V, TMA>;
    if (prim >= P_SPIN_SEM_UNIQ1 && prim <= P_SPIN_SEM_UNIQ120) return k_sem<false, true, MODE, V, TMA>;
    if (prim >= P_EBO_SEM_UNIQ1 && prim <= P_EBO_SEM_UNIQ120) return k_sem<true, true, MODE, V, TMA>;
    switch (prim) {
      case P_SPIN_MUTEX: return k_mutex<MK_SPIN, false, MODE, V, TMA>;
      case P_EBO_MUTEX: return k_mutex<MK_EBO, false, MODE, V, TMA>;
      case P_SLEEP_MUTEX: return k_mutex<MK_SLEEP, false, MODE, V, TMA>;
      case P_FA_MUTEX: return k_mutex<MK_FA, false, MODE, V, TMA>;
      case P_SPIN_MUTEX_UNIQ: return k_mutex<MK_SPIN, true, MODE, V, TMA>;
      case P_EBO_MUTEX_UNIQ: return k_mutex<MK_EBO, true, MODE, V, TMA>;
      case P_SLEEP_MUTEX_UNIQ: return k_mutex<MK_SLEEP, true, MODE, V, TMA>;
      case P_FA_MUTEX_UNIQ: return k_mutex<MK_FA, true, MODE, V, TMA>;
      default: return nullptr;
    }
  } else {
    switch (prim) {
      case P_SPIN_MUTEX: return k_mutex<MK_SPIN, false, MODE, V>;
      case P_EBO_MUTEX: return k_mutex<MK_EBO, false, MODE, V>;
      case P_SLEEP_MUTEX: return k_mutex<MK_SLEEP, false, MODE, V>;
      case P_FA_MUTEX: return k_mutex<MK_FA, false, MODE, V>;
      case P_SPIN_MUTEX_UNIQ: return k_mutex<MK_SPIN, true, MODE, V>;
      case P_EBO_MUTEX_UNIQ: return k_mutex<MK_EBO, true, MODE, V>;
      case P_SLEEP_MUTEX_UNIQ: return k_mutex<MK_SLEEP, true, MODE, V>;
      case P_FA_MUTEX_UNIQ: return k_mutex<MK_FA, true, MODE, V>;
      default: return nullptr;
    }
  }
}

template <int V, bool TMA>
static KernelFn pick_v(int prim, int mode) {
  switch (mode) {
    case M_REF: return pick<M_REF, V, TMA>(prim);
    case M_INC: return pick<M_INC, V, TMA>(prim);
    case M_SLICE: return TMA ? nullptr : pick<M_SLICE, V, false>(prim);
    default: return nullptr;
  }
}

// Kernel choice for a run.  Mutex and semaphore kernels with numLdSt > 32 whose
// chunk fits in shared memory take the TMA path (dynamic shared memory = one
// chunk); otherwise the register path with the deepest vector variant the
// thread count allows.  Barrier kernels (every TB co-resident, four 256-thread
// TBs per SM) with numLdSt > 32 stage their chunks through 48 KB tiles.
constexpr size_t kBarrierStageBytes = 48u * 1024u;
KernelFn syncprim_plan(int prim, int mode, int threads, int num_ldst, size_t* smem_bytes, bool bulk = true) {
  const bool barrier = prim >= P_ATOMIC_TREE && prim <= P_LF_TREE_EXCH;
  const size_t chunk = (size_t)threads * (num_ldst + 1) * 4;
  *smem_bytes = 0;
  if (bulk && barrier && mode != M_SLICE && threads <= 256 && num_ldst > 32) {
    *smem_bytes = chunk < kBarrierStageBytes ? chunk : kBarrierStageBytes;
    return pick_v<8, true>(prim, mode);
  }
  if (bulk && !barrier && mode != M_SLICE && threads <= 256 && num_ldst > 32 && chunk <= kTmaMaxBytes) {
    *smem_bytes = chunk;
    return pick_v<8, true>(prim, mode);
  }
  if (threads > 512) return pick_v<4, false>(prim, mode);
  return pick_v<8, false>(prim, mode);
}

// Dynamic shared memory of a barrier launch whose plan took the bulk-copy path
// (base > 0): the shared memory the co-resident TBs of one SM leave free, so one
// TB per SM stages a whole chunk and four take 48 KB tiles (whole half-warp
// regions, at most the bulk-copy path's cap).  phys_nsm is the device's SM count.
size_t barrier_tile_bytes(int threads, int num_ldst, int num_tbs, int phys_nsm, size_t base) {
  if (base == 0 || phys_nsm <= 0) return base;
  const size_t chunk = (size_t)threads * (num_ldst + 1) * 4;
  const size_t region = (size_t)64 * (num_ldst + 1);
  const int per_sm = (num_tbs + phys_nsm - 1) / phys_nsm;
  size_t budget = per_sm > 0 ? (size_t)(216 * 1024) / (size_t)per_sm : base;
  budget = std::min(budget, (size_t)kTmaMaxBytes) / region * region;
  return std::max(base, std::min(chunk, budget));
}

KernelFn syncprim_kernel(int prim, int mode, int threads, int num_ldst) {
  size_t smem = 0;
  return syncprim_plan(prim, mode, threads, num_ldst, &smem);
}

// Allow the kernel its dynamic shared memory (once per function).
// Global mutexes and semaphores with a bulk-copy critical section (numLdSt >
// 32): one thread-block cluster per logical TB.  Rank 0 takes and releases the
// lock or semaphore (the same words and rules as k_mutex / k_sem), and every
// rank moves its slice of the chunk's half-warp regions through its own
// bulk-copy engine (cl_mutex_op / cl_sem_op, shared with the batched kernel),
// so one critical section's ~200 KB at numLdSt 100 moves over several SMs.
// All ranks agree on every stop (cl_grant / cl_end), so none is left at a
// cluster barrier.
template <int MODE>
__global__ void __launch_bounds__(256) k_prim_cluster(RunDesc d) {
  __shared__ int s_slot;
  __shared__ int s_ok[1 + 8];
  __shared__ unsigned long long s_mbar;
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  TmaCtx tma;
  tma_init(tma, &s_mbar, dyn_smem);
  tma.cap = dyn_smem_bytes();
  const HsEnv env{d.status, d.timeout_ns};
  const int cl = d.cluster;
  const int cr = (int)cluster_ctarank();
  const int b = (int)blockIdx.x / cl;
  const bool mutex = is_mutex_prim(d.prim);
  for (int j = 0; j < d.iters; ++j) {
    const bool ok = mutex ? cl_mutex_op<MODE>(d, b, cr, cl, &s_slot, s_ok, tma, env)
                          : cl_sem_op<MODE>(d, b, cr, cl, s_ok, tma, env);
    if (!ok) break;
  }
  cl_barrier(cl);  // rank 0's shared words stay valid until every rank is done
}

KernelFn prim_cluster_kernel(int mode) {
  if (mode == M_REF) return k_prim_cluster<M_REF>;
  if (mode == M_INC) return k_prim_cluster<M_INC>;
  return nullptr;
}

cudaError_t prepare_smem(KernelFn fn, size_t smem_bytes) {
  if (smem_bytes <= 32 * 1024) return cudaSuccess;  // dynamic + static must stay under the 48 KB default
  return cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTmaMaxBytes);
}

__global__ void k_fill_lines(unsigned* base, size_t n, size_t stride, unsigned value) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    base[i * stride] = value;
}

cudaError_t launch_fill_lines(unsigned* base, size_t n, size_t stride, unsigned value, cudaStream_t st) {
  k_fill_lines<<<(unsigned)((n + 255) / 256 > 152 ? 152 : (n + 255) / 256), 256, 0, st>>>(base, n, stride, value);
  return cudaGetLastError();
}

cudaError_t launch_ring_init(unsigned* ring, unsigned slots_per_group, unsigned groups, cudaStream_t st) {
  k_ring_init<<<152, 256, 0, st>>>(ring, slots_per_group, groups);
  return cudaGetLastError();
}

}  // namespace hs
