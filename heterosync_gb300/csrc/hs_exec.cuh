// hs_exec.cuh -- executing one SyncPrims instance on a gang of co-resident
// CTAs: shared by the batched kernel (many instances, static gangs) and the
// server kernel (requests admitted into slots as they arrive).
//
// A gang of c CTAs runs an instance's numTBs logical TBs.  Mutex and semaphore
// instances: one executor per ecl CTAs (a whole thread-block cluster, or one
// CTA); executor x runs the logical TBs congruent to x, one operation at a
// time; within a cluster, rank 0 takes and releases the lock or semaphore and
// every rank moves a slice of the critical section's half-warp regions.
// Barrier instances: every gang CTA works through the logical TBs congruent to
// its rank, with a counter barrier among the gang after each data phase.
#pragma once
#include "hs_cs.cuh"

namespace hs {

__device__ __forceinline__ bool is_mutex_prim(int p) { return (p >= 4 && p <= 7) || (p >= 20 && p <= 23); }
__device__ __forceinline__ bool is_sem_prim(int p) { return (p >= 8 && p <= 15) || (p >= 24 && p <= 31); }

// Bytes of dynamic shared memory this launch gave the CTA (the staging
// buffer of the bulk-copy critical section).
__device__ __forceinline__ unsigned dyn_smem_bytes() {
  unsigned r;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

// The cluster's share of one chunk's critical section: rank cr of cl moves
// regions [cr*R/cl, (cr+1)*R/cl) through its own bulk-copy engine.
template <int MODE>
__device__ __forceinline__ bool cl_cs(const RunDesc& d, int chunk, int cr, int cl, TmaCtx& t, const HsEnv& env) {
  const int R = d.T >> 4;
  const int lo = cr * R / cl, hi = (cr + 1) * R / cl;
  if (lo >= hi) return true;
  if (cl == 1 && d.L <= 16) {
    cs_chunk<MODE, 4>(d, chunk);
    return true;
  }
  return cs_chunk_tma_tiled<MODE>(d, chunk, t, t.cap, env, lo, hi);
}

__device__ __forceinline__ void cl_barrier(int cl) {
  if (cl > 1) cluster_sync_all();
}

// End of a cluster operation: every rank has finished its share, and all ranks
// agree on whether every share succeeded (each rank's flag goes to the leader's
// s_ok[1 + rank] through distributed shared memory before the barrier).
__device__ __forceinline__ bool cl_end(int* s_ok, bool cs_ok, int cr, int cl) {
  if (cl == 1) return cs_ok;
  if (is_master()) *reinterpret_cast<volatile int*>(map_shared_rank(s_ok + 1 + cr, 0)) = cs_ok ? 1 : 0;
  cluster_sync_all();
  const volatile int* f = map_shared_rank(s_ok + 1, 0);
  bool all = true;
  for (int i = 0; i < cl; ++i) all = all && f[i] != 0;
  return all;
}

// After the leader's wait: every rank learns whether it succeeded (the leader's
// flag read through distributed shared memory).
__device__ __forceinline__ bool cl_grant(int* s_ok, int leader_ok, int cr, int cl) {
  if (cl == 1) return __syncthreads_and(is_master() ? leader_ok : 1) != 0;
  if (cr == 0 && is_master()) *s_ok = leader_ok;
  cluster_sync_all();
  const int* leader = map_shared_rank(s_ok, 0);
  return *reinterpret_cast<const volatile int*>(leader) != 0;
}

// One critical section of mutex logical TB b at iteration j, executed by the
// whole cluster: rank 0 takes and releases the lock, every rank moves its share.
template <int MODE>
__device__ __noinline__ bool cl_mutex_op(const RunDesc& d, int b, int cr, int cl, int* s_slot, int* s_ok, TmaCtx& t,
                                         const HsEnv& env) {
  const bool uniq = d.prim >= 20;
  const int kind = d.prim % 4;  // 0 spin, 1 EBO, 2 ring, 3 ticket (main.cu:1224-1256 order)
  const int g = uniq ? (b % d.nsm) : 0;
  unsigned* w0 = group_line(d, g, 0);
  unsigned* w1 = group_line(d, g, 1);
  unsigned* w2 = group_line(d, g, 2);
  unsigned* ring = d.ring + (size_t)g * (d.ring_max + 1) * kRingStride;
  const unsigned wrap = uniq ? 100000000u : 1000000000u;
  int ok = 1, slot = 0;
  if (cr == 0) {
    if (kind == 0) ok = spin_lock<GPU>(w0, env);
    else if (kind == 1) ok = ebo_lock<GPU>(w0, d.bo_min, d.bo_max, env);
    else if (kind == 3) ok = ticket_lock<GPU>(w0, w1, wrap, d.bo_unit, d.bo_max, env);
    else {
      slot = queue_lock<GPU>(w2, ring, kRingStride, d.ring_max, d.bo_unit, env, s_slot);
      ok = slot >= 0;
    }
  }
  if (!cl_grant(s_ok, ok, cr, cl)) return false;
  const bool cs_ok = cl_end(s_ok, cl_cs<MODE>(d, g, cr, cl, t, env), cr, cl);
  if (cr == 0) {
    if (kind <= 1) spin_unlock<GPU>(w0);
    else if (kind == 3) ticket_unlock<GPU>(w1, wrap);
    else queue_unlock<GPU>(ring, kRingStride, d.ring_max, (unsigned)slot);
  }
  return cs_ok;
}

// One wait/CS/post of semaphore logical TB b, executed by the whole cluster.
template <int MODE>
__device__ __noinline__ bool cl_sem_op(const RunDesc& d, int b, int cr, int cl, int* s_ok, TmaCtx& t,
                                       const HsEnv& env) {
  const bool uniq = d.prim >= 24;
  const bool ebo = (d.prim >= 12 && d.prim <= 15) || d.prim >= 28;
  const int Gd = d.num_tbs;
  const int numSM = Gd < d.nsm ? Gd : d.nsm;
  const int smID = b % numSM, k = ceil_div(Gd, numSM), p = b / numSM;
  const bool writer = (p == smID % k);
  unsigned* st = group_line(d, uniq ? smID : 0, 0);
  int ok = 1;
  if (cr == 0) ok = sem_wait<GPU>(st, writer, d.sem_max, ebo, !uniq, d.bo_min, d.bo_max, env);
  if (!cl_grant(s_ok, ok, cr, cl)) return false;
  bool cs_ok = true;
  if (writer) {
    int cur = uniq ? b : 0;
    for (int j = 0; j < k && cs_ok; ++j) {
      cs_ok = cl_cs<MODE>(d, cur, cr, cl, t, env);
      cur = uniq ? (cur + numSM) % Gd : cur + 1;
    }
  } else {
    const int R = d.T >> 4, lo = cr * R / cl, hi = (cr + 1) * R / cl;
    const int rc = uniq ? b : p;
    if (cl == 1 && d.L <= 16) cs_read(d.data + (size_t)rc * chunk_words(d.T, d.L), d.T, d.L, d.sink + b);
    else if (lo < hi) cs_ok = cs_read_tma_tiled(d, rc, t, t.cap, env, d.sink + b, lo, hi);
  }
  cs_ok = cl_end(s_ok, cs_ok, cr, cl);
  if (cr == 0) sem_post<GPU>(st, writer, d.sem_max);
  return cs_ok;
}

// Counter barrier among the gang's CTAs (instance's global barrier lines).
__device__ __forceinline__ bool gang_barrier(const RunDesc& d, unsigned n, unsigned& gen, const HsEnv& env) {
  __syncthreads();  // every thread's critical-section stores precede the master's release
  int ok = 1;
  if (is_master()) {
    bool okb = true;
    counter_barrier<GPU>(d.locks + (size_t)(d.l_glob + 0) * kLineWords, d.locks + (size_t)(d.l_glob + 1) * kLineWords,
                         n, gen, d.bo_unit, env, HS_SITE_BATCH, [] { return true; }, &okb);
    ok = okb;
  }
  gen += 1u;
  return __syncthreads_or(!ok) == 0;
}

// Tree-barrier instance: every logical TB's chunk once per phase, a gang
// barrier after each phase (LocalExch: a second phase on the chunk
// numBlocksAtBarr TBs ahead, main.cu:153-211).  Each gang CTA handles the
// logical TBs congruent to its rank.
template <int MODE>
__device__ __noinline__ void batch_barrier(const RunDesc& d, int rank, int c, unsigned gen, TmaCtx& t,
                                           const HsEnv& env) {
  const int G = d.num_tbs, nb = G < d.nsm ? G : d.nsm, kmax = ceil_div(G, nb);
  const bool exch = (d.prim == 1 || d.prim == 3) && kmax > 1;
  for (int e = 0; e < d.iters; ++e) {
    const long long base = exch ? (long long)e * (nb + 1) : (long long)e;
    for (int b = rank; b < G; b += c)
      if (!cl_cs<MODE>(d, (int)((b + base) % G), 0, 1, t, env)) return;
    if (!gang_barrier(d, (unsigned)c, gen, env)) return;
    if (exch) {
      for (int b = rank; b < G; b += c)
        if (!cl_cs<MODE>(d, (int)((b + base + nb) % G), 0, 1, t, env)) return;
      if (!gang_barrier(d, (unsigned)c, gen, env)) return;
    }
  }
}

}  // namespace hs
