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
    if (cl == 1 && d.L <= 16) {
      int cur = uniq ? b : 0;
      for (int j = 0; j < k && cs_ok; ++j) {
        cs_chunk<MODE, 4>(d, cur);
        cur = uniq ? (cur + numSM) % Gd : cur + 1;
      }
    } else {  // the k chunks' shares packed into shared tiles
      const int R = d.T >> 4, lo = cr * R / cl, hi = (cr + 1) * R / cl;
      cs_ok = cs_chunks_tma_tiled<MODE>(d, uniq ? b : 0, k, uniq ? numSM : 1, uniq ? Gd : (k > 0 ? k : 1), t, t.cap,
                                        env, lo, hi);
    }
  } else {
    const int R = d.T >> 4, lo = cr * R / cl, hi = (cr + 1) * R / cl;
    const int rc = uniq ? b : p;
    const unsigned* c = d.data + (size_t)rc * chunk_words(d.T, d.L);
    if (cl == 1 && d.L <= 16) cs_read(c, d.T, d.L, d.sink + b);
    else if (cl > 1 && lo < hi)  // a cluster rank's slice is small: vector loads beat a bulk-copy round trip
      cs_read_regions(c + (size_t)lo * 16 * (d.L + 1), hi - lo, d.T, d.L, d.sink + b);
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

// ---------------------------------------------------------------------------
// Relaxed-atomics instances (the batch's four extra kinds).  One operation of
// logical TB b at iteration j; no operation waits on a logical TB that is not
// running (the seqlock writer waits only for a writer that holds the lock), so
// any executor count is deadlock-free.  Storage layouts and final states:
//   RefCounter   : ref[L], total[L]; every thread t takes and drops a reference
//                  on ref[(b+j+t) % L] (relaxed +1, release -1) and counts it in
//                  total: ref unchanged, total += number of (b, j, t) per slot
//                  (refCounter_kernel.cu:4-55 at instance scale).
//   SplitCounter : one 64-bit partial per logical SM; every warp adds 32*L to
//                  partial[b % NUM_SM] and the CTA then reads all partials
//                  (splitCounter_kernel.cu:10-103 with per-SM 64-bit partials).
//   Seqlock      : 4 x 64-bit payload + torn-read count; the sequence word is
//                  lock state.  TBs b % 4 == 0 write (CAS even -> odd, payload,
//                  release +1), the others read with the seqlock retry rule and
//                  count payloads that do not match their sequence number
//                  (seqlocks_kernel.cu:17-232 with a 4 x u64 payload).
//   Flags        : data[L] + violation count; the flag word is lock state.  TB 0
//                  writes data = j+1 then releases flag = j+1; the others acquire
//                  the flag and count data words below it (flags_kernel.cu
//                  stop/dirty message passing, without waiting).
// ---------------------------------------------------------------------------
enum : int { P_REFCOUNT = 60, P_SPLITCOUNT = 61, P_SEQLOCK = 62, P_FLAGS = 63 };
__device__ __forceinline__ bool is_relaxed_prim(int p) { return p >= P_REFCOUNT && p <= P_FLAGS; }

__device__ __forceinline__ unsigned long long seq_pattern(unsigned seq, int i) {
  return (unsigned long long)seq * 0x9E3779B97F4A7C15ull + (unsigned long long)i;
}

static __device__ __noinline__ bool relaxed_op(const RunDesc& d, int b, int j, const HsEnv& env) {
  __shared__ unsigned s_v;
  const int t = threadIdx.x, T = d.T;
  unsigned* st = d.data;
  if (d.prim == P_REFCOUNT) {
    const int L = d.L;
    if (t < T) {
      const int k = (b + j + t) % L;
      asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(st + k) : "memory");
      asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" :: "l"(st + L + k) : "memory");
      asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(st + k), "r"(0xFFFFFFFFu) : "memory");
    }
    return true;
  }
  if (d.prim == P_SPLITCOUNT) {
    unsigned long long* part = reinterpret_cast<unsigned long long*>(st);
    if ((t & 31) == 0 && t < T) {
      asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;"
                   :: "l"(part + (b % d.nsm)), "l"((unsigned long long)32 * (unsigned long long)d.L) : "memory");
    }
    unsigned long long sum = 0;
    for (int s2 = t; s2 < d.nsm; s2 += blockDim.x) {
      unsigned long long v;
      asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(part + s2) : "memory");
      sum += v;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((t & 31) == 0 && sum) atomicAdd(d.sink + b, (unsigned)(sum & 0xFFFFFFFFu));
    return true;
  }
  unsigned* lockw = d.locks + (size_t)d.l_grp * kLineWords;
  if (d.prim == P_SEQLOCK) {
    unsigned long long* pay = reinterpret_cast<unsigned long long*>(st);
    unsigned* torn = st + 8;
    int ok = 1;
    if (is_master()) {
      if (b % 4 == 0) {
        unsigned cur = 0;
        ok = wait_until_p([&] {
               cur = ld_relaxed<GPU>(lockw);
               return (cur & 1u) == 0u && atom_cas_acquire<GPU>(lockw, cur, cur + 1u) == cur;
             }, [&] { return ld_relaxed<GPU>(lockw); }, [] {}, env, HS_SITE_RELAXED);
        if (ok) {
          asm volatile("fence.acq_rel.gpu;" ::: "memory");  // payload stores stay after the odd sequence number
          const unsigned v = cur + 2u;
          for (int i = 0; i < 4; ++i)
            asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(pay + i), "l"(seq_pattern(v, i)) : "memory");
          st_release<GPU>(lockw, v);
        }
      } else {
        for (int tries = 0; tries < 64; ++tries) {
          const unsigned s1 = ld_acquire<GPU>(lockw);
          if (s1 & 1u) continue;
          unsigned long long p[4];
          for (int i = 0; i < 4; ++i)
            asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(p[i]) : "l"(pay + i) : "memory");
          asm volatile("fence.acq_rel.gpu;" ::: "memory");
          if (ld_relaxed<GPU>(lockw) != s1) continue;
          bool good = true;
          if (s1 != 0u)
            for (int i = 0; i < 4; ++i) good = good && p[i] == seq_pattern(s1, i);
          if (!good) atomicAdd(torn, 1u);
          break;
        }
      }
    }
    return __syncthreads_or(!ok) == 0;
  }
  // P_FLAGS
  const int L = d.L;
  unsigned* data = st;
  unsigned* viol = st + L;
  if (b == 0) {
    for (int k = t; k < L; k += blockDim.x) st_relaxed<GPU>(data + k, (unsigned)j + 1u);
    __syncthreads();
    if (is_master()) st_release<GPU>(lockw, (unsigned)j + 1u);
  } else {
    if (is_master()) s_v = ld_acquire<GPU>(lockw);
    __syncthreads();
    const unsigned f = s_v;
    for (int k = t; k < L; k += blockDim.x)
      if (ld_relaxed<GPU>(data + k) < f) atomicAdd(viol, 1u);
    __syncthreads();
  }
  return true;
}

}  // namespace hs
