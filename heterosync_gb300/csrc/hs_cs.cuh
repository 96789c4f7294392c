// hs_cs.cuh -- critical-section bodies shared by the SyncPrims kernels and the
// batched persistent kernel (heterosync cuda/syncPrims/uvm/main.cu:60-100).
#pragma once
#include <cuda_runtime.h>
#include "hs_internal.h"
#include "../../include/hs/hs_device.cuh"

namespace hs {

// ---------------------------------------------------------------------------
// Critical-section bodies.  A "chunk" is the data of one reference TB: T/16
// half-warp regions of (L+1) lines x 16 words (main.cu:60-72, 1304-1308).
// ---------------------------------------------------------------------------
__device__ __forceinline__ size_t chunk_words(int T, int L) { return (size_t)T * (L + 1); }

// REF: line n+1 <- line n for n = L-1..0 in every region of the chunk.
// Passes of up to 32 lines go from the top down; each pass loads everything
// into registers, one CTA barrier, then stores.  Stores of a pass never touch
// lines a later pass loads, and a later pass only overwrites lines an earlier
// pass already loaded, so one barrier per pass suffices.
// `tid` is the thread's index within the T threads that work on the chunk
// (threadIdx.x, or its index within a sub-block when one CTA hosts several
// logical TBs; every sub-block then passes through the same CTA barriers).
template <int MAXV>
__device__ __forceinline__ void cs_ref_shift(unsigned* chunk, int T, int L, int tid = threadIdx.x) {
  const int R = T >> 4;
  const int rw4 = (L + 1) * 4;
  uint4* c4 = reinterpret_cast<uint4*>(chunk);
  const int lpp = 4 * MAXV;  // lines per pass: MAXV*T items / (R regions * 4 vectors)
  for (int hi = L; hi > 0; hi -= lpp) {
    const int lo = hi - lpp > 0 ? hi - lpp : 0;
    const int per_region = (hi - lo) * 4;
    const int nitems = R * per_region;
    uint4 v[MAXV];
    int idx[MAXV];
#pragma unroll
    for (int u = 0; u < MAXV; ++u) {
      const int t = tid + u * T;
      idx[u] = -1;
      if (t < nitems) {
        const int h = t / per_region;
        idx[u] = h * rw4 + lo * 4 + (t - h * per_region);
        v[u] = c4[idx[u]];
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXV; ++u)
      if (idx[u] >= 0) c4[idx[u] + 4] = v[u];
  }
}

// INC: every word of lines 1..L of every region gets +1.
template <int MAXV>
__device__ __forceinline__ void cs_inc(unsigned* chunk, int T, int L, int tid = threadIdx.x) {
  const int R = T >> 4;
  const int rw4 = (L + 1) * 4;
  const int per_region = L * 4;
  const int nitems = R * per_region;
  uint4* c4 = reinterpret_cast<uint4*>(chunk);
  for (int base = 0; base < nitems; base += MAXV * T) {
    uint4 v[MAXV];
    int idx[MAXV];
#pragma unroll
    for (int u = 0; u < MAXV; ++u) {
      const int t = base + tid + u * T;
      idx[u] = -1;
      if (t < nitems) {
        const int h = t / per_region;
        idx[u] = h * rw4 + 4 + (t - h * per_region);
        v[u] = c4[idx[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < MAXV; ++u)
      if (idx[u] >= 0) {
        v[u].x += 1u; v[u].y += 1u; v[u].z += 1u; v[u].w += 1u;
        c4[idx[u]] = v[u];
      }
  }
}

// SLICE: words [s*L, s*L+L) get +1, one thread per word.
__device__ __forceinline__ void cs_slice(unsigned* data, int s, int L) {
  unsigned* p = data + (size_t)s * L;
  for (int w = threadIdx.x; w < L; w += blockDim.x) p[w] += 1u;
}

// Semaphore reader: load lines 0..L-1 of the chunk (main.cu:89-100); the loaded
// values are folded into one word per TB so the loads are not dead.
// Reader over R consecutive half-warp regions starting at `chunk` (a whole
// chunk: R = T / 16).
__device__ __forceinline__ void cs_read_regions(const unsigned* chunk, int R, int T, int L, unsigned* sink_slot) {
  const int rw4 = (L + 1) * 4;
  const int per_region = L * 4;
  const int nitems = R * per_region;
  const uint4* c4 = reinterpret_cast<const uint4*>(chunk);
  unsigned acc = 0;
  // eight independent loads in flight per thread per step
  for (int base = threadIdx.x; base < nitems; base += 8 * T) {
    uint4 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = base + u * T;
      if (t < nitems) {
        const int h = t / per_region;
        v[u] = c4[h * rw4 + (t - h * per_region)];
      } else {
        v[u] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) acc += v[u].x ^ v[u].y ^ v[u].z ^ v[u].w;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc == 0x9E3779B9u) *sink_slot = acc;  // practically never taken
}

__device__ __forceinline__ void cs_read(const unsigned* chunk, int T, int L, unsigned* sink_slot) {
  cs_read_regions(chunk, T >> 4, T, L, sink_slot);
}

// ---------------------------------------------------------------------------
// TMA path for large chunks (numLdSt > 32, chunk <= kTmaMaxBytes): one
// cp.async.bulk copies the whole chunk into shared memory (completion counted
// on an mbarrier), then one bulk store per half-warp region writes lines
// 0..L-1 back one line up (INC: lines 1..L after +1 in shared memory).  The
// copy engine keeps the whole chunk in flight, which roughly doubles one SM's
// throughput on the critical section over vector loads.
// Ordering: the acquire (generic proxy) is followed by fence.proxy.async before
// the bulk load; the bulk stores are completed (wait_group 0) and followed by
// fence.proxy.async before the release.
// ---------------------------------------------------------------------------
constexpr unsigned kTmaMaxBytes = 200u * 1024u;
constexpr int kTmaParts = 4;  // bulk loads per whole-chunk reference-mode critical section

struct TmaCtx {
  unsigned char* buf;  // dynamic shared memory, chunk bytes
  unsigned mbar;       // shared address of the mbarrier (of part 0)
  unsigned phase;
  unsigned cap;        // bytes of buf (tiled paths)
  int parts;           // mbarriers at mbar, mbar + 8, ... (whole-chunk REF path)
};

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// mbar_storage holds `parts` consecutive mbarriers (1 for every path but the
// whole-chunk reference-mode critical section, which loads in parts).
__device__ __forceinline__ void tma_init(TmaCtx& t, unsigned long long* mbar_storage, unsigned char* dyn,
                                         int parts = 1) {
  t.buf = dyn;
  t.mbar = smem_addr(mbar_storage);
  t.phase = 0;
  t.cap = 0;
  t.parts = parts;
  if (is_master()) {
    for (int p = 0; p < parts; ++p)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(t.mbar + 8u * p) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

__device__ __forceinline__ bool mbar_done(unsigned mbar, unsigned phase) {
  unsigned done;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
  return done != 0;
}

// Wait for this CTA's own bulk copy.  The copy completes in hardware whatever
// other CTAs do, so this wait does not give up when another CTA has already
// failed (abandoning it would leave the copy writing into shared memory and the
// mbarrier a phase ahead of its owner); it has only its own time limit.
constexpr unsigned long long kTmaWaitNs = 1000000000ull;
__device__ __forceinline__ bool tma_wait(const TmaCtx& t, const HsEnv& env) {
  if (mbar_done(t.mbar, t.phase)) return true;
  const unsigned long long t0 = globaltimer();
  for (unsigned i = 1;; ++i) {
    if (mbar_done(t.mbar, t.phase)) return true;
    if ((i & 63u) == 0u && globaltimer() - t0 > kTmaWaitNs) {
      fail(env, HS_DEV_TIMEOUT, HS_SITE_TMA);
      return false;
    }
  }
}

// Load a chunk into shared memory; returns the CTA-wide success.
__device__ __forceinline__ bool tma_load_chunk(const unsigned* chunk, unsigned bytes, TmaCtx& t, const HsEnv& env) {
  if (is_master()) {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(t.mbar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(t.buf)), "l"(chunk), "r"(bytes), "r"(t.mbar) : "memory");
  }
  const bool ok = is_master() ? tma_wait(t, env) : true;
  t.phase ^= 1u;
  return __syncthreads_and(ok) != 0;
}

// Store lines [first, first+L) of every region of the staged chunk to lines
// [1, L] of the chunk in global memory, and complete the writes.
__device__ __forceinline__ void tma_store_shifted(unsigned* chunk, int T, int L, unsigned first, TmaCtx& t) {
  if (is_master()) {
    const int R = T >> 4;
    const unsigned rb = (unsigned)(16 * (L + 1) * 4);
    const unsigned sbase = smem_addr(t.buf);
    for (int h = 0; h < R; ++h) {
      unsigned char* dst = reinterpret_cast<unsigned char*>(chunk) + (size_t)h * rb + 64u;
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                   :: "l"(dst), "r"(sbase + h * rb + first * 64u), "r"((unsigned)(64 * L)) : "memory");
    }
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
}

// Reference mode in parts: the master loads the chunk's regions as t.parts
// bulk copies, each completing on its own mbarrier, and issues a part's
// shifted stores as soon as that part has landed, so stores of the first
// regions overlap the loads of the last.  Only the master touches the buffer
// (no CTA barrier between parts).  One CTA moved a numLdSt-100 chunk in 2.21
// us in four parts against 2.42 us in one.
__device__ __forceinline__ bool cs_chunk_tma_ref_parts(unsigned* chunk, int T, int L, TmaCtx& t, const HsEnv& env) {
  int ok = 1;
  if (is_master()) {
    const int R = T >> 4;
    const int P = t.parts < R ? t.parts : R;
    const int rp = (R + P - 1) / P;
    const unsigned rb = (unsigned)(64 * (L + 1));
    const unsigned sbase = smem_addr(t.buf);
    unsigned char* c = reinterpret_cast<unsigned char*>(chunk);
    asm volatile("fence.proxy.async.global;" ::: "memory");
    for (int p = 0; p < P; ++p) {
      const int lo = p * rp, hi = (lo + rp < R) ? lo + rp : R;
      if (lo >= hi) continue;
      const unsigned mb = t.mbar + 8u * p, bytes = (unsigned)(hi - lo) * rb;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(mb), "r"(bytes) : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   :: "r"(sbase + lo * rb), "l"(c + (size_t)lo * rb), "r"(bytes), "r"(mb) : "memory");
    }
    for (int p = 0; p < P && ok; ++p) {
      const int lo = p * rp, hi = (lo + rp < R) ? lo + rp : R;
      if (lo >= hi) continue;
      const unsigned mb = t.mbar + 8u * p;
      if (!mbar_done(mb, t.phase)) {
        const unsigned long long t0 = globaltimer();
        for (unsigned i = 1; !mbar_done(mb, t.phase); ++i) {
          if ((i & 63u) == 0u && globaltimer() - t0 > kTmaWaitNs) {
            fail(env, HS_DEV_TIMEOUT, HS_SITE_TMA);
            ok = 0;
            break;
          }
        }
        if (!ok) break;
      }
      for (int h = lo; h < hi; ++h)
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(c + (size_t)h * rb + 64u), "r"(sbase + h * rb), "r"((unsigned)(64 * L)) : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  t.phase ^= 1u;
  return __syncthreads_and(ok) != 0;
}

template <int MODE>
__device__ __forceinline__ bool cs_chunk_tma(const RunDesc& d, int chunk, TmaCtx& t, const HsEnv& env) {
  unsigned* c = d.data + (size_t)chunk * chunk_words(d.T, d.L);
  const unsigned bytes = (unsigned)(d.T * (d.L + 1) * 4);
  if (MODE == M_REF && t.parts > 1) return cs_chunk_tma_ref_parts(c, d.T, d.L, t, env);
  if (!tma_load_chunk(c, bytes, t, env)) return false;
  if constexpr (MODE == M_REF) {
    tma_store_shifted(c, d.T, d.L, 0u, t);
  } else {
    const int R = d.T >> 4, per_region = d.L * 4, rw4 = (d.L + 1) * 4;
    uint4* s4 = reinterpret_cast<uint4*>(t.buf);
    for (int i = threadIdx.x; i < R * per_region; i += d.T) {
      const int h = i / per_region;
      uint4& v = s4[h * rw4 + 4 + (i - h * per_region)];
      v.x += 1u; v.y += 1u; v.z += 1u; v.w += 1u;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic smem writes -> bulk store reads
    __syncthreads();
    // lines 1..L of smem go to lines 1..L of global: same offsets, so "shift" from line 1 to line 1
    if (is_master()) {
      const unsigned rb = (unsigned)(16 * (d.L + 1) * 4);
      const unsigned sbase = smem_addr(t.buf);
      for (int h = 0; h < R; ++h) {
        unsigned char* dst = reinterpret_cast<unsigned char*>(c) + (size_t)h * rb + 64u;
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(dst), "r"(sbase + h * rb + 64u), "r"((unsigned)(64 * d.L)) : "memory");
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
      asm volatile("fence.proxy.async.global;" ::: "memory");
    }
  }
  return true;
}

// Tiled TMA critical section: whole half-warp regions are independent, so a
// chunk can be staged through a buffer smaller than the chunk, a tile of
// regions at a time (one bulk load per tile, one bulk store per region).  Used
// where shared memory must stay small (the batched kernel keeps four CTAs per
// SM).  The buffer is reused only after the previous tile's stores have read
// it (wait_group.read).
template <int MODE>
__device__ __forceinline__ bool cs_chunk_tma_tiled(const RunDesc& d, int chunk, TmaCtx& t, unsigned buf_bytes,
                                                   const HsEnv& env, int r_lo = 0, int r_hi = -1) {
  unsigned* c = d.data + (size_t)chunk * chunk_words(d.T, d.L);
  const int R = r_hi < 0 ? (d.T >> 4) : r_hi;
  const unsigned rb = (unsigned)(64 * (d.L + 1));
  int per = (int)(buf_bytes / rb);
  if (per < 1) per = 1;
  const unsigned sbase = smem_addr(t.buf);
  for (int r0 = r_lo; r0 < R; r0 += per) {
    const int n = (R - r0 < per) ? (R - r0) : per;
    unsigned char* src = reinterpret_cast<unsigned char*>(c) + (size_t)r0 * rb;
    if (!tma_load_chunk(reinterpret_cast<const unsigned*>(src), (unsigned)n * rb, t, env)) return false;
    unsigned first = 0u;
    if constexpr (MODE == M_INC) {
      const int per_region = d.L * 4, rw4 = (d.L + 1) * 4;
      uint4* s4 = reinterpret_cast<uint4*>(t.buf);
      for (int i = threadIdx.x; i < n * per_region; i += d.T) {
        const int h = i / per_region;
        uint4& v = s4[h * rw4 + 4 + (i - h * per_region)];
        v.x += 1u; v.y += 1u; v.z += 1u; v.w += 1u;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      first = 1u;
    }
    if (is_master()) {
      for (int h = 0; h < n; ++h) {
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(src + (size_t)h * rb + 64u), "r"(sbase + h * rb + first * 64u), "r"((unsigned)(64 * d.L))
                     : "memory");
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // buffer free for the next tile
    }
    __syncthreads();
  }
  if (is_master()) {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // writes complete before the release
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  return true;
}

// Several chunks' critical sections through one staging buffer: the k chunks
// (first + i*add) mod mod, regions [r_lo, r_hi) of each, are packed into
// tiles of whole regions; a tile issues one bulk load per contiguous run (all
// completing on the one mbarrier), then one bulk store per region.  A
// semaphore writer's numTBs_perSM chunks thus share tiles instead of paying a
// load-store round trip each.
template <int MODE>
__device__ __forceinline__ bool cs_chunks_tma_tiled(const RunDesc& d, int first, int k, int add, int mod, TmaCtx& t,
                                                    unsigned buf_bytes, const HsEnv& env, int r_lo, int r_hi) {
  const int nr = r_hi - r_lo;
  if (nr <= 0 || k <= 0) return true;
  const unsigned rb = (unsigned)(64 * (d.L + 1));
  const size_t cw = chunk_words(d.T, d.L);
  int per = (int)(buf_bytes / rb);
  if (per < 1) per = 1;
  const unsigned sbase = smem_addr(t.buf);
  const int total = k * nr;
  auto region_ptr = [&](int p) {
    const int i = p / nr, r = r_lo + p % nr;
    const int c = (int)(((long long)first + (long long)i * add) % mod);
    return reinterpret_cast<unsigned char*>(d.data + (size_t)c * cw) + (size_t)r * rb;
  };
  for (int p0 = 0; p0 < total; p0 += per) {
    const int n = (total - p0 < per) ? (total - p0) : per;
    if (is_master()) {
      asm volatile("fence.proxy.async.global;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(t.mbar), "r"((unsigned)n * rb)
                   : "memory");
      int q = 0;
      while (q < n) {  // one bulk load per run of regions contiguous in memory
        int e = q + 1;
        while (e < n && (p0 + e) % nr != 0) ++e;
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     :: "r"(sbase + (unsigned)q * rb), "l"(region_ptr(p0 + q)), "r"((unsigned)(e - q) * rb),
                        "r"(t.mbar)
                     : "memory");
        q = e;
      }
    }
    const bool ok = is_master() ? tma_wait(t, env) : true;
    t.phase ^= 1u;
    if (__syncthreads_and(ok) == 0) return false;
    unsigned first_line = 0u;
    if constexpr (MODE == M_INC) {
      const int per_region = d.L * 4, rw4 = (d.L + 1) * 4;
      uint4* s4 = reinterpret_cast<uint4*>(t.buf);
      for (int i = threadIdx.x; i < n * per_region; i += d.T) {
        const int h = i / per_region;
        uint4& v = s4[h * rw4 + 4 + (i - h * per_region)];
        v.x += 1u; v.y += 1u; v.z += 1u; v.w += 1u;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      first_line = 1u;
    }
    if (is_master()) {
      for (int h = 0; h < n; ++h) {
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(region_ptr(p0 + h) + 64u), "r"(sbase + h * rb + first_line * 64u),
                        "r"((unsigned)(64 * d.L))
                     : "memory");
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
    __syncthreads();
  }
  if (is_master()) {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  return true;
}

// Semaphore reader through the staging buffer, a tile of regions at a time.
__device__ __forceinline__ bool cs_read_tma_tiled(const RunDesc& d, int chunk, TmaCtx& t, unsigned buf_bytes,
                                                  const HsEnv& env, unsigned* sink_slot, int r_lo = 0, int r_hi = -1) {
  const unsigned* c = d.data + (size_t)chunk * chunk_words(d.T, d.L);
  const int R = r_hi < 0 ? (d.T >> 4) : r_hi;
  const unsigned rb = (unsigned)(64 * (d.L + 1));
  int per = (int)(buf_bytes / rb);
  if (per < 1) per = 1;
  const int per_region = d.L * 4, rw4 = (d.L + 1) * 4;
  unsigned acc = 0;
  for (int r0 = r_lo; r0 < R; r0 += per) {
    const int n = (R - r0 < per) ? (R - r0) : per;
    if (!tma_load_chunk(c + (size_t)r0 * (rb / 4), (unsigned)n * rb, t, env)) return false;
    const uint4* s4 = reinterpret_cast<const uint4*>(t.buf);
    for (int i = threadIdx.x; i < n * per_region; i += d.T) {
      const int h = i / per_region;
      const uint4 v = s4[h * rw4 + (i - h * per_region)];
      acc += v.x ^ v.y ^ v.z ^ v.w;
    }
    __syncthreads();  // buffer reused by the next tile
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc == 0x9E3779B9u) *sink_slot = acc;
  return true;
}

// Semaphore reader on the TMA path: stage the chunk, fold lines 0..L-1.
__device__ __forceinline__ bool cs_read_tma(const RunDesc& d, int chunk, TmaCtx& t, const HsEnv& env,
                                            unsigned* sink_slot) {
  const unsigned* c = d.data + (size_t)chunk * chunk_words(d.T, d.L);
  if (!tma_load_chunk(c, (unsigned)(d.T * (d.L + 1) * 4), t, env)) return false;
  const int R = d.T >> 4, per_region = d.L * 4, rw4 = (d.L + 1) * 4;
  const uint4* s4 = reinterpret_cast<const uint4*>(t.buf);
  unsigned acc = 0;
  for (int i = threadIdx.x; i < R * per_region; i += d.T) {
    const int h = i / per_region;
    const uint4 v = s4[h * rw4 + (i - h * per_region)];
    acc += v.x ^ v.y ^ v.z ^ v.w;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc == 0x9E3779B9u) *sink_slot = acc;
  __syncthreads();  // the buffer is reused by the next load
  return true;
}

// Tiled bulk-copy critical section run by ONE sub-block of a CTA that hosts a
// whole logical-SM group (the group-CTA tree barrier at numLdSt > 64): the T
// threads [r*T, (r+1)*T) work on their own chunk through their own buffer and
// mbarrier, thread tid 0 issuing the copies, and synchronise on named barrier
// `bar` (1..15) instead of the CTA barrier.  Each member thus keeps its own
// load and stores in flight, as one-CTA-per-TB launches do: one CTA moving all
// the group's chunks through shared buffers ran at half their speed.
__device__ __forceinline__ void sub_sync(int bar, int T) {
  asm volatile("bar.sync %0, %1;" :: "r"(bar), "r"(T) : "memory");
}
__device__ __forceinline__ bool sub_and(int bar, int T, int v) {
  int r;
  asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.and.pred q, %2, %3, p;\n\t"
               "selp.s32 %0, 1, 0, q;\n\t}"
               : "=r"(r) : "r"(v), "r"(bar), "r"(T) : "memory");
  return r != 0;
}

template <int MODE>
__device__ __forceinline__ bool cs_chunk_tma_sub(const RunDesc& d, int chunk, TmaCtx& t, unsigned buf_bytes,
                                                 const HsEnv& env, int bar, int tid) {
  unsigned char* c = reinterpret_cast<unsigned char*>(d.data + (size_t)chunk * chunk_words(d.T, d.L));
  const int T = d.T, R = T >> 4;
  const unsigned rb = (unsigned)(64 * (d.L + 1));
  int per = (int)(buf_bytes / rb);
  if (per < 1) per = 1;
  const unsigned sbase = smem_addr(t.buf);
  for (int r0 = 0; r0 < R; r0 += per) {
    const int n = (R - r0 < per) ? (R - r0) : per;
    unsigned char* src = c + (size_t)r0 * rb;
    int ok = 1;
    if (tid == 0) {
      asm volatile("fence.proxy.async.global;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(t.mbar), "r"((unsigned)n * rb)
                   : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   :: "r"(sbase), "l"(src), "r"((unsigned)n * rb), "r"(t.mbar) : "memory");
      ok = tma_wait(t, env);
    }
    t.phase ^= 1u;
    if (!sub_and(bar, T, ok)) {
      if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // earlier tiles' stores
      return false;
    }
    unsigned first = 0u;
    if constexpr (MODE == M_INC) {
      const int per_region = d.L * 4, rw4 = (d.L + 1) * 4;
      uint4* s4 = reinterpret_cast<uint4*>(t.buf);
      for (int i = tid; i < n * per_region; i += T) {
        const int h = i / per_region;
        uint4& v = s4[h * rw4 + 4 + (i - h * per_region)];
        v.x += 1u; v.y += 1u; v.z += 1u; v.w += 1u;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      sub_sync(bar, T);
      first = 1u;
    }
    if (tid == 0) {
      for (int h = 0; h < n; ++h) {
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(src + (size_t)h * rb + 64u), "r"(sbase + h * rb + first * 64u), "r"((unsigned)(64 * d.L))
                     : "memory");
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // buffer free for the next tile
    }
    sub_sync(bar, T);
  }
  if (tid == 0) {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // writes complete before the release
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  return true;
}

// Vector depth V = 16-byte vectors each thread keeps in flight per pass.  The
// launch bound follows from it: V 4 -> 1024 threads, 8 -> 512, 26 -> 256 (a
// 256-thread TB then moves numLdSt <= 104 lines of its chunk in one pass).
template <int V> struct Bounds { static constexpr int kThreads = V <= 4 ? 1024 : (V <= 8 ? 512 : 256); };

template <int MODE, int V>
__device__ __forceinline__ void cs_chunk(const RunDesc& d, int chunk, int tid = threadIdx.x) {
  unsigned* c = d.data + (size_t)chunk * chunk_words(d.T, d.L);
  if constexpr (MODE == M_REF) cs_ref_shift<V>(c, d.T, d.L, tid);
  else cs_inc<V>(c, d.T, d.L, tid);
}

__device__ __forceinline__ unsigned* group_line(const RunDesc& d, int g, int k) {
  return d.locks + (size_t)(d.l_grp + 4 * g + k) * kLineWords;
}

}  // namespace hs
