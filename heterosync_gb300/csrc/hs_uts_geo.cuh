// hs_uts_geo.cuh -- geometric UTS walk (SHA-1 node generator, work stealing
// over per-CTA lock-free queues); shared by the standalone kernel
// (hs_uts_geo.cu) and the server's tree-search requests (hs_serve.cu).
#pragma once
#include "../../include/hs/hs_device.cuh"

namespace hs {


constexpr int kGeoMaxDepth = 30;
constexpr int kGeoTable = 128;
constexpr unsigned kGeoQueueCap = 512;  // items per CTA queue (power of two)

struct GeoItem {  // children [first, end) of the node with state s at `depth`
  unsigned s[5];
  unsigned depth, first, end;
};

struct GeoArgs {
  unsigned* qseq;         // nq * cap cell sequence numbers
  GeoItem* qitem;         // nq * cap items
  unsigned* qpos;         // per queue: [q * 64] enqueue position, [q * 64 + 32] dequeue position
  unsigned* work;         // queued items + busy threads
  unsigned* idle;         // threads looking for work
  unsigned long long* out;  // [0] nodes, [8] leaves, [16] deepest level
  const unsigned* table;
  int nt, limit, nq;
  unsigned seed;
  unsigned* status;
  unsigned long long timeout_ns;
};

__device__ __forceinline__ unsigned rotl32(unsigned x, int n) { return __funnelshift_l(x, x, n); }

// SHA-1 (FIPS 180-4) of one padded 64-byte block given as 16 big-endian words.
__device__ __forceinline__ void sha1_block(unsigned w[16], unsigned h[5]) {
  unsigned a = 0x67452301u, b = 0xEFCDAB89u, c = 0x98BADCFEu, d = 0x10325476u, e = 0xC3D2E1F0u;
#pragma unroll
  for (int t = 0; t < 80; ++t) {
    unsigned wt;
    if (t < 16) {
      wt = w[t];
    } else {
      wt = rotl32(w[(t - 3) & 15] ^ w[(t - 8) & 15] ^ w[(t - 14) & 15] ^ w[t & 15], 1);
      w[t & 15] = wt;
    }
    unsigned f, k;
    if (t < 20) { f = (b & c) | (~b & d); k = 0x5A827999u; }
    else if (t < 40) { f = b ^ c ^ d; k = 0x6ED9EBA1u; }
    else if (t < 60) { f = (b & c) | (b & d) | (c & d); k = 0x8F1BBCDCu; }
    else { f = b ^ c ^ d; k = 0xCA62C1D6u; }
    const unsigned tmp = rotl32(a, 5) + f + e + k + wt;
    e = d; d = c; c = rotl32(b, 30); b = a; a = tmp;
  }
  h[0] = 0x67452301u + a; h[1] = 0xEFCDAB89u + b; h[2] = 0x98BADCFEu + c; h[3] = 0x10325476u + d;
  h[4] = 0xC3D2E1F0u + e;
}

__device__ __forceinline__ void geo_child(const unsigned p[5], unsigned i, unsigned out[5]) {
  unsigned w[16] = {p[0], p[1], p[2], p[3], p[4], i, 0x80000000u, 0, 0, 0, 0, 0, 0, 0, 0, 192u};
  sha1_block(w, out);
}

__device__ __forceinline__ void geo_root(unsigned seed, unsigned out[5]) {
  unsigned w[16] = {0, 0, 0, 0, seed, 0x80000000u, 0, 0, 0, 0, 0, 0, 0, 0, 0, 160u};
  sha1_block(w, out);
}

__device__ __forceinline__ int geo_nchildren(const unsigned s[5], int depth, int limit, const unsigned* t, int nt) {
  if (depth >= limit) return 0;
  const unsigned r = s[4] & 0x7fffffffu;
  int m = 0;
  while (m < nt && r < t[m]) ++m;
  return m;
}

// Bounded multi-producer multi-consumer ring (per-cell sequence numbers).
static __device__ bool q_push(const GeoArgs& a, int q, const GeoItem& it) {
  unsigned* enq = a.qpos + (size_t)q * 64;
  unsigned* seq = a.qseq + (size_t)q * kGeoQueueCap;
  GeoItem* items = a.qitem + (size_t)q * kGeoQueueCap;
  unsigned pos = ld_relaxed<GPU>(enq);
  for (int tries = 0; tries < 64; ++tries) {
    const unsigned sq = ld_acquire<GPU>(seq + (pos & (kGeoQueueCap - 1)));
    const int dif = (int)(sq - pos);
    if (dif == 0) {
      if (atomicCAS(enq, pos, pos + 1u) == pos) {
        items[pos & (kGeoQueueCap - 1)] = it;
        st_release<GPU>(seq + (pos & (kGeoQueueCap - 1)), pos + 1u);
        return true;
      }
      pos = ld_relaxed<GPU>(enq);
    } else if (dif < 0) {
      return false;  // full
    } else {
      pos = ld_relaxed<GPU>(enq);
    }
  }
  return false;
}

static __device__ bool q_pop(const GeoArgs& a, int q, GeoItem& it) {
  unsigned* deq = a.qpos + (size_t)q * 64 + 32;
  unsigned* seq = a.qseq + (size_t)q * kGeoQueueCap;
  const GeoItem* items = a.qitem + (size_t)q * kGeoQueueCap;
  unsigned pos = ld_relaxed<GPU>(deq);
  for (int tries = 0; tries < 64; ++tries) {
    const unsigned sq = ld_acquire<GPU>(seq + (pos & (kGeoQueueCap - 1)));
    const int dif = (int)(sq - (pos + 1u));
    if (dif == 0) {
      if (atomicCAS(deq, pos, pos + 1u) == pos) {
        it = items[pos & (kGeoQueueCap - 1)];
        st_release<GPU>(seq + (pos & (kGeoQueueCap - 1)), pos + kGeoQueueCap);
        return true;
      }
      pos = ld_relaxed<GPU>(deq);
    } else if (dif < 0) {
      return false;  // empty
    } else {
      pos = ld_relaxed<GPU>(deq);
    }
  }
  return false;
}

struct GeoFrame {
  unsigned s[5];
  int next, end;
};

// The walk, run by every thread of the walking CTAs (rank = this CTA's index
// among them): the standalone kernel's grid, or a server slot's CTAs.  Each
// CTA pushes to queue rank % nq and steals from random others.
static __device__ void uts_geo_walk(const GeoArgs& a, unsigned rank) {
  __shared__ unsigned s_t[kGeoTable];
  for (int i = threadIdx.x; i < kGeoTable; i += blockDim.x) s_t[i] = i < a.nt ? a.table[i] : 0u;
  __syncthreads();
  const HsEnv env{a.status, a.timeout_ns};
  const int myq = (int)(rank % (unsigned)a.nq);
  unsigned rng = 0x9E3779B9u * (rank * blockDim.x + threadIdx.x + 1u);
  GeoFrame st[kGeoMaxDepth + 1];
  int sp = 0;  // frames on the stack; frame f holds a node at depth base + f
  unsigned base = 0;
  unsigned long long nodes = 0, leaves = 0;
  unsigned deepest = 0;
  bool busy = false;
  if (rank == 0 && threadIdx.x == 0) {  // the root; work starts at 1 for this thread
    unsigned r[5];
    geo_root(a.seed, r);
    nodes = 1;
    const int m = geo_nchildren(r, 0, a.limit, s_t, a.nt);
    if (m == 0) {
      leaves = 1;
      asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(a.work), "r"(0xFFFFFFFFu) : "memory");
    } else {
      for (int k = 0; k < 5; ++k) st[0].s[k] = r[k];
      st[0].next = 0;
      st[0].end = m;
      sp = 1;
      base = 0;
      busy = true;
    }
  }
  bool counted_idle = false;
  unsigned long long t0 = 0;
  unsigned last_work = 0;
  unsigned nap = 64;
  for (;;) {
    if (busy) {
      // walk up to 64 nodes, then consider giving work away
      for (int step = 0; step < 64 && sp > 0; ++step) {
        GeoFrame& f = st[sp - 1];
        if (f.next == f.end) {
          --sp;
          continue;
        }
        unsigned c[5];
        geo_child(f.s, (unsigned)f.next, c);
        f.next += 1;
        const unsigned d = base + (unsigned)sp;  // the child's depth
        ++nodes;
        if (d > deepest) deepest = d;
        const int m = geo_nchildren(c, (int)d, a.limit, s_t, a.nt);
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
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(a.work), "r"(0xFFFFFFFFu) : "memory");
        continue;
      }
      if (ld_relaxed<GPU>(a.idle) != 0u) {
        // give away the upper half of the oldest frame with two or more children left
        for (int f = 0; f < sp; ++f) {
          const int left = st[f].end - st[f].next;
          if (left >= 2) {
            GeoItem it;
            for (int k = 0; k < 5; ++k) it.s[k] = st[f].s[k];
            it.depth = base + (unsigned)f;
            it.first = (unsigned)(st[f].next + left / 2);
            it.end = (unsigned)st[f].end;
            atomicAdd(a.work, 1u);
            if (q_push(a, myq, it)) st[f].end = (int)it.first;
            else asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" :: "l"(a.work), "r"(0xFFFFFFFFu) : "memory");
            break;
          }
        }
      }
      continue;
    }
    // idle: own queue first, then a few random victims
    GeoItem it;
    bool got = q_pop(a, myq, it);
    for (int v = 0; v < 4 && !got; ++v) {
      rng ^= rng << 13; rng ^= rng >> 17; rng ^= rng << 5;
      got = q_pop(a, (int)(rng % (unsigned)a.nq), it);
    }
    if (got) {
      if (counted_idle) {
        atomicSub(a.idle, 1u);
        counted_idle = false;
      }
      for (int k = 0; k < 5; ++k) st[0].s[k] = it.s[k];
      st[0].next = (int)it.first;
      st[0].end = (int)it.end;
      base = it.depth;
      sp = 1;
      busy = true;
      nap = 64;
      t0 = 0;
      continue;
    }
    if (!counted_idle) {
      atomicAdd(a.idle, 1u);
      counted_idle = true;
    }
    const unsigned w = ld_acquire<GPU>(a.work);
    if (w == 0u) break;
    // bounded: the work count must move within the time limit
    const unsigned long long now = globaltimer();
    if (t0 == 0 || w != last_work) {
      t0 = now;
      last_work = w;
    } else if (now - t0 > a.timeout_ns || ld_relaxed<GPU>(a.status) != 0u) {
      if (ld_relaxed<GPU>(a.status) == 0u) fail(env, HS_DEV_TIMEOUT, HS_SITE_UTS);
      break;
    }
    sleep_ns(nap);
    nap = nap < 1024u ? nap * 2u : 1024u;
  }
  if (counted_idle) atomicSub(a.idle, 1u);
  atomicAdd(a.out, nodes);
  atomicAdd(a.out + 8, leaves);
  atomicMax(a.out + 16, (unsigned long long)deepest);
}

}  // namespace hs
