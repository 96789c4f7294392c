// hs_uts_geo.cuh -- geometric UTS walk (SHA-1 node generator, work stealing
// over per-CTA lock-free queues); shared by the standalone kernel
// (hs_uts_geo.cu), the cooperative CPU+GPU walk (hs_uts_geo.cu, with host
// threads through the bridge below) and the server's tree-search requests
// (hs_serve.cu).  The node generator is __host__ __device__: the host walkers
// of the cooperative walk hash with the same code.
#pragma once
#include "../../include/hs/hs_device.cuh"

namespace hs {


constexpr int kGeoMaxDepth = 30;
constexpr int kGeoTable = 128;
constexpr unsigned kGeoQueueCap = 512;  // items per CTA queue (power of two)
constexpr unsigned kBridgeCap = 1024;   // items per CPU<->GPU bridge ring (power of two)
constexpr int kHostLevels = 7;          // the GPU gives host walkers subtrees with 3..kHostLevels levels left
constexpr int kHostMinLevels = 3;

struct GeoItem {  // children [first, end) of the node with state s at `depth`
  unsigned s[5];
  unsigned depth, first, end;
};

// Cooperative walk: GPU CTAs and host threads share one tree through two
// bounded rings in mapped pinned host memory.  Each ring has one producer side
// and one consumer side: a side's own position word lives in its own memory
// (the GPU's in device memory, the host's in host memory), so the rings need
// no atomics across the link; the cells' sequence numbers carry the
// hand-off (release/acquire at system scope).  Only the global count takes
// system-scope atomics from both sides.
//   ctl (host memory, one word per 128-byte line):
//     [0]   global count: active sides (a side is active while its own count
//           of queued items plus busy walkers is non-zero) plus items in the
//           two rings; the walk is over when it reaches zero
//     [32]  idle host walkers        [64]  the GPU has idle threads (host walkers give work)
//     [96]  abort (a side timed out) [128] GPU->host ring dequeue position (host only)
//     [160] host->GPU ring enqueue position (host only)
//     [192] GPU heartbeat            [224] host heartbeat
//   dev (device memory): [0] GPU->host enqueue position, [32] host->GPU
//     dequeue position, [64] done (a poller saw the global count at zero),
//     [96] the pollers' last view of the host (progress signature)
static_assert(sizeof(GeoItem) == 32, "bridge cells copy items as 8 words");

struct GeoBridge {
  unsigned* ctl;
  unsigned* g2h_seq;
  GeoItem* g2h_item;
  unsigned* h2g_seq;
  GeoItem* h2g_item;
  unsigned* dev;
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
  GeoBridge br;  // cooperative walk only
};

__host__ __device__ __forceinline__ unsigned rotl32(unsigned x, int n) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(x, x, n);
#else
  return (x << n) | (x >> (32 - n));
#endif
}

// SHA-1 (FIPS 180-4) of one padded 64-byte block given as 16 big-endian words.
__host__ __device__ __forceinline__ void sha1_block(unsigned w[16], unsigned h[5]) {
  unsigned a = 0x67452301u, b = 0xEFCDAB89u, c = 0x98BADCFEu, d = 0x10325476u, e = 0xC3D2E1F0u;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
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

__host__ __device__ __forceinline__ void geo_child(const unsigned p[5], unsigned i, unsigned out[5]) {
  unsigned w[16] = {p[0], p[1], p[2], p[3], p[4], i, 0x80000000u, 0, 0, 0, 0, 0, 0, 0, 0, 192u};
  sha1_block(w, out);
}

__host__ __device__ __forceinline__ void geo_root(unsigned seed, unsigned out[5]) {
  unsigned w[16] = {0, 0, 0, 0, seed, 0x80000000u, 0, 0, 0, 0, 0, 0, 0, 0, 0, 160u};
  sha1_block(w, out);
}

__host__ __device__ __forceinline__ int geo_nchildren(const unsigned s[5], int depth, int limit, const unsigned* t,
                                                      int nt) {
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

// GPU side of the bridge rings: producer of the GPU->host ring, consumer of
// the host->GPU ring.  Items cross the link word by word at system scope.
static __device__ bool g2h_push(const GeoBridge& br, const GeoItem& it) {
  unsigned* enq = br.dev;
  unsigned pos = ld_relaxed<GPU>(enq);
  for (int tries = 0; tries < 16; ++tries) {
    const unsigned c = pos & (kBridgeCap - 1);
    const int dif = (int)(ld_acquire<SYS>(br.g2h_seq + c) - pos);
    if (dif == 0) {
      if (atomicCAS(enq, pos, pos + 1u) == pos) {
        unsigned* dst = reinterpret_cast<unsigned*>(br.g2h_item + c);
        const unsigned* src = reinterpret_cast<const unsigned*>(&it);
#pragma unroll
        for (int k = 0; k < 8; ++k) st_relaxed<SYS>(dst + k, src[k]);
        st_release<SYS>(br.g2h_seq + c, pos + 1u);
        return true;
      }
    } else if (dif < 0) {
      return false;  // full
    }
    pos = ld_relaxed<GPU>(enq);
  }
  return false;
}

static __device__ bool h2g_pop(const GeoBridge& br, GeoItem& it) {
  unsigned* deq = br.dev + 32;
  unsigned pos = ld_relaxed<GPU>(deq);
  for (int tries = 0; tries < 16; ++tries) {
    const unsigned c = pos & (kBridgeCap - 1);
    const int dif = (int)(ld_acquire<SYS>(br.h2g_seq + c) - (pos + 1u));
    if (dif == 0) {
      if (atomicCAS(deq, pos, pos + 1u) == pos) {
        const unsigned* src = reinterpret_cast<const unsigned*>(br.h2g_item + c);
        unsigned* dst = reinterpret_cast<unsigned*>(&it);
#pragma unroll
        for (int k = 0; k < 8; ++k) dst[k] = ld_relaxed<SYS>(src + k);
        st_release<SYS>(br.h2g_seq + c, pos + kBridgeCap);
        return true;
      }
    } else if (dif < 0) {
      return false;  // empty
    }
    pos = ld_relaxed<GPU>(deq);
  }
  return false;
}

struct GeoFrame {
  unsigned s[5];
  int next, end;
};

// Work count of this side: every lane of the warp adds its change (a lane
// that received a subtree from a warp-mate: +1; a lane whose subtree is done:
// -1) and lane 0 applies the warp's sum with one atomic.  A subtree handed over
// inside a warp stays counted through its donor, so the count never passes
// through zero while work is left.
template <bool COOP>
static __device__ __forceinline__ void geo_work_delta(const GeoArgs& a, int delta) {
  const int sum = __reduce_add_sync(0xFFFFFFFFu, delta);
  if ((threadIdx.x & 31u) == 0u && sum != 0) {
    if constexpr (COOP) {
      const unsigned old = atom_add_acqrel<GPU>(a.work, (unsigned)sum);
      if (sum < 0 && old + (unsigned)sum == 0u) atom_add_acqrel<SYS>(a.br.ctl, 0xFFFFFFFFu);  // the side went idle
    } else {
      asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(a.work), "r"((unsigned)sum) : "memory");
    }
  }
  __syncwarp();  // the warp's count change is ordered before its lanes' next reads of the count
}

// The walk, run by every thread of the walking CTAs (rank = this CTA's index
// among them): the standalone kernel's grid, or a server slot's CTAs.
//
// Each lane walks its own subtrees depth first (a stack of frames), 16 nodes
// per round.  The warp stays converged: after every round, lanes with nothing
// left receive the upper half of the oldest frame of a warp-mate that has two
// or more children left there, through shuffles (no global memory, no
// atomics); only lanes the warp cannot feed go to the CTA queues (own queue
// first, then random victims).  Busy lanes give work to those queues while
// threads anywhere are idle.  Each CTA pushes to queue rank % nq.
//
// COOP: host threads walk the same tree (hs_uts_geo.cu).  A busy thread gives
// host walkers that are idle a subtree near the depth limit (3 to 7 levels
// left: small, since a host core hashes some 40x slower than the GPU); idle
// threads elect one poller per CTA at a time, at most one poll per kPollNs,
// which takes work the host walkers gave back, asks for more once over half
// of the grid is idle (the tail of the walk), and ends the walk for everyone
// when the global count is zero.  The GPU side's own count (work) is then one of
// the two sides the global count tracks.
template <bool COOP = false>
static __device__ void uts_geo_walk(const GeoArgs& a, unsigned rank) {
  constexpr unsigned long long kPollNs = 16000;  // a poll costs a few link round trips
  constexpr unsigned kFull = 0xFFFFFFFFu;
  __shared__ unsigned s_t[kGeoTable];
  __shared__ unsigned s_poll;
  __shared__ unsigned long long s_poll_t;
  for (int i = threadIdx.x; i < kGeoTable; i += blockDim.x) s_t[i] = i < a.nt ? a.table[i] : 0u;
  if (threadIdx.x == 0) {
    s_poll = 0u;
    s_poll_t = 0ull;
  }
  __syncthreads();
  const HsEnv env{a.status, a.timeout_ns};
  const int myq = (int)(rank % (unsigned)a.nq);
  const unsigned lane = threadIdx.x & 31u, lanes_below = (1u << lane) - 1u;
  unsigned rng = 0x9E3779B9u * (rank * blockDim.x + threadIdx.x + 1u);
  GeoFrame st[kGeoMaxDepth + 1];
  int sp = 0;  // frames on the stack; frame f holds a node at depth base + f
  unsigned base = 0;
  unsigned long long nodes = 0, leaves = 0;
  unsigned deepest = 0;
  bool busy = false;
  unsigned batches = 0;
  if (rank == 0 && threadIdx.x == 0) {  // the root; work starts at 1 for this thread
    unsigned r[5];
    geo_root(a.seed, r);
    nodes = 1;
    const int m = geo_nchildren(r, 0, a.limit, s_t, a.nt);
    if (m == 0) {
      leaves = 1;
      if constexpr (COOP) {
        if (atom_add_acqrel<GPU>(a.work, 0xFFFFFFFFu) == 1u) atom_add_acqrel<SYS>(a.br.ctl, 0xFFFFFFFFu);
      } else {
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(a.work), "r"(0xFFFFFFFFu) : "memory");
      }
    } else {
      for (int k = 0; k < 5; ++k) st[0].s[k] = r[k];
      st[0].next = 0;
      st[0].end = m;
      sp = 1;
      base = 0;
      busy = true;
    }
  }
  bool counted_idle = false, stop = false;
  unsigned long long t0 = 0;
  unsigned last_work = 0;
  unsigned nap = 64;
  for (;;) {
    int delta = 0;
    if (busy) {
      for (int step = 0; step < 16; ++step) {
        // exhausted frames are popped first, so every lane with work left
        // hashes in the same iteration (the SHA-1 rounds run with full warps)
        while (sp > 0 && st[sp - 1].next == st[sp - 1].end) --sp;
        if (sp == 0) break;
        GeoFrame& f = st[sp - 1];
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
      while (sp > 0 && st[sp - 1].next == st[sp - 1].end) --sp;
      if (sp == 0) {
        busy = false;
        delta = -1;
      } else {
        if constexpr (COOP) {
          if ((++batches & 63u) == 0u) {  // every 1024 nodes: heartbeat, and feed idle host walkers
            if (threadIdx.x == 0) st_relaxed<SYS>(a.br.ctl + 192, (unsigned)(globaltimer() >> 16));
            const unsigned hidle = ld_relaxed<SYS>(a.br.ctl + 32);
            if (hidle != 0u && ld_relaxed<GPU>(a.br.dev) - ld_relaxed<SYS>(a.br.ctl + 128) < hidle) {
              for (int f = 0; f < sp; ++f) {
                const int left = st[f].end - st[f].next;
                const int levels = a.limit - (int)(base + (unsigned)f);
                if (left >= 2 && levels <= kHostLevels && levels >= kHostMinLevels) {
                  GeoItem it;
                  for (int k = 0; k < 5; ++k) it.s[k] = st[f].s[k];
                  it.depth = base + (unsigned)f;
                  it.first = (unsigned)(st[f].next + left / 2);
                  it.end = (unsigned)st[f].end;
                  atom_add_acqrel<SYS>(a.br.ctl, 1u);
                  if (g2h_push(a.br, it)) st[f].end = (int)it.first;
                  else atom_add_acqrel<SYS>(a.br.ctl, 0xFFFFFFFFu);
                  break;
                }
              }
            }
          }
        }
        if (ld_relaxed<GPU>(a.idle) != 0u) {
          // threads elsewhere are idle: the upper half of the oldest frame with two or more children left
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
      }
    }
    // hand-overs inside the warp: idle lanes take the upper half of a warp-mate's oldest divisible frame
    const unsigned idle_m = __ballot_sync(kFull, !busy && !stop);
    if (idle_m != 0u) {
      int fd = -1;
      if (busy)
        for (int f = 0; f < sp; ++f)
          if (st[f].end - st[f].next >= 2) {
            fd = f;
            break;
          }
      const unsigned donor_m = __ballot_sync(kFull, fd >= 0);
      const int pairs = min(__popc(idle_m), __popc(donor_m));
      if (pairs > 0) {
        unsigned v[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        if (fd >= 0) {
          const int left = st[fd].end - st[fd].next;
          for (int k = 0; k < 5; ++k) v[k] = st[fd].s[k];
          v[5] = base + (unsigned)fd;
          v[6] = (unsigned)(st[fd].next + left / 2);
          v[7] = (unsigned)st[fd].end;
        }
        const int ir = __popc(idle_m & lanes_below), dr = __popc(donor_m & lanes_below);
        const bool recv = ((idle_m >> lane) & 1u) && ir < pairs;
        const int src = recv ? (int)__fns(donor_m, 0u, ir + 1) : (int)lane;
        unsigned g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) g[k] = __shfl_sync(kFull, v[k], src);
        if (fd >= 0 && dr < pairs) st[fd].end = (int)v[6];  // a matched donor keeps the lower half
        if (recv) {
          for (int k = 0; k < 5; ++k) st[0].s[k] = g[k];
          base = g[5];
          st[0].next = (int)g[6];
          st[0].end = (int)g[7];
          sp = 1;
          busy = true;
          delta += 1;
          nap = 64;
          t0 = 0;
          if (counted_idle) {
            atomicSub(a.idle, 1u);
            counted_idle = false;
          }
        }
      }
    }
    geo_work_delta<COOP>(a, delta);
    // lanes the warp could not feed: the CTA queues, then (cooperative) the host
    const bool warp_idle = __all_sync(kFull, !busy);
    if (!busy && !stop) {
      GeoItem it;
      bool got = q_pop(a, myq, it);
      for (int v = 0; v < 4 && !got; ++v) {
        rng ^= rng << 13; rng ^= rng >> 17; rng ^= rng << 5;
        got = q_pop(a, (int)(rng % (unsigned)a.nq), it);
      }
      unsigned w = 0;
      if constexpr (COOP) {
        if (!got && ld_relaxed<GPU>(a.br.dev + 64) != 0u) stop = true;  // done
        const unsigned long long now = globaltimer();
        if (!got && !stop && now - *(volatile unsigned long long*)&s_poll_t >= kPollNs &&
            atomicCAS(&s_poll, 0u, 1u) == 0u) {
          s_poll_t = now;
          if (h2g_pop(a.br, it)) {
            got = true;
            // the item's share of the global count becomes this side's, unless the side was active already
            if (atom_add_acqrel<GPU>(a.work, 1u) != 0u) atom_add_acqrel<SYS>(a.br.ctl, 0xFFFFFFFFu);
          } else {
            const unsigned gc = ld_acquire<SYS>(a.br.ctl);
            const unsigned ab = ld_relaxed<SYS>(a.br.ctl + 96);
            if (gc == 0u || ab != 0u) {
              if (ab != 0u) fail(env, HS_DEV_TIMEOUT, HS_SITE_UTS);
              st_release<GPU>(a.br.dev + 64, 1u);
              stop = true;
            } else {
              // ask the host walkers for work once more than half of this side's threads are idle
              if (ld_relaxed<GPU>(a.work) < gridDim.x * blockDim.x / 2u && ld_relaxed<SYS>(a.br.ctl + 64) == 0u)
                st_relaxed<SYS>(a.br.ctl + 64, 1u);
              st_relaxed<GPU>(a.br.dev + 96, gc * 0x9E3779B1u ^ ld_relaxed<SYS>(a.br.ctl + 224));
            }
          }
          atomicExch(&s_poll, 0u);
        }
        if (!got && !stop) w = ld_acquire<GPU>(a.work) ^ (ld_relaxed<GPU>(a.br.dev + 96) * 0x85EBCA77u);
      }
      if (got) {  // a queue item's count passes to this lane (queued items and busy lanes are both counted)
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
      } else if (!stop) {
        if (!counted_idle) {
          atomicAdd(a.idle, 1u);
          counted_idle = true;
        }
        if constexpr (!COOP) {
          w = ld_acquire<GPU>(a.work);
          if (w == 0u) stop = true;
        }
        if (!stop) {
          // bounded: the work count (and, cooperative, the host's view) must move within the time limit
          const unsigned long long now = globaltimer();
          if (t0 == 0 || w != last_work) {
            t0 = now;
            last_work = w;
          } else if (now - t0 > a.timeout_ns || ld_relaxed<GPU>(a.status) != 0u) {
            if (ld_relaxed<GPU>(a.status) == 0u) fail(env, HS_DEV_TIMEOUT, HS_SITE_UTS);
            if constexpr (COOP) {
              st_relaxed<SYS>(a.br.ctl + 96, 1u);  // the host walkers stop too
              st_release<GPU>(a.br.dev + 64, 1u);
            }
            stop = true;
          }
          if (!stop && warp_idle) {  // only a warp with no busy lane waits
            sleep_ns(nap);
            nap = nap < 1024u ? nap * 2u : 1024u;
          }
        }
      }
    }
    if (__all_sync(kFull, stop)) break;
  }
  if (counted_idle) atomicSub(a.idle, 1u);
  atomicAdd(a.out, nodes);
  atomicAdd(a.out + 8, leaves);
  atomicMax(a.out + 16, (unsigned long long)deepest);
}

}  // namespace hs
