// hs_device.cuh -- sm_103a synchronization primitives for the HeteroSync hot path.
//
// Every primitive here is block-collective in the same sense as the reference's
// device API (all threads of the CTA call it; thread 0 performs the atomics), but
// it is built on scoped PTX (ld.acquire / st.release / atom / red at .gpu or
// .cluster scope) instead of volatile accesses plus __threadfence, it polls with a
// single lane, broadcasts with one bar.red (__syncthreads_or) instead of one
// __syncthreads per failed poll, and every wait is bounded: a wait that exceeds
// HsEnv::timeout_ns, or that sees another CTA's error in HsEnv::status, gives up,
// records HS_DEV_TIMEOUT and the wait site, and returns false so the kernel can
// exit cleanly (no __trap, no assert, no unbounded spin).
//
// Reference algorithms restated here (heterosync, cuda/syncPrims/uvm/):
//   spin mutex            cudaLocksMutexSpin.cu:13-95
//   EBO mutex             cudaLocksMutexEBO.cu:13-133
//   fetch-and-add mutex   cudaLocksMutexFA.cu:13-133
//   sleep (ring) mutex    cudaLocksMutexSleep.cu:20-199
//   spin/EBO semaphore    cudaLocksSemaphoreSpin.cu:25-405, cudaLocksSemaphoreEBO.cu:23-457
//   atomic tree barrier   cudaLocksBarrierAtomic.cu:6-172
//   lock-free barrier     cudaLocksBarrierFast.cu:10-330
// The reference-signature wrappers (same names and parameters as those files)
// are in hs_device_ref.cuh.
#pragma once
#include <cstdint>

namespace hs {

// ---------------------------------------------------------------------------
// Status words shared by all CTAs of one instance.
//   status[0] : error bits (nonzero means "abort": every waiter gives up)
//   status[1] : site code of the first failing wait
// ---------------------------------------------------------------------------
enum : unsigned {
  HS_DEV_TIMEOUT = 1u,   // a bounded wait ran out
  HS_DEV_BADARG  = 2u,   // a kernel saw arguments it cannot honour
  HS_DEV_TORN    = 4u,   // a semaphore reader saw a torn snapshot (inc mode check)
};

// Wait-site codes (status[1]); one per spin loop so a timeout names its loop.
enum : unsigned {
  HS_SITE_SPIN_LOCK = 1, HS_SITE_EBO_LOCK = 2, HS_SITE_FA_LOCK = 3, HS_SITE_SLEEP_LOCK = 4,
  HS_SITE_SEM_WAIT = 5, HS_SITE_BAR_LOCAL = 6, HS_SITE_BAR_GLOBAL = 7, HS_SITE_BAR_SCAN = 8,
  HS_SITE_BAR_GO = 9, HS_SITE_BATCH = 10, HS_SITE_SERVE = 11, HS_SITE_RELAXED = 12,
  HS_SITE_UTS = 13, HS_SITE_EXCH = 14, HS_SITE_TMA = 15,
};

struct HsEnv {
  unsigned* status;                 // 2 words, see above
  unsigned long long timeout_ns;    // per-wait limit
};

// Padding: one lock word per 128-byte L2 line.
constexpr int kLineWords = 32;

// ---------------------------------------------------------------------------
// Scoped memory operations (generic addressing: global or distributed shared).
// ---------------------------------------------------------------------------
enum Scope { GPU = 0, CLUSTER = 1, CTA = 2, SYS = 3 };  // SYS: host memory shared with CPU threads

template <int S> __device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  if constexpr (S == CLUSTER) asm volatile("ld.acquire.cluster.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  else if constexpr (S == CTA) asm volatile("ld.acquire.cta.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  else if constexpr (S == SYS) asm volatile("ld.acquire.sys.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  else asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
template <int S> __device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
  unsigned v;
  if constexpr (S == CLUSTER) asm volatile("ld.relaxed.cluster.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  else if constexpr (S == CTA) asm volatile("ld.relaxed.cta.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  else if constexpr (S == SYS) asm volatile("ld.relaxed.sys.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  else asm volatile("ld.relaxed.gpu.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
template <int S> __device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  if constexpr (S == CLUSTER) asm volatile("st.release.cluster.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else if constexpr (S == CTA) asm volatile("st.release.cta.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else if constexpr (S == SYS) asm volatile("st.release.sys.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else asm volatile("st.release.gpu.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
template <int S> __device__ __forceinline__ void st_relaxed(unsigned* p, unsigned v) {
  if constexpr (S == CLUSTER) asm volatile("st.relaxed.cluster.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else if constexpr (S == CTA) asm volatile("st.relaxed.cta.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else if constexpr (S == SYS) asm volatile("st.relaxed.sys.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else asm volatile("st.relaxed.gpu.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
// atom.inc: old = *p; *p = (old >= lim) ? 0 : old + 1   (same wrap rule as atomicInc)
template <int S> __device__ __forceinline__ unsigned atom_inc_relaxed(unsigned* p, unsigned lim) {
  unsigned o;
  if constexpr (S == CLUSTER) asm volatile("atom.relaxed.cluster.inc.u32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(lim) : "memory");
  else asm volatile("atom.relaxed.gpu.inc.u32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(lim) : "memory");
  return o;
}
template <int S> __device__ __forceinline__ void red_release_inc(unsigned* p, unsigned lim) {
  if constexpr (S == CLUSTER) asm volatile("red.release.cluster.inc.u32 [%0], %1;" :: "l"(p), "r"(lim) : "memory");
  else asm volatile("red.release.gpu.inc.u32 [%0], %1;" :: "l"(p), "r"(lim) : "memory");
}
template <int S> __device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  if constexpr (S == CLUSTER) asm volatile("red.release.cluster.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
  else asm volatile("red.release.gpu.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
template <int S> __device__ __forceinline__ unsigned atom_add_acqrel(unsigned* p, unsigned v) {
  unsigned o;
  if constexpr (S == CLUSTER) asm volatile("atom.acq_rel.cluster.add.u32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(v) : "memory");
  else if constexpr (S == SYS) asm volatile("atom.acq_rel.sys.add.u32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(v) : "memory");
  else asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(v) : "memory");
  return o;
}
template <int S> __device__ __forceinline__ unsigned atom_cas_acquire(unsigned* p, unsigned cmp, unsigned val) {
  unsigned o;
  if constexpr (S == CLUSTER) asm volatile("atom.acquire.cluster.cas.b32 %0, [%1], %2, %3;" : "=r"(o) : "l"(p), "r"(cmp), "r"(val) : "memory");
  else asm volatile("atom.acquire.gpu.cas.b32 %0, [%1], %2, %3;" : "=r"(o) : "l"(p), "r"(cmp), "r"(val) : "memory");
  return o;
}
template <int S> __device__ __forceinline__ unsigned atom_or_relaxed(unsigned* p, unsigned v) {
  unsigned o;
  if constexpr (S == CLUSTER) asm volatile("atom.relaxed.cluster.or.b32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(v) : "memory");
  else asm volatile("atom.relaxed.gpu.or.b32 %0, [%1], %2;" : "=r"(o) : "l"(p), "r"(v) : "memory");
  return o;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void sleep_ns(unsigned ns) {
  if (ns) __nanosleep(ns);
}

// Record a failure (first site wins) and raise the abort bit for everyone.
__device__ __forceinline__ void fail(const HsEnv& env, unsigned bits, unsigned site) {
  atomicOr(env.status, bits);
  atomicCAS(env.status + 1, 0u, site);
}

// Bounded wait executed by ONE thread.  cond() is re-evaluated after backoff();
// every 16 polls the status word and the timer are checked.  Returns true once
// cond() holds, false on timeout or when another CTA has already failed.
//
// progress() names a word other waiters' progress changes (a ticket lock's turn,
// a semaphore's state): whenever its value moves, the timer restarts, so a
// waiter that is legitimately behind many others (a reader held off by a long
// writer phase) never times out while the system advances; a wait times out
// only after timeout_ns with no observed progress.
template <class Cond, class Progress, class Backoff>
__device__ __forceinline__ bool wait_until_p(Cond cond, Progress progress, Backoff backoff, const HsEnv& env,
                                             unsigned site) {
  if (cond()) return true;
  unsigned long long t0 = globaltimer();
  unsigned last = progress();
  unsigned polls = 0;
  for (;;) {
    backoff();
    if (cond()) return true;
    if ((++polls & 15u) == 0u) {
      if (ld_relaxed<GPU>(env.status) != 0u) return false;
      const unsigned long long now = globaltimer();
      const unsigned p = progress();
      if (p != last) {
        last = p;
        t0 = now;
      } else if (now - t0 > env.timeout_ns) {
        fail(env, HS_DEV_TIMEOUT, site);
        return false;
      }
    }
  }
}

template <class Cond, class Backoff>
__device__ __forceinline__ bool wait_until(Cond cond, Backoff backoff, const HsEnv& env, unsigned site) {
  return wait_until_p(cond, [] { return 0u; }, backoff, env, site);
}

__device__ __forceinline__ bool is_master() {
  return threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0;
}

// Capped exponential sequence used by the reference EBO primitives:
// b -> ((b << 1) + 1) & (cap - 1)   (1, 3, 7, ..., cap-1; cap a power of two)
__device__ __forceinline__ unsigned ebo_next(unsigned b, unsigned cap) {
  return ((b << 1) + 1u) & (cap - 1u);
}

// ---------------------------------------------------------------------------
// Mutexes.  lock_* returns (to every thread) whether the lock was taken.
// unlock_* must follow a successful lock_* and is called by all threads.
// ---------------------------------------------------------------------------

// Spin (test-and-test-and-set) mutex: CAS 0->1 with acquire, release store 0.
template <int S>
__device__ __forceinline__ bool spin_lock(unsigned* lock, const HsEnv& env) {
  int ok = 0;  // non-masters contribute 0, so the bar.red OR is the master's result
  if (is_master()) {
    ok = wait_until([&] { return ld_relaxed<S>(lock) == 0u && atom_cas_acquire<S>(lock, 0u, 1u) == 0u; },
                    [] {}, env, HS_SITE_SPIN_LOCK);
  }
  return __syncthreads_or(ok) != 0;
}
template <int S>
__device__ __forceinline__ void spin_unlock(unsigned* lock) {
  __syncthreads();  // every thread's critical-section stores precede the release
  if (is_master()) st_release<S>(lock, 0u);
}

// Exponential-backoff mutex: as spin, sleeping b ns after each failed try,
// b following the reference's capped sequence starting at bmin (cap bmax, pow2).
template <int S>
__device__ __forceinline__ bool ebo_lock(unsigned* lock, unsigned bmin, unsigned bmax, const HsEnv& env) {
  int ok = 0;  // non-masters contribute 0, so the bar.red OR is the master's result
  if (is_master()) {
    unsigned b = bmin;
    ok = wait_until([&] { return ld_relaxed<S>(lock) == 0u && atom_cas_acquire<S>(lock, 0u, 1u) == 0u; },
                    [&] { sleep_ns(b); b = ebo_next(b, bmax); }, env, HS_SITE_EBO_LOCK);
  }
  return __syncthreads_or(ok) != 0;
}

// Fetch-and-add (ticket) mutex.  ticket/turn wrap at `wrap` like atomicInc.
// The wait sleeps in proportion to the number of tickets ahead (unit ns per
// position, capped at bmax); unit == 0 spins.
template <int S>
__device__ __forceinline__ bool ticket_lock(unsigned* ticket, unsigned* turn, unsigned wrap,
                                            unsigned unit, unsigned bmax, const HsEnv& env) {
  int ok = 0;  // non-masters contribute 0, so the bar.red OR is the master's result
  if (is_master()) {
    const unsigned my = atom_inc_relaxed<S>(ticket, wrap);
    unsigned cur = 0;
    ok = wait_until_p([&] { cur = ld_acquire<S>(turn); return cur == my; }, [&] { return cur; },
                    [&] {
                      if (unit) {
                        unsigned ahead = (my >= cur) ? (my - cur) : (my + wrap + 1u - cur);
                        unsigned ns = ahead > 1u ? (ahead - 1u) * unit : 0u;
                        sleep_ns(ns < bmax ? ns : bmax);
                      }
                    },
                    env, HS_SITE_FA_LOCK);
  }
  return __syncthreads_or(ok) != 0;
}
template <int S>
__device__ __forceinline__ void ticket_unlock(unsigned* turn, unsigned wrap) {
  __syncthreads();
  if (is_master()) red_release_inc<S>(turn, wrap);
}

// ---------------------------------------------------------------------------
// Cohort (die-aware) mutexes.  A GB300 has two dies; an L2 line is homed on
// one of them.  A lock hand-off between two SMs of the die that homes the lock
// word costs ~450 ns, any hand-off that crosses the dies ~750 ns (and an
// atomic ~150 against ~330 ns).  A cohort lock keeps hand-offs on one die: each
// die has a local lock homed on it, and the global lock (the primitive's own
// word) is taken only by a TB that did not inherit it.  The local lock is a
// ticket queue whose turn word also counts the passes.  A releasing holder
// with local waiters passes the local lock together with the global one, at
// most kCohortMaxPass times in a row; otherwise it releases both.  Mutual
// exclusion is the global lock's (held by one cohort) and the local lock's
// (one holder in the cohort).
// ---------------------------------------------------------------------------
constexpr unsigned kCohortMaxPass = 63;

// Ticket cohort: a ticket lock per die over the global ticket lock.  The local
// turn word carries the pass count: turn = (ticket << 6) | passes, written
// only by the holder; local tickets wrap at kCohortTicketWrap.  The holder
// snapshots the local ticket counter as soon as it holds the lock, so the
// waiter check costs nothing at release.
constexpr unsigned kCohortTicketWrap = (1u << 25) - 1u;
__device__ __forceinline__ bool cohort_ticket_lock(unsigned* lt, unsigned* lu, unsigned* gt, unsigned* gu,
                                                   unsigned wrap, unsigned unit, unsigned bmax, const HsEnv& env,
                                                   unsigned& my, unsigned& pc, unsigned& snap) {
  int ok = 0;
  if (is_master()) {
    my = atom_inc_relaxed<GPU>(lt, kCohortTicketWrap);
    unsigned cur = 0;
    ok = wait_until_p([&] { cur = ld_acquire<GPU>(lu); return (cur >> 6) == my; }, [&] { return cur; },
                      [&] {
                        if (unit) {
                          const unsigned t = cur >> 6;
                          const unsigned ahead = (my >= t) ? (my - t) : (my + kCohortTicketWrap + 1u - t);
                          const unsigned ns = ahead > 1u ? (ahead - 1u) * unit : 0u;
                          sleep_ns(ns < bmax ? ns : bmax);
                        }
                      },
                      env, HS_SITE_FA_LOCK);
    pc = cur & 63u;
    if (ok && pc == 0u) {
      const unsigned g = atom_inc_relaxed<GPU>(gt, wrap);
      unsigned gc = 0;
      ok = wait_until_p([&] { gc = ld_acquire<GPU>(gu); return gc == g; }, [&] { return gc; },
                        [&] {
                          if (unit) {
                            const unsigned ahead = (g >= gc) ? (g - gc) : (g + wrap + 1u - gc);
                            const unsigned ns = ahead > 1u ? (ahead - 1u) * unit : 0u;
                            sleep_ns(ns < bmax ? ns : bmax);
                          }
                        },
                        env, HS_SITE_FA_LOCK);
    }
  }
  const bool got = __syncthreads_or(ok) != 0;
  // tickets taken so far, read after the CTA barrier so that the barrier does
  // not wait for it (its value is needed only at release; a ticket taken after
  // the read only means one global release more)
  if (is_master()) snap = ld_relaxed<GPU>(lt);
  return got;
}
__device__ __forceinline__ void cohort_ticket_unlock(unsigned* lu, unsigned* gu, unsigned wrap, unsigned my,
                                                     unsigned pc, unsigned snap) {
  __syncthreads();
  if (is_master()) {
    const unsigned next = (my >= kCohortTicketWrap) ? 0u : my + 1u;
    if (snap != next && pc + 1u < kCohortMaxPass) {
      st_release<GPU>(lu, (next << 6) | (pc + 1u));  // pass the global lock on within the die
    } else {
      red_release_inc<GPU>(gu, wrap);
      st_release<GPU>(lu, next << 6);
    }
  }
}

// Ticket cohort over a global lock (the spin and EBO mutexes' test-and-set word).  The
// local layer is cohort_ticket_lock's (turn = (ticket << 6) | passes, written
// only by the holder).  A TB whose turn comes without a pass runs `acquire`
// (master thread; false on timeout) to take the global lock; the releasing
// holder passes both locks to the next ticket of its die (at most
// kCohortMaxPass times in a row) or runs `release` and advances the turn.
// Only one TB per die touches the global lock word, and a pass is one release
// store to a line homed on the die, with no atomic at all.
template <class Acquire>
__device__ __forceinline__ bool cohort_queue_lock(unsigned* lt, unsigned* lu, Acquire acquire, const HsEnv& env,
                                                  unsigned site, unsigned& my, unsigned& pc, unsigned& snap) {
  int ok = 0;
  if (is_master()) {
    my = atom_inc_relaxed<GPU>(lt, kCohortTicketWrap);
    unsigned cur = 0;
    ok = wait_until_p([&] { cur = ld_acquire<GPU>(lu); return (cur >> 6) == my; }, [&] { return cur; }, [] {}, env,
                      site);
    pc = cur & 63u;
    if (ok && pc == 0u) ok = acquire();
  }
  const bool got = __syncthreads_or(ok) != 0;
  if (is_master()) snap = ld_relaxed<GPU>(lt);  // as in cohort_ticket_lock
  return got;
}
template <class Release>
__device__ __forceinline__ void cohort_queue_unlock(unsigned* lu, Release release, unsigned my, unsigned pc,
                                                    unsigned snap) {
  __syncthreads();  // every thread's critical-section stores precede the release
  if (is_master()) {
    const unsigned next = (my >= kCohortTicketWrap) ? 0u : my + 1u;
    if (snap != next && pc + 1u < kCohortMaxPass) {
      st_release<GPU>(lu, (next << 6) | (pc + 1u));  // pass the global lock on within the die
    } else {
      release();
      st_release<GPU>(lu, next << 6);
    }
  }
}

// Ring-buffer (array queue) "sleep" mutex.  A waiter takes slot
// atomicInc(tail, max_slot) and waits for ring[slot] == 1; unlock writes -1 to
// its slot and 1 to the next (wrapping after max_slot).  Slots are `stride`
// words apart.  The slot is returned to every thread through shared memory.
template <int S>
__device__ __forceinline__ int queue_lock(unsigned* tail, unsigned* ring, unsigned stride,
                                          unsigned max_slot, unsigned spin_ns, const HsEnv& env,
                                          int* s_slot) {
  int ok = 0;  // non-masters contribute 0, so the bar.red OR is the master's result
  if (is_master()) {
    const unsigned slot = atom_inc_relaxed<S>(tail, max_slot);
    *s_slot = (int)slot;
    unsigned* mine = ring + (size_t)slot * stride;
    unsigned* prev = ring + (size_t)(slot == 0u ? max_slot : slot - 1u) * stride;
    ok = wait_until_p([&] { return ld_acquire<S>(mine) == 1u; }, [&] { return ld_relaxed<S>(prev); },
                      [&] { sleep_ns(spin_ns); }, env, HS_SITE_SLEEP_LOCK);
  }
  if (!__syncthreads_or(ok)) return -1;
  return *s_slot;
}
template <int S>
__device__ __forceinline__ void queue_unlock(unsigned* ring, unsigned stride, unsigned max_slot, unsigned slot) {
  __syncthreads();
  if (is_master()) {
    const unsigned next = (slot >= max_slot) ? 0u : slot + 1u;
    st_relaxed<S>(ring + (size_t)slot * stride, 0xFFFFFFFFu);
    st_release<S>(ring + (size_t)next * stride, 1u);
  }
}

// ---------------------------------------------------------------------------
// Reader/writer semaphore on ONE packed word:
//   bits 0..30 : count (starts at N+1 == maxc), bit 31 : writer-waiting flag.
// Admission rules are the reference's (cudaLocksSemaphoreSpin.cu:70-127):
//   writer needs count == maxc, then count -= maxc and clears writer-waiting;
//   a refused writer sets writer-waiting;
//   reader needs writer-waiting == 0 and count > 1, then count -= 1.
// Post: writer count += maxc, reader count += 1 -- a single red.release.
// Backoff policy (EBO variants): writers exponential, readers +5 ns linear
// (reader_linear == true) or exponential (Local variants).
// ---------------------------------------------------------------------------
constexpr unsigned kSemWW = 0x80000000u;
constexpr unsigned kSemCnt = 0x7FFFFFFFu;

template <int S>
__device__ __forceinline__ bool sem_try_once(unsigned* st, bool writer, unsigned maxc) {
  const unsigned s = ld_relaxed<S>(st);
  if (writer) {
    if ((s & kSemCnt) == maxc) return atom_cas_acquire<S>(st, s, 0u) == s;
    if (!(s & kSemWW)) atom_or_relaxed<S>(st, kSemWW);
    return false;
  }
  if (!(s & kSemWW) && (s & kSemCnt) > 1u) return atom_cas_acquire<S>(st, s, s - 1u) == s;
  return false;
}

template <int S>
__device__ __forceinline__ bool sem_wait(unsigned* st, bool writer, unsigned maxc, bool ebo, bool reader_linear,
                                         unsigned bmin, unsigned bmax, const HsEnv& env) {
  int ok = 0;  // non-masters contribute 0, so the bar.red OR is the master's result
  if (is_master()) {
    unsigned b = bmin;
    ok = wait_until_p([&] { return sem_try_once<S>(st, writer, maxc); }, [&] { return ld_relaxed<S>(st); },
                    [&] {
                      if (ebo) {
                        sleep_ns(b);
                        if (writer || !reader_linear) b = ebo_next(b, bmax);
                        else b = (b + 5u < bmax) ? b + 5u : bmax;
                      }
                    },
                    env, HS_SITE_SEM_WAIT);
  }
  return __syncthreads_or(ok) != 0;
}
// Die-aware (cohort) writers of a global semaphore.  Writers exclude one
// another and every reader, so, like the cohort mutexes, the writers of one die
// form a cohort queued on a ticket lock homed on that die (the
// cohort_ticket_lock encoding: local turn = (ticket << 6) | passes).  A writer
// whose turn comes without a pass takes the semaphore by the reference's writer
// rule (count == maxc, else set writer-waiting); on release, a writer with
// writers queued behind it on its die hands the semaphore to the next one (at
// most kCohortMaxPass times in a row) instead of posting, otherwise it posts
// (count += maxc) and advances the turn.  A hand-over is what the reference's
// rules would give as well: a waiting writer has writer-waiting set, so no
// reader can enter between the post and that writer's acquisition; here the
// count simply stays 0 across it.  A hand-over touches only the die's own
// lines (no CAS at all), and only one writer per die polls the semaphore word.
__device__ __forceinline__ bool cohort_sem_writer_wait(unsigned* lt, unsigned* lu, unsigned* st, unsigned maxc,
                                                       bool ebo, unsigned bmin, unsigned bmax, const HsEnv& env,
                                                       unsigned& my, unsigned& pc, unsigned& snap) {
  int ok = 0;
  if (is_master()) {
    unsigned b = bmin;
    auto backoff = [&] {
      if (ebo) {
        sleep_ns(b);
        b = ebo_next(b, bmax);
      }
    };
    my = atom_inc_relaxed<GPU>(lt, kCohortTicketWrap);
    unsigned cur = 0;
    // the die's ticket queue is this build's own and has no backoff; the EBO
    // backoff applies where the reference's writers back off, on the semaphore
    ok = wait_until_p([&] { cur = ld_acquire<GPU>(lu); return (cur >> 6) == my; }, [&] { return cur; }, [] {}, env,
                      HS_SITE_SEM_WAIT);
    pc = cur & 63u;
    // tickets taken so far, read before the semaphore wait and the CTA barrier:
    // measured faster here than after the barrier (the mutexes read it after)
    snap = ld_relaxed<GPU>(lt);
    if (ok && pc == 0u) {  // the die's cohort does not hold the semaphore: take it by the writer rule
      ok = wait_until_p(
          [&] {
            const unsigned s = ld_relaxed<GPU>(st);
            if ((s & kSemCnt) == maxc) return atom_cas_acquire<GPU>(st, s, 0u) == s;
            if (!(s & kSemWW)) atom_or_relaxed<GPU>(st, kSemWW);
            return false;
          },
          [&] { return ld_relaxed<GPU>(st); }, backoff, env, HS_SITE_SEM_WAIT);
    }
  }
  return __syncthreads_or(ok) != 0;
}
__device__ __forceinline__ void cohort_sem_writer_post(unsigned* lu, unsigned* st, unsigned maxc, unsigned my,
                                                       unsigned pc, unsigned snap) {
  __syncthreads();  // every thread's critical-section stores precede the release
  if (is_master()) {
    const unsigned next = (my >= kCohortTicketWrap) ? 0u : my + 1u;
    if (snap != next && pc + 1u < kCohortMaxPass) {
      st_release<GPU>(lu, (next << 6) | (pc + 1u));  // hand the semaphore to the next writer of this die
    } else {
      red_release_add<GPU>(st, maxc);
      st_release<GPU>(lu, next << 6);
    }
  }
}

template <int S>
__device__ __forceinline__ void sem_post(unsigned* st, bool writer, unsigned maxc) {
  __syncthreads();
  if (is_master()) red_release_add<S>(st, writer ? maxc : 1u);
}

// ---------------------------------------------------------------------------
// Barriers.  All state is generation-valued and monotonic, so nothing is reset
// between episodes or launches (the reference's two-counter "facsimile sense
// reversal", cudaLocksBarrierAtomic.cu:67-81, and its in/out flag resets,
// cudaLocksBarrierFast.cu:109-161, are replaced by one generation word).
// ---------------------------------------------------------------------------

// Counter barrier among n arrivals (one thread each).  The last arriver resets
// the counter and publishes gen+1.  Returns 1 if this thread was the last.
// `gen` is the caller's copy of the generation for this episode.
template <int S, class OnLast>
__device__ __forceinline__ int counter_barrier(unsigned* count, unsigned* genw, unsigned n, unsigned gen,
                                               unsigned poll_ns, const HsEnv& env, unsigned site,
                                               OnLast on_last, bool* ok) {
  const unsigned old = atom_add_acqrel<S>(count, 1u);
  if (old == n - 1u) {
    st_relaxed<S>(count, 0u);
    *ok = on_last();
    st_release<S>(genw, gen + 1u);
    return 1;
  }
  *ok = wait_until([&] { return ld_acquire<S>(genw) != gen; }, [&] { sleep_ns(poll_ns); }, env, site);
  return 0;
}

// Flag wait: all n flags (dense, generation-valued) must reach `target`.
// Executed by every thread of the CTA (strided scan, like the reference's main
// TB, cudaLocksBarrierFast.cu:26-61); returns the CTA-wide result.
template <int S>
__device__ __forceinline__ bool scan_flags(const unsigned* flags, unsigned n, unsigned target, unsigned poll_ns,
                                           const HsEnv& env, unsigned site) {
  int ok = 1;
  for (unsigned i = threadIdx.x; i < n && ok; i += blockDim.x) {
    ok = wait_until([&] { return (int)(ld_acquire<S>(flags + i) - target) >= 0; }, [&] { sleep_ns(poll_ns); },
                    env, site);
  }
  return __syncthreads_and(ok) != 0;
}

// Hardware cluster barrier (all threads of all CTAs in the cluster).
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_id_x() {
  unsigned r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

// Map a local shared-memory address to the same address in CTA `rank` of the
// cluster (distributed shared memory), as a generic pointer.
template <class T>
__device__ __forceinline__ T* map_shared_rank(T* p, unsigned rank) {
  T* r;
  asm volatile("mapa.u64 %0, %1, %2;" : "=l"(r) : "l"(p), "r"(rank));
  return r;
}

}  // namespace hs
