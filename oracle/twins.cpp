// twins.cpp -- ORACLE (test infrastructure and the host-thread CPU baseline).
//
// std::thread / std::atomic runs of the reference's SyncPrims algorithms on the
// host's cores.  Each logical TB is a small state machine whose every step is
// non-blocking (a lock attempt, a poll, a critical section), and the logical
// TBs are dealt cyclically onto min(numTBs, threads) std::threads that keep
// stepping their TBs; a wait therefore never blocks a thread that hosts the TB
// being waited for.  One "launch" (repeat) ends when every TB has finished its
// iterations, as a kernel launch does.
//
// Algorithms (heterosync cuda/syncPrims/uvm/):
//   spin / EBO mutex   CAS 0->1, release store 0     cudaLocksMutexSpin.cu:13-50, MutexEBO.cu:13-70
//   ticket mutex       fetch-add ticket, poll turn    cudaLocksMutexFA.cu:13-69
//   ring mutex         slot = inc(tail) mod max+1     cudaLocksMutexSleep.cu:20-108
//   semaphores         reader/writer admission rules  cudaLocksSemaphoreSpin.cu:25-213
//   tree barriers      counter barrier with a local   cudaLocksBarrierAtomic.cu, main.cu:104-315
//                      exchange stage (LocalExch)
// Data accesses are the reference's (main.cu:60-100) and the build's INC and
// SLICE modes, so a run's final storage equals the oracle golden.
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace {

struct alignas(64) AU {
  std::atomic<uint32_t> v{0};
};

struct Shared {
  int prim, T, L, G, iters, nsm, mode;
  uint32_t* data;
  std::vector<AU> lock, ticket, turn, tail, sem;  // per group
  std::vector<std::unique_ptr<std::atomic<int32_t>[]>> ring;
  uint32_t ring_max;
  AU gcount, ggen;
  std::vector<AU> lcount, lgen;
  std::atomic<uint32_t> sink{0};
};

bool is_barrier(int p) { return p <= 3; }
bool is_gmutex(int p) { return p >= 4 && p <= 7; }
bool is_gsem(int p) { return p >= 8 && p <= 15; }
bool is_umutex(int p) { return p >= 20 && p <= 23; }

size_t chunk_words(const Shared& s) { return (size_t)s.T * (s.L + 1); }

// One critical section on chunk c (REF: one-line shift; INC: +1 on lines 1..L).
void cs_chunk(Shared& s, long c) {
  uint32_t* base = s.data + (size_t)c * chunk_words(s);
  const int R = s.T / 16;
  for (int h = 0; h < R; ++h) {
    uint32_t* reg = base + (size_t)h * 16 * (s.L + 1);
    if (s.mode == 0) std::memmove(reg + 16, reg, (size_t)16 * s.L * 4);
    else
      for (int i = 16; i < 16 * (s.L + 1); ++i) reg[i] += 1u;
  }
}
void cs_slice(Shared& s, long slice) {
  uint32_t* p = s.data + (size_t)slice * s.L;
  for (int w = 0; w < s.L; ++w) p[w] += 1u;
}
void cs_read(Shared& s, long c) {
  const uint32_t* base = s.data + (size_t)c * chunk_words(s);
  uint32_t acc = 0;
  const int R = s.T / 16;
  for (int h = 0; h < R; ++h)
    for (int i = 0; i < 16 * s.L; ++i) acc += base[(size_t)h * 16 * (s.L + 1) + i];
  s.sink.fetch_add(acc & 1u, std::memory_order_relaxed);
}

struct TB {
  int b = 0, j = 0, phase = 0;
  uint32_t ticket = 0, slot = 0, gen = 0, bo = 1, skip = 0;
  long cur = 0;
  bool done = false;
};

uint32_t atomic_inc_wrap(std::atomic<uint32_t>& a, uint32_t lim,
                         std::memory_order mo = std::memory_order_relaxed) {  // atomicInc semantics
  uint32_t o = a.load(std::memory_order_relaxed);
  while (!a.compare_exchange_weak(o, o >= lim ? 0u : o + 1u, mo, std::memory_order_relaxed)) {
  }
  return o;
}

// ---- one non-blocking step of a logical TB; returns true if it progressed ----
bool step_mutex(Shared& s, TB& t) {
  const bool uniq = is_umutex(s.prim);
  const int g = uniq ? t.b % s.nsm : 0;
  const int kind = (s.prim % 4 == 0) ? 0 : (s.prim % 4 == 1) ? 1 : (s.prim % 4 == 2) ? 2 : 3;  // spin, EBO, sleep, FA
  auto cs = [&] {
    if (s.mode == 2) {
      const int Gs = uniq ? s.nsm : 1, r = t.b / Gs, m = (s.G - g + Gs - 1) / Gs;
      cs_slice(s, g + (long)((r + t.j) % m) * Gs);
    } else {
      cs_chunk(s, g);
    }
  };
  if (kind <= 1) {
    if (t.skip) { --t.skip; return false; }
    auto& L = s.lock[g].v;
    uint32_t z = 0;
    if (L.load(std::memory_order_relaxed) == 0 && L.compare_exchange_strong(z, 1u, std::memory_order_acquire)) {
      cs();
      L.store(0u, std::memory_order_release);
      ++t.j;
      t.bo = 1;
      return true;
    }
    if (kind == 1) { t.skip = t.bo; t.bo = ((t.bo << 1) + 1u) & 1023u; }
    return false;
  }
  if (kind == 3) {
    if (t.phase == 0) {
      t.ticket = atomic_inc_wrap(s.ticket[g].v, uniq ? 100000000u : 1000000000u);
      t.phase = 1;
      return true;
    }
    if (s.turn[g].v.load(std::memory_order_acquire) != t.ticket) return false;
    cs();
    atomic_inc_wrap(s.turn[g].v, uniq ? 100000000u : 1000000000u, std::memory_order_release);
    ++t.j;
    t.phase = 0;
    return true;
  }
  // ring mutex
  if (t.phase == 0) {
    t.slot = atomic_inc_wrap(s.tail[g].v, s.ring_max);
    t.phase = 1;
    return true;
  }
  std::atomic<int32_t>* ring = s.ring[g].get();
  if (ring[t.slot].load(std::memory_order_acquire) != 1) return false;
  cs();
  const uint32_t next = t.slot >= s.ring_max ? 0u : t.slot + 1u;
  ring[t.slot].store(-1, std::memory_order_relaxed);
  ring[next].store(1, std::memory_order_release);
  ++t.j;
  t.phase = 0;
  return true;
}

bool step_sem(Shared& s, TB& t, unsigned maxc) {
  const bool uniq = !is_gsem(s.prim);
  const int numSM = s.G < s.nsm ? s.G : s.nsm;
  const int smID = t.b % numSM, k = (s.G + numSM - 1) / numSM, p = t.b / numSM;
  const bool writer = (p == smID % k);
  auto& st = s.sem[uniq ? smID : 0].v;
  const bool ebo = (s.prim >= 12 && s.prim <= 15) || s.prim >= 28;
  if (t.skip) { --t.skip; return false; }
  uint32_t cur = st.load(std::memory_order_relaxed);
  bool got = false;
  if (writer) {
    if ((cur & 0x7FFFFFFFu) == maxc) got = st.compare_exchange_strong(cur, 0u, std::memory_order_acquire);
    else if (!(cur & 0x80000000u)) st.fetch_or(0x80000000u, std::memory_order_relaxed);
  } else if (!(cur & 0x80000000u) && (cur & 0x7FFFFFFFu) > 1u) {
    got = st.compare_exchange_strong(cur, cur - 1u, std::memory_order_acquire);
  }
  if (!got) {
    if (ebo) {
      t.skip = t.bo;
      t.bo = (writer || uniq) ? (((t.bo << 1) + 1u) & 1023u) : (t.bo + 5u > 1023u ? 1023u : t.bo + 5u);
    }
    return false;
  }
  if (writer) {
    if (uniq) {
      long c = t.b;
      for (int i = 0; i < k; ++i) { cs_chunk(s, c); c = (c + numSM) % s.G; }
    } else {
      for (int i = 0; i < k; ++i) cs_chunk(s, i);
    }
  } else {
    cs_read(s, uniq ? t.b : p);
  }
  st.fetch_add(writer ? maxc : 1u, std::memory_order_release);
  ++t.j;
  t.bo = 1;
  return true;
}

bool step_barrier(Shared& s, TB& t) {
  const int nb = s.G < s.nsm ? s.G : s.nsm;
  const int g = t.b % nb, m = (s.G - g + nb - 1) / nb, kmax = (s.G + nb - 1) / nb;
  const bool exch = (s.prim == 1 || s.prim == 3) && kmax > 1;
  switch (t.phase) {
    case 0:
      if (s.mode == 0 || s.mode == 1) cs_chunk(s, t.cur);
      t.phase = exch ? 1 : 3;
      return true;
    case 1: {  // local arrival
      t.gen = s.lgen[g].v.load(std::memory_order_relaxed);
      if (s.lcount[g].v.fetch_add(1u, std::memory_order_acq_rel) == (uint32_t)m - 1u) {
        s.lcount[g].v.store(0u, std::memory_order_relaxed);
        s.lgen[g].v.store(t.gen + 1u, std::memory_order_release);
      }
      t.phase = 2;
      return true;
    }
    case 2:
      if (s.lgen[g].v.load(std::memory_order_acquire) == t.gen) return false;
      t.cur = (t.cur + nb) % s.G;
      cs_chunk(s, t.cur);
      t.phase = 3;
      return true;
    case 3: {  // global arrival
      t.gen = s.ggen.v.load(std::memory_order_relaxed);
      if (s.gcount.v.fetch_add(1u, std::memory_order_acq_rel) == (uint32_t)s.G - 1u) {
        s.gcount.v.store(0u, std::memory_order_relaxed);
        s.ggen.v.store(t.gen + 1u, std::memory_order_release);
      }
      t.phase = 4;
      return true;
    }
    default:
      if (s.ggen.v.load(std::memory_order_acquire) == t.gen) return false;
      t.cur = (t.cur + 1) % s.G;
      ++t.j;
      t.phase = 0;
      return true;
  }
}

}  // namespace

// Run `repeats` launches of primitive `prim` on `storage` with up to `nthreads`
// host threads (0 = hardware concurrency).  mode 0 REF, 1 INC, 2 SLICE.
// Returns 0 and the wall time in *secs; -1 on bad arguments.
extern "C" int hs_twin_run(int prim, int T, int L, int G, int iters, int repeats, int nsm, int mode,
                           uint32_t* storage, long words, int nthreads, double* secs) {
  if (T % 16 || L <= 0 || G <= 0 || nsm <= 0 || iters < 0 || !storage) return -1;
  if (mode == 2 && !(is_gmutex(prim) || is_umutex(prim))) return -1;
  Shared s;
  s.prim = prim; s.T = T; s.L = L; s.G = G; s.iters = iters; s.nsm = nsm; s.mode = mode; s.data = storage;
  const int groups = nsm > 1 ? nsm : 1;
  s.lock = std::vector<AU>(groups); s.ticket = std::vector<AU>(groups); s.turn = std::vector<AU>(groups);
  s.tail = std::vector<AU>(groups); s.sem = std::vector<AU>(groups);
  s.lcount = std::vector<AU>(groups); s.lgen = std::vector<AU>(groups);
  s.ring_max = (uint32_t)G;
  int sem_count = 0;
  switch (prim % 4) { case 0: sem_count = 1; break; case 1: sem_count = 2; break; case 2: sem_count = 10; break; default: sem_count = 120; }
  const bool sem = (prim >= 8 && prim <= 15) || (prim >= 24 && prim <= 31);
  const unsigned maxc = (unsigned)sem_count + 1u;
  for (auto& x : s.sem) x.v.store(maxc);
  if (prim == 6 || prim == 22) {
    for (int g = 0; g < (prim == 22 ? groups : 1); ++g) {
      s.ring.emplace_back(new std::atomic<int32_t>[s.ring_max + 1]);
      for (uint32_t i = 0; i <= s.ring_max; ++i) s.ring.back()[i].store(i == 0 ? 1 : -1);
    }
    while ((int)s.ring.size() < groups) s.ring.emplace_back(nullptr);
  }
  int nt = nthreads > 0 ? nthreads : (int)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > G) nt = G;
  (void)words;

  const auto t0 = std::chrono::steady_clock::now();
  for (int rep = 0; rep < repeats; ++rep) {
    std::vector<std::thread> th;
    for (int w = 0; w < nt; ++w) {
      th.emplace_back([&, w] {
        std::vector<TB> mine;
        for (int b = w; b < G; b += nt) { TB t; t.b = b; t.cur = b; mine.push_back(t); }
        size_t left = mine.size();
        while (left) {
          bool progress = false;
          for (auto& t : mine) {
            if (t.done) continue;
            bool p;
            if (is_barrier(prim)) p = step_barrier(s, t);
            else if (sem) p = step_sem(s, t, maxc);
            else p = step_mutex(s, t);
            progress |= p;
            if (t.j >= iters && (!is_barrier(prim) || t.phase == 0)) { t.done = true; --left; }
          }
          if (!progress) std::this_thread::yield();
        }
      });
    }
    for (auto& x : th) x.join();
  }
  *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return 0;
}
