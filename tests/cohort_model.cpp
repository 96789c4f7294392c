// Host model of the cohort (die-aware) protocols of include/hs/hs_device.cuh
// (cohort_queue_lock / _unlock over a test-and-set word,
// cohort_ticket_lock / cohort_ticket_unlock,
// and the semaphore's cohort writers, cohort_sem_writer_wait / _post, beside
// readers that follow sem_try_once's reader rule), run by std::threads standing
// for TBs, split over two "dies".  The encodings are the device code's; the
// ticket wraps and the pass limit are parameters, so that small values drive
// the wrap-around and global-release branches often.  Checks: mutual exclusion
// (a non-atomic counter and an owner word inside the critical section; for the
// semaphore, no reader beside a writer and at most N readers at once) and the
// final state of every lock word.  Test code only.
//
//   cohort_model tas|ticket <threads> <iters> <max_pass> <local_wrap> <global_wrap>
//   cohort_model sem <threads> <iters> <max_pass> <readers> <N> [local_wrap]
// prints "ok <counter>" or "FAIL <reason>" and exits 0 / 1.
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

using u32 = uint32_t;
std::atomic<u32> g_word{0}, g_ticket{0}, g_turn{0};
std::atomic<u32> l_ticket[2], l_turn[2];
std::atomic<int> owner{-1};
std::atomic<bool> bad{false};
unsigned long long counter = 0;  // guarded by the lock under test
u32 kMaxPass = 63, kLocalWrap = (1u << 25) - 1u, kGlobalWrap = 1000000000u;

// atom.inc: old = *p; *p = (old >= lim) ? 0 : old + 1
u32 atom_inc(std::atomic<u32>& p, u32 lim) {
  u32 old = p.load(std::memory_order_relaxed);
  while (!p.compare_exchange_weak(old, old >= lim ? 0u : old + 1u, std::memory_order_relaxed)) {
  }
  return old;
}

void critical_section(int me) {
  int expect = -1;
  if (!owner.compare_exchange_strong(expect, me)) bad = true;
  counter += 1;  // a lost update shows a broken exclusion
  expect = me;
  if (!owner.compare_exchange_strong(expect, -1)) bad = true;
}

// --- queue cohort (cohort_queue_lock / _unlock): the die's ticket queue over a
// global test-and-set word (spin and EBO mutexes)
void tas_thread(int me, int die, int iters) {
  for (int i = 0; i < iters; ++i) {
    const u32 my = atom_inc(l_ticket[die], kLocalWrap);
    u32 cur;
    while (((cur = l_turn[die].load(std::memory_order_acquire)) >> 6) != my) {
    }
    const u32 pc = cur & 63u;
    const u32 snap = l_ticket[die].load(std::memory_order_relaxed);
    if (pc == 0u) {
      for (;;) {
        u32 z = 0;
        if (g_word.load(std::memory_order_relaxed) == 0u &&
            g_word.compare_exchange_weak(z, 1u, std::memory_order_acquire))
          break;
      }
    }
    critical_section(me);
    const u32 next = (my >= kLocalWrap) ? 0u : my + 1u;
    if (snap != next && pc + 1u < kMaxPass) {
      l_turn[die].store((next << 6) | (pc + 1u), std::memory_order_release);
    } else {
      g_word.store(0u, std::memory_order_release);
      l_turn[die].store(next << 6, std::memory_order_release);
    }
  }
}

// --- ticket cohort: local turn = (ticket << 6) | passes
void ticket_thread(int me, int die, int iters) {
  for (int i = 0; i < iters; ++i) {
    const u32 my = atom_inc(l_ticket[die], kLocalWrap);
    u32 cur;
    while (((cur = l_turn[die].load(std::memory_order_acquire)) >> 6) != my) {
    }
    const u32 pc = cur & 63u;
    const u32 snap = l_ticket[die].load(std::memory_order_relaxed);
    if (pc == 0u) {
      const u32 g = atom_inc(g_ticket, kGlobalWrap);
      while (g_turn.load(std::memory_order_acquire) != g) {
      }
    }
    critical_section(me);
    const u32 next = (my >= kLocalWrap) ? 0u : my + 1u;
    if (snap != next && pc + 1u < kMaxPass) {
      l_turn[die].store((next << 6) | (pc + 1u), std::memory_order_release);
    } else {
      // red.release.inc on the global turn
      u32 t = g_turn.load(std::memory_order_relaxed);
      while (!g_turn.compare_exchange_weak(t, t >= kGlobalWrap ? 0u : t + 1u, std::memory_order_release)) {
      }
      l_turn[die].store(next << 6, std::memory_order_release);
    }
  }
}

// --- semaphore: one word, [30:0] count (starts at maxc = N + 1), [31] writer-waiting
constexpr u32 kWW = 0x80000000u, kCnt = 0x7FFFFFFFu;
std::atomic<u32> sem{0};
std::atomic<int> writers_in{0}, readers_in{0};
std::atomic<unsigned long long> reader_ops{0};
u32 kMaxc = 2;

void sem_writer_thread(int me, int die, int iters) {
  for (int i = 0; i < iters; ++i) {
    const u32 my = atom_inc(l_ticket[die], kLocalWrap);
    u32 cur;
    while (((cur = l_turn[die].load(std::memory_order_acquire)) >> 6) != my) {
    }
    const u32 pc = cur & 63u;
    const u32 snap = l_ticket[die].load(std::memory_order_relaxed);
    if (pc == 0u) {  // take the semaphore by the writer rule
      for (;;) {
        u32 s = sem.load(std::memory_order_relaxed);
        if ((s & kCnt) == kMaxc) {
          if (sem.compare_exchange_strong(s, 0u, std::memory_order_acquire)) break;
          continue;
        }
        if (!(s & kWW)) sem.fetch_or(kWW, std::memory_order_relaxed);
      }
    }
    if (writers_in.fetch_add(1) != 0 || readers_in.load() != 0) bad = true;
    critical_section(me);
    if (readers_in.load() != 0 || writers_in.fetch_sub(1) != 1) bad = true;
    const u32 next = (my >= kLocalWrap) ? 0u : my + 1u;
    if (snap != next && pc + 1u < kMaxPass) {
      l_turn[die].store((next << 6) | (pc + 1u), std::memory_order_release);
    } else {
      sem.fetch_add(kMaxc, std::memory_order_release);
      l_turn[die].store(next << 6, std::memory_order_release);
    }
  }
}

void sem_reader_thread(int, int, int iters) {
  for (int i = 0; i < iters; ++i) {
    for (;;) {
      u32 s = sem.load(std::memory_order_relaxed);
      if (!(s & kWW) && (s & kCnt) > 1u && sem.compare_exchange_strong(s, s - 1u, std::memory_order_acquire)) break;
    }
    const int r = readers_in.fetch_add(1);
    if (r >= (int)kMaxc - 1 || writers_in.load() != 0) bad = true;
    reader_ops.fetch_add(1);
    readers_in.fetch_sub(1);
    sem.fetch_add(1u, std::memory_order_release);
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 7 && !(argc == 8 && std::strcmp(argv[1], "sem") == 0)) {
    std::fprintf(stderr, "usage: cohort_model tas|ticket threads iters max_pass local_wrap global_wrap\n"
                         "       cohort_model sem threads iters max_pass readers N\n");
    return 2;
  }
  const bool tas = std::strcmp(argv[1], "tas") == 0;
  const int n = std::atoi(argv[2]), iters = std::atoi(argv[3]);
  if (std::strcmp(argv[1], "sem") == 0) {
    kMaxPass = (u32)std::atoi(argv[4]);
    if (argc > 7) kLocalWrap = (u32)std::strtoul(argv[7], nullptr, 10);
    const int readers = std::atoi(argv[5]);
    kMaxc = (u32)std::atoi(argv[6]) + 1u;
    sem = kMaxc;
    for (int d = 0; d < 2; ++d) {
      l_ticket[d] = 0;
      l_turn[d] = 0;
    }
    std::vector<std::thread> ts;
    for (int t = 0; t < n; ++t) ts.emplace_back(sem_writer_thread, t, t % 2, iters);
    for (int t = 0; t < readers; ++t) ts.emplace_back(sem_reader_thread, n + t, 0, iters);
    for (auto& t : ts) t.join();
    const unsigned long long want = (unsigned long long)n * (unsigned long long)iters;
    if (bad.load()) return std::puts("FAIL a reader beside a writer, two writers, or too many readers"), 1;
    if (counter != want) return std::printf("FAIL counter %llu of %llu\n", counter, want), 1;
    if (reader_ops.load() != (unsigned long long)readers * iters) return std::puts("FAIL reader count"), 1;
    if (sem.load() != kMaxc) return std::printf("FAIL semaphore word %#x at the end\n", sem.load()), 1;
    for (int d = 0; d < 2; ++d)
      if ((l_turn[d].load() >> 6) != l_ticket[d].load() || (l_turn[d].load() & 63u) != 0u)
        return std::printf("FAIL die %d ticket %u turn %#x at the end\n", d, l_ticket[d].load(), l_turn[d].load()), 1;
    std::printf("ok %llu\n", counter);
    return 0;
  }
  kMaxPass = (u32)std::atoi(argv[4]);
  kLocalWrap = (u32)std::strtoul(argv[5], nullptr, 10);
  kGlobalWrap = (u32)std::strtoul(argv[6], nullptr, 10);
  for (int d = 0; d < 2; ++d) {
    l_ticket[d] = 0;
    l_turn[d] = 0;
  }
  std::vector<std::thread> ts;
  for (int t = 0; t < n; ++t) ts.emplace_back(tas ? tas_thread : ticket_thread, t, t % 2, iters);
  for (auto& t : ts) t.join();
  const unsigned long long want = (unsigned long long)n * (unsigned long long)iters;
  if (bad.load()) return std::puts("FAIL two holders at once"), 1;
  if (counter != want) return std::printf("FAIL counter %llu of %llu\n", counter, want), 1;
  if (tas && g_word.load() != 0u) return std::puts("FAIL global word held at the end"), 1;
  if (!tas && g_ticket.load() != g_turn.load()) return std::puts("FAIL global ticket and turn differ"), 1;
  {
    for (int d = 0; d < 2; ++d)
      if ((l_turn[d].load() >> 6) != l_ticket[d].load() || (l_turn[d].load() & 63u) != 0u)
        return std::printf("FAIL die %d ticket %u turn %#x at the end\n", d, l_ticket[d].load(), l_turn[d].load()), 1;
  }
  std::printf("ok %llu\n", counter);
  return 0;
}
