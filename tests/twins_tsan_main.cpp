// Driver for the thread-sanitizer run of the host-thread twins (oracle/twins.cpp):
// every SyncPrims family at a small size on 4 host threads, in INC mode, each
// final storage compared with the oracle golden (oracle/golden.c).  Built with
// -fsanitize=thread by tests/test_tsan_cpu.py; a data race makes the sanitizer
// fail the process.  Test code only.
#include <cstdint>
#include <cstdio>
#include <vector>

extern "C" int hs_twin_run(int prim, int T, int L, int G, int iters, int repeats, int nsm, int mode,
                           uint32_t* storage, long words, int nthreads, double* secs);
extern "C" int hs_oracle_golden(int syncPrim, int T, int L, int numTBs, int iters, int repeats, int NUM_SM, int inc,
                                uint32_t* storage, long numStorageLocs);
extern "C" long hs_oracle_storage_words(int prim, int T, int L, int numTBs, int NUM_SM);

int main() {
  // spin/EBO/ring/ticket mutexes, semaphores of 1 and 10 (global and per-SM),
  // both tree barriers with and without local exchange
  const int prims[] = {4, 5, 6, 7, 8, 10, 12, 20, 21, 22, 23, 24, 26, 0, 1, 2, 3};
  const int T = 32, L = 3, G = 12, iters = 40, nsm = 4;
  int failed = 0;
  for (int p : prims) {
    const long n = hs_oracle_storage_words(p, T, L, G, nsm);
    std::vector<uint32_t> a(n), b(n);
    for (long i = 0; i < n; ++i) a[i] = b[i] = (uint32_t)(i * 2654435761u);
    double secs = 0;
    if (hs_twin_run(p, T, L, G, iters, 2, nsm, 1, a.data(), n, 4, &secs) != 0 ||
        hs_oracle_golden(p, T, L, G, iters, 2, nsm, 1, b.data(), n) != 0 || a != b) {
      std::printf("FAIL prim %d\n", p);
      failed = 1;
    }
  }
  if (!failed) std::puts("ok");
  return failed;
}
