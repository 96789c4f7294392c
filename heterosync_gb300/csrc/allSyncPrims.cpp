// allSyncPrims.cpp -- drop-in for the reference's allSyncPrims-1kernel binary.
//
//   allSyncPrims-1kernel <syncPrim> <numLdSt> <numTBs> <numCSIters>
//
// Same arguments, primitive names, stdout lines and exit codes as heterosync
// cuda/syncPrims/uvm/main.cu:1130-1821 (usage text 1132-1172, sizes 1176-1195,
// storage sizing 1283-1308, labels 1352-1451, timing line 1618, golden
// comparison 1790-1808).  The work runs through libhsgb300 (include/hs/hs.h).
//
// Extensions (environment variables; defaults reproduce the reference):
//   HS_THREADS       threads per TB (reference: 32)
//   HS_MODE          ref | inc      (data mode, see hs.h)
//   HS_NSM           NUM_SM used in the index math (default: device SM count)
//   HS_TIMEOUT_MS    per-wait device timeout
//   HS_NO_SYNC_EACH  1: do not host-synchronise after each of the 10 launches
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "../../include/hs/hs.h"

static const int NUM_REPEATS = 10;  // main.cu:21

static void usage() {
  std::fprintf(stderr, "./allSyncPrims-1kernel <syncPrim> <numLdSt> <numTBs> <numCSIters>\n");
  std::fprintf(stderr, "where:\n");
  std::fprintf(stderr,
               "\t<syncPrim>: a string that represents which synchronization primitive to run.\n"
               "\t\tatomicTreeBarrUniq - Atomic Tree Barrier\n"
               "\t\tatomicTreeBarrUniqLocalExch - Atomic Tree Barrier with local exchange\n"
               "\t\tlfTreeBarrUniq - Lock-Free Tree Barrier\n"
               "\t\tlfTreeBarrUniqLocalExch - Lock-Free Tree Barrier with local exchange\n"
               "\t\tspinMutex - Spin Lock Mutex\n"
               "\t\tspinMutexEBO - Spin Lock Mutex with Backoff\n"
               "\t\tsleepMutex - Sleep Mutex\n"
               "\t\tfaMutex - Fetch-and-Add Mutex\n"
               "\t\tspinSem1 - Spin Semaphore (Max: 1)\n"
               "\t\tspinSem2 - Spin Semaphore (Max: 2)\n"
               "\t\tspinSem10 - Spin Semaphore (Max: 10)\n"
               "\t\tspinSem120 - Spin Semaphore (Max: 120)\n"
               "\t\tspinSemEBO1 - Spin Semaphore with Backoff (Max: 1)\n"
               "\t\tspinSemEBO2 - Spin Semaphore with Backoff (Max: 2)\n"
               "\t\tspinSemEBO10 - Spin Semaphore with Backoff (Max: 10)\n"
               "\t\tspinSemEBO120 - Spin Semaphore with Backoff (Max: 120)\n"
               "\t\tspinMutexUniq - Spin Lock Mutex -- accesses to unique locations per TB\n"
               "\t\tspinMutexEBOUniq - Spin Lock Mutex with Backoff -- accesses to unique locations per TB\n"
               "\t\tsleepMutexUniq - Sleep Mutex -- accesses to unique locations per TB\n"
               "\t\tfaMutexUniq - Fetch-and-Add Mutex -- accesses to unique locations per TB\n"
               "\t\tspinSemUniq1 - Spin Semaphore (Max: 1) -- accesses to unique locations per TB\n"
               "\t\tspinSemUniq2 - Spin Semaphore (Max: 2) -- accesses to unique locations per TB\n"
               "\t\tspinSemUniq10 - Spin Semaphore (Max: 10) -- accesses to unique locations per TB\n"
               "\t\tspinSemUniq120 - Spin Semaphore (Max: 120) -- accesses to unique locations per TB\n"
               "\t\tspinSemEBOUniq1 - Spin Semaphore with Backoff (Max: 1) -- accesses to unique locations per TB\n"
               "\t\tspinSemEBOUniq2 - Spin Semaphore with Backoff (Max: 2) -- accesses to unique locations per TB\n"
               "\t\tspinSemEBOUniq10 - Spin Semaphore with Backoff (Max: 10) -- accesses to unique locations per TB\n"
               "\t\tspinSemEBOUniq120 - Spin Semaphore with Backoff (Max: 120) -- accesses to unique locations per TB\n"
               "\tAlso accepted (the HIP build's extra primitives):\n"
               "\t\tPRspinSem{1,2,10,120}, PRspinSemEBO{1,2,10,120} - Priority Spin Semaphores\n"
               "\t\tatomicTreeBarrUniq[LocalExch]{SRB,NaiveSRB,NaiveAllSRB} - Sense Reversing Barriers\n");
  std::fprintf(stderr, "\t<numLdSt>: the # of LDs and STs to do for each thread in the critical section.\n");
  std::fprintf(stderr, "\t<numTBs>: the # of TBs to execute (want to be divisible by the number of SMs).\n");
  std::fprintf(stderr, "\t<numCSIters>: number of iterations of the critical section.\n");
}

static int env_int(const char* k, int dflt) {
  const char* v = std::getenv(k);
  return (v && *v) ? std::atoi(v) : dflt;
}

int main(int argc, char** argv) {
  if (argc != 5) {
    usage();
    std::exit(-1);
  }
  int nsm_dev = 0, ccM = 0, ccm = 0, max_tpb = 0;
  int s = hs_device_info(0, &nsm_dev, &ccM, &ccm, &max_tpb);
  if (s == HS_ENODEV) {
    std::fprintf(stderr, "There is no device supporting CUDA\n");
    std::exit(-1);
  }
  if (s) {
    std::fprintf(stderr, "ERROR Begin - %s\n", hs_last_error());
    std::exit(-1);
  }
  std::fprintf(stdout, "GPU Compute Capability: %d.%d\n", ccM, ccm);

  const int T = env_int("HS_THREADS", 32);
  const int NUM_SM = env_int("HS_NSM", nsm_dev);
  const int maxTBPerSM = max_tpb / T;
  const int MAX_BLOCKS = maxTBPerSM * NUM_SM;
  std::fprintf(stdout, "# SM: %d, Max Thrs/TB: %d, Max TB/SM: %d, Max # TB: %d\n", NUM_SM, max_tpb, maxTBPerSM,
               MAX_BLOCKS);

  const char* name = argv[1];
  const int NUM_LDST = std::atoi(argv[2]);
  const int numTBs = std::atoi(argv[3]);
  const int NUM_ITERS = std::atoi(argv[4]);
  if (numTBs > MAX_BLOCKS) {
    std::fprintf(stderr, "ERROR: numTBs (%d) > Max # TB (%d)\n", numTBs, MAX_BLOCKS);
    std::exit(-1);
  }
  const int prim = hs_prim_id(name);
  if (prim < 0) {
    std::fprintf(stderr, "ERROR: Unknown synchronization primitive: %s\n", name);
    std::exit(-1);
  }

  hs_run_config cfg;
  hs_run_config_default(&cfg);
  cfg.prim = prim;
  cfg.num_ldst = NUM_LDST;
  cfg.num_tbs = numTBs;
  cfg.num_iters = NUM_ITERS;
  cfg.threads = T;
  cfg.repeats = NUM_REPEATS;
  cfg.nsm = NUM_SM;
  const char* mode = std::getenv("HS_MODE");
  cfg.mode = (mode && std::strcmp(mode, "inc") == 0) ? HS_MODE_INC : HS_MODE_REF;
  if (env_int("HS_TIMEOUT_MS", 0) > 0) cfg.timeout_ns = (unsigned long long)env_int("HS_TIMEOUT_MS", 0) * 1000000ull;
  cfg.flags = env_int("HS_NO_SYNC_EACH", 0) ? 0 : HS_RUN_SYNC_EACH;

  size_t words = 0;
  if ((s = hs_storage_words(&cfg, NUM_SM, &words)) != HS_OK) {
    std::fprintf(stderr, "ERROR: %s\n", hs_last_error());
    std::exit(-1);
  }
  const int numUniqLocsAccPerTB = T * (NUM_LDST + 1);
  const int numLocsMult = (int)(words / (size_t)numUniqLocsAccPerTB);

  hs_ctx* ctx = nullptr;
  if ((s = hs_ctx_create(0, &ctx)) != HS_OK) {
    std::fprintf(stderr, "ERROR After cudaLocksInit - %s\n", hs_last_error());
    std::exit(-1);
  }
  // the reference's lock-data initialisation (cudaLocksInit(MAX_BLOCKS, 8 * NUM_SM,
  // 24 * NUM_SM, ...), main.cu:1277-1279), whose timed ring copy is line "H->D 1"
  // (with few SMs the reference's stride can round to no room for the ring:
  // the lock data then gets the next size that leaves room)
  int lock_blocks = MAX_BLOCKS;
  while ((lock_blocks + NUM_SM) / 16 * 16 <= lock_blocks) ++lock_blocks;
  if ((s = cudaLocksInit(lock_blocks, 8 * NUM_SM, 24 * NUM_SM, false, NUM_SM)) != 0) {
    std::fprintf(stderr, "ERROR After cudaLocksInit - error %d\n", s);
    std::exit(-1);
  }
  std::fprintf(stdout, "\tmemcpy H->D 1 elapsed time: %f ms\n", hs_locks_init_copy_ms());
  std::fprintf(stdout, "# TBs: %d, # Ld/St: %d, # Locs Mult: %d, # Uniq Locs/TB: %d, # Storage Locs: %d\n", numTBs,
               NUM_LDST, numLocsMult, numUniqLocsAccPerTB, (int)words);

  // storage[i] = i (main.cu:1315), as float in reference mode, as uint32 in inc mode
  std::vector<uint32_t> storage(words), init(words), golden(words);
  for (size_t i = 0; i < words; ++i) {
    if (cfg.mode == HS_MODE_REF) {
      float f = (float)i;
      std::memcpy(&init[i], &f, 4);
    } else {
      init[i] = (uint32_t)i;
    }
  }
  storage = init;

  char label[128];
  hs_prim_label(prim, NUM_ITERS, label, sizeof(label));
  hs_run_result res;
  s = hs_run(ctx, &cfg, storage.data(), 0, nullptr, &res);
  std::fprintf(stdout, "\tmemcpy H->D 2 elapsed time: %f ms\n", res.h2d_ms);
  std::fprintf(stdout, "%s\n", label);
  std::fflush(stdout);
  if (s != HS_OK) {
    std::fprintf(stderr, "ERROR cudaDeviceSynchronize (%s) - %s: %s\n", name, hs_status_string(s), hs_last_error());
    std::exit(-1);
  }
  std::printf("elapsed time: %f ms, average: %f ms\n", res.elapsed_ms, res.avg_ms);
  std::fflush(stdout);
  std::fprintf(stdout, "\tmemcpy D->H elapsed time: %f ms\n", res.d2h_ms);
  std::fflush(stdout);

  hs_expected_storage(&cfg, NUM_SM, init.data(), golden.data(), words);
  std::fprintf(stdout, "Comparing GPU results to golden results:\n");
  unsigned numErrors = 0;
  for (size_t i = 0; i < words; ++i) {
    if (storage[i] != golden[i]) {
      if (cfg.mode == HS_MODE_REF) {
        float a, b;
        std::memcpy(&a, &storage[i], 4);
        std::memcpy(&b, &golden[i], 4);
        std::fprintf(stderr, "\tERROR: storage[%d] = %f, golden[%d] = %f\n", (int)i, a, (int)i, b);
      } else {
        std::fprintf(stderr, "\tERROR: storage[%d] = %u, golden[%d] = %u\n", (int)i, storage[i], (int)i, golden[i]);
      }
      ++numErrors;
    }
  }
  hs_ctx_destroy(ctx);
  cudaLocksDestroy();
  if (numErrors > 0) {
    std::fprintf(stderr, "ERROR: %s has %u output errors\n", name, numErrors);
    std::exit(-1);
  }
  std::fprintf(stdout, "PASSED!\n");
  return 0;
}
