// relaxed_cli.cpp -- drop-ins for the reference's relaxed-atomics and UTS
// programs: refCounter, splitCounter, seqlocks, flags (cuda/relaxedAtomics/uvm/*)
// and uts (cuda/uts/uvm/uts.cu).  One executable; the program is chosen by the
// name it is invoked under (the build installs it under each name).  Same
// arguments, output lines and checks as the reference's mains, through
// libhsgb300 (include/hs/hs.h).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/hs/hs.h"

static int prog_refcounter(int argc, char** argv) {  // refCounter.cu:5-155
  if (argc != 5) {
    std::fprintf(stderr, "./refCounter <numSharersPerGroup> <numTBs> <tbSize> <numRepeats>\n");
    std::fprintf(stderr, "where:\n");
    std::fprintf(stderr, "\t<numSharersPerGroup>: number of thread blocks sharing a counter\n");
    std::fprintf(stderr, "\t<numTBs>: number of thread blocks to launch\n");
    std::fprintf(stderr, "\t<tbSize>: number of threads in a thread block\n");
    std::fprintf(stderr, "\t<numRepeats>: how many times to have the 'main' TB read its data before setting stop\n");
    std::exit(-1);
  }
  const int sharers = std::atoi(argv[1]), numTBs = std::atoi(argv[2]), tbSize = std::atoi(argv[3]),
            reps = std::atoi(argv[4]);
  if (sharers <= 0 || sharers > numTBs || tbSize <= 0 || tbSize > 256) {
    std::fprintf(stderr, "ERROR: need 0 < numSharersPerGroup <= numTBs and tbSize <= 256\n");
    std::exit(-1);
  }
  const unsigned numThrs = (unsigned)tbSize * numTBs, numCounters = numThrs / sharers,
                 groups = numTBs / sharers, perGroup = numCounters / groups;
  std::fprintf(stdout, "# Thr: %d, # TB: %d, # Counters: %d, # Sharers: %d, # Groups: %d, # Counters/Group: %d\n",
               numThrs, numTBs, numCounters, sharers, groups, perGroup);
  std::fprintf(stdout, "Initializing data...\n...allocating memory.\n...initializing memory.\n");
  std::vector<unsigned> c0(numCounters, 0), c1(numCounters, 0), d0(numThrs, 0), d1(numThrs, 0);
  std::fprintf(stdout, "Launching kernel - %d runs with %d TBs and %d threads/TB\n", 1, numTBs, tbSize);
  hs_relaxed_result r;
  if (hs_refcounter(sharers, numTBs, tbSize, reps, c0.data(), c1.data(), d0.data(), d1.data(), &r)) {
    std::fprintf(stderr, "ERROR: %s\n", hs_relaxed_last_error());
    std::exit(-1);
  }
  bool pass = true;
  for (unsigned i = 0; i < numCounters; ++i)
    if (c0[i]) { std::fprintf(stderr, "ERROR: h_counters0[%d]: %d\n", i, c0[i]); pass = false; }
  for (unsigned i = 0; i < numCounters; ++i)
    if (c1[i]) { std::fprintf(stderr, "ERROR: h_counters1[%d]: %d\n", i, c1[i]); pass = false; }
  bool any0 = false, any1 = false;
  for (unsigned i = 0; i < numThrs; ++i) { any0 |= d0[i] != 0; any1 |= d1[i] != 0; }
  if (!any0) { std::fprintf(stderr, "ERROR: none of d_del0 array locations set\n"); pass = false; }
  if (!any1) { std::fprintf(stderr, "ERROR: none of d_del1 array locations set\n"); pass = false; }
  std::fprintf(stderr, pass ? "TEST PASSED!\n" : "TEST FAILED!\n");
  return 0;
}

static int prog_splitcounter(int argc, char** argv) {  // splitCounter.cu:5-98
  if (argc != 3) {
    std::fprintf(stderr, "./splitCounter <numTBs> <tbSize>\n");
    std::fprintf(stderr, "where:\n");
    std::fprintf(stderr, "\t<numTBs>: number of thread blocks to launch\n");
    std::fprintf(stderr, "\t<tbSize>: number of threads in a thread block\n");
    std::exit(-1);
  }
  const int numTBs = std::atoi(argv[1]), tbSize = std::atoi(argv[2]);
  const unsigned numThrs = (unsigned)numTBs * tbSize;
  std::fprintf(stdout, "Initializing data...\n...allocating memory.\n...initializing memory.\n");
  std::vector<unsigned> counters(numThrs / 2, 0), out(numThrs, 0);
  std::fprintf(stdout, "Launching kernel - %d runs with %d TBs and %d threads/TB\n", 1, numTBs, tbSize);
  hs_relaxed_result r;
  if (hs_splitcounter(numTBs, tbSize, counters.data(), out.data(), &r)) {
    std::fprintf(stderr, "ERROR: %s\n", hs_relaxed_last_error());
    std::exit(-1);
  }
  bool pass = true;
  for (unsigned i = 0; i < numThrs / 2; ++i)
    if (counters[i] != 1u) { std::fprintf(stderr, "ERROR: h_counters[%d] != %d, = %u\n", i, 1, counters[i]); pass = false; }
  // Readers' sums are approximate by design: each lies between 0 and the number
  // of counters its half-warp read (the reference checks them against 0, which
  // assumes every reader ran before every writer).
  const unsigned perHalfWarp = (numThrs / 2) / (unsigned)(tbSize / 2) * 16u;
  for (unsigned i = 0; i < numThrs; ++i)
    if (out[i] > perHalfWarp) { std::fprintf(stderr, "\tThread %d: %u, > %u\n", i, out[i], perHalfWarp); pass = false; }
  std::fprintf(stdout, pass ? "PASSED\n" : "FAILED\n");
  return 0;
}

static int prog_seqlocks(int argc, char** argv) {  // seqlocks.cu:5-111
  if (argc != 5) {
    std::fprintf(stderr, "./seqlocks <numTBs> <tbSize> <groupSize_seqlock> <pageAlign> <useTFs>\n");
    std::fprintf(stderr, "where:\n");
    std::fprintf(stderr, "\t<numTBs>: number of thread blocks to launch\n");
    std::fprintf(stderr, "\t<tbSize>: number of threads in a thread block\n");
    std::fprintf(stderr, "\t<groupSize_seqlock>: how many TBs share a seqlock\n");
    std::fprintf(stderr, "\t<useTFs>: if 1, use weaker version with more fully relaxed atomics and TFs to enforce ordering\n");
    std::exit(-1);
  }
  const int numTBs = std::atoi(argv[1]), tbSize = std::atoi(argv[2]), group = std::atoi(argv[3]),
            useTFs = std::atoi(argv[4]) == 1;
  const int numThrs = numTBs * tbSize, numSeq = numTBs / group;
  std::fprintf(stdout, "Initializing data...\n...allocating memory.\n...initializing memory.\n");
  std::vector<unsigned> seq((size_t)(numSeq > 0 ? numSeq : 1), 0);
  std::vector<int> d0(32, 0), d1(32, 0), out((size_t)numThrs, -1);
  std::fprintf(stdout, "Launching kernel - %d runs with %d TBs and %d threads/TB\n", 1, numTBs, tbSize);
  hs_relaxed_result r;
  if (hs_seqlocks(numTBs, tbSize, group, useTFs, seq.data(), d0.data(), d1.data(), out.data(), 0, &r)) {
    std::fprintf(stderr, "ERROR: %s\n", hs_relaxed_last_error());
    std::exit(-1);
  }
  for (int i = 0; i < numSeq; ++i) {
    if (seq[i] % 2 != 0) std::fprintf(stderr, "ERROR: seqlock should be a multiple of 2!\n");
    // exact count: every writer TB on this seqlock advances it by 2 per iteration (NUM_ITERS = 10)
    unsigned writers = 0;
    for (int b = 0; b < numTBs; ++b)
      if (b % 16 == 0 && b % group == i) ++writers;
    if (seq[i] != 2u * 10u * writers)
      std::fprintf(stderr, "ERROR: seqlock[%d] = %u, expected %u\n", i, seq[i], 2u * 10u * writers);
  }
  return 0;
}

static int prog_flags(int argc, char** argv) {  // flags.cu:19-176
  if (argc != 8) {
    std::fprintf(stderr, "./flags <numTBs> <tbSize> <numAccsPerThr> <numRepeats> <cutoffVal> <numIters> <pageAlign>\n");
    std::fprintf(stderr, "where:\n");
    std::fprintf(stderr, "\t<numTBs>: number of thread blocks to launch\n");
    std::fprintf(stderr, "\t<tbSize>: number of threads in a thread block\n");
    std::fprintf(stderr, "\t<numAccsPerThr>: number of data accesses each thread does in the kernel\n");
    std::fprintf(stderr, "\t<numRepeats>: how many times to have the 'main' TB read its data before setting stop\n");
    std::fprintf(stderr, "\t<cutoffVal>: the cutoff value for comparing the random values to (all > will be accepted)\n");
    std::fprintf(stderr, "\t<numIters>: number of iterations for worker TB's loop\n");
    std::fprintf(stderr, "\t<pageAlign>: if 1 the arrays will be page aligned, else arrays will be unaligned.\n");
    std::exit(-1);
  }
  const int numTBs = std::atoi(argv[1]), tbSize = std::atoi(argv[2]), accs = std::atoi(argv[3]),
            reps = std::atoi(argv[4]), iters = std::atoi(argv[6]);
  const float cutoff = (float)std::atof(argv[5]);
  const unsigned numThrs = (unsigned)tbSize * numTBs, numAccs = (unsigned)iters * numTBs;
  if (numAccs > (64u * 1024u) * 10u || numAccs == 0) { std::fprintf(stderr, "ERROR: numIters*numTBs out of range\n"); std::exit(-1); }
  std::fprintf(stdout, "Initializing data...\n...allocating memory.\n");
  srand(2018);  // flags.cu:92
  std::fprintf(stdout, "...initializing memory.\n");
  std::vector<unsigned> out(numThrs, 0);
  std::vector<float> rnd(numAccs);
  for (unsigned i = 0; i < numAccs; ++i) rnd[i] = (float)rand() / (float)((unsigned)-1);
  std::fprintf(stdout, "Launching kernel - %d runs with %d TBs and %d threads/TB, %u iterations of worker TB loop\n",
               1, numTBs, tbSize, iters);
  hs_relaxed_result r;
  unsigned dirty = 0;
  if (hs_flags(numTBs, tbSize, accs, reps, cutoff, iters, rnd.data(), (int)numAccs, out.data(), &dirty, 0, &r)) {
    std::fprintf(stderr, "ERROR: %s\n", hs_relaxed_last_error());
    std::exit(-1);
  }
  std::fprintf(stdout, "isDirty - %d\n", dirty);
  bool pass = true;
  const unsigned expected = (unsigned)reps * accs * accs;
  for (unsigned i = 0; i < numThrs; ++i) {
    const bool mainSlice = i >= (unsigned)tbSize * (numTBs - 1);
    const unsigned want = (dirty != 0 && mainSlice) ? expected : 0u;
    if (out[i] != want) {
      std::fprintf(stderr, "ERROR: outArr[%d] != %u, = %u\n", i, want, out[i]);
      pass = false;
    }
  }
  std::fprintf(stdout, "Test %s!\n", pass ? "PASSED" : "FAILED");
  return 0;
}

static int prog_uts(int argc, char** argv) {  // uts.cu:550-587, callGPU 244-455
  if (argc != 6) {
    std::fprintf(stderr, "Invalid arguments passed in, expected:\n");
    std::fprintf(stderr, "./uts <numThreads> <numElements> <fertility> <local_stack_size> <N_active_blocks>\n");
    std::exit(-1);
  }
  const int threads = std::atoi(argv[1]), N = std::atoi(argv[2]), fert = std::atoi(argv[3]),
            blocks = std::atoi(argv[5]);
  std::printf("# CPU threads that do work:%d\n", threads);
  const int num_nodes = N + ((N % 2) ? 0 : 1);
  std::printf("Running with N_elements=%d N_active_blocks=%d\n", num_nodes, blocks);
  std::vector<hs_uts_node> tree((size_t)num_nodes);
  unsigned leaves_g = 0, sum_g = 0, restarts = 0;
  if (hs_uts_tree_build(num_nodes, fert, 200, tree.data(), &leaves_g, &sum_g, &restarts)) {
    std::fprintf(stderr, "Error: %s\n", hs_uts_last_error());
    std::exit(-1);
  }
  const int cores_used = blocks > 15 ? 15 : blocks;  // NUM_PHYSICAL_CORES, uts.cu:19, 258
  std::vector<int> frontier((size_t)cores_used * 16 + 2);
  int nf = 0;
  unsigned host_processed = 0;
  if (hs_uts_frontier(tree.data(), num_nodes, cores_used, frontier.data(), &nf, &host_processed)) {
    std::printf("Error: %s\n", hs_uts_last_error());
    std::exit(-1);
  }
  std::printf("done processing nodes\n");
  std::printf("done initing work stack\n");
  std::printf("Launch uts kernel...\n");
  hs_uts_result res;
  if (hs_uts_run(tree.data(), num_nodes, frontier.data(), nf, host_processed, blocks, 128, 0, &res)) {
    std::fprintf(stderr, "ERROR %s\n", hs_uts_last_error());
    std::exit(-1);
  }
  std::printf("Kernel completed.\n");
  std::printf("Created uts tree size %d with %d leaves, %d leaf sum, %d fertility, and %d restarts:\n", num_nodes,
              leaves_g, sum_g, fert, restarts);
  std::printf("kernel found %d leaf nodes\n", res.leaves_found);
  std::printf("kernel found %d leaf sum\n", res.leaf_sum);
  std::printf("nodes_processed:%d\n", res.nodes_processed);
  if (res.leaves_found != leaves_g) { std::printf("Error: leaves_found %d != %d\n", res.leaves_found, leaves_g); std::exit(-1); }
  if (res.leaf_sum != sum_g) { std::printf("Error: leaf_sum %d != %d\n", res.leaf_sum, sum_g); std::exit(-1); }
  if (res.nodes_processed != (unsigned)num_nodes) {
    std::printf("Error: nodes_processed %d != %d\n", res.nodes_processed, num_nodes);
    std::exit(-1);
  }
  std::printf("SUCCESS!\n");
  return 0;
}

int main(int argc, char** argv) {
  std::string name = argv[0];
  const size_t slash = name.find_last_of('/');
  if (slash != std::string::npos) name = name.substr(slash + 1);
  if (name == "refCounter") return prog_refcounter(argc, argv);
  if (name == "splitCounter") return prog_splitcounter(argc, argv);
  if (name == "seqlocks") return prog_seqlocks(argc, argv);
  if (name == "flags") return prog_flags(argc, argv);
  if (name == "uts") return prog_uts(argc, argv);
  std::fprintf(stderr, "invoke as refCounter, splitCounter, seqlocks, flags or uts\n");
  return 2;
}
