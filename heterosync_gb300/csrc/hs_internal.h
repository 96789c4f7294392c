// hs_internal.h -- descriptors shared by the host runtime and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>

namespace hs {

// Reference syncPrim ids (cuda/syncPrims/uvm/main.cu:1224-1256).
enum Prim : int {
  P_ATOMIC_TREE = 0, P_ATOMIC_TREE_EXCH = 1, P_LF_TREE = 2, P_LF_TREE_EXCH = 3,
  P_SPIN_MUTEX = 4, P_EBO_MUTEX = 5, P_SLEEP_MUTEX = 6, P_FA_MUTEX = 7,
  P_SPIN_SEM1 = 8, P_SPIN_SEM2 = 9, P_SPIN_SEM10 = 10, P_SPIN_SEM120 = 11,
  P_EBO_SEM1 = 12, P_EBO_SEM2 = 13, P_EBO_SEM10 = 14, P_EBO_SEM120 = 15,
  P_SPIN_MUTEX_UNIQ = 20, P_EBO_MUTEX_UNIQ = 21, P_SLEEP_MUTEX_UNIQ = 22, P_FA_MUTEX_UNIQ = 23,
  P_SPIN_SEM_UNIQ1 = 24, P_SPIN_SEM_UNIQ2 = 25, P_SPIN_SEM_UNIQ10 = 26, P_SPIN_SEM_UNIQ120 = 27,
  P_EBO_SEM_UNIQ1 = 28, P_EBO_SEM_UNIQ2 = 29, P_EBO_SEM_UNIQ10 = 30, P_EBO_SEM_UNIQ120 = 31,
};

// Data modes.
//  REF   : the reference's critical section, a one-line copy shift of each
//          half-warp region (main.cu:60-72), on 32-bit words;
//  INC   : same locations, but every written word is incremented (exact count oracle);
//  SLICE : uint32[numTBs*numLdSt]; TB b at iteration j adds 1 to slice (b+j) mod numTBs
//          (per group for the Uniq mutexes).
enum Mode : int { M_REF = 0, M_INC = 1, M_SLICE = 2 };

// Mutex kinds.
enum MutexKind : int { MK_SPIN = 0, MK_EBO = 1, MK_SLEEP = 2, MK_FA = 3 };

constexpr int kRingStride = 8;  // ring slot stride in words (32-byte sectors)

// Everything one launch of one primitive instance needs, passed by value.
struct RunDesc {
  unsigned* data;       // shared data (storage), 32-bit words
  unsigned* locks;      // lock-state lines (kLineWords words each)
  unsigned* ring;       // ring-mutex slots, (ring_max+1)*kRingStride words per group
  unsigned* status;     // 2 words: error bits, first failing site
  unsigned* sink;       // one word per TB for semaphore readers' loads
  int prim, mode, T, L, num_tbs, iters, nsm;
  unsigned sem_max;     // semaphore count + 1
  unsigned bo_min, bo_max, bo_unit;
  unsigned ring_max;    // highest ring slot index (slots 0..ring_max)
  unsigned long long timeout_ns;
  int skip_tb;          // logical TB that never arrives at a barrier (-1: none)
  int cluster;          // CTAs per cluster for barrier kernels (1: no clusters)
  int grp;              // tree barriers: logical TBs one CTA hosts (0 or 1: one CTA per TB)
  unsigned tile_cap;    // group-CTA bulk-copy barrier: bytes per staging buffer
  // line offsets inside `locks`
  int l_glob;           // global barrier: +0 count, +1 gen, +2 go
  int l_gflag;          // global barrier flags (dense, one word per group)
  int l_grp;            // per-group lines: 4 per group
  int l_lflag;          // per-group member flags (dense), lflag_lines per group
  int lflag_lines;
  int variant;          // HIP-extension variant of the primitive (PrimVariant)
  // Cohort (die-aware) global mutexes: cohort != 0 enables them.  die_map[smid]
  // is the SM's die (0/1); coh[3 * die + i] are three lock lines homed on that die.
  int cohort;
  const unsigned char* die_map;
  unsigned* coh[6];
};

// Variants the HIP build of the reference adds to the CUDA primitives
// (hip/syncPrims/uvm/main.hip.cpp:2040-2090): they run the CUDA primitive's
// kernel with the variant's barrier form; the critical sections, and so the
// final storage, are the CUDA primitive's.
enum PrimVariant : int {
  PV_NONE = 0,
  PV_PRIORITY = 1,   // PRspinSem*, PRspinSemEBO*: exiting TBs go first
  PV_SRB = 2,        // atomicTreeBarrUniq*SRB: sense-reversing tree barrier
  PV_NAIVE = 3,      // *NaiveSRB: every TB joins one global barrier (no local stage)
  PV_NAIVE_ALL = 4,  // *NaiveAllSRB: every thread joins one global barrier
};

// Cohort pool (one per context): a die map of 256 bytes (one per SM id), then
// candidate lock lines whose home die calibration finds (hs_cohort.cu).
constexpr int kCohortMapWords = 64;
constexpr int kCohortCandidates = 128;
bool hs_cohort_calibrate(int device, unsigned* pool, int ncand, int sel[2][3]);

// Lock-state layout for a run: line offsets and total size.
struct Layout {
  int l_glob, l_gflag, l_grp, l_lflag, lflag_lines, lines;
  int groups;
  size_t ring_words;
};

#ifdef __CUDACC__
__host__ __device__
#endif
inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

}  // namespace hs
