/* hs.h -- C ABI of the GB300-native HeteroSync hot path (libhsgb300.so).
 *
 * Plain C types only.  Every function returns an int status (HS_OK == 0) unless
 * stated otherwise.  Device memory pointers are plain `void*`; streams are the
 * `cudaStream_t` value cast to `void*` (NULL = the legacy default stream).
 *
 * Two groups of entry points:
 *  1. The reference's own host API, same names and arguments (so a program
 *     written against heterosync's cudaLocks.h links against this library):
 *     cudaLocksInit / cudaLocksDestroy / cudaMutexCreate* / cudaSemaphoreCreate*.
 *  2. hs_* entry points that replace the reference's per-primitive host
 *     launch wrappers (invoke*, cuda/syncPrims/uvm/main.cu:838-1128) and its
 *     command line (main.cu:1130-1821), plus the batch, serving and probe paths
 *     this build adds.
 */
#ifndef HS_H_
#define HS_H_

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
enum {
  HS_OK = 0,
  HS_EINVAL = 1,       /* bad argument (sizes, unknown primitive, mode not supported) */
  HS_ETIMEDOUT = 2,    /* a bounded device wait ran out (device status has the site) */
  HS_ENORES = 3,       /* the launch cannot be co-resident (barriers) or memory is short */
  HS_ECUDA = 4,        /* a CUDA runtime call failed (hs_last_error() has the text) */
  HS_ENODEV = 5,       /* no CUDA device */
  HS_EMISMATCH = 6     /* a self-check found results that differ from the expected ones */
};

/* ---- data modes ------------------------------------------------------------ */
enum {
  HS_MODE_REF = 0,     /* reference critical section: one-line copy shift of 32-bit words */
  HS_MODE_INC = 1,     /* same locations, every written word += 1 (exact count check) */
  HS_MODE_SLICE = 2    /* uint32[numTBs*numLdSt]; TB b, iteration j: slice (b+j) mod numTBs += 1 (mutexes) */
};

/* ---- run flags --------------------------------------------------------------- */
enum {
  HS_RUN_SYNC_EACH = 1,   /* host-synchronise after every launch, as main.cu:844-854 does */
  HS_RUN_KEEP_STATE = 2,  /* do not re-initialise lock state before the repeats */
  HS_RUN_NO_CLUSTER = 4,  /* tree barriers: keep the local stage in L2 instead of on thread-block clusters */
  HS_RUN_REGISTER_CS = 8, /* critical sections on the register path only (no bulk copies through shared memory) */
  HS_RUN_GRAPH = 16,      /* the repeats as one CUDA graph: captured once per context and launch shape, then
                             replayed (not with HS_RUN_SYNC_EACH); the lock state is still reset before it */
  HS_RUN_NO_COHORT = 32,  /* global spin, EBO and ticket mutexes and global semaphores' writers: the
                             primitive's lock alone instead of the die-aware cohort (a ticket queue per die,
                             homed on it, in front of the lock, which is handed on within the die) */
  HS_RUN_CLUSTER_CS = 64, /* global mutexes and semaphores with numLdSt > 32: one thread-block cluster per
                             logical TB, the critical section split over its SMs, for every such run (by
                             default only semaphores whose writers own 4 or more chunks, where it is faster) */
  HS_RUN_NO_GROUP_CTA = 128 /* tree barriers: one CTA per logical TB even where a whole logical-SM group
                               fits one CTA (by default such a group runs as one CTA of numTBs_perSM x
                               threads, its local stage the CTA barrier: register critical sections up
                               to numLdSt 64, a bulk-copy buffer per member above) */
};

/* One run of one SyncPrims primitive: `repeats` launches of `num_tbs` TBs of
 * `threads` threads, each TB doing `num_iters` critical sections / episodes. */
typedef struct hs_run_config {
  int prim;             /* reference syncPrim id, see hs_prim_id() */
  int num_ldst;         /* <numLdSt> */
  int num_tbs;          /* <numTBs> */
  int num_iters;        /* <numCSIters> */
  int threads;          /* threads per TB (reference: 32, main.cu:8); multiple of 16, <= 1024 */
  int repeats;          /* launches (reference: NUM_REPEATS = 10, main.cu:21) */
  int mode;             /* HS_MODE_* */
  int nsm;              /* NUM_SM used in the reference index math; 0 = device SM count */
  unsigned backoff_min_ns;   /* EBO start (reference 1) */
  unsigned backoff_max_ns;   /* EBO cap, power of two (reference MAX_BACKOFF = 1024) */
  unsigned backoff_unit_ns;  /* ticket-lock per-position sleep / poll sleep (0 = spin) */
  unsigned long long timeout_ns; /* per-wait limit without observed progress, 0 = 10 s */
  int skip_tb;          /* fault injection for barriers: this TB never arrives (-1 = none) */
  int flags;            /* HS_RUN_* */
} hs_run_config;

typedef struct hs_run_result {
  int status;                   /* HS_OK, HS_ETIMEDOUT, ... */
  unsigned dev_error_bits;      /* device status word 0 */
  unsigned dev_error_site;      /* device status word 1 (wait site) */
  float elapsed_ms;             /* device time of all launches (CUDA events on the launch stream) */
  float avg_ms;                 /* elapsed_ms / repeats: the reference's "average" */
  float h2d_ms, d2h_ms;         /* storage copies when storage is host memory */
  unsigned long long ops;       /* num_tbs * num_iters * repeats */
  unsigned launches;            /* kernels launched by this call */
  int cluster;                  /* tree barriers: CTAs per thread-block cluster (1: no clusters) */
  int cohort;                   /* global mutexes and semaphores: 1 if the die-aware cohort form ran */
  int tbs_per_cta;              /* tree barriers: logical TBs per CTA (1: one CTA per TB) */
} hs_run_result;

typedef struct hs_ctx hs_ctx;

/* ---- library / device -------------------------------------------------------- */
int hs_version(void);
const char* hs_last_error(void);
const char* hs_status_string(int status);
/* Multiprocessor count, compute capability and max threads/block of `device`. */
int hs_device_info(int device, int* nsm, int* cc_major, int* cc_minor, int* max_threads_per_block);
/* Total kernels this library has launched in this process (all entry points). */
unsigned long long hs_launch_count(void);

/* ---- primitive names (main.cu:1224-1256) ------------------------------------- */
/* Reference name -> syncPrim id (0-15, 20-31); -1 if unknown. */
int hs_prim_id(const char* name);
/* syncPrim id -> reference name; NULL if unknown. */
const char* hs_prim_name(int prim);
/* The label the reference prints before timing (main.cu:1352-1451), e.g.
 * "fetchadd_mutex_100"; returns the length written (snprintf semantics). */
int hs_prim_label(int prim, int num_iters, char* buf, int buflen);
/* Semaphore size for semaphore prims (1, 2, 10, 120), 0 otherwise. */
int hs_prim_sem_count(int prim);
/* The CUDA primitive a HIP-build-only id runs (PRspinSem* -> spinSem*,
 * PRspinSemEBO* -> spinSemEBO*, atomicTreeBarrUniq*SRB -> atomicTreeBarrUniq(LocalExch)),
 * and its variant (1 priority, 2 sense-reversing tree, 3 naive, 4 naive all
 * threads); other ids map to themselves, variant 0. */
int hs_prim_base(int prim, int* variant);
/* Storage words a run needs (numLocsMult * threads * (numLdSt+1), main.cu:1283-1308;
 * numTBs * numLdSt for HS_MODE_SLICE). */
int hs_storage_words(const hs_run_config* cfg, int nsm, size_t* words);

/* ---- runs (replace invoke*, main.cu:838-1128) -------------------------------- */
int hs_ctx_create(int device, hs_ctx** out);
int hs_ctx_destroy(hs_ctx* ctx);
/* Fill *cfg with the reference defaults (threads 32, repeats 10, REF mode, ...). */
void hs_run_config_default(hs_run_config* cfg);
/* Run one primitive.  `storage` holds hs_storage_words() 32-bit words, on the
 * device (storage_on_device != 0) or in host memory (copied in and out inside
 * the call and timed in h2d_ms / d2h_ms).  Synchronises before returning. */
int hs_run(hs_ctx* ctx, const hs_run_config* cfg, void* storage, int storage_on_device, void* stream,
           hs_run_result* result);
/* Expected final storage of a run, from its initial contents (closed form of
 * the reference's golden replay, main.cu:1633-1788).  Host arrays. */
int hs_expected_storage(const hs_run_config* cfg, int nsm, const uint32_t* init, uint32_t* expected, size_t words);

/* ---- runs without device allocation ------------------------------------------ */
/* No counterpart in the reference.  hs_run() for callers that cannot allocate
 * device memory -- host frameworks that own all device memory through their own
 * pool, processes under a device-memory budget fixed at start-up, and
 * latency-critical loops that cannot afford cudaMalloc's implicit device-wide
 * synchronisation.  The lock state lives in one fixed device array of
 * HS_NOALLOC_SCRATCH_BYTES that the library holds on every GPU that loads it;
 * runs whose state does not fit are rejected with HS_EINVAL.  `storage` must be
 * device memory.  The first call on a device looks up the array's address:
 * make it before any stream capture.  All calls share the array, so calls that
 * overlap on the GPU race; each call clears the state it needs.  elapsed_ms is
 * host wall time around the launches (no events are created).  Runs are always
 * the flat form (one CTA per TB, no clusters, plain rather than die-aware
 * locks, fresh lock state): cfg->flags may hold HS_RUN_SYNC_EACH,
 * HS_RUN_NO_CLUSTER, HS_RUN_REGISTER_CS and HS_RUN_NO_COHORT, and any other
 * flag is rejected with HS_EINVAL.  Barriers whose TBs cannot all be resident
 * with the shared memory they launch with are rejected with HS_ENORES before
 * anything is launched. */
#define HS_NOALLOC_SCRATCH_BYTES (1u << 20)
int hs_run_noalloc(const hs_run_config* cfg, void* storage, void* stream, hs_run_result* result);
const char* hs_noalloc_last_error(void);

/* ---- batched mixed instances: one persistent, graph-replayed launch --------------- */
/* No counterpart in the reference (its runs are one primitive per process).
 * Instance i runs numTBs logical TBs on a gang of ceil(numTBs / v) co-resident
 * CTAs; every instance has its own storage and lock state; 256 threads per TB. */
typedef struct hs_batch_instance { int prim, num_ldst, num_tbs, num_iters; } hs_batch_instance;
/* Batch-only instance kinds beside the 28 SyncPrims ids: the relaxed-atomics
 * microbenchmarks at instance scale (refCounter_kernel.cu, splitCounter_kernel.cu,
 * seqlocks_kernel.cu, flags_kernel.cu); 256 threads per TB, numLdSt sets the
 * counter / data width. */
enum { HS_BATCH_REFCOUNTER = 60, HS_BATCH_SPLITCOUNTER = 61, HS_BATCH_SEQLOCK = 62, HS_BATCH_FLAGS = 63 };
int hs_batch_instance_words(const hs_batch_instance* inst, int nsm, size_t* words);
/* Closed-form final storage of one instance after one run (mode: HS_MODE_INC or HS_MODE_REF). */
int hs_batch_expected_storage(const hs_batch_instance* inst, int nsm, int mode, const uint32_t* init,
                              uint32_t* out, size_t words);
typedef struct hs_batch_result {
  float elapsed_ms;             /* device time of the batch (or of all serial launches) */
  unsigned long long ops;       /* sum of numTBs * numCSIters */
  unsigned launches;            /* kernels launched */
  int grid;                     /* CTAs of the persistent launch (0 for the serial form) */
  int tbs_per_cta;              /* v */
  unsigned dev_error_bits;
  int failed_instance;          /* -1 if none */
} hs_batch_result;
typedef struct hs_batch hs_batch;
const char* hs_batch_last_error(void);
/* The mixed batch (32 kinds), drawn from std::mt19937_64(seed). */
int hs_batch_generate(unsigned long long seed, int n, int nsm, int iter_div, hs_batch_instance* out);
int hs_batch_create(const hs_batch_instance* inst, int n, int threads, int mode, hs_batch** out);
int hs_batch_destroy(hs_batch* b);
size_t hs_batch_storage_words(hs_batch* b, int i);
int hs_batch_set_storage(hs_batch* b, int i, const uint32_t* host);
int hs_batch_get_storage(hs_batch* b, int i, uint32_t* host);
/* Gang plan with v logical TBs per CTA; HS_ENORES if the gangs cannot be co-resident. */
int hs_batch_plan(hs_batch* b, int v, int* grid, int* capacity);
/* General plan, launched with thread-block clusters of cl CTAs (1, 2, 4 or 8).
 * Instances whose operations serialise on one lock or semaphore (global mutexes
 * and semaphores) get executors in proportion to numTBs * numCSIters *
 * (numLdSt + 1), serial_execs for the heaviest (0 = ceil(numTBs / v) each); with
 * numLdSt >= 33 each executor is a whole cluster (the holder's critical section
 * split over its SMs), else one CTA.  The other instances get ceil(numTBs / v)
 * one-CTA executors. */
int hs_batch_plan_ex(hs_batch* b, int cl, int serial_execs, int v, int* grid, int* capacity);
int hs_batch_get_plan(hs_batch* b, int* cl, int* serial_execs, int* v, int* grid);
/* Exponential-backoff bounds (ns; bo_max a power of two) of the batched launch;
 * the per-launch form keeps the reference's 1..1024.  The autotuner sets them. */
int hs_batch_set_backoff(hs_batch* b, unsigned bo_min, unsigned bo_max);
int hs_batch_get_backoff(hs_batch* b, unsigned* bo_min, unsigned* bo_max);
/* Staging bytes per CTA for bulk-copy critical sections (0 = the largest chunk:
 * whole-chunk copies, fewer CTAs per SM).  Default 40 KiB.  Invalidates the plan. */
int hs_batch_set_stage(hs_batch* b, unsigned bytes);
unsigned hs_batch_get_stage(hs_batch* b);
/* Try v = 1, 2, 4, ... and keep the fastest plan that fits (storage is restored after each try). */
int hs_batch_autotune(hs_batch* b, void* stream, int* best_v, float* best_ms);
/* Lock-state reset + persistent kernel, captured once per plan into a CUDA graph and replayed. */
int hs_batch_run(hs_batch* b, void* stream, hs_batch_result* result);
/* Comparison point: one standalone launch per instance on the same stream. */
int hs_batch_run_serial(hs_batch* b, void* stream, hs_batch_result* result);

/* ---- relaxed-atomics microbenchmarks (cuda/relaxedAtomics/uvm) ----------------- */
/* Host arrays in and out (the reference's managed arrays); the kernel alone is
 * timed.  Sizes and array lengths are the reference's. */
typedef struct hs_relaxed_result {
  float elapsed_ms;
  unsigned long long ops;
  unsigned dev_error_bits, dev_error_site;
} hs_relaxed_result;
const char* hs_relaxed_last_error(void);
/* refCounter.cu:5-155: counters0/1 [numTBs*tbSize/numSharersPerGroup], del0/1 [numTBs*tbSize] */
int hs_refcounter(int numSharersPerGroup, int numTBs, int tbSize, int numRepeats, unsigned* counters0,
                  unsigned* counters1, unsigned* del0, unsigned* del1, hs_relaxed_result* result);
/* splitCounter.cu:5-98: counters [numTBs*tbSize/2], outArr [numTBs*tbSize] */
int hs_splitcounter(int numTBs, int tbSize, unsigned* counters, unsigned* outArr, hs_relaxed_result* result);
/* seqlocks.cu:5-111: seqlock [numTBs/groupSize], data0/1 [32], outArr [numTBs*tbSize] */
int hs_seqlocks(int numTBs, int tbSize, int groupSize, int useTFs, unsigned* seqlock, int* data0, int* data1,
                int* outArr, unsigned long long timeout_ns, hs_relaxed_result* result);
/* flags.cu:19-176: randArr [randLen], outArr [numTBs*tbSize], *dirty_out = final dirty count */
int hs_flags(int numTBs, int tbSize, int numAccsPerThr, int numRepeats, float cutoffVal, int numIters,
             const float* randArr, int randLen, unsigned* outArr, unsigned* dirty_out, unsigned long long timeout_ns,
             hs_relaxed_result* result);

/* ---- UTS (cuda/uts/uvm/uts.cu) -------------------------------------------------- */
/* Same layout as the reference's uts_node (uts.cu:40-46). */
typedef struct hs_uts_node {
  unsigned int value;
  unsigned int depth;
  unsigned int to_add;
  int child_a;
  int child_b;
} hs_uts_node;
typedef struct hs_uts_result {
  unsigned nodes_processed, leaves_found, leaf_sum;
  float elapsed_ms;
  unsigned dev_error_bits;
} hs_uts_result;
const char* hs_uts_last_error(void);
/* uts.cu:290-339: binary tree of num_nodes (odd) nodes from srand(seed); golden leaf count and sum. */
int hs_uts_tree_build(int num_nodes, int fertility, unsigned seed, hs_uts_node* tree, unsigned* leaves,
                      unsigned* leaf_sum, unsigned* restarts);
/* uts.cu:341-383: initial frontier of cores_used*16 nodes and the internal nodes expanded on the host. */
int hs_uts_frontier(const hs_uts_node* tree, int num_nodes, int cores_used, int* frontier, int* count,
                    unsigned* host_processed);
/* Replaces access_shared (uts.cu:91-242): process every remaining node on the GPU. */
int hs_uts_run(const hs_uts_node* tree, int num_nodes, const int* frontier, int n_frontier, unsigned host_processed,
               int blocks, int threads, unsigned long long timeout_ns, hs_uts_result* out);

/* ---- geometric UTS with a SHA-1 node generator ----------------------------------- */
/* No counterpart in the reference repository (its UTS is the rand() binary
 * tree, hs_uts_run): the published Unbalanced Tree Search geometric tree.
 * root = SHA-1(16 zero bytes || seed), child i = SHA-1(parent || i) (4-byte
 * big-endian integers), r = last state word & 0x7fffffff, children = 0 at
 * depth >= depth_limit, else #{k >= 1 : r < T[k-1]} with T from
 * hs_uts_geo_table (geometric, mean `branching`).  Work stealing over per-CTA
 * lock-free queues; the node count is exact. */
typedef struct hs_uts_geo_result {
  unsigned long long nodes, leaves;
  unsigned max_depth;
  float elapsed_ms;
  unsigned dev_error_bits;
} hs_uts_geo_result;
const char* hs_uts_geo_last_error(void);
/* T[k-1] = floor(2^31 q^k), q = b / (1 + b), q^k formed by repeated IEEE double
 * multiplication; returns the number of nonzero entries. */
int hs_uts_geo_table(double branching, uint32_t* table, int n);
int hs_uts_geo_run(unsigned seed, int depth_limit, double branching, int blocks, int threads,
                   unsigned long long timeout_ns, hs_uts_geo_result* r);

/* Cooperative CPU+GPU walk of the same tree: `blocks` CTAs and `host_threads`
 * host threads balance load dynamically through two rings in mapped pinned
 * host memory (README.txt:30 of the reference names CPU+GPU load balancing for
 * UTS; its uts.cu:457-539 host threads do no tree work).  The GPU gives idle
 * host walkers subtrees with 3 to 7 levels left; host walkers give the GPU
 * the upper half of their oldest frame once over half of its threads idle.
 * host_threads < 0: the host's cores minus one.  blocks == 0: host threads
 * only, with no CUDA call (the walk runs on a machine without a GPU).  GPU and
 * host threads together need a link with native host atomics
 * (cudaDevAttrHostNativeAtomicSupported, NVLink-C2C); HS_EINVAL otherwise.
 * Waits are bounded on both sides: no progress for timeout_ns → HS_ETIMEDOUT. */
typedef struct hs_uts_coop_result {
  unsigned long long nodes, leaves;
  unsigned max_depth;
  unsigned long long gpu_nodes, host_nodes; /* nodes each side expanded */
  unsigned long long to_host, to_gpu;       /* items that crossed the link each way */
  int host_threads;                         /* walkers that ran */
  float elapsed_ms;                         /* wall time, launch to both sides done */
  unsigned dev_error_bits;
} hs_uts_coop_result;
int hs_uts_geo_coop_run(unsigned seed, int depth_limit, double branching, int blocks, int threads, int host_threads,
                        unsigned long long timeout_ns, hs_uts_coop_result* r);

/* ---- tree barrier with local exchange on thread-block clusters ----------------- */
/* The LocalExch tree barriers (main.cu:153-270; joinBarrier_helper,
 * cudaLocksBarrierAtomic.cu:147-172; joinLFBarrier_helper,
 * cudaLocksBarrierFast.cu:315-330) with the local level on clusters of
 * `cluster` CTAs (1, 2, 4, 8): n resident CTAs each own `elems` words; each of
 * `episodes` episodes rotates every CTA's buffer to CTA (b + 1) mod n through
 * distributed shared memory (within a cluster) or an L2 staging slot (between
 * clusters) and ends with one tree barrier (lf = 0: generation counter among the
 * cluster leaders; lf = 1: per-cluster flags scanned by a master CTA).  host_out
 * receives the final buffers: host_in rotated by `episodes` CTAs. */
typedef struct hs_exchange_result {
  float elapsed_ms;          /* kernel time (CUDA events) */
  double episodes_per_s;
  double exchange_gbs;       /* 2 * n * elems * 4 bytes per episode / time */
  int clusters;
  unsigned dev_error_bits, wait_site;
} hs_exchange_result;
const char* hs_exchange_last_error(void);
/* words uniform fp32 in [-1, 1): (int32)(r >> 40) * 2^-23 - 1 over std::mt19937_64(seed) draws r. */
int hs_exchange_fill(unsigned long long seed, size_t words, uint32_t* out);
int hs_exchange_run(const uint32_t* host_in, uint32_t* host_out, int n, int elems, int cluster, int lf, int episodes,
                    unsigned long long timeout_ns, hs_exchange_result* r);

/* ---- served request loop -------------------------------------------------------- */
/* A persistent server kernel of `slots` slots x `gang` co-resident CTAs admits
 * requests as they arrive (oldest first, when a slot is free and the device
 * arena has pages for the request's storage and lock state), executes each on
 * its slot's CTAs and publishes a completion.  No counterpart in the reference
 * (whose programs run one instance per launch); the instances themselves are
 * its SyncPrims (main.cu:104-836) in increment mode, 256 threads per TB.
 * Between hs_serve_start and hs_serve_stop the server kernel occupies the
 * device: the process must not make synchronising CUDA calls on it
 * (cudaDeviceSynchronize, cudaMalloc, cudaFree) until the server stopped. */
enum { HS_REQ_SYNCPRIM = 0, HS_REQ_UTS_GEO = 1 };
typedef struct hs_serve_request {
  int kind;                                  /* HS_REQ_SYNCPRIM or HS_REQ_UTS_GEO */
  int prim, num_ldst, num_tbs, num_iters;    /* SYNCPRIM: a SyncPrims id or an HS_BATCH_* kind */
  unsigned seed;                             /* UTS_GEO: the geometric tree (hs_uts_geo_run) */
  int depth_limit;
  double branching;
} hs_serve_request;
/* A tree-search request's input may be NULL (the server builds the walk's
 * initial state); its output (hs_serve_request_words words) holds the final
 * state, from which this reads the counts. */
int hs_serve_uts_geo_counts(const uint32_t* final_words, size_t words, unsigned long long* nodes,
                            unsigned long long* leaves, unsigned* deepest);
typedef struct hs_serve_completion {
  unsigned long long id;
  int status;                 /* HS_OK; HS_ENORES: larger than the arena; HS_ETIMEDOUT: a wait ran out */
  unsigned dev_error_bits, wait_site;
  double latency_us;          /* submission (or due time, hs_serve_drive) to completion seen by the host */
  double service_us;          /* on the device: state laid out -> final storage copied back */
  double admit_to_end_us;     /* on the device: admission -> completion */
} hs_serve_completion;
typedef struct hs_server hs_server;
const char* hs_serve_last_error(void);
int hs_serve_start(int slots, int gang, unsigned long long arena_bytes, unsigned long long staging_bytes,
                   double idle_timeout_s, hs_server** out);
int hs_serve_request_words(const hs_serve_request* r, int nsm, size_t* words);
/* Copies `input` (the instance's initial storage) into the staging pool and
 * publishes the request; `output` receives the final storage when
 * hs_serve_poll returns its completion.  HS_ENORES: ring or staging pool full. */
int hs_serve_submit(hs_server* s, const hs_serve_request* r, const uint32_t* input, uint32_t* output,
                    unsigned long long* id);
int hs_serve_poll(hs_server* s, hs_serve_completion* out, int max, int* n);
int hs_serve_pending(hs_server* s, unsigned long long* in_flight);
int hs_serve_stop(hs_server* s, double timeout_s);
int hs_serve_destroy(hs_server* s);
/* Open-loop driver: request i is published at arrival_s[i] seconds after the
 * start; comps[i] receives its completion (latency from the due time). */
int hs_serve_drive(hs_server* s, const hs_serve_request* reqs, int n, const uint32_t* const* inputs,
                   uint32_t* const* outputs, const double* arrival_s, double timeout_s, hs_serve_completion* comps,
                   double* wall_s);

/* ---- roofline probes --------------------------------------------------------- */
/* Aggregate L2 atomic rate: blocks x threads threads each issue `iters`
 * red.add to their own 128-byte-spaced word (same_address = 0: contention-free
 * peak), or one lane per block to a single word (same_address = 1: the rate one
 * contended lock word sustains).  Result in atomics per second. */
int hs_probe_l2_atomics(int blocks, int threads, int iters, int same_address, double* atomics_per_s);

/* L2-resident copy bandwidth: two buffers of bytes/2 each (together well under
 * the L2's size), copied `reps` times in one launch with loads and stores that
 * bypass L1, after one warm-up launch.  Result: bytes read + written per second,
 * in GB/s. */
int hs_probe_l2_bandwidth(size_t bytes, int reps, double* copy_gbs);

/* The latencies a lock hand-off is made of, each measured by one thread:
 *  handoff: CTA 0 and each other CTA (one per SM, cooperative launch) ping-pong
 *           a flag `rounds` times (st.release.gpu, then ld.acquire.gpu polls until
 *           the answer shows); one hand-off = half a round trip.  Median, min and
 *           max over the partners (SMs on both dies).
 *  atomic:  a dependent chain of atom.add.gpu over 64 lines spread across L2.
 *  load:    a dependent chain of ld.relaxed.gpu (L2 hits, L1 bypassed) over a
 *           randomly linked 512 KiB cycle of 128-byte lines.
 * Waits are bounded (2 s); a timeout sets dev_error_bits and returns HS_ETIMEDOUT. */
typedef struct hs_latency_result {
  double handoff_ns_median, handoff_ns_min, handoff_ns_max;
  double atomic_rtt_ns, load_rtt_ns;
  int partners;
  unsigned dev_error_bits;
} hs_latency_result;
int hs_probe_latency(int rounds, hs_latency_result* r);

/* ---- the reference's host API (cuda/syncPrims/uvm/cudaLocks.h:4-26) ----------- */
/* Same field order as cudaLockData_t (cudaLocks.h:4-16). */
typedef struct hs_lock_data {
  int maxBufferSize;
  int arrayStride;
  int mutexCount;
  int semaphoreCount;
  unsigned int* barrierBuffers;
  int* mutexBuffers;
  unsigned int* mutexBufferHeads;
  unsigned int* mutexBufferTails;
  unsigned int* semaphoreBuffers;
} hs_lock_data;

/* cudaLocks.cu:3-81.  Returns a cudaError_t value (0 = cudaSuccess).  Sizes whose
 * arrayStride, (maxBlocksPerKernel + NUM_SM) / 16 * 16, would not exceed
 * maxBlocksPerKernel (a ring of maxBlocksPerKernel + 1 slots would overrun into
 * the next; a stride of 0 leaves no barrier buffer) return cudaErrorInvalidValue. */
int cudaLocksInit(const int maxBlocksPerKernel, const int numMutexes, const int numSemaphores, const bool pageAlign,
                  const int NUM_SM);
/* cudaLocks.cu:83-95 (this one also frees barrierBuffers). */
int cudaLocksDestroy(void);
/* The lock data cudaLocksInit filled in (the reference's cpuLockData, pinned host memory). */
hs_lock_data* hs_lock_data_get(void);
/* Device time (CUDA events) of the last cudaLocksInit's host-to-device copy of
 * the ring-buffer slots: the figure the reference prints as "memcpy H->D 1"
 * (cudaLocks.cu:66-74). */
float hs_locks_init_copy_ms(void);
/* cudaLocksMutexSpin.cu:4, cudaLocksMutexEBO.cu:6, cudaLocksMutexFA.cu:6, cudaLocksMutexSleep.cu:6 */
int cudaMutexCreateSpin(unsigned int* const handle, const int mutexNumber);
int cudaMutexCreateEBO(unsigned int* const handle, const int mutexNumber);
int cudaMutexCreateFA(unsigned int* const handle, const int mutexNumber);
int cudaMutexCreateSleep(unsigned int* const handle, const int mutexNumber);
/* cudaLocksSemaphoreSpin.cu:6-23, cudaLocksSemaphoreEBO.cu:4-21 */
int cudaSemaphoreCreateSpin(unsigned int* const handle, const int semaphoreNumber, const unsigned int count,
                            const int NUM_SM);
int cudaSemaphoreCreateEBO(unsigned int* const handle, const int semaphoreNumber, const unsigned int count,
                           const int NUM_SM);

#ifdef __cplusplus
}
#endif
#endif /* HS_H_ */
