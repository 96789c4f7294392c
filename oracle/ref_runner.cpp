// ref_runner.cpp -- ORACLE / reference arm (test and benchmark infrastructure).
//
// Runs the reference's OWN SyncPrims kernels -- compiled unmodified from
// heterosync cuda/syncPrims/uvm/main.cu by oracle/build_ref.sh into
// oracle/_ref/*.cubin -- on the local GPU, through the CUDA driver API.  The
// host side restates what the reference's main() does around its kernels:
//   lock state        cudaLocksInit, cudaLocks.cu:3-81, with (MAX_BLOCKS,
//                     8*NUM_SM mutexes, 24*NUM_SM semaphores) as main.cu:1267
//   per-SM barriers   NUM_SM*MAX_BLOCKS*2 zeroed words, main.cu:1281, 1317
//   handles           mutex/semaphore numbers and counts of main.cu:1352-1451,
//                     semaphore words {count+1,0,0,count+1} (cudaLocksSemaphoreSpin.cu:12-22)
//   launches          NUM_REPEATS launches of <<<numTBs, T>>> each followed by a
//                     device synchronise, timed with events (main.cu:838-1128, 1494-1618)
// The lock-data struct lives in mapped pinned host memory and is passed by
// pointer, as the reference passes cpuLockData.
//
// Refuses (returns 3) launches that would deadlock in the reference: barrier
// kernels whose TBs cannot all be co-resident, or whose numTBs is neither <=
// NUM_SM nor a multiple of it (README.txt:80; main.cu:131-133).
#include <cuda.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct RefLockData {  // cudaLockData_t, cudaLocks.h:4-16
  int maxBufferSize;
  int arrayStride;
  int mutexCount;
  int semaphoreCount;
  unsigned* barrierBuffers;
  int* mutexBuffers;
  unsigned* mutexBufferHeads;
  unsigned* mutexBufferTails;
  unsigned* semaphoreBuffers;
};

std::string g_msg;
std::map<std::string, CUmodule> g_mods;
CUcontext g_ctx = nullptr;

#define CK(x)                                              \
  do {                                                     \
    CUresult r_ = (x);                                     \
    if (r_ != CUDA_SUCCESS) {                              \
      const char* s_ = nullptr;                            \
      cuGetErrorString(r_, &s_);                           \
      g_msg = std::string(#x) + ": " + (s_ ? s_ : "?");    \
      return 4;                                            \
    }                                                      \
  } while (0)

int ensure_ctx() {
  if (g_ctx) return 0;
  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  CK(cuDevicePrimaryCtxRetain(&g_ctx, dev));
  CK(cuCtxSetCurrent(g_ctx));
  return 0;
}

int find_kernel(CUmodule mod, const char* name, CUfunction* out) {
  unsigned n = 0;
  CK(cuModuleGetFunctionCount(&n, mod));
  std::vector<CUfunction> fs(n);
  CK(cuModuleEnumerateFunctions(fs.data(), n, mod));
  char prefix[128];
  std::snprintf(prefix, sizeof(prefix), "_Z%zu%s", std::strlen(name), name);
  for (CUfunction f : fs) {
    const char* fn = nullptr;
    if (cuFuncGetName(&fn, f) != CUDA_SUCCESS || !fn) continue;
    if (std::strncmp(fn, prefix, std::strlen(prefix)) == 0) {
      *out = f;
      return 0;
    }
  }
  g_msg = std::string("kernel not found in module: ") + name;
  return 1;
}

// syncPrim id -> (kernel name, kind, handle number, semaphore count).  main.cu:1224-1451.
struct RefPrim {
  int id;
  const char* kernel;
  int kind;  // 0 barrier, 1 mutex, 2 global semaphore, 3 uniq semaphore
  int handle;
  unsigned count;
};
const RefPrim kRef[] = {
    {0, "kernelAtomicTreeBarrierUniq", 0, 0, 0},
    {1, "kernelAtomicTreeBarrierUniqLocalExch", 0, 0, 0},
    {2, "kernelFBSTreeBarrierUniq", 0, 0, 0},
    {3, "kernelFBSTreeBarrierUniqLocalExch", 0, 0, 0},
    {4, "kernelSpinLockMutex", 1, 0, 0},
    {5, "kernelEBOMutex", 1, 1, 0},
    {6, "kernelSleepingMutex", 1, 2, 0},
    {7, "kernelFetchAndAddMutex", 1, 3, 0},
    {8, "kernelSpinLockSemaphore", 2, 0, 1},
    {9, "kernelSpinLockSemaphore", 2, 1, 2},
    {10, "kernelSpinLockSemaphore", 2, 2, 10},
    {11, "kernelSpinLockSemaphore", 2, 3, 120},
    {12, "kernelEBOSemaphore", 2, 4, 1},
    {13, "kernelEBOSemaphore", 2, 5, 2},
    {14, "kernelEBOSemaphore", 2, 6, 10},
    {15, "kernelEBOSemaphore", 2, 7, 120},
    {20, "kernelSpinLockMutexUniq", 1, 4, 0},
    {21, "kernelEBOMutexUniq", 1, 5, 0},
    {22, "kernelSleepingMutexUniq", 1, 6, 0},
    {23, "kernelFetchAndAddMutexUniq", 1, 7, 0},
    {24, "kernelSpinLockSemaphoreUniq", 3, 12, 1},
    {25, "kernelSpinLockSemaphoreUniq", 3, 13, 2},
    {26, "kernelSpinLockSemaphoreUniq", 3, 14, 10},
    {27, "kernelSpinLockSemaphoreUniq", 3, 15, 120},
    {28, "kernelEBOSemaphoreUniq", 3, 16, 1},
    {29, "kernelEBOSemaphoreUniq", 3, 17, 2},
    {30, "kernelEBOSemaphoreUniq", 3, 18, 10},
    {31, "kernelEBOSemaphoreUniq", 3, 19, 120},
};

}  // namespace

extern "C" const char* hs_ref_last_error(void) { return g_msg.c_str(); }

extern "C" int hs_ref_device(int* nsm, int* max_tpb) {
  int r = ensure_ctx();
  if (r) return r;
  CUdevice dev;
  CK(cuCtxGetDevice(&dev));
  CK(cuDeviceGetAttribute(nsm, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
  CK(cuDeviceGetAttribute(max_tpb, CU_DEVICE_ATTRIBUTE_MAX_THREADS_PER_BLOCK, dev));
  return 0;
}

// Run one reference primitive.  `storage` holds the initial contents (the
// reference uses storage[i] = i as float) and receives the final ones.
// Returns 0 ok, 1 bad arguments, 3 refused (would deadlock), 4 CUDA error.
extern "C" int hs_ref_run(const char* cubin, int T, int prim, int L, int numTBs, int iters, int repeats,
                          int sync_each, uint32_t* storage, long words, float* elapsed_ms) {
  int r = ensure_ctx();
  if (r) return r;
  CK(cuCtxSetCurrent(g_ctx));
  const RefPrim* rp = nullptr;
  for (const auto& p : kRef)
    if (p.id == prim) rp = &p;
  if (!rp || T <= 0 || L <= 0 || numTBs <= 0) { g_msg = "bad arguments"; return 1; }
  CUmodule mod;
  auto it = g_mods.find(cubin);
  if (it == g_mods.end()) {
    CK(cuModuleLoad(&mod, cubin));
    g_mods[cubin] = mod;
  } else {
    mod = it->second;
  }
  CUfunction fn;
  if ((r = find_kernel(mod, rp->kernel, &fn))) return r;

  int NUM_SM = 0, max_tpb = 0;
  if ((r = hs_ref_device(&NUM_SM, &max_tpb))) return r;
  const int MAX_BLOCKS = (max_tpb / T) * NUM_SM;  // main.cu:1192-1195
  if (numTBs > MAX_BLOCKS) { g_msg = "numTBs > MAX_BLOCKS"; return 1; }
  if (rp->kind == 3) {
    // The reference's per-SM semaphore kernels (kernelSpinLockSemaphoreUniq /
    // kernelEBOSemaphoreUniq) did not finish on GB300 (spinSemUniq1, 304 TBs x 32
    // threads: killed after 900 s).  cudaSemaphore*TryWaitLocal reads the count
    // with a plain load after only __threadfence_block(), so a CTA can keep
    // reading a stale copy and retry forever.  Never launched again.
    g_msg = "reference Uniq semaphore kernels livelock on this GPU (stale per-SM count reads); not run";
    return 3;
  }
  if (rp->kind == 2) {
    // The reference's global semaphore kernels (kernelSpinLockSemaphore /
    // kernelEBOSemaphore) read maxSemCount from the live count word at kernel
    // start (main.cu:542-543, 695-696).  A CTA that starts after another writer
    // took the semaphore reads 0; as a writer it then waits for count == 0,
    // which never recurs once every other writer has finished.  A bench run
    // whose reference arm launched them did not finish (killed after 600 s).
    // Never launched again.
    g_msg = "reference global semaphore kernels can wait forever on GB300 (maxSemCount race at kernel start); not run";
    return 3;
  }
  if (rp->kind == 0) {
    if (!(numTBs <= NUM_SM || numTBs % NUM_SM == 0)) {
      g_msg = "barrier numTBs neither <= NUM_SM nor a multiple of it: the reference kernel would deadlock";
      return 3;
    }
    int per_sm = 0;
    CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, 0));
    if ((long long)per_sm * NUM_SM < numTBs) { g_msg = "barrier TBs cannot all be co-resident"; return 3; }
  }
  // storage size check (numLocsMult, main.cu:1283-1301)
  const int perSM = (numTBs + NUM_SM - 1) / NUM_SM;
  long mult = 0;
  if (rp->kind == 0 || rp->kind == 3) mult = numTBs;
  else if (rp->kind == 1) mult = (prim >= 20) ? (numTBs < NUM_SM ? numTBs : NUM_SM) : 1;
  else mult = perSM;
  const long numStorageLocs = mult * (long)T * (L + 1);
  if (words < numStorageLocs) { g_msg = "storage too small"; return 1; }

  // cudaLocksInit(MAX_BLOCKS, 8*NUM_SM, 24*NUM_SM, false, NUM_SM)
  RefLockData* ld = nullptr;
  CK(cuMemHostAlloc((void**)&ld, sizeof(RefLockData), CU_MEMHOSTALLOC_DEVICEMAP | CU_MEMHOSTALLOC_PORTABLE));
  const int numMutexes = 8 * NUM_SM, numSems = 24 * NUM_SM;
  ld->maxBufferSize = MAX_BLOCKS;
  ld->arrayStride = (MAX_BLOCKS + NUM_SM) / 16 * 16;
  ld->mutexCount = numMutexes;
  ld->semaphoreCount = numSems;
  const size_t stride = (size_t)ld->arrayStride;
  CUdeviceptr bb, mb, mh, mt, sb, persm, st;
  CK(cuMemAlloc(&bb, 4 * stride * 2));
  CK(cuMemAlloc(&mb, 4 * stride * numMutexes));
  CK(cuMemAlloc(&mh, 4 * (size_t)numMutexes));
  CK(cuMemAlloc(&mt, 4 * (size_t)numMutexes));
  CK(cuMemAlloc(&sb, 4 * 4 * (size_t)numSems));
  CK(cuMemsetD32(bb, 0, stride * 2));
  CK(cuMemsetD32(mh, 0, numMutexes));
  CK(cuMemsetD32(mt, 0, numMutexes));
  CK(cuMemsetD32(sb, 0, 4 * (size_t)numSems));
  {
    std::vector<int> ring(stride * numMutexes, -1);  // cudaLocks.cu:58-65
    for (size_t i = 0; i < ring.size(); i += stride) ring[i] = 1;
    CK(cuMemcpyHtoD(mb, ring.data(), ring.size() * 4));
  }
  ld->barrierBuffers = (unsigned*)bb;
  ld->mutexBuffers = (int*)mb;
  ld->mutexBufferHeads = (unsigned*)mh;
  ld->mutexBufferTails = (unsigned*)mt;
  ld->semaphoreBuffers = (unsigned*)sb;
  CUdeviceptr ld_dev;
  CK(cuMemHostGetDevicePointer(&ld_dev, ld, 0));
  const size_t persm_words = (size_t)NUM_SM * MAX_BLOCKS * 2;
  CK(cuMemAlloc(&persm, persm_words * 4));
  CK(cuMemsetD32(persm, 0, persm_words));
  CK(cuMemAlloc(&st, (size_t)numStorageLocs * 4));
  CK(cuMemcpyHtoD(st, storage, (size_t)numStorageLocs * 4));
  if (rp->kind >= 2) {  // cudaSemaphoreCreate{Spin,EBO}(&h, handle, count, NUM_SM)
    std::vector<unsigned> w((size_t)4 * NUM_SM);
    for (int id = 0; id < NUM_SM; ++id) {
      w[4 * id] = rp->count + 1;
      w[4 * id + 1] = 0;
      w[4 * id + 2] = 0;
      w[4 * id + 3] = rp->count + 1;
    }
    CK(cuMemcpyHtoD(sb + (size_t)rp->handle * 4 * NUM_SM * 4, w.data(), w.size() * 4));
  }

  unsigned handle = (unsigned)rp->handle;
  unsigned nlocs = (unsigned)numStorageLocs;
  float* stp = (float*)st;
  RefLockData* ldp = (RefLockData*)ld_dev;
  unsigned* persmp = (unsigned*)persm;
  int NUM_LDST = L, ITER = iters, NSM = NUM_SM, MB = MAX_BLOCKS;
  void* a_bar[] = {&stp, &ldp, &persmp, &ITER, &NUM_LDST, &NSM, &MB};
  void* a_mtx[] = {&handle, &stp, &ldp, &ITER, &NUM_LDST, &NSM};
  void* a_gsem[] = {&handle, &stp, &ldp, &nlocs, &ITER, &NUM_LDST, &NSM};
  void** args = rp->kind == 0 ? a_bar : rp->kind == 1 ? a_mtx : rp->kind == 2 ? a_gsem : a_mtx;

  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  CK(cuCtxSynchronize());
  CK(cuEventRecord(e0, 0));
  for (int rep = 0; rep < repeats; ++rep) {
    CK(cuLaunchKernel(fn, numTBs, 1, 1, T, 1, 1, 0, 0, args, nullptr));
    if (sync_each) CK(cuCtxSynchronize());
  }
  CK(cuCtxSynchronize());
  CK(cuEventRecord(e1, 0));
  CK(cuEventSynchronize(e1));
  CK(cuEventElapsedTime(elapsed_ms, e0, e1));
  CK(cuMemcpyDtoH(storage, st, (size_t)numStorageLocs * 4));
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  cuMemFree(bb);
  cuMemFree(mb);
  cuMemFree(mh);
  cuMemFree(mt);
  cuMemFree(sb);
  cuMemFree(persm);
  cuMemFree(st);
  cuMemFreeHost(ld);
  return 0;
}

// The reference's refCounter kernel (cuda/relaxedAtomics/uvm/refCounter/
// refCounter_kernel.cu:4-55) with its host's sizes and one launch
// (refCounter.cu:24-82, numRuns = 1): numCounters = numThrs / numSharers,
// numSharingGroups = numTBs / numSharers, numCounters_perSharingGroup =
// numCounters / numSharingGroups.  The kernel has no waits (uniform loops of
// atomics and CTA barriers), so it cannot hang.  Returns the final counters0/1
// (numCounters words each) and del0/1 (numThrs words each).  Sizes whose
// counter index (sharing group * per-group + threadIdx.x) would leave the
// arrays are refused (1).
extern "C" int hs_ref_refcounter(const char* cubin, int numSharers, int numTBs, int tbSize, int numRepeats,
                                 uint32_t* counters0, uint32_t* counters1, uint32_t* del0, uint32_t* del1,
                                 float* elapsed_ms) {
  int r = ensure_ctx();
  if (r) return r;
  CK(cuCtxSetCurrent(g_ctx));
  if (numSharers <= 0 || numTBs <= 0 || tbSize <= 0 || tbSize > 256 || numSharers > numTBs || numRepeats < 0 ||
      numTBs % numSharers != 0) {
    g_msg = "bad arguments";
    return 1;
  }
  const unsigned numThrs = (unsigned)tbSize * (unsigned)numTBs;
  const unsigned numCounters = numThrs / (unsigned)numSharers;
  const unsigned numGroups = (unsigned)numTBs / (unsigned)numSharers;
  const unsigned perGroup = numCounters / numGroups;
  if ((numGroups - 1u) * perGroup + (unsigned)tbSize > numCounters) { g_msg = "counter index out of range"; return 1; }
  CUmodule mod;
  auto it = g_mods.find(cubin);
  if (it == g_mods.end()) {
    CK(cuModuleLoad(&mod, cubin));
    g_mods[cubin] = mod;
  } else {
    mod = it->second;
  }
  CUfunction fn;
  if ((r = find_kernel(mod, "refCounter_kernel", &fn))) return r;
  CUdeviceptr c0, c1, d0, d1;
  CK(cuMemAlloc(&c0, (size_t)numCounters * 4));
  CK(cuMemAlloc(&c1, (size_t)numCounters * 4));
  CK(cuMemAlloc(&d0, (size_t)numThrs * 4));
  CK(cuMemAlloc(&d1, (size_t)numThrs * 4));
  CK(cuMemsetD32(c0, 0, numCounters));
  CK(cuMemsetD32(c1, 0, numCounters));
  CK(cuMemsetD32(d0, 0, numThrs));
  CK(cuMemsetD32(d1, 0, numThrs));
  unsigned reps = (unsigned)numRepeats, sharers = (unsigned)numSharers, nc = numCounters, ng = numGroups,
           pg = perGroup;
  void* args[] = {&c0, &c1, &d0, &d1, &reps, &sharers, &nc, &ng, &pg};
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  CK(cuEventRecord(e0, 0));
  CK(cuLaunchKernel(fn, numTBs, 1, 1, tbSize, 1, 1, 0, 0, args, nullptr));
  CK(cuEventRecord(e1, 0));
  CK(cuEventSynchronize(e1));
  CK(cuEventElapsedTime(elapsed_ms, e0, e1));
  CK(cuMemcpyDtoH(counters0, c0, (size_t)numCounters * 4));
  CK(cuMemcpyDtoH(counters1, c1, (size_t)numCounters * 4));
  CK(cuMemcpyDtoH(del0, d0, (size_t)numThrs * 4));
  CK(cuMemcpyDtoH(del1, d1, (size_t)numThrs * 4));
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  cuMemFree(c0);
  cuMemFree(c1);
  cuMemFree(d0);
  cuMemFree(d1);
  return 0;
}
