/* golden.c -- ORACLE (test infrastructure only; never linked into the product).
 *
 * A plain-C restatement of the reference's host golden for the SyncPrims
 * benchmark, heterosync cuda/syncPrims/uvm/main.cu:
 *   accessData_golden          main.cu:33-51
 *   storage sizing             main.cu:1283-1308
 *   golden replay per class    main.cu:1633-1788
 * generalised only in the parameters the reference fixes at compile time or
 * reads from the device (threads per TB T, NUM_SM, NUM_REPEATS), and with a
 * second operation: in "inc" mode every location the golden would write is
 * incremented instead of copied (the exact-count check of the build's
 * HS_MODE_INC).  The loops are the reference's loops, in the reference's order,
 * so it is slow (O(repeats * iters * numTBs * T * numLdSt)) and meant for the
 * small sizes the parity tests use.
 *
 * Also: the SLICE workload replay (uint32[numTBs*numLdSt], TB b at iteration j
 * adds 1 to slice (b+j) mod numTBs, per logical-SM group for the Uniq mutexes).
 */
#include <stdint.h>
#include <stddef.h>

#define HALFWARP 16
#define WORDS_PER_LINE 16

static long ceil_div_l(long a, long b) { return (a + b - 1) / b; }

/* numLocsMult, main.cu:1283-1301 (-1: unknown primitive). */
long hs_oracle_locs_mult(int prim, int numTBs, int NUM_SM) {
  if (prim < 4 || (prim >= 24 && prim <= 35)) return numTBs;
  if (prim >= 4 && prim <= 7) return 1;
  if (prim >= 8 && prim <= 19) return ceil_div_l(numTBs, NUM_SM);
  if ((prim >= 20 && prim <= 23) || prim == 36) return numTBs < NUM_SM ? numTBs : NUM_SM;
  return -1;
}

long hs_oracle_storage_words(int prim, int T, int L, int numTBs, int NUM_SM) {
  long m = hs_oracle_locs_mult(prim, numTBs, NUM_SM);
  return m < 0 ? -1 : m * (long)T * (L + 1);
}

/* accessData_golden (main.cu:33-51): a location that is not in the first line
 * of its half-warp region takes the value of the same word one line below. */
static void access_golden(uint32_t* s, long loc, int L, int inc) {
  if (loc % ((long)HALFWARP * (L + 1)) >= WORDS_PER_LINE) {
    if (inc) s[loc] += 1u;
    else s[loc] = s[loc - WORDS_PER_LINE];
  }
}

/* The golden replay, main.cu:1637-1788.  `storage` holds the initial contents
 * (the reference uses storage[i] = i as float) and receives the result.
 * Returns 0, or -1 for an unknown primitive / too-small storage. */
int hs_oracle_golden(int syncPrim, int T, int L, int numTBs, int iters, int repeats, int NUM_SM, int inc,
                     uint32_t* storage, long numStorageLocs) {
  const long numUniqLocsAccPerTB = (long)T * (L + 1);
  const int numTBs_perSM = (int)ceil_div_l(numTBs, NUM_SM); /* main.cu:1219 */
  long numLocsAccessed = 0, currLoc = 0;
  if (numStorageLocs < hs_oracle_storage_words(syncPrim, T, L, numTBs, NUM_SM)) return -1;
  if (hs_oracle_locs_mult(syncPrim, numTBs, NUM_SM) < 0) return -1;

  for (int repeat = 0; repeat < repeats; ++repeat) {
    for (int j = 0; j < iters; ++j) {
      if (syncPrim < 4) {
        /* barriers: every TB's region once per episode (main.cu:1650-1668) */
        numLocsAccessed = numTBs * numUniqLocsAccPerTB;
        for (long i = numLocsAccessed - 1; i >= 0; --i) {
          currLoc = (i + (long)j * numUniqLocsAccPerTB) % numLocsAccessed;
          access_golden(storage, currLoc, L, inc);
        }
        /* local exchange: a second pass when several TBs share an SM (1672-1686) */
        if ((syncPrim == 1 || syncPrim == 3) && numTBs_perSM > 1) {
          for (long i = numLocsAccessed - 1; i >= 0; --i) {
            currLoc = (i + (long)numTBs_perSM * numUniqLocsAccPerTB) % numLocsAccessed;
            currLoc = (currLoc + (long)j * numUniqLocsAccPerTB) % numLocsAccessed;
            access_golden(storage, currLoc, L, inc);
          }
        }
      } else if (syncPrim >= 4 && syncPrim <= 7) {
        /* global mutexes: every TB updates the same region (1692-1703) */
        for (int block = 0; block < numTBs; ++block)
          for (long i = numUniqLocsAccPerTB - 1; i >= 0; --i) access_golden(storage, i, L, inc);
      } else if (syncPrim >= 8 && syncPrim <= 19) {
        /* global semaphores: one writer TB per SM updates numTBs_perSM regions (1710-1743) */
        const int numSM = numTBs < NUM_SM ? numTBs : NUM_SM;
        for (int tb = 0; tb < numTBs; ++tb) {
          const int smID = tb % numSM;
          const int perSM_tbID = tb / numSM;
          const int isWriter = (perSM_tbID == (smID % numTBs_perSM));
          if (isWriter) {
            for (int k = 0; k < numTBs_perSM; ++k)
              for (long i = numUniqLocsAccPerTB - 1; i >= 0; --i) {
                currLoc = (i + (long)k * numUniqLocsAccPerTB) % numStorageLocs;
                access_golden(storage, currLoc, L, inc);
              }
          }
        }
      } else if (syncPrim >= 20 && syncPrim <= 23) {
        /* Uniq mutexes: TBs wrap onto the region of their SM (1753-1765) */
        numLocsAccessed = numTBs * numUniqLocsAccPerTB;
        for (long i = numLocsAccessed - 1; i >= 0; --i) {
          currLoc = i % ((long)NUM_SM * numUniqLocsAccPerTB);
          access_golden(storage, currLoc, L, inc);
        }
      } else {
        /* Uniq semaphores: every region once (1775-1786) */
        numLocsAccessed = numTBs * numUniqLocsAccPerTB;
        for (long i = numLocsAccessed - 1; i >= 0; --i) access_golden(storage, i, L, inc);
      }
    }
  }
  return 0;
}

/* SLICE workload replay: for every launch, iteration and TB, +1 on the TB's
 * slice.  Global mutexes (uniq == 0): slice (b + j) mod numTBs.  Uniq mutexes:
 * group g = b mod NUM_SM with members g + r*NUM_SM; slice g + ((r + j) mod m_g)*NUM_SM. */
int hs_oracle_slice(int uniq, int L, int numTBs, int iters, int repeats, int NUM_SM, uint32_t* data, long words) {
  if (words < (long)numTBs * L) return -1;
  const int G = uniq ? NUM_SM : 1;
  for (int rep = 0; rep < repeats; ++rep)
    for (int j = 0; j < iters; ++j)
      for (int b = 0; b < numTBs; ++b) {
        const int g = b % G, r = b / G;
        const int m = (numTBs - g + G - 1) / G;
        const long s = g + (long)((r + j) % m) * G;
        for (int w = 0; w < L; ++w) data[s * L + w] += 1u;
      }
  return 0;
}
