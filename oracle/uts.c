/* uts.c -- ORACLE (test infrastructure only; never linked into the product).
 *
 * Plain-C restatement of the reference UTS host code, heterosync
 * cuda/uts/uvm/uts.cu:
 *   tree generation and golden   uts.cu:290-339 (srand(seed), BFS over undecided
 *                                nodes, value rand()%100, fertile if
 *                                rand()%100 < fertility, new leaves go to the
 *                                front of the leaf list, restart from the leaf
 *                                list when no undecided node is left, leftovers
 *                                become leaves of value 1)
 *   initial frontier             uts.cu:341-383
 * glibc rand() is the reference's random source, so the tree is a function of
 * (num_nodes, fertility, seed) on any glibc host.
 */
#include <stdlib.h>
#include <string.h>

typedef struct { unsigned value, depth, to_add; int child_a, child_b; } oracle_uts_node;

int hs_oracle_uts_tree(int num_nodes, int fertility, unsigned seed, oracle_uts_node* tree, unsigned* leaves,
                       unsigned* leaf_sum, unsigned* restarts) {
  if (num_nodes <= 0 || (num_nodes % 2) == 0) return -1;
  memset(tree, 0, sizeof(oracle_uts_node) * (size_t)num_nodes);
  /* undecided: FIFO queue; leaf list kept in insertion order, read back reversed */
  int* und = (int*)malloc(sizeof(int) * (size_t)num_nodes * 2 + 16);
  int* leaf = (int*)malloc(sizeof(int) * (size_t)num_nodes + 16);
  int uh = 0, ut = 0, nl = 0;
  unsigned rs = 0;
  srand(seed);
  und[ut++] = 0;
  int next = 1;
  while (next != num_nodes) {
    if (uh == ut) {               /* undecided_nodes = leaf_nodes (front = most recent leaf) */
      uh = ut = 0;
      for (int i = nl - 1; i >= 0; --i) und[ut++] = leaf[i];
      nl = 0;
      ++rs;
    }
    const int cur = und[uh];
    tree[cur].value = (unsigned)(rand() % 100);
    tree[cur].depth = 0;
    tree[cur].to_add = 0;
    if ((rand() % 100) < fertility) {
      tree[cur].child_a = next;
      und[ut++] = next++;
      tree[cur].child_b = next;
      und[ut++] = next++;
    } else {
      tree[cur].child_a = 0;
      tree[cur].child_b = 0;
      leaf[nl++] = cur;
    }
    ++uh;
    if (ut > num_nodes * 2 - 4 && uh > 0) { /* compact the queue */
      memmove(und, und + uh, sizeof(int) * (size_t)(ut - uh));
      ut -= uh;
      uh = 0;
    }
  }
  unsigned sum = 0;
  for (int i = uh; i < ut; ++i) {
    const int n = und[i];
    tree[n].child_a = tree[n].child_b = 0;
    tree[n].value = 1;
    tree[n].depth = 0;
    tree[n].to_add = 0;
    sum += 1;
  }
  for (int i = 0; i < nl; ++i) sum += tree[leaf[i]].value;
  *leaves = (unsigned)(nl + (ut - uh));
  *leaf_sum = sum;
  *restarts = rs;
  free(und);
  free(leaf);
  return 0;
}

/* uts.cu:341-383.  frontier must hold cores_used*16 + 2 ints. */
int hs_oracle_uts_frontier(const oracle_uts_node* tree, int num_nodes, int cores_used, int* frontier, int* count,
                           unsigned* host_processed) {
  const int want = cores_used * 16;
  const int cap = want + 4;
  int* q = (int*)malloc(sizeof(int) * (size_t)cap * 2);
  int h = 0, t = 0;
  unsigned processed = 0;
  long guard = 0;
  q[t++] = 0;
  while (t - h < want) {
    if (t == h || ++guard > (long)num_nodes * 4 + 1024) { free(q); return -1; }
    const int n = q[h++];
    if (tree[n].child_a > 0) {
      q[t++] = tree[n].child_a;
      q[t++] = tree[n].child_b;
      ++processed;
    } else {
      q[t++] = n;
    }
    if (t > cap * 2 - 4) { memmove(q, q + h, sizeof(int) * (size_t)(t - h)); t -= h; h = 0; }
  }
  for (int i = h; i < t; ++i) frontier[i - h] = q[i];
  *count = t - h;
  *host_processed = processed;
  free(q);
  return 0;
}
