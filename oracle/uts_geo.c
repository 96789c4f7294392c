/* ORACLE (test infrastructure only): geometric UTS tree with a SHA-1
 * splittable node generator, counted by a depth-first walk on the host.
 *
 * The reference ships no geometric tree (its UTS, cuda/uts/uvm/uts.cu, builds
 * a binary tree from rand()); this workload follows the published Unbalanced
 * Tree Search benchmark's geometric shape and SHA-1 node generator, restated
 * here and in the CUDA kernel from one definition:
 *   root state    = SHA-1(16 zero bytes || seed, 4 bytes big-endian)
 *   child i state = SHA-1(parent state (20 bytes) || i, 4 bytes big-endian)
 *   r             = bytes 16..19 of a node's state, big-endian, & 0x7fffffff
 *   children      = 0 at depth >= depth_limit (root depth 0), else the number
 *                   of k >= 1 with r < T[k-1], where T[k-1] = floor(2^31 q^k),
 *                   q = b / (1 + b) and q^k is formed by k - 1 multiplications
 *                   in IEEE double (a geometric count with mean b).
 * SHA-1 is FIPS 180-4 (one 64-byte block suffices: messages are 20 or 24
 * bytes); tests check it against Python's hashlib.  Parity with a reference
 * implementation is unpinned: none exists in the reference repository.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint32_t rotl(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }

/* SHA-1 of a message of len <= 55 bytes (one block). */
void hs_oracle_sha1(const uint8_t* msg, int len, uint8_t out[20]) {
  uint8_t block[64];
  memset(block, 0, sizeof(block));
  memcpy(block, msg, (size_t)len);
  block[len] = 0x80;
  const uint64_t bits = (uint64_t)len * 8u;
  for (int i = 0; i < 8; ++i) block[63 - i] = (uint8_t)(bits >> (8 * i));
  uint32_t w[80];
  for (int t = 0; t < 16; ++t)
    w[t] = ((uint32_t)block[4 * t] << 24) | ((uint32_t)block[4 * t + 1] << 16) | ((uint32_t)block[4 * t + 2] << 8) |
           (uint32_t)block[4 * t + 3];
  for (int t = 16; t < 80; ++t) w[t] = rotl(w[t - 3] ^ w[t - 8] ^ w[t - 14] ^ w[t - 16], 1);
  uint32_t h[5] = {0x67452301u, 0xEFCDAB89u, 0x98BADCFEu, 0x10325476u, 0xC3D2E1F0u};
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4];
  for (int t = 0; t < 80; ++t) {
    uint32_t f, k;
    if (t < 20) { f = (b & c) | (~b & d); k = 0x5A827999u; }
    else if (t < 40) { f = b ^ c ^ d; k = 0x6ED9EBA1u; }
    else if (t < 60) { f = (b & c) | (b & d) | (c & d); k = 0x8F1BBCDCu; }
    else { f = b ^ c ^ d; k = 0xCA62C1D6u; }
    const uint32_t tmp = rotl(a, 5) + f + e + k + w[t];
    e = d; d = c; c = rotl(b, 30); b = a; a = tmp;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e;
  for (int i = 0; i < 5; ++i) {
    out[4 * i] = (uint8_t)(h[i] >> 24);
    out[4 * i + 1] = (uint8_t)(h[i] >> 16);
    out[4 * i + 2] = (uint8_t)(h[i] >> 8);
    out[4 * i + 3] = (uint8_t)h[i];
  }
}

/* Thresholds T[0..n-1]; returns how many are nonzero. */
int hs_oracle_geo_table(double b, uint32_t* t, int n) {
  const double q = b / (1.0 + b);
  double p = q;
  int nz = 0;
  for (int k = 0; k < n; ++k) {
    const double v = p * 2147483648.0;
    t[k] = v >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)v;
    if (t[k]) nz = k + 1;
    p *= q;
  }
  return nz;
}

static int geo_children(const uint8_t s[20], int depth, int limit, const uint32_t* t, int nt) {
  if (depth >= limit) return 0;
  const uint32_t r = (((uint32_t)s[16] << 24) | ((uint32_t)s[17] << 16) | ((uint32_t)s[18] << 8) | s[19]) &
                     0x7fffffffu;
  int m = 0;
  while (m < nt && r < t[m]) ++m;
  return m;
}

void hs_oracle_geo_root(uint32_t seed, uint8_t out[20]) {
  uint8_t msg[20];
  memset(msg, 0, sizeof(msg));
  msg[16] = (uint8_t)(seed >> 24);
  msg[17] = (uint8_t)(seed >> 16);
  msg[18] = (uint8_t)(seed >> 8);
  msg[19] = (uint8_t)seed;
  hs_oracle_sha1(msg, 20, out);
}

void hs_oracle_geo_child(const uint8_t parent[20], uint32_t i, uint8_t out[20]) {
  uint8_t msg[24];
  memcpy(msg, parent, 20);
  msg[20] = (uint8_t)(i >> 24);
  msg[21] = (uint8_t)(i >> 16);
  msg[22] = (uint8_t)(i >> 8);
  msg[23] = (uint8_t)i;
  hs_oracle_sha1(msg, 24, out);
}

/* Depth-first count of the whole tree: nodes, leaves, deepest level. */
int hs_oracle_geo_count(uint32_t seed, int depth_limit, double b, unsigned long long* nodes,
                        unsigned long long* leaves, int* max_depth) {
  if (depth_limit < 0 || depth_limit > 64 || b <= 0.0) return 1;
  uint32_t t[128];
  const int nt = hs_oracle_geo_table(b, t, 128);
  struct Frame { uint8_t s[20]; int next, end; } st[66];
  unsigned long long n = 1, lv = 0;
  int md = 0, sp = 0;
  uint8_t root[20];
  hs_oracle_geo_root(seed, root);
  const int m0 = geo_children(root, 0, depth_limit, t, nt);
  if (m0 == 0) lv = 1;
  else {
    memcpy(st[0].s, root, 20);
    st[0].next = 0;
    st[0].end = m0;
    sp = 1;
  }
  while (sp > 0) {
    struct Frame* f = &st[sp - 1];
    if (f->next == f->end) { --sp; continue; }
    uint8_t c[20];
    hs_oracle_geo_child(f->s, (uint32_t)f->next, c);
    f->next += 1;
    const int d = sp;  /* depth of the child */
    ++n;
    if (d > md) md = d;
    const int m = geo_children(c, d, depth_limit, t, nt);
    if (m == 0) { ++lv; continue; }
    memcpy(st[sp].s, c, 20);
    st[sp].next = 0;
    st[sp].end = m;
    ++sp;
  }
  *nodes = n;
  *leaves = lv;
  *max_depth = md;
  return 0;
}
