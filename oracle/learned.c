/*
 * Oracle (test infrastructure only): per-node features of the learned reinsertion scorer.
 * The reference has no learned part (it selects nodes by the inefficiency of
 * lib/builder/Bittner13CUDA.cu:480-500); this restates the product's feature definition so the
 * GPU feature kernels can be checked. Parity unpinned: see oracle.h.
 *
 * Feature row (24 floats) of inner node x with children l, r, parent p and grand parent g
 * (p = g = the root where they do not exist), SA = surface area, all raw values clamped to
 * [-64, 64] (NaN -> -64):
 *   0 log2 SA(x)              5 log2 leaves(l)            10 rank of the inefficiency
 *   1 SA(x) / SA(p)           6 log2 leaves(r)            11 rank of SA(x) / min(SA(l), SA(r))
 *   2 SA(x) / SA(g)           7 log2 (SA(x) / SA(root))   12 rank of SA(x) / (SA(l) + SA(r))
 *   3 SA(x) / (SA(l)+SA(r))   8 log2 (SA(x) / min(l, r))  13 rank of SA(x)
 *   4 min(depth, 256) / log2(#leaves)   9 log2 inefficiency   14..23 zero
 * A rank is (#values in lower bins + half the own bin) / #inner nodes over a 65536-bin histogram
 * of the order-preserving integer image of the value (its top 16 bits); NaN values rank as 0.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define NONE 0xFFFFFFFFu
#define RANK_BINS 65536u
#define DEPTH_CAP 256u

static uint32_t f2ord(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
static float clampf(float v) { return fminf(fmaxf(v, -64.0f), 64.0f); }
static float nz(float v) { return isnan(v) ? 0.0f : v; }

float orc_lr_inv_log2_leaves(uint32_t n_leaves) { return 1.0f / log2f((float)(n_leaves > 2 ? n_leaves : 2)); }

uint32_t orc_lr_features(const orc_node *t, uint32_t n_nodes, uint32_t root, float *feat, uint32_t *inner_out) {
  uint32_t *depth = malloc(sizeof(uint32_t) * (n_nodes ? n_nodes : 1));
  uint32_t *leaves = calloc(n_nodes ? n_nodes : 1, sizeof(uint32_t));
  uint32_t *stack = malloc(sizeof(uint32_t) * (n_nodes ? n_nodes : 1));
  uint32_t n_leaves = 0, n_inner = 0;
  for (uint32_t i = 0; i < n_nodes; ++i) depth[i] = NONE;
  /* depth top-down from the root */
  uint32_t sp = 0;
  if (root < n_nodes) {
    depth[root] = 0;
    stack[sp++] = root;
  }
  while (sp) {
    const uint32_t x = stack[--sp];
    if (t[x].isLeafFlag) continue;
    const uint32_t c[2] = {t[x].left, t[x].right};
    for (int k = 0; k < 2; ++k) {
      if (c[k] >= n_nodes || depth[c[k]] != NONE) continue;
      depth[c[k]] = depth[x] + 1;
      stack[sp++] = c[k];
    }
  }
  /* leaf counts: every leaf adds one to itself and each ancestor */
  for (uint32_t i = 0; i < n_nodes; ++i) {
    if (!t[i].isLeafFlag) continue;
    n_leaves++;
    uint32_t x = i;
    for (uint32_t k = 0; k <= n_nodes; ++k) {
      leaves[x]++;
      if (x == root || t[x].parent >= n_nodes) break;
      x = t[x].parent;
    }
  }
  const float inv_l = orc_lr_inv_log2_leaves(n_leaves);
  const float sroot = t[root].surfaceArea;
  uint32_t *hist = calloc((size_t)RANK_BINS * 8, sizeof(uint32_t));
  float *src = malloc(sizeof(float) * 4 * (n_nodes ? n_nodes : 1));
  for (uint32_t x = 0; x < n_nodes; ++x) {
    if (t[x].isLeafFlag) continue;
    const uint32_t i = n_inner++;
    if (inner_out) inner_out[i] = x;
    const float sa = t[x].surfaceArea;
    const float sl = t[t[x].left].surfaceArea, sr = t[t[x].right].surfaceArea;
    const uint32_t p = x == root ? root : t[x].parent;
    const uint32_t g = p == root ? root : t[p].parent;
    const float mn = sl < sr ? sl : sr;
    const float sum = sl + sr;
    const float cost = orc_inefficiency(t, x);
    const uint32_t d = depth[x] > DEPTH_CAP ? DEPTH_CAP : depth[x];
    float f[10];
    f[0] = log2f(sa);
    f[1] = sa / t[p].surfaceArea;
    f[2] = sa / t[g].surfaceArea;
    f[3] = sa / sum;
    f[4] = (float)d * inv_l;
    f[5] = log2f((float)leaves[t[x].left]);
    f[6] = log2f((float)leaves[t[x].right]);
    f[7] = log2f(sa / sroot);
    f[8] = log2f(sa / mn);
    f[9] = log2f(cost);
    float *o = feat + (size_t)i * ORC_LR_FEATURES;
    for (int k = 0; k < 10; ++k) o[k] = clampf(f[k]);
    for (int k = 14; k < ORC_LR_FEATURES; ++k) o[k] = 0.0f;
    float *s = src + (size_t)i * 4;
    s[0] = nz(cost);
    s[1] = nz(sa / mn);
    s[2] = nz(sa / sum);
    s[3] = nz(sa);
    for (int r = 0; r < 4; ++r) hist[(size_t)r * RANK_BINS + (f2ord(s[r]) >> 16)]++;
  }
  /* exclusive prefix per histogram, stored in the second half */
  for (int r = 0; r < 4; ++r) {
    uint32_t run = 0;
    for (uint32_t b = 0; b < RANK_BINS; ++b) {
      hist[(size_t)(4 + r) * RANK_BINS + b] = run;
      run += hist[(size_t)r * RANK_BINS + b];
    }
  }
  const float fn = (float)n_inner;
  for (uint32_t i = 0; i < n_inner; ++i) {
    const float *s = src + (size_t)i * 4;
    float *o = feat + (size_t)i * ORC_LR_FEATURES;
    for (int r = 0; r < 4; ++r) {
      const uint32_t b = f2ord(s[r]) >> 16;
      const float below = (float)hist[(size_t)(4 + r) * RANK_BINS + b];
      const float own = (float)hist[(size_t)r * RANK_BINS + b];
      o[10 + r] = (below + 0.5f * own) / fn;
    }
  }
  free(hist);
  free(src);
  free(depth);
  free(leaves);
  free(stack);
  return n_inner;
}
