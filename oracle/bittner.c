/*
 * Oracle (test infrastructure only): Bittner et al. 2013 reinsertion optimizer.
 *  - orc_bittner_seq:     the sequential CPU optimizer, lib/builder/Bittner13.cpp:71-312.
 *  - orc_bittner_chunked: the chunked parallel GPU algorithm, lib/builder/Bittner13CUDA.cu:141-772
 *                         with lib/base/BVHPatch.hpp:87-335, items of a chunk evaluated against
 *                         the chunk-start tree, conflicts resolved by batch rank.
 * Both are pinned to the reference's own code (oracle.h): orc_bittner_seq to Bittner13.cpp, the
 * chunked form with Bittner13Par's rules to Bittner13Par.cpp.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NNODE 10
#define P_GRAND_PARENT 0
#define P_1ST_ROOT 1
#define P_1ST_BEST 2
#define P_NODE 3
#define P_1ST_INSERT 4
#define P_2ND_ROOT 5
#define P_2ND_BEST 6
#define P_2ND_INSERT 7
#define P_SIBLING 8
#define P_PARENT 9
#define NONE 0xFFFFFFFFu

static void merge_into(orc_aabb *a, const orc_aabb *b) {
  for (int k = 0; k < 3; ++k) {
    a->mn[k] = a->mn[k] < b->mn[k] ? a->mn[k] : b->mn[k];
    a->mx[k] = a->mx[k] > b->mx[k] ? a->mx[k] : b->mx[k];
  }
}

/* kCalcCost (Bittner13CUDA.cu:480-500): (SA^3 * 2) / ((SA_L + SA_R) * min(SA_L, SA_R)). */
float orc_inefficiency(const orc_node *nodes, uint32_t i) {
  const orc_node *nd = &nodes[i];
  if (nd->isLeafFlag) return 0.0f;
  float sa = nd->surfaceArea;
  float l = nodes[nd->left].surfaceArea;
  float r = nodes[nd->right].surfaceArea;
  float num = sa * sa;
  num = num * sa;
  num = num * 2.0f;
  float den = l + r;
  den = den * (l < r ? l : r);
  return num / den;
}

/* ---- binary heap with the hole-based sift of the C++ standard library heap algorithms,
 *      restated from lib/builder/CUDAHeap.hpp:33-112. "less(a, b)" is a.cost > b.cost, so the
 *      front of the heap holds the smallest cost. ------------------------------------------- */
typedef struct hitem {
  uint32_t node;
  float cost;
} hitem;

static int hless(const hitem *a, const hitem *b) { return a->cost > b->cost; }

static void sift_up(hitem *h, long hole, long top, hitem v) {
  long parent = (hole - 1) / 2;
  while (hole > top && hless(&h[parent], &v)) {
    h[hole] = h[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h[hole] = v;
}

static void heap_push(hitem *h, long len_after) { sift_up(h, len_after - 1, 0, h[len_after - 1]); }

static void heap_pop(hitem *h, long len) {
  if (len <= 1) return;
  long last = len - 1;
  hitem v = h[last];
  h[last] = h[0];
  long n = last, hole = 0, top = 0, second = 0;
  while (second < (n - 1) / 2) {
    second = 2 * (second + 1);
    if (hless(&h[second], &h[second - 1])) second--;
    h[hole] = h[second];
    hole = second;
  }
  if ((n & 1) == 0 && second == (n - 2) / 2) {
    second = 2 * (second + 1);
    h[hole] = h[second - 1];
    hole = second - 1;
  }
  sift_up(h, hole, top, v);
}

/* ================================ sequential (Bittner13.cpp) ================================ */

/* findNodeForReinsertion (Bittner13.cpp:71-113). */
static uint32_t seq_find_node(const orc_node *t, uint32_t root, uint32_t n, hitem *pq, uint32_t cap) {
  float best_cost = INFINITY;
  uint32_t best = 0;
  const orc_node *nd = &t[n];
  float sarea = nd->surfaceArea;
  long size = 1;
  pq[0].node = root;
  pq[0].cost = 0.0f;
  while (size > 0) {
    hitem cur = pq[0];
    const orc_node *cn = &t[cur.node];
    heap_pop(pq, size);
    size--;
    if (cur.cost + sarea >= best_cost) break;
    orc_aabb m = nd->bbox; /* directCost: node's box merged with the candidate's */
    merge_into(&m, &cn->bbox);
    float direct = orc_surface_area(&m);
    float total = cur.cost + direct;
    if (total < best_cost) {
      best_cost = total;
      best = cur.node;
    }
    float induced = total - cn->surfaceArea;
    if (induced + sarea < best_cost && !cn->isLeafFlag) {
      if ((uint32_t)size + 2 <= cap) {
        pq[size].node = cn->left; pq[size].cost = induced;
        pq[size + 1].node = cn->right; pq[size + 1].cost = induced;
        heap_push(pq, size + 1);
        heap_push(pq, size + 2);
        size += 2;
      }
    }
  }
  return best;
}

/* fixTree (Bittner13.cpp:198-220). */
static void seq_fix_tree(orc_node *t, uint32_t root, uint32_t x) {
  int last_left = 1;
  orc_aabb b = t[t[x].left].bbox;
  for (;;) {
    uint32_t sib = last_left ? t[x].right : t[x].left;
    merge_into(&b, &t[sib].bbox);
    t[x].bbox = b;
    t[x].surfaceArea = orc_surface_area(&b);
    if (x == root) return;
    last_left = t[x].isLeft != 0;
    x = t[x].parent;
  }
}

static uint32_t sibling_of(const orc_node *t, uint32_t x) {
  const orc_node *p = &t[t[x].parent];
  return t[x].isLeft ? p->right : p->left;
}

/* removeNode (Bittner13.cpp:115-158). */
static int seq_remove(orc_node *t, uint32_t root, uint32_t x, uint32_t ins[2], uint32_t unused[2]) {
  if (t[x].isLeafFlag || x == root) return 0;
  uint32_t s = sibling_of(t, x);
  uint32_t p = t[x].parent;
  uint32_t g = t[p].parent;
  float lsa = t[t[x].left].surfaceArea, rsa = t[t[x].right].surfaceArea;
  if (p == root) return 0;
  if (t[p].isLeft) {
    t[g].left = s;
    t[s].isLeft = 1;
  } else {
    t[g].right = s;
    t[s].isLeft = 0;
  }
  t[s].parent = g;
  seq_fix_tree(t, root, g);
  if (lsa > rsa) { ins[0] = t[x].left; ins[1] = t[x].right; }
  else { ins[0] = t[x].right; ins[1] = t[x].left; }
  unused[0] = x;
  unused[1] = p;
  return 1;
}

/* reinsert (Bittner13.cpp:161-196). */
static void seq_reinsert(orc_node *t, uint32_t *root, uint32_t x, uint32_t u, hitem *pq, uint32_t cap) {
  uint32_t best = seq_find_node(t, *root, x, pq, cap);
  uint32_t r = t[best].parent;
  if (best == *root) {
    *root = u;
    r = u;
  } else {
    if (t[best].isLeft) { t[r].left = u; t[u].isLeft = 1; }
    else { t[r].right = u; t[u].isLeft = 0; }
  }
  t[u].parent = r;
  t[u].left = best;
  t[u].right = x;
  t[best].parent = u;
  t[best].isLeft = 1;
  t[x].parent = u;
  t[x].isLeft = 0;
  seq_fix_tree(t, *root, u);
}

typedef struct cost_item {
  float cost;
  uint32_t idx;
} cost_item;

static int cmp_cost_desc(const void *a, const void *b) {
  const cost_item *x = a, *y = b;
  if (x->cost > y->cost) return -1;
  if (x->cost < y->cost) return 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

int orc_bittner_seq(orc_node *t, uint32_t n_nodes, uint32_t *root, uint32_t iters, float batch_percent,
                    double *sah_trace) {
  if (batch_percent <= 0.01f) batch_percent = 0.01f;
  if (batch_percent >= 75.0f) batch_percent = 75.0f;
  uint32_t k = (uint32_t)((batch_percent / 100.0f) * (float)n_nodes);
  const uint32_t cap = 16384; /* Bittner13::QUEUE_SIZE */
  hitem *pq = malloc(sizeof(hitem) * cap);
  uint32_t *todo = malloc(sizeof(uint32_t) * (n_nodes ? n_nodes : 1));
  if (sah_trace) sah_trace[0] = orc_sah(t, n_nodes, *root);
  for (uint32_t it = 0; it < iters; ++it) {
    /* nth_element + sort of the first k (Bittner13.cpp:258-283), with the same library calls. */
    const uint32_t m = orc_std_select(t, n_nodes, k, 1, todo);
    for (uint32_t j = 0; j < m; ++j) {
      uint32_t ins[2], un[2];
      if (!seq_remove(t, *root, todo[j], ins, un)) continue;
      seq_reinsert(t, root, ins[0], un[0], pq, cap);
      seq_reinsert(t, root, ins[1], un[1], pq, cap);
    }
    if (sah_trace) sah_trace[it + 1] = orc_sah(t, n_nodes, *root);
  }
  free(pq);
  free(todo);
  return 0;
}

/* ============================ chunked GPU algorithm (Bittner13CUDA.cu) ========================= */

typedef struct npatch {
  uint32_t parent, left, right;
  uint16_t isLeafFlag, isLeft;
} npatch;

/* BVHPatch (BVHPatch.hpp:87-335), ENABLE_AABB_PATH = 0 variant. */
typedef struct bpatch {
  npatch nd[NNODE];
  uint32_t idx[NNODE];
  uint32_t apath[4];
  orc_aabb abox[4];
  const orc_node *t;
  uint32_t root;
} bpatch;

static npatch to_patch(const orc_node *n) {
  npatch p = {n->parent, n->left, n->right, n->isLeafFlag, n->isLeft};
  return p;
}
static void bp_clear(bpatch *p) {
  for (int i = 0; i < NNODE; ++i) p->idx[i] = NONE;
  for (int i = 0; i < 4; ++i) p->apath[i] = NONE;
}
static uint32_t bp_index_subset(const bpatch *p, uint32_t x) {
  if (p->idx[0] == x) return 0;
  if (p->idx[1] == NONE) return NONE;
  if (p->idx[1] == x) return 1;
  if (p->idx[2] == x) return 2;
  if (p->idx[3] == x) return 3;
  return NONE;
}
static uint32_t bp_index(const bpatch *p, uint32_t x) {
  for (uint32_t i = 0; i < NNODE; ++i)
    if (p->idx[i] == x) return i;
  return NONE;
}
static npatch bp_get(const bpatch *p, uint32_t x) {
  uint32_t i = bp_index(p, x);
  return i == NONE ? to_patch(&p->t[x]) : p->nd[i];
}
static npatch bp_get_subset(const bpatch *p, uint32_t x) {
  uint32_t i = bp_index_subset(p, x);
  return i == NONE ? to_patch(&p->t[x]) : p->nd[i];
}
static npatch *bp_patch_node(bpatch *p, uint32_t x, uint32_t slot) {
  p->idx[slot] = x;
  p->nd[slot] = to_patch(&p->t[x]);
  return &p->nd[slot];
}
static npatch *bp_move(bpatch *p, uint32_t from, uint32_t to) {
  p->idx[to] = p->idx[from];
  p->idx[from] = NONE;
  p->nd[to] = p->nd[from];
  return &p->nd[to];
}
static uint32_t bp_sibling(const bpatch *p, const npatch *n) {
  npatch par = bp_get(p, n->parent);
  return n->isLeft == 0 ? par.left : par.right;
}
static orc_aabb bp_get_aabb(const bpatch *p, uint32_t x) {
  for (int i = 0; i < 4; ++i)
    if (p->apath[i] == x) return p->abox[i];
  return p->t[x].bbox;
}
/* patchAABBFrom (BVHPatch.hpp:293-316): two levels of temporary boxes from x upwards. */
static void bp_patch_aabb_from(bpatch *p, uint32_t x, uint32_t pidx) {
  uint32_t ni = x;
  npatch nd = bp_get_subset(p, ni);
  orc_aabb b = bp_get_aabb(p, nd.left);
  int last_left = 1;
  for (uint32_t i = 0; i < 2; ++i) {
    uint32_t sib = last_left ? nd.right : nd.left;
    orc_aabb sb = bp_get_aabb(p, sib);
    merge_into(&b, &sb);
    p->abox[pidx * 2 + i] = b;
    p->apath[pidx * 2 + i] = ni;
    last_left = nd.isLeft != 0;
    if (ni == p->root) break;
    ni = nd.parent;
    nd = bp_get_subset(p, ni);
  }
}

/* findNode1 (Bittner13CUDA.cu:141-191). */
static uint32_t gpu_find_node(const bpatch *p, uint32_t n, hitem *pq, uint32_t cap, uint64_t *overflow) {
  float best_cost = INFINITY;
  uint32_t best = 0;
  const orc_node *nd = &p->t[n];
  orc_aabb nbox = nd->bbox;
  float sarea = nd->surfaceArea;
  long size = 1;
  pq[0].node = p->root;
  pq[0].cost = 0.0f;
  while (size > 0) {
    hitem cur = pq[0];
    if (cur.cost + sarea >= best_cost) break;
    heap_pop(pq, size);
    size--;
    npatch cn = bp_get_subset(p, cur.node);
    orc_aabb b = bp_get_aabb(p, cur.node);
    float induced = -1.0f * orc_surface_area(&b);
    merge_into(&b, &nbox);
    float direct = orc_surface_area(&b);
    float total = cur.cost + direct;
    if (total < best_cost) {
      best_cost = total;
      best = cur.node;
    }
    induced = induced + total;
    if (induced + sarea < best_cost && !cn.isLeafFlag) {
      if ((uint32_t)size + 2 <= cap) {
        pq[size].node = cn.left; pq[size].cost = induced;
        pq[size + 1].node = cn.right; pq[size + 1].cost = induced;
        heap_push(pq, size + 1);
        heap_push(pq, size + 2);
        size += 2;
      } else {
        (*overflow)++;
      }
    }
  }
  return best;
}

/* removeNode (Bittner13CUDA.cu:267-305). out: ins[2], unused[2], grand parent. */
static int gpu_remove(bpatch *p, uint32_t x, uint32_t ins[2], uint32_t un[2], uint32_t *g_out) {
  if (p->t[x].isLeafFlag || x == p->root) return 0;
  npatch *nn = bp_patch_node(p, x, P_NODE);
  uint32_t s = bp_sibling(p, nn);
  uint32_t pi = nn->parent;
  if (pi == p->root) return 0;
  npatch *sp = bp_patch_node(p, s, P_SIBLING);
  npatch *pp = bp_patch_node(p, pi, P_PARENT);
  uint32_t gi = pp->parent;
  npatch *gp = bp_patch_node(p, gi, P_GRAND_PARENT);
  if (pp->isLeft) {
    gp->left = s;
    sp->isLeft = 1;
  } else {
    gp->right = s;
    sp->isLeft = 0;
  }
  sp->parent = gi;
  bp_patch_aabb_from(p, gi, 0);
  if (p->t[nn->left].surfaceArea > p->t[nn->right].surfaceArea) { ins[0] = nn->left; ins[1] = nn->right; }
  else { ins[0] = nn->right; ins[1] = nn->left; }
  un[0] = x;
  un[1] = pi;
  *g_out = gi;
  return 1;
}

/* Batched best-first search (the GPU kernels' default search). Same cost model and pruning as
 * findNode1, but in rounds over the whole frontier: every frontier entry whose bound cost + SA(n)
 * is below the best total so far is evaluated; the best total among them (ties: the entry first
 * in (cost, node) order) replaces the best if strictly smaller; every evaluated inner node whose
 * induced cost still passes the bound against the updated best pushes both children; if more
 * than BF_CAP children were pushed, the BF_CAP lowest in (cost, node) order are kept (the rest
 * are counted as overflow). The frontier's order plays no other part. */
#define BF_CAP 128

typedef struct fent {
  float c;
  uint32_t n;
} fent;

static int fent_cmp(const void *a, const void *b) {
  const fent *x = a, *y = b;
  if (x->c < y->c) return -1;
  if (x->c > y->c) return 1;
  return x->n < y->n ? -1 : (x->n > y->n);
}

static uint32_t gpu_find_node_batched(const bpatch *p, uint32_t n, uint64_t *overflow, uint64_t *visits) {
  float best_cost = INFINITY;
  uint32_t best = 0;
  const orc_node *nd = &p->t[n];
  orc_aabb nbox = nd->bbox;
  float sarea = nd->surfaceArea;
  fent f[BF_CAP], nf[2 * BF_CAP];
  size_t fn = 1;
  f[0].c = 0.0f;
  f[0].n = p->root;
  for (;;) {
    float tot[BF_CAP], ind[BF_CAP];
    npatch cn[BF_CAP];
    size_t cand[BF_CAP], nv = 0;
    for (size_t i = 0; i < fn; ++i)
      if (f[i].c + sarea < best_cost) cand[nv++] = i;
    if (nv == 0) break;
    if (visits) *visits += nv;
    size_t bi = 0;
    for (size_t v = 0; v < nv; ++v) {
      const fent *e = &f[cand[v]];
      cn[v] = bp_get_subset(p, e->n);
      orc_aabb b = bp_get_aabb(p, e->n);
      float induced = -1.0f * orc_surface_area(&b);
      merge_into(&b, &nbox);
      float direct = orc_surface_area(&b);
      tot[v] = e->c + direct;
      ind[v] = induced + tot[v];
      if (v > 0 && (tot[v] < tot[bi] || (tot[v] == tot[bi] && fent_cmp(e, &f[cand[bi]]) < 0))) bi = v;
    }
    if (tot[bi] < best_cost) {
      best_cost = tot[bi];
      best = f[cand[bi]].n;
    }
    size_t m = 0;
    for (size_t v = 0; v < nv; ++v) {
      if (cn[v].isLeafFlag || !(ind[v] + sarea < best_cost)) continue;
      nf[m].c = ind[v]; nf[m].n = cn[v].left; m++;
      nf[m].c = ind[v]; nf[m].n = cn[v].right; m++;
    }
    if (m > BF_CAP) {
      qsort(nf, m, sizeof(fent), fent_cmp);
      *overflow += m - BF_CAP;
      m = BF_CAP;
    }
    memcpy(f, nf, m * sizeof(fent));
    fn = m;
  }
  return best;
}

/* reinsert (Bittner13CUDA.cu:308-358). mode 0: batched search, 1: findNode1 heap order. */
/* findNode2 (Bittner13CUDA.cu:194-264, the same as Bittner13Par.cpp:131-187 with its queue of
 * altFindNodeQueueSize entries): the approximate search of altFindNode. A fixed array of qsize
 * (cost, node) slots, empty = +inf; each step pops the first slot of smallest cost; an expanded
 * node's left child takes the popped slot and its right child the slot that the previous scan
 * found to hold the largest cost (the first empty one while there is one, else the worst entry,
 * which is dropped); the scan keeps its previous max slot when no cost exceeds 0. */
#define ALT_QUEUE_MAX 64
static uint32_t gpu_find_node_alt(const bpatch *p, uint32_t n, uint32_t qsize, uint64_t *visits) {
  float best_cost = INFINITY;
  uint32_t best = 0;
  const orc_node *nd = &p->t[n];
  orc_aabb nbox = nd->bbox;
  float sarea = nd->surfaceArea;
  float co[ALT_QUEUE_MAX];
  uint32_t nl[ALT_QUEUE_MAX];
  if (qsize > ALT_QUEUE_MAX) qsize = ALT_QUEUE_MAX;
  for (uint32_t i = 0; i < qsize; ++i) { co[i] = INFINITY; nl[i] = 0; }
  uint32_t mn_i = 0, mx_i = 1;
  float mn = 0.0f;
  nl[0] = p->root;
  co[0] = 0.0f;
  while (mn < INFINITY) {
    const uint32_t cur = nl[mn_i];
    const float cc = co[mn_i];
    co[mn_i] = INFINITY;
    if (cc + sarea >= best_cost) break;
    if (visits) (*visits)++;
    npatch cn = bp_get_subset(p, cur);
    orc_aabb b = bp_get_aabb(p, cur);
    float induced = -1.0f * orc_surface_area(&b);
    merge_into(&b, &nbox);
    float direct = orc_surface_area(&b);
    float total = cc + direct;
    if (total < best_cost) {
      best_cost = total;
      best = cur;
    }
    induced = induced + total;
    if (induced + sarea < best_cost && !cn.isLeafFlag) {
      nl[mn_i] = cn.left;
      nl[mx_i] = cn.right;
      co[mn_i] = induced;
      co[mx_i] = induced;
    }
    mn = INFINITY;
    float mx = 0.0f;
    for (uint32_t i = 0; i < qsize; ++i) {
      if (co[i] < mn) { mn = co[i]; mn_i = i; }
      if (co[i] > mx) { mx = co[i]; mx_i = i; }
    }
  }
  return best;
}

static int gpu_reinsert(bpatch *p, uint32_t x, uint32_t unused, int update, hitem *pq, uint32_t cap,
                        uint64_t *overflow, int mode, uint64_t *visits) {
  uint32_t best = mode == 0   ? gpu_find_node_batched(p, x, overflow, visits)
                  : mode == 2 ? gpu_find_node_alt(p, x, cap, visits)
                              : gpu_find_node(p, x, pq, cap, overflow);
  if (best == p->root) return 0;
  uint32_t bpi = bp_index(p, best);
  npatch *b;
  if (bpi == NONE) b = bp_patch_node(p, best, update ? P_1ST_BEST : P_2ND_BEST);
  else if (bpi == P_GRAND_PARENT) b = &p->nd[P_GRAND_PARENT];
  else b = bp_move(p, bpi, update ? P_1ST_BEST : P_2ND_BEST);
  npatch *nn = bp_patch_node(p, x, update ? P_1ST_INSERT : P_2ND_INSERT);
  npatch *u = &p->nd[update ? P_NODE : P_PARENT];
  uint32_t ri = b->parent;
  uint32_t rpi = bp_index(p, ri);
  npatch *r = rpi == NONE ? bp_patch_node(p, ri, update ? P_1ST_ROOT : P_2ND_ROOT)
                          : bp_move(p, rpi, update ? P_1ST_ROOT : P_2ND_ROOT);
  if (b->isLeft) {
    r->left = unused;
    u->isLeft = 1;
  } else {
    r->right = unused;
    u->isLeft = 0;
  }
  u->parent = ri;
  u->left = best;
  u->right = x;
  b->parent = unused;
  b->isLeft = 1;
  nn->parent = unused;
  nn->isLeft = 0;
  if (update) bp_patch_aabb_from(p, unused, 1);
  return 1;
}

static int cmp_u32(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : x > y;
}

typedef struct dnode {
  uint32_t depth, idx;
} dnode;
static int cmp_depth_desc(const void *a, const void *b) {
  const dnode *x = a, *y = b;
  if (x->depth != y->depth) return x->depth > y->depth ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* kFixTree3_1/3_2 (Bittner13CUDA.cu:407-467): refit every node on a path from a fix node to
 * the root, children first. Same boxes as the full refit of kFixTree1. */
static void refit_paths(orc_node *t, uint32_t root, const uint32_t *fix, uint32_t nfix, uint8_t *mark,
                        dnode *buf) {
  uint32_t nd = 0;
  for (uint32_t i = 0; i < nfix; ++i) {
    uint32_t x = fix[i];
    if (x == NONE) continue;
    for (;;) {
      if (mark[x]) break;
      mark[x] = 1;
      buf[nd].idx = x;
      buf[nd].depth = 0;
      nd++;
      if (x == root || t[x].parent == x) break;
      x = t[x].parent;
    }
  }
  for (uint32_t i = 0; i < nd; ++i) {
    uint32_t x = buf[i].idx, d = 0;
    while (x != root && t[x].parent != x) { x = t[x].parent; d++; }
    buf[i].depth = d;
  }
  qsort(buf, nd, sizeof(dnode), cmp_depth_desc);
  for (uint32_t i = 0; i < nd; ++i) {
    orc_node *x = &t[buf[i].idx];
    mark[buf[i].idx] = 0;
    if (x->isLeafFlag) continue;
    orc_aabb b = t[x->left].bbox;
    merge_into(&b, &t[x->right].bbox);
    x->bbox = b;
    x->surfaceArea = orc_surface_area(&b);
  }
}

/* One iteration of the chunked algorithm over a given batch order (order[pos] = the node at batch
 * position pos, as the sorted todo list of bn13_selectNodes). Work buffers live in w. */
typedef struct chunk_work {
  bpatch *patches;
  uint8_t *valid;
  uint32_t *fix, *owner;
  uint8_t *mark;
  dnode *dbuf;
  hitem *pqs;
  uint64_t *ovf, *vis;
  uint32_t nthreads;
} chunk_work;

static void chunk_work_init(chunk_work *w, uint32_t n_nodes, uint32_t csize, uint32_t cap) {
  w->patches = malloc(sizeof(bpatch) * (csize ? csize : 1));
  w->valid = malloc(csize ? csize : 1);
  w->fix = malloc(sizeof(uint32_t) * 3 * (csize ? csize : 1));
  w->owner = malloc(sizeof(uint32_t) * (n_nodes ? n_nodes : 1));
  w->mark = calloc(n_nodes ? n_nodes : 1, 1);
  w->dbuf = malloc(sizeof(dnode) * (n_nodes ? n_nodes : 1));
  for (uint32_t i = 0; i < n_nodes; ++i) w->owner[i] = NONE;
  w->nthreads = (uint32_t)orc_num_threads();
  w->pqs = malloc(sizeof(hitem) * cap * w->nthreads);
  w->ovf = calloc(w->nthreads, sizeof(uint64_t));
  w->vis = calloc(w->nthreads, sizeof(uint64_t));
}

static void chunk_work_free(chunk_work *w, orc_bn13_stats *st) {
  for (uint32_t i = 0; i < w->nthreads; ++i) {
    st->heap_overflow += w->ovf[i];
    st->nodes_visited += w->vis[i];
  }
  free(w->patches); free(w->valid); free(w->fix); free(w->owner); free(w->mark); free(w->dbuf);
  free(w->pqs); free(w->ovf); free(w->vis);
}

static uint32_t chunk_size(uint32_t n_nodes, const orc_bn13_cfg *cfg, uint32_t *numc_out) {
  float bp = cfg->batch_percent;
  if (bp <= 0.01f) bp = 0.01f;
  if (bp >= 75.0f) bp = 75.0f;
  uint32_t numc = cfg->num_chunks ? cfg->num_chunks : 1;
  uint32_t lnum = (uint32_t)((bp / 100.0f) * (float)n_nodes);
  *numc_out = numc;
  return lnum / numc;
}

static void run_iteration(orc_node *t, uint32_t root, const uint32_t *order, uint32_t n_order, uint32_t numc,
                          uint32_t csize, uint32_t cap, const orc_bn13_cfg *cfg, chunk_work *w, orc_bn13_stats *st) {
  const int mode = (int)cfg->search_mode;
  for (uint32_t c = 0; c < numc; ++c) {
    /* kRemoveAndReinsert (:504-564) against the chunk-start tree. */
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t kk = 0; kk < (int64_t)csize; ++kk) {
      uint32_t k = (uint32_t)kk;
#ifdef _OPENMP
      int tid = omp_get_thread_num();
#else
      int tid = 0;
#endif
      hitem *pq = w->pqs + (size_t)cap * tid;
      uint32_t pos = cfg->offset_access ? k * numc + c : c * csize + k;
      uint32_t node = pos < n_order ? order[pos] : NONE;
      bpatch *p = &w->patches[k];
      p->t = t;
      p->root = root;
      bp_clear(p);
      w->valid[k] = 0;
      w->fix[3 * k] = w->fix[3 * k + 1] = w->fix[3 * k + 2] = NONE;
      if (node == NONE) continue;
      uint32_t ins[2], un[2], g;
      if (!gpu_remove(p, node, ins, un, &g)) continue;
      if (!gpu_reinsert(p, ins[0], un[0], 1, pq, cap, &w->ovf[tid], mode, &w->vis[tid])) continue;
      if (!gpu_reinsert(p, ins[1], un[1], 0, pq, cap, &w->ovf[tid], mode, &w->vis[tid])) continue;
      w->valid[k] = 1;
      w->fix[3 * k] = g;
      w->fix[3 * k + 1] = un[0];
      w->fix[3 * k + 2] = un[1];
    }
    /* Conflict rule 0: claim every patched node with the item's rank; lowest rank wins.
     * Rule 1: in batch order, an item takes its nodes only if none is taken yet. */
    for (uint32_t k = 0; k < csize; ++k) {
      if (!w->valid[k]) continue;
      if (cfg->conflict_rule == 1) {
        int free_all = 1;
        for (int s = 0; s < NNODE; ++s) {
          uint32_t x = w->patches[k].idx[s];
          if (x != NONE && w->owner[x] != NONE) free_all = 0;
        }
        if (!free_all) continue;
      }
      for (int s = 0; s < NNODE; ++s) {
        uint32_t x = w->patches[k].idx[s];
        if (x != NONE && k < w->owner[x]) w->owner[x] = k;
      }
    }
    uint32_t nwin = 0;
    for (uint32_t k = 0; k < csize; ++k) {
      st->items++;
      if (!w->valid[k]) { st->skipped_invalid++; continue; }
      int ok = 1;
      for (int s = 0; s < NNODE; ++s) {
        uint32_t x = w->patches[k].idx[s];
        if (x != NONE && w->owner[x] != k) ok = 0;
      }
      if (!ok) {
        st->skipped_conflict++;
        w->valid[k] = 0;
        w->fix[3 * k] = w->fix[3 * k + 1] = w->fix[3 * k + 2] = NONE;
        continue;
      }
      nwin++;
    }
    /* kApplyPatches (:612-627) for the winners, then release every claim. */
    for (uint32_t k = 0; k < csize; ++k) {
      for (int s = 0; s < NNODE; ++s) {
        uint32_t x = w->patches[k].idx[s];
        if (x == NONE) continue;
        if (w->valid[k]) {
          t[x].parent = w->patches[k].nd[s].parent;
          t[x].left = w->patches[k].nd[s].left;
          t[x].right = w->patches[k].nd[s].right;
          t[x].isLeft = w->patches[k].nd[s].isLeft;
        }
      }
    }
    for (uint32_t k = 0; k < csize; ++k)
      for (int s = 0; s < NNODE; ++s)
        if (w->patches[k].idx[s] != NONE) w->owner[w->patches[k].idx[s]] = NONE;
    st->applied += nwin;
    refit_paths(t, root, w->fix, 3 * csize, w->mark, w->dbuf);
  }
}

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

int orc_bittner_chunked(orc_node *t, uint32_t n_nodes, uint32_t root, uint32_t iters,
                        const orc_bn13_cfg *cfg, double *sah_trace, orc_bn13_stats *stats) {
  return orc_bittner_chunked_until(t, n_nodes, root, iters, cfg, 0.0, sah_trace, NULL, stats, NULL);
}

int orc_bittner_chunked_until(orc_node *t, uint32_t n_nodes, uint32_t root, uint32_t iters,
                              const orc_bn13_cfg *cfg, double stop_sah, double *sah_trace, double *iter_ms,
                              orc_bn13_stats *stats, uint32_t *done) {
  uint32_t numc;
  const uint32_t csize = chunk_size(n_nodes, cfg, &numc);
  const uint32_t cap = cfg->heap_cap ? cfg->heap_cap : 4096;
  orc_bn13_stats st;
  memset(&st, 0, sizeof(st));

  /* initData (Bittner13CUDA.cu:939-987): the inner-node list in ascending index order. */
  uint32_t n_inner = 0;
  for (uint32_t i = 0; i < n_nodes; ++i) n_inner += t[i].isLeafFlag == 0;
  uint32_t *inner = malloc(sizeof(uint32_t) * (n_inner ? n_inner : 1));
  for (uint32_t i = 0, j = 0; i < n_nodes; ++i) if (!t[i].isLeafFlag) inner[j++] = i;
  cost_item *todo = malloc(sizeof(cost_item) * (n_inner ? n_inner : 1));
  uint32_t *order = malloc(sizeof(uint32_t) * (n_inner ? n_inner : 1));
  uint32_t *order_all = cfg->std_select ? malloc(sizeof(uint32_t) * (n_nodes ? n_nodes : 1)) : NULL;
  chunk_work w;
  chunk_work_init(&w, n_nodes, csize, cap);

  if (sah_trace) sah_trace[0] = orc_sah(t, n_nodes, root);
  uint32_t it = 0;
  for (; it < iters; ++it) {
    const double t0 = now_ms();
    uint32_t n_order = n_inner;
    if (cfg->std_select) {
      /* Bittner13Par.cpp:421-437: nth_element + sort of the chunk-rounded batch over all nodes. */
      n_order = orc_std_select(t, n_nodes, numc * csize, 1, order_all);
      run_iteration(t, root, order_all, n_order, numc, csize, cap, cfg, &w, &st);
    } else {
      /* bn13_selectNodes (:659-726): kCalcCost + stable descending sort of (cost, node). */
      for (uint32_t j = 0; j < n_inner; ++j) {
        todo[j].idx = inner[j];
        todo[j].cost = orc_inefficiency(t, inner[j]);
      }
      qsort(todo, n_inner, sizeof(cost_item), cmp_cost_desc);
      for (uint32_t j = 0; j < n_inner; ++j) order[j] = todo[j].idx;
      run_iteration(t, root, order, n_order, numc, csize, cap, cfg, &w, &st);
    }
    if (iter_ms) iter_ms[it] = now_ms() - t0;
    if (sah_trace || stop_sah > 0.0) {
      const double sah = orc_sah(t, n_nodes, root);
      if (sah_trace) sah_trace[it + 1] = sah;
      if (stop_sah > 0.0 && sah <= stop_sah) {
        ++it;
        break;
      }
    }
  }
  if (done) *done = it;
  chunk_work_free(&w, &st);
  if (stats) *stats = st;
  free(inner); free(todo); free(order); free(order_all);
  (void)cmp_u32;
  return 0;
}

int orc_bittner_iteration_ordered(orc_node *t, uint32_t n_nodes, uint32_t root, const uint32_t *order,
                                  uint32_t n_order, const orc_bn13_cfg *cfg, orc_bn13_stats *stats) {
  uint32_t numc;
  const uint32_t csize = chunk_size(n_nodes, cfg, &numc);
  const uint32_t cap = cfg->heap_cap ? cfg->heap_cap : 4096;
  orc_bn13_stats st;
  memset(&st, 0, sizeof(st));
  chunk_work w;
  chunk_work_init(&w, n_nodes, csize, cap);
  run_iteration(t, root, order, n_order, numc, csize, cap, cfg, &w, &st);
  chunk_work_free(&w, &st);
  if (stats) *stats = st;
  return 0;
}

/* ---- isolated realised gain of one reinsertion ---------------------------------------------
 * The patch changes the children of three nodes only: the grand parent (its child becomes the
 * sibling) and the two reused nodes (new parents of the reinserted children). A node's box changes
 * iff it lies on a path from one of these to the root in the patched tree, and only those nodes'
 * surface areas change, so the SAH reduction (cInner = 1) is the sum of old minus new surface
 * area over the union of the three paths, divided by the root's area. The union is a tree with at
 * most two join points: path 1 (from the first reused node) meets path 0 (from the grand parent) at
 * J1 = lca(s1, s0); path 2 meets path 0 or the private part of path 1 at J2, the deeper of
 * lca(s2, s0) and lca(s2, s1). New boxes are computed bottom-up in the order: private part of
 * path 2, private part of path 1, path 0 to the root; a child's new box is the running box of the
 * walk, the last box of a private part at its join node, or else the child's unchanged box. */
typedef struct gwalk {
  uint32_t prev, last1, j1, last2, j2;
  orc_aabb prevbox, box1, box2;
} gwalk;

static uint32_t np_parent(const bpatch *p, uint32_t x) { return bp_get(p, x).parent; }

static int new_depth(const bpatch *p, uint32_t x, uint32_t n_nodes, uint32_t *d) {
  uint32_t k = 0;
  while (x != p->root) {
    if (x >= n_nodes || k > n_nodes) return 0;
    x = np_parent(p, x);
    k++;
  }
  *d = k;
  return 1;
}

static uint32_t lca(const bpatch *p, uint32_t a, uint32_t da, uint32_t b, uint32_t db, uint32_t *dout) {
  while (da > db) { a = np_parent(p, a); da--; }
  while (db > da) { b = np_parent(p, b); db--; }
  while (a != b && da > 0) { a = np_parent(p, a); b = np_parent(p, b); da--; }
  *dout = da;
  return a;
}

static orc_aabb child_box(const bpatch *p, const gwalk *w, uint32_t x, uint32_t c) {
  if (c == w->prev) return w->prevbox;
  if (x == w->j1 && c == w->last1) return w->box1;
  if (x == w->j2 && c == w->last2) return w->box2;
  return p->t[c].bbox;
}

/* Walk from x up to (not including) stop, or through the root when stop is NONE. */
static void gain_walk(const bpatch *p, gwalk *w, uint32_t x, uint32_t stop, uint32_t n_nodes, double *acc, int *ok) {
  w->prev = NONE;
  for (uint32_t k = 0; x != stop; ++k) {
    if (x >= n_nodes || k > n_nodes) { *ok = 0; return; }
    npatch n = bp_get(p, x);
    if (n.left >= n_nodes || n.right >= n_nodes) { *ok = 0; return; }
    orc_aabb b = child_box(p, w, x, n.left);
    orc_aabb rb = child_box(p, w, x, n.right);
    merge_into(&b, &rb);
    *acc += (double)p->t[x].surfaceArea - (double)orc_surface_area(&b);
    w->prev = x;
    w->prevbox = b;
    if (x == p->root) return;
    x = n.parent;
  }
}

static float isolated_gain(const bpatch *p, uint32_t s0, uint32_t s1, uint32_t s2, uint32_t n_nodes, int *ok) {
  uint32_t d0, d1, d2, dj1, d20, d21;
  if (!new_depth(p, s0, n_nodes, &d0) || !new_depth(p, s1, n_nodes, &d1) || !new_depth(p, s2, n_nodes, &d2)) {
    *ok = 0;
    return 0.0f;
  }
  const uint32_t j1 = lca(p, s1, d1, s0, d0, &dj1);
  const uint32_t l20 = lca(p, s2, d2, s0, d0, &d20);
  const uint32_t l21 = lca(p, s2, d2, s1, d1, &d21);
  const uint32_t j2 = d20 >= d21 ? l20 : l21;
  gwalk w;
  memset(&w, 0, sizeof(w));
  w.last1 = w.j1 = w.last2 = w.j2 = NONE;
  double acc = 0.0;
  gain_walk(p, &w, s2, j2, n_nodes, &acc, ok);
  w.last2 = w.prev;
  w.box2 = w.prevbox;
  w.j2 = j2;
  gain_walk(p, &w, s1, j1, n_nodes, &acc, ok);
  w.last1 = w.prev;
  w.box1 = w.prevbox;
  w.j1 = j1;
  gain_walk(p, &w, s0, NONE, n_nodes, &acc, ok);
  if (!*ok) return 0.0f;
  return (float)(acc / (double)p->t[p->root].surfaceArea);
}

void orc_bn13_gains(const orc_node *t, uint32_t n_nodes, uint32_t root, const uint32_t *cand, uint32_t n,
                    float *gain, uint8_t *ok_out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    bpatch p;
    p.t = t;
    p.root = root;
    bp_clear(&p);
    uint64_t ovf = 0, vis = 0;
    uint32_t ins[2], un[2], g;
    const uint32_t x = cand[i];
    int ok = x < n_nodes && gpu_remove(&p, x, ins, un, &g) && gpu_reinsert(&p, ins[0], un[0], 1, NULL, 0, &ovf, 0, &vis) &&
             gpu_reinsert(&p, ins[1], un[1], 0, NULL, 0, &ovf, 0, &vis);
    float v = 0.0f;
    if (ok) v = isolated_gain(&p, g, un[0], un[1], n_nodes, &ok);
    gain[i] = ok ? v : 0.0f;
    if (ok_out) ok_out[i] = (uint8_t)ok;
  }
}
