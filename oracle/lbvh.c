/*
 * Oracle (test infrastructure only): LBVH build, SAH, levels and the Validate command,
 * restated in plain C from the reference's files cited per function. Parity unpinned: see
 * oracle.h.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* AABB::surfaceArea (lib/base/BVH.hpp:62-65): 2 * (dx*dy + dx*dz + dy*dz), each product and
 * sum rounded separately (the file is compiled with -ffp-contract=off). */
float orc_surface_area(const orc_aabb *b) {
  float dx = b->mx[0] - b->mn[0];
  float dy = b->mx[1] - b->mn[1];
  float dz = b->mx[2] - b->mn[2];
  float xy = dx * dy;
  float xz = dx * dz;
  float yz = dy * dz;
  float s = xy + xz;
  s = s + yz;
  return 2.0f * s;
}

/* AABB::mergeWith (BVH.hpp:67-74): a = a < b ? a : b per component for the minimum,
 * a > b ? a : b for the maximum; 'a' is the box being grown. */
static void merge_into(orc_aabb *a, const orc_aabb *b) {
  for (int k = 0; k < 3; ++k) {
    a->mn[k] = a->mn[k] < b->mn[k] ? a->mn[k] : b->mn[k];
    a->mx[k] = a->mx[k] > b->mx[k] ? a->mx[k] : b->mx[k];
  }
}

/* kInitTriData (LBVH_CUDA.cu:60-96) for one triangle. */
static void tri_box(const float *vert, const uint32_t *face, orc_aabb *box, float *centroid) {
  const float *v1 = vert + 3 * (size_t)face[0];
  const float *v2 = vert + 3 * (size_t)face[1];
  const float *v3 = vert + 3 * (size_t)face[2];
  for (int k = 0; k < 3; ++k) {
    float mn = v1[k];
    float mx = v2[k];
    if (v2[k] < mn) mn = v2[k];
    if (v3[k] < mn) mn = v3[k];
    if (v1[k] > mx) mx = v1[k];
    if (v3[k] > mx) mx = v3[k];
    box->mn[k] = mn - FLT_EPSILON;
    box->mx[k] = mx + FLT_EPSILON;
    if (centroid) {
      float s = v1[k] + v2[k];
      s = s + v3[k];
      centroid[k] = s / 3.0f;
    }
  }
}

void orc_tri_data(const float *vert, const uint32_t *faces, uint32_t n, orc_aabb *bbox_out,
                  float *centroid_out, orc_aabb *scene_out) {
  /* ReduceRootAABB over all triangle boxes, initial value = the box [(0,0,0),(0,0,0)]
   * (LBVH_CUDA.cu:104-106,112-113). min/max are exact, so the order does not matter. */
  orc_aabb scene = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
#pragma omp parallel
  {
    orc_aabb local = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
#pragma omp for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      orc_aabb b;
      float c[3];
      tri_box(vert, faces + 3 * i, &b, c);
      if (bbox_out) bbox_out[i] = b;
      if (centroid_out) memcpy(centroid_out + 3 * i, c, sizeof(c));
      merge_into(&local, &b);
    }
#pragma omp critical
    merge_into(&scene, &local);
  }
  if (scene_out) *scene_out = scene;
}

/* LBVH_calcMortonCodes host part (LBVH_CUDA.cu:168-180). */
void orc_morton_params(const orc_aabb *scene, float offset[3], float scale[3]) {
  for (int k = 0; k < 3; ++k) {
    offset[k] = 0.0f - scene->mn[k];
    float mx = scene->mx[k] + offset[k];
    scale[k] = 1.0f / mx;
  }
}

/* Bit interleave written as a plain loop (the reference uses multiply/mask magic numbers,
 * LBVH_CUDA.cu:132-138; both insert two zeros after every input bit). */
static uint64_t spread3(uint64_t v, int bits) {
  uint64_t r = 0;
  for (int b = 0; b < bits; ++b) r |= ((v >> b) & 1ull) << (3 * b);
  return r;
}

/* kCalcMortonCodes (LBVH_CUDA.cu:140-166) with 2^bits cells per axis. */
static uint32_t quantise(float c, float off, float scale, float cells, float maxcell) {
  c = c + off;
  c = c * scale;
  c = c * cells;
  if (c < 0.0f) c = 0.0f;
  if (c > maxcell) c = maxcell;
  return (uint32_t)c;
}

void orc_morton30(const float *centroid, uint32_t n, const float offset[3], const float scale[3],
                  uint32_t *codes) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint32_t q[3];
    for (int k = 0; k < 3; ++k)
      q[k] = quantise(centroid[3 * i + k], offset[k], scale[k], 1024.0f, 1023.0f);
    /* x * 4 + y * 2 + z (LBVH_CUDA.cu:164) */
    codes[i] = (uint32_t)(spread3(q[0], 10) * 4u + spread3(q[1], 10) * 2u + spread3(q[2], 10));
  }
}

void orc_morton63(const float *centroid, uint32_t n, const float offset[3], const float scale[3],
                  uint64_t *codes) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint32_t q[3];
    for (int k = 0; k < 3; ++k)
      q[k] = quantise(centroid[3 * i + k], offset[k], scale[k], 2097152.0f, 2097151.0f);
    codes[i] = spread3(q[0], 21) * 4u + spread3(q[1], 21) * 2u + spread3(q[2], 21);
  }
}

/* Stable ascending LSD radix sort, 8 bits per pass (the semantics of cub::DeviceRadixSort). */
static void lsd_sort(const void *keys, int key_bytes, uint32_t n, void *keys_out, uint32_t *vals_out) {
  size_t kb = (size_t)key_bytes;
  uint8_t *ka = malloc(kb * (n ? n : 1)), *kbuf = malloc(kb * (n ? n : 1));
  uint32_t *va = malloc(sizeof(uint32_t) * (n ? n : 1)), *vb = malloc(sizeof(uint32_t) * (n ? n : 1));
  memcpy(ka, keys, kb * n);
  for (uint32_t i = 0; i < n; ++i) va[i] = i;
  for (int pass = 0; pass < key_bytes; ++pass) {
    size_t cnt[257];
    memset(cnt, 0, sizeof(cnt));
    for (uint32_t i = 0; i < n; ++i) cnt[ka[(size_t)i * kb + pass] + 1]++;
    for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
    for (uint32_t i = 0; i < n; ++i) {
      size_t dst = cnt[ka[(size_t)i * kb + pass]]++;
      memcpy(kbuf + dst * kb, ka + (size_t)i * kb, kb);
      vb[dst] = va[i];
    }
    uint8_t *t = ka; ka = kbuf; kbuf = t;
    uint32_t *tv = va; va = vb; vb = tv;
  }
  if (keys_out) memcpy(keys_out, ka, kb * n);
  if (vals_out) memcpy(vals_out, va, sizeof(uint32_t) * n);
  free(ka); free(kbuf); free(va); free(vb);
}

void orc_sort_pairs32(const uint32_t *keys, uint32_t n, uint32_t *keys_out, uint32_t *vals_out) {
  lsd_sort(keys, 4, n, keys_out, vals_out);
}
void orc_sort_pairs64(const uint64_t *keys, uint32_t n, uint64_t *keys_out, uint32_t *vals_out) {
  lsd_sort(keys, 8, n, keys_out, vals_out);
}

/* ---- Karras topology (LBVH_CUDA.cu:205-324) ----------------------------------------------- */

typedef struct topo_ctx {
  const uint32_t *k32;
  const uint64_t *k64;
  uint32_t n;
  int mode;
} topo_ctx;

static int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }
static int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

/* delta(i, j) (LBVH_CUDA.cu:208-212). refCompat: __clz(int) applied to the 64-bit
 * (morton << 32 | index) XOR keeps only its low 32 bits, i.e. clz32(i ^ j). karras: the
 * common-prefix length of the full (morton, index) key. */
static int32_t delta(const topo_ctx *c, uint32_t i, uint32_t j) {
  if (j >= c->n) return -1;
  if (c->mode == ORC_TOPO_REFCOMPAT) return clz32(i ^ j);
  if (c->k64) {
    uint64_t a = c->k64[i], b = c->k64[j];
    if (a != b) return clz64(a ^ b);
    return 64 + clz32(i ^ j);
  }
  uint32_t a = c->k32[i], b = c->k32[j];
  if (a != b) return clz32(a ^ b);
  return 32 + clz32(i ^ j);
}

/* findSplit (LBVH_CUDA.cu:214-246). The keys compared are unique (index-augmented), so the
 * reference's "identical codes" early exit never triggers. */
static uint32_t find_split(const topo_ctx *c, uint32_t first, uint32_t last) {
  int32_t common = delta(c, first, last);
  uint32_t split = first;
  uint32_t step = last - first;
  do {
    step = (step + 1) >> 1;
    uint32_t ns = split + step;
    if (ns < last) {
      if (delta(c, first, ns) > common) split = ns;
    }
  } while (step > 1);
  return split;
}

/* determineRange (LBVH_CUDA.cu:249-271), all index arithmetic in wrapping uint32. */
static void determine_range(const topo_ctx *c, uint32_t i, uint32_t *lo, uint32_t *hi) {
  int32_t dd = delta(c, i, i + 1) - delta(c, i, i - 1);
  int32_t d = dd > 0 ? 1 : -1;
  uint32_t du = (uint32_t)d;
  int32_t dmin = delta(c, i, i - du);
  uint32_t lmax = 2;
  while (delta(c, i, i + lmax * du) > dmin) lmax *= 2;
  uint32_t l = 0;
  do {
    lmax >>= 1;
    if (delta(c, i, i + (l + lmax) * du) > dmin) l += lmax;
  } while (lmax > 1);
  uint32_t j = i + l * du;
  if (i < j) { *lo = i; *hi = j; } else { *lo = j; *hi = i; }
}

void orc_build_topology(const uint32_t *keys32, const uint64_t *keys64, uint32_t n, int mode,
                        orc_node *nodes) {
  topo_ctx c = {keys32, keys64, n, mode};
  if (n == 0) return;
  /* kBuildTree (LBVH_CUDA.cu:294-324): every inner node writes its children and the
   * children's parent / isLeft fields. */
#pragma omp parallel for schedule(static)
  for (int64_t ii = 0; ii < (int64_t)n - 1; ++ii) {
    uint32_t i = (uint32_t)ii, first, last;
    determine_range(&c, i, &first, &last);
    uint32_t split = find_split(&c, first, last);
    uint32_t a = split, b = split + 1;
    if (a == first) a += n - 1;
    if (b == last) b += n - 1;
    nodes[i].left = a;
    nodes[i].right = b;
    nodes[i].isLeafFlag = 0;
    nodes[i].level = 0;
    nodes[i].pad = 0;
    nodes[a].parent = i;
    nodes[a].isLeft = 1;
    nodes[b].parent = i;
    nodes[b].isLeft = 0;
  }
  /* The reference never writes the root's parent and relies on zero-filled memory for
   * root.parent == root (Validate.cpp:62, LBVH_CUDA.cu:370); it is written explicitly here. */
  nodes[0].parent = 0;
  nodes[0].isLeft = 0;
}

/* kGenLeafNodes (LBVH_CUDA.cu:273-292): leaf i of the sorted order lives at n - 1 + i. */
void orc_gen_leaves(const float *vert, const uint32_t *faces, const uint32_t *sorted_idx, uint32_t n,
                    orc_node *nodes) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    orc_node *nd = &nodes[n - 1 + i];
    uint32_t f = sorted_idx[i];
    tri_box(vert, faces + 3 * (size_t)f, &nd->bbox, NULL);
    nd->parent = UINT32_MAX;
    nd->isLeafFlag = 1;
    nd->left = f;
    nd->right = 1;
    nd->level = 255; /* UINT8_MAX stored into the uint16 level (LBVH_CUDA.cu:287) */
    nd->isLeft = 0;
    nd->pad = 0;
    nd->surfaceArea = orc_surface_area(&nd->bbox);
  }
}

/* kFixAABBTree (LBVH_CUDA.cu:341-374) evaluated children-first: bbox = left merged with
 * right, SA recomputed. Iterative pre-order, processed in reverse. */
void orc_refit(orc_node *nodes, uint32_t n_nodes, uint32_t root) {
  if (n_nodes == 0) return;
  uint32_t *order = malloc(sizeof(uint32_t) * n_nodes);
  uint32_t *stack = malloc(sizeof(uint32_t) * (n_nodes + 1));
  uint32_t no = 0, sp = 0;
  stack[sp++] = root;
  while (sp && no < n_nodes) {
    uint32_t x = stack[--sp];
    order[no++] = x;
    if (!nodes[x].isLeafFlag) {
      stack[sp++] = nodes[x].right;
      stack[sp++] = nodes[x].left;
    }
  }
  for (uint32_t k = no; k-- > 0;) {
    orc_node *x = &nodes[order[k]];
    if (x->isLeafFlag) continue;
    orc_aabb b = nodes[x->left].bbox;
    merge_into(&b, &nodes[x->right].bbox);
    x->bbox = b;
    x->surfaceArea = orc_surface_area(&b);
  }
  free(order);
  free(stack);
}

int orc_lbvh_build(const float *vert, const uint32_t *faces, uint32_t n, int morton_bits, int mode,
                   orc_node *nodes, void *sorted_keys_out, uint32_t *sorted_idx_out) {
  if (n == 0) return 0;
  if (morton_bits != 30 && morton_bits != 63) return -1;
  float *cen = malloc(sizeof(float) * 3 * (size_t)n);
  uint32_t *idx = malloc(sizeof(uint32_t) * n);
  orc_aabb scene;
  float off[3], sc[3];
  orc_tri_data(vert, faces, n, NULL, cen, &scene);
  orc_morton_params(&scene, off, sc);
  uint32_t *k32 = NULL, *s32 = NULL;
  uint64_t *k64 = NULL, *s64 = NULL;
  if (morton_bits == 30) {
    k32 = malloc(sizeof(uint32_t) * n);
    s32 = malloc(sizeof(uint32_t) * n);
    orc_morton30(cen, n, off, sc, k32);
    orc_sort_pairs32(k32, n, s32, idx);
  } else {
    k64 = malloc(sizeof(uint64_t) * n);
    s64 = malloc(sizeof(uint64_t) * n);
    orc_morton63(cen, n, off, sc, k64);
    orc_sort_pairs64(k64, n, s64, idx);
  }
  orc_gen_leaves(vert, faces, idx, n, nodes);
  orc_build_topology(s32, s64, n, mode, nodes);
  if (n == 1) { nodes[0].parent = 0; nodes[0].isLeft = 0; }
  orc_refit(nodes, 2 * n - 1, 0);
  if (sorted_keys_out) memcpy(sorted_keys_out, morton_bits == 30 ? (void *)s32 : (void *)s64,
                              (morton_bits == 30 ? 4u : 8u) * (size_t)n);
  if (sorted_idx_out) memcpy(sorted_idx_out, idx, sizeof(uint32_t) * n);
  free(cen); free(idx); free(k32); free(s32); free(k64); free(s64);
  return 0;
}

/* BVH::calcSAH (BVH.cpp:23-37). */
double orc_sah(const orc_node *nodes, uint32_t n_nodes, uint32_t root) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < (int64_t)n_nodes; ++i)
    if ((uint32_t)i != root) s += (double)nodes[i].surfaceArea;
  return s / (double)nodes[root].surfaceArea;
}

/* BVH::fixLevels (BVH.cpp:39-70). */
uint32_t orc_fix_levels(orc_node *nodes, uint32_t n_nodes, uint32_t root) {
  if (!n_nodes) return 0;
  uint32_t *st = malloc(sizeof(uint32_t) * (n_nodes + 1));
  uint32_t sp = 0, maxl = 0;
  nodes[root].level = 0;
  st[sp++] = root;
  while (sp) {
    uint32_t x = st[--sp];
    if (nodes[x].level > maxl) maxl = nodes[x].level;
    if (!nodes[x].isLeafFlag) {
      nodes[nodes[x].left].level = (uint16_t)(nodes[x].level + 1);
      nodes[nodes[x].right].level = (uint16_t)(nodes[x].level + 1);
      st[sp++] = nodes[x].right;
      st[sp++] = nodes[x].left;
    }
  }
  free(st);
  return maxl;
}

/* Validate::checkTree/checkBBoxes/checkBBoxesStrict/checkSurfaceArea/checkTris
 * (Validate.cpp:42-263). */
int orc_validate(const orc_node *nodes, uint32_t n_nodes, uint32_t root, const float *vert,
                 const uint32_t *faces, uint32_t n_faces, int check_levels, uint32_t errs[5]) {
  memset(errs, 0, 5 * sizeof(uint32_t));
  if (!n_nodes) return 0;
  /* checkTree */
  uint8_t *seen = calloc(n_nodes, 1);
  uint32_t *st = malloc(sizeof(uint32_t) * 2 * (n_nodes + 1));
  uint32_t sp = 0;
  if (nodes[root].parent != root) errs[0]++;
  st[sp++] = root;
  st[sp++] = 0;
  while (sp) {
    uint32_t lvl = st[--sp];
    uint32_t x = st[--sp];
    if (x >= n_nodes || seen[x]) { errs[0]++; continue; }
    seen[x] = 1;
    if (check_levels && nodes[x].level != lvl) errs[0]++;
    if (x != root) {
      const orc_node *p = &nodes[nodes[x].parent];
      if (nodes[x].isLeft && p->left != x) errs[0]++;
      if (!nodes[x].isLeft && p->right != x) errs[0]++;
    }
    if (!nodes[x].isLeafFlag) {
      const orc_node *nd = &nodes[x];
      if (nd->left == nd->right || nd->left == x || nd->right == x) { errs[0]++; continue; }
      if (nd->left >= n_nodes || nd->right >= n_nodes) { errs[0]++; continue; }
      if (nodes[nd->left].parent != x) errs[0]++;
      if (nodes[nd->right].parent != x) errs[0]++;
      st[sp++] = nd->right; st[sp++] = lvl + 1;
      st[sp++] = nd->left;  st[sp++] = lvl + 1;
    }
  }
  for (uint32_t i = 0; i < n_nodes; ++i) if (!seen[i]) errs[0]++;
  free(seen);
  free(st);
  /* checkBBoxes, checkBBoxesStrict, checkSurfaceArea */
  for (uint32_t i = 0; i < n_nodes; ++i) {
    const orc_node *nd = &nodes[i];
    float dsa = nd->surfaceArea - orc_surface_area(&nd->bbox);
    if (!(fabsf(dsa) < 0.000001f)) errs[3]++;
    if (nd->isLeafFlag) continue;
    if (nd->left >= n_nodes || nd->right >= n_nodes) { errs[1]++; errs[2]++; continue; }
    const orc_aabb *b = &nd->bbox, *l = &nodes[nd->left].bbox, *r = &nodes[nd->right].bbox;
    int e = 0, es = 0;
    for (int k = 0; k < 3; ++k) {
      if (!(b->mn[k] <= l->mn[k])) e++;
      if (!(b->mx[k] >= l->mx[k])) e++;
      if (!(b->mn[k] <= r->mn[k])) e++;
      if (!(b->mx[k] >= r->mx[k])) e++;
      if (!(b->mn[k] == fminf(l->mn[k], r->mn[k]))) es++;
      if (!(b->mx[k] == fmaxf(l->mx[k], r->mx[k]))) es++;
    }
    if (e) errs[1]++;
    if (es) errs[2]++;
  }
  /* checkTris */
  if (vert && faces) {
    uint8_t *cov = calloc(n_faces ? n_faces : 1, 1);
    for (uint32_t i = 0; i < n_nodes; ++i) {
      const orc_node *nd = &nodes[i];
      if (!nd->isLeafFlag) continue;
      int e = 0;
      for (uint32_t j = nd->left; j < nd->left + nd->right; ++j) {
        if (j >= n_faces) { e++; continue; }
        cov[j] = 1;
        for (int v = 0; v < 3; ++v) {
          const float *p = vert + 3 * (size_t)faces[3 * (size_t)j + v];
          for (int k = 0; k < 3; ++k)
            if (!(nd->bbox.mn[k] <= p[k]) || !(nd->bbox.mx[k] >= p[k])) e++;
        }
      }
      if (e) errs[4]++;
    }
    for (uint32_t j = 0; j < n_faces; ++j) if (!cov[j]) errs[4]++;
    free(cov);
  }
  return (int)(errs[0] + errs[1] + errs[2] + errs[3] + errs[4]);
}

/* adler32 (RFC 1950), used by the reference's BVH export format (BVHExport.cpp). */
uint32_t orc_adler32(const uint8_t *data, size_t len) {
  uint32_t a = 1, b = 0;
  for (size_t i = 0; i < len; ++i) {
    a = (a + data[i]) % 65521u;
    b = (b + a) % 65521u;
  }
  return (b << 16) | a;
}
