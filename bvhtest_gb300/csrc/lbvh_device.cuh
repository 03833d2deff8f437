// Device side of the LBVH build (lib/builder/LBVH_CUDA.cu), shared by the single-mesh kernels
// (lbvh.cu) and the batched ones (batch.cu).
#pragma once

#include "common.cuh"

namespace bvhgb {
namespace {

// kInitTriData (LBVH_CUDA.cu:60-96): box from the three vertices with the reference's compare
// order, grown by FLT_EPSILON; centroid ((v1 + v2) + v3) / 3.
__device__ __forceinline__ void tri_box(const float *__restrict__ vert, const uint32_t *__restrict__ faces, uint32_t f,
                                        Box &b, float *c) {
  uint32_t i1 = __ldg(faces + 3 * (size_t)f), i2 = __ldg(faces + 3 * (size_t)f + 1), i3 = __ldg(faces + 3 * (size_t)f + 2);
  float v1[3], v2[3], v3[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v1[k] = __ldg(vert + 3 * (size_t)i1 + k);
    v2[k] = __ldg(vert + 3 * (size_t)i2 + k);
    v3[k] = __ldg(vert + 3 * (size_t)i3 + k);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float mn = v1[k], mx = v2[k];
    if (v2[k] < mn) mn = v2[k];
    if (v3[k] < mn) mn = v3[k];
    if (v1[k] > mx) mx = v1[k];
    if (v3[k] > mx) mx = v3[k];
    b.mn[k] = fsub(mn, FLT_EPSILON);
    b.mx[k] = fadd(mx, FLT_EPSILON);
    if (c) c[k] = fdiv(fadd(fadd(v1[k], v2[k]), v3[k]), 3.0f);
  }
}

// Expands the low 10 / 21 bits of v so that two zero bits follow every bit.
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__device__ __forceinline__ uint64_t spread21(uint64_t v) {
  v &= 0x1FFFFFull;
  v = (v | (v << 32)) & 0x001F00000000FFFFull;
  v = (v | (v << 16)) & 0x001F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

// kCalcMortonCodes (LBVH_CUDA.cu:140-166): (c + offset) * scale * cells, clamped, truncated.
__device__ __forceinline__ uint32_t quantise(float c, float off, float scale, float cells, float maxcell) {
  c = fadd(c, off);
  c = fmul(c, scale);
  c = fmul(c, cells);
  if (c < 0.0f) c = 0.0f;
  if (c > maxcell) c = maxcell;
  return (uint32_t)c;
}

// Host part of LBVH_calcMortonCodes (LBVH_CUDA.cu:171-180) from the order-mapped scene box.
__device__ __forceinline__ void morton_params(const uint32_t *scene, float off[3], float sc[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float mn = ord2f(scene[k]), mx = ord2f(scene[3 + k]);
    off[k] = fsub(0.0f, mn);
    sc[k] = fdiv(1.0f, fadd(mx, off[k]));
  }
}

// 30-bit (10 per axis) or 63-bit (21 per axis) Morton key of a centroid (kCalcMortonCodes).
template <int BITS>
__device__ __forceinline__ uint64_t morton_key(const float c[3], const float off[3], const float sc[3]) {
  if (BITS == 30) {
    const uint32_t x = quantise(c[0], off[0], sc[0], 1024.0f, 1023.0f);
    const uint32_t y = quantise(c[1], off[1], sc[1], 1024.0f, 1023.0f);
    const uint32_t z = quantise(c[2], off[2], sc[2], 1024.0f, 1023.0f);
    return spread10(x) * 4u + spread10(y) * 2u + spread10(z);
  }
  const uint64_t x = quantise(c[0], off[0], sc[0], 2097152.0f, 2097151.0f);
  const uint64_t y = quantise(c[1], off[1], sc[1], 2097152.0f, 2097151.0f);
  const uint64_t z = quantise(c[2], off[2], sc[2], 2097152.0f, 2097151.0f);
  return spread21(x) * 4u + spread21(y) * 2u + spread21(z);
}

// delta(i, j) (LBVH_CUDA.cu:208-212) for in-range i != j.
template <int MODE, typename K>
__device__ __forceinline__ int delta(const K *__restrict__ keys, uint32_t i, uint32_t j) {
  if (MODE == BVHGB_TOPO_REFCOMPAT) return __clz((int)(i ^ j));
  K a = __ldg(keys + i), b = __ldg(keys + j);
  if (a != b) return sizeof(K) == 8 ? __clzll((long long)(a ^ b)) : __clz((int)(a ^ b));
  return (int)(8 * sizeof(K)) + __clz((int)(i ^ j));
}

// True when the node covering [l, r] is the LEFT child of its parent (parent split = r).
template <int MODE, typename K>
__device__ __forceinline__ bool parent_is_right(const K *keys, uint32_t l, uint32_t r, uint32_t n) {
  if (l == 0) return true;
  if (r == n - 1) return false;
  return delta<MODE, K>(keys, r, r + 1) > delta<MODE, K>(keys, l - 1, l);
}

__device__ __forceinline__ void store_record(bvhgb_node *nd, const Box &b, uint32_t parent, uint32_t left,
                                             uint32_t right, uint32_t leaf, uint32_t isLeft, uint32_t level) {
  float4 *p = reinterpret_cast<float4 *>(nd);
  float sa = surface_area(b);
  p[0] = make_float4(b.mn[0], b.mn[1], b.mn[2], b.mx[0]);
  p[1] = make_float4(b.mx[1], b.mx[2], __uint_as_float(parent), __uint_as_float(left));
  p[2] = make_float4(__uint_as_float(right), __uint_as_float(leaf | (isLeft << 16)), __uint_as_float(level),
                     sa);
}

__device__ __forceinline__ void set_parent(bvhgb_node *nd, uint32_t parent, uint16_t isLeft) {
  nd->parent = parent;
  nd->isLeft = isLeft;
}

// From node [l, r] with box 'box' (right: the node is its parent's left child, so the parent's
// split is r; otherwise l - 1) climb through the tree's exchange slots: at each split the first
// thread to arrive leaves its far end in the slot and stops; the second merges the boxes, writes
// the parent with the Karras node index the reference assigns and goes on (kBuildTree +
// kFixAABBTree, LBVH_CUDA.cu:273-374). The node [l, r] itself must already be written.
template <int MODE, typename K>
__device__ __forceinline__ void lbvh_climb_from(uint32_t l, uint32_t r, bool right, Box box, uint32_t n,
                                                const K *__restrict__ keys, bvhgb_node *nodes, uint32_t *slots,
                                                uint32_t *err) {
  // Each step strictly grows [l, r], so n - 1 steps reach the root; the bound and the range checks
  // turn corrupted exchange slots into an error, not a hang.
  for (uint32_t step = 0;; ++step) {
    const uint32_t split = right ? r : l - 1;
    const uint32_t other = atom_exch_acq_rel(&slots[split], right ? l : r);
    if (other == kNone) return;
    const uint32_t L = right ? l : other, R = right ? other : r;
    if (step >= n || L > split || split + 1 > R || R >= n) {
      atomicOr(err, kErrBadIndex);
      return;
    }
    const uint32_t a = (L == split) ? n - 1 + split : split;          // left child  [L, split]
    const uint32_t b = (split + 1 == R) ? n - 1 + split + 1 : split + 1;  // right child [split+1, R]
    const Box sib = load_box_cg(nodes + (right ? b : a));
    Box pb;
    if (right) { pb = box; merge_into(pb, sib); }   // left child's box merged with the right's
    else { pb = sib; merge_into(pb, box); }
    l = L;
    r = R;
    const bool root = (l == 0 && r == n - 1);
    uint32_t pidx = 0;
    if (!root) {
      right = parent_is_right<MODE, K>(keys, l, r, n);
      pidx = right ? r : l;  // Karras index: a left child is numbered by its last key, a right child by its first
    }
    store_record(nodes + pidx, pb, root ? 0u : kNone, a, b, 0u, 0u, 0u);
    set_parent(nodes + a, pidx, 1);
    set_parent(nodes + b, pidx, 0);
    if (root) return;
    box = pb;
  }
}

// One sorted leaf of a tree of n leaves: write the leaf (left = the face's index in its mesh) and
// climb (kGenLeafNodes + the climb above). keys, nodes and slots are the tree's own arrays.
template <int MODE, typename K>
__device__ __forceinline__ void lbvh_climb(uint32_t i, uint32_t n, const K *__restrict__ keys, uint32_t face,
                                           Box box, bvhgb_node *nodes, uint32_t *slots, uint32_t *err) {
  const uint32_t leafIdx = n - 1 + i;
  if (n == 1) {
    store_record(nodes + leafIdx, box, 0u, face, 1u, 1u, 0u, 255u);
    return;
  }
  store_record(nodes + leafIdx, box, kNone, face, 1u, 1u, 0u, 255u);
  lbvh_climb_from<MODE, K>(i, i, parent_is_right<MODE, K>(keys, i, i, n), box, n, keys, nodes, slots, err);
}

}  // namespace
}  // namespace bvhgb
