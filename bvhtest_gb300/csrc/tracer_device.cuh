// Device side of the closest-hit tracer (lib/tracer/CUDAKernels.cu:66-223, restated with a
// watertight triangle test and a short stack), shared by the single-tree kernels (tracer.cu) and
// the batched ones (batch.cu). Errors are OR-ed into the word the caller passes.
#pragma once

#include "common.cuh"

namespace bvhgb {
namespace {

constexpr int kStack = 96;
constexpr float kFarScale = 1.0000004f;   // 1 + 2 * gamma(3), gamma(n) = n u / (1 - n u), u = 2^-24
constexpr float kBestSlack = 1.0000153f;  // relative slack on the best t when culling boxes

struct RayPre {
  float o[3], d[3], inv[3];
  float sx, sy, sz;
  int kx, ky, kz;
};

__device__ __forceinline__ void setup_ray(RayPre &r) {
#pragma unroll
  for (int k = 0; k < 3; ++k) r.inv[k] = fdiv(1.0f, r.d[k]);
  float ax = fabsf(r.d[0]), ay = fabsf(r.d[1]), az = fabsf(r.d[2]);
  int kz = (ax >= ay) ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  float dz = kz == 0 ? r.d[0] : (kz == 1 ? r.d[1] : r.d[2]);
  if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  float dx = kx == 0 ? r.d[0] : (kx == 1 ? r.d[1] : r.d[2]);
  float dy = ky == 0 ? r.d[0] : (ky == 1 ? r.d[1] : r.d[2]);
  r.sx = fdiv(dx, dz);
  r.sy = fdiv(dy, dz);
  r.sz = fdiv(1.0f, dz);
}

__device__ __forceinline__ float pick(const float *v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }

// Watertight ray/triangle test; every operation rounds once (matches the oracle bit for bit).
__device__ __forceinline__ bool ray_tri(const RayPre &r, const float *v0, const float *v1, const float *v2, float tmin,
                                        float tmax, bool cull, float &tout) {
  float A[3], B[3], C[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    A[k] = fsub(v0[k], r.o[k]);
    B[k] = fsub(v1[k], r.o[k]);
    C[k] = fsub(v2[k], r.o[k]);
  }
  const float Akz = pick(A, r.kz), Bkz = pick(B, r.kz), Ckz = pick(C, r.kz);
  const float Ax = fsub(pick(A, r.kx), fmul(r.sx, Akz)), Ay = fsub(pick(A, r.ky), fmul(r.sy, Akz));
  const float Bx = fsub(pick(B, r.kx), fmul(r.sx, Bkz)), By = fsub(pick(B, r.ky), fmul(r.sy, Bkz));
  const float Cx = fsub(pick(C, r.kx), fmul(r.sx, Ckz)), Cy = fsub(pick(C, r.ky), fmul(r.sy, Ckz));
  float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
  float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
  float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
    V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
    W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
  }
  if (cull) {
    if (U < 0.0f || V < 0.0f || W < 0.0f) return false;
  } else {
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  }
  const float det = fadd(fadd(U, V), W);
  if (det == 0.0f) return false;
  const float Az = fmul(r.sz, Akz), Bz = fmul(r.sz, Bkz), Cz = fmul(r.sz, Ckz);
  const float T = fadd(fadd(fmul(U, Az), fmul(V, Bz)), fmul(W, Cz));
  const float t = fdiv(T, det);
  if (!(t > tmin) || !(t <= tmax)) return false;
  tout = t;
  return true;
}

// Robust slab test; sign-selected planes make 0 * inf NaNs drop out of the min/max.
__device__ __forceinline__ bool box_hit(const RayPre &r, float4 a, float4 b, float tmin, float tmax, float &tn) {
  const float mn[3] = {a.x, a.y, a.z};
  const float mx[3] = {a.w, b.x, b.y};
  float t0 = tmin, t1 = tmax;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const bool neg = r.inv[k] < 0.0f || (r.inv[k] == 0.0f && signbit(r.inv[k]));
    const float nearP = neg ? mx[k] : mn[k], farP = neg ? mn[k] : mx[k];
    const float tNear = fmul(fsub(nearP, r.o[k]), r.inv[k]);
    const float tFar = fmul(fmul(fsub(farP, r.o[k]), r.inv[k]), kFarScale);
    t0 = fmaxf(t0, tNear);
    t1 = fminf(t1, tFar);
  }
  tn = t0;
  return t0 <= t1;
}

struct Hit {
  uint32_t prim;
  float t;
};

__device__ __forceinline__ void load_tri(const float *__restrict__ vert, const uint32_t *__restrict__ faces, uint32_t f,
                                         float *v0, float *v1, float *v2) {
  const uint32_t a = __ldg(faces + 3 * (size_t)f), b = __ldg(faces + 3 * (size_t)f + 1), c = __ldg(faces + 3 * (size_t)f + 2);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v0[k] = __ldg(vert + 3 * (size_t)a + k);
    v1[k] = __ldg(vert + 3 * (size_t)b + k);
    v2[k] = __ldg(vert + 3 * (size_t)c + k);
  }
}

__device__ __forceinline__ void test_leaf(const RayPre &r, const float *__restrict__ vert,
                                          const uint32_t *__restrict__ faces, uint32_t first, uint32_t count,
                                          float tmin, float tmax, bool cull, Hit &h) {
  for (uint32_t f = first; f < first + count; ++f) {
    float v0[3], v1[3], v2[3], t;
    load_tri(vert, faces, f, v0, v1, v2);
    if (ray_tri(r, v0, v1, v2, tmin, tmax, cull, t)) {
      if (h.prim == kNone || t < h.t || (t == h.t && f < h.prim)) {
        h.t = t;
        h.prim = f;
      }
    }
  }
}

// Closest hit through the 48-byte node array. Returns the number of inner nodes visited.
__device__ __forceinline__ uint32_t traverse(const RayPre &r, const bvhgb_node *__restrict__ nodes, uint32_t numNodes,
                                             uint32_t root, const float *__restrict__ vert,
                                             const uint32_t *__restrict__ faces, float tmin, float tmax, bool cull,
                                             Hit &h, uint32_t *err) {
  uint2 stack[kStack];
  int sp = 0;
  uint32_t visits = 0;
  h.prim = kNone;
  h.t = tmax;
  float4 a, b, c;
  load_node(nodes, root, a, b, c);
  float tn;
  if (!box_hit(r, a, b, tmin, tmax, tn)) return 0;
  uint32_t left = __float_as_uint(b.w), right = __float_as_uint(c.x);
  bool leaf = (__float_as_uint(c.y) & 0xFFFFu) != 0;
  // A tree visits each node at most once; the bound turns a cyclic (corrupted) input into an error.
  for (uint32_t it = 0;; ++it) {
    if (it > numNodes) {
      atomicOr(err, kErrBadIndex);
      break;
    }
    if (leaf) {
      test_leaf(r, vert, faces, left, right, tmin, tmax, cull, h);
    } else {
      ++visits;
      if (left >= numNodes || right >= numNodes) {
        atomicOr(err, kErrBadIndex);
      } else {
        float4 la, lb, lc, ra, rb, rc;
        load_node(nodes, left, la, lb, lc);
        load_node(nodes, right, ra, rb, rc);
        const float lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
        float tl, tr;
        const bool hl = box_hit(r, la, lb, tmin, lim, tl);
        const bool hr = box_hit(r, ra, rb, tmin, lim, tr);
        if (hl && hr) {
          const bool lfirst = tl <= tr;
          const uint32_t farIdx = lfirst ? right : left;
          if (sp < kStack) stack[sp++] = make_uint2(farIdx, __float_as_uint(lfirst ? tr : tl));
          else atomicOr(err, kErrStackOverflow);
          const float4 &nb = lfirst ? lb : rb;
          const float4 &nc = lfirst ? lc : rc;
          left = __float_as_uint(nb.w);
          right = __float_as_uint(nc.x);
          leaf = (__float_as_uint(nc.y) & 0xFFFFu) != 0;
          continue;
        }
        if (hl || hr) {
          const float4 &nb = hl ? lb : rb;
          const float4 &nc = hl ? lc : rc;
          left = __float_as_uint(nb.w);
          right = __float_as_uint(nc.x);
          leaf = (__float_as_uint(nc.y) & 0xFFFFu) != 0;
          continue;
        }
      }
    }
    // Pop the next subtree whose entry distance can still beat the best hit.
    bool found = false;
    while (sp > 0) {
      const uint2 e = stack[--sp];
      const float lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
      if (__uint_as_float(e.y) <= lim) {
        const float4 *p = reinterpret_cast<const float4 *>(nodes + e.x);
        const float4 nb = __ldg(p + 1), nc = __ldg(p + 2);
        left = __float_as_uint(nb.w);
        right = __float_as_uint(nc.x);
        leaf = (__float_as_uint(nc.y) & 0xFFFFu) != 0;
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return visits;
}


// ---- traversal records --------------------------------------------------------------------------
// Traversal record of an inner node: both children's boxes and references in 64 bytes (one aligned
// pair of sectors), so a visit loads one record instead of the children's two 48-byte nodes, and a
// leaf child's faces are known without loading the leaf. ref = the node id of an inner child, the
// first face of a leaf child; count = 0 for an inner child, the leaf's face count. Built from the
// drop-in node array before a trace (the boxes are copied bit for bit, so hits do not change).
struct __align__(64) TravNode {
  float4 q0;  // left mn.xyz, left mx.x
  float4 q1;  // left mx.y mx.z, right mn.x mn.y
  float4 q2;  // right mn.z, right mx.xyz
  uint4 q3;   // left ref, right ref, left count, right count
};


__device__ __forceinline__ void build_trav(const bvhgb_node *__restrict__ nodes, uint32_t numNodes, uint32_t x,
                                           TravNode *__restrict__ out, uint32_t *err) {
  const float4 *p = reinterpret_cast<const float4 *>(nodes + x);
  const float4 b = __ldg(p + 1), c = __ldg(p + 2);
  if (__float_as_uint(c.y) & 0xFFFFu) return;  // leaves have no record
  const uint32_t l = __float_as_uint(b.w), r = __float_as_uint(c.x);
  TravNode t;
  if (l >= numNodes || r >= numNodes) {  // no child can be hit: an empty box on both sides
    atomicOr(err, kErrBadIndex);
    const float inf = __int_as_float(0x7f800000);
    t.q0 = make_float4(inf, inf, inf, -inf);
    t.q1 = make_float4(-inf, -inf, inf, inf);
    t.q2 = make_float4(inf, -inf, -inf, -inf);
    t.q3 = make_uint4(0u, 0u, 0u, 0u);
  } else {
    const float4 *pl = reinterpret_cast<const float4 *>(nodes + l);
    const float4 *pr = reinterpret_cast<const float4 *>(nodes + r);
    const float4 la = __ldg(pl), lb = __ldg(pl + 1), lc = __ldg(pl + 2);
    const float4 ra = __ldg(pr), rb = __ldg(pr + 1), rc = __ldg(pr + 2);
    const bool lleaf = (__float_as_uint(lc.y) & 0xFFFFu) != 0, rleaf = (__float_as_uint(rc.y) & 0xFFFFu) != 0;
    t.q0 = la;
    t.q1 = make_float4(lb.x, lb.y, ra.x, ra.y);
    t.q2 = make_float4(ra.z, ra.w, rb.x, rb.y);
    t.q3 = make_uint4(lleaf ? __float_as_uint(lb.w) : l, rleaf ? __float_as_uint(rb.w) : r,
                      lleaf ? __float_as_uint(lc.x) : 0u, rleaf ? __float_as_uint(rc.x) : 0u);
  }
  out[x] = t;
}

// Closest hit through the traversal records (same hits as traverse(): the boxes and triangle tests
// are the same and the closest-hit rule does not depend on the order of the tests). A leaf child
// is tested as soon as its box is hit, so the stack holds inner nodes only. Returns the number of
// inner nodes visited.
__device__ __forceinline__ uint32_t traverse_records(const RayPre &r, const bvhgb_node *__restrict__ nodes,
                                                     const TravNode *__restrict__ trav, uint32_t numNodes,
                                                     uint32_t root, const float *__restrict__ vert,
                                                     const uint32_t *__restrict__ faces, float tmin, float tmax,
                                                     bool cull, Hit &h, uint32_t *err) {
  uint2 stack[kStack];
  int sp = 0;
  uint32_t visits = 0;
  h.prim = kNone;
  h.t = tmax;
  float4 a, b, c;
  load_node(nodes, root, a, b, c);
  float tn;
  if (!box_hit(r, a, b, tmin, tmax, tn)) return 0;
  if (__float_as_uint(c.y) & 0xFFFFu) {
    test_leaf(r, vert, faces, __float_as_uint(b.w), __float_as_uint(c.x), tmin, tmax, cull, h);
    return 0;
  }
  uint32_t cur = root;
  for (uint32_t it = 0;; ++it) {
    if (it > numNodes) {  // a tree visits each node at most once: a cyclic (corrupted) input
      atomicOr(err, kErrBadIndex);
      break;
    }
    ++visits;
    const float4 *q = reinterpret_cast<const float4 *>(trav + cur);
    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
    const uint4 q3 = __ldg(reinterpret_cast<const uint4 *>(q + 3));
    float lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
    float tl, tr;
    bool hl = box_hit(r, q0, make_float4(q1.x, q1.y, 0.0f, 0.0f), tmin, lim, tl);
    bool hr = box_hit(r, make_float4(q1.z, q1.w, q2.x, q2.y), make_float4(q2.z, q2.w, 0.0f, 0.0f), tmin, lim, tr);
    if (hl && q3.z) {
      test_leaf(r, vert, faces, q3.x, q3.z, tmin, tmax, cull, h);
      hl = false;
    }
    if (hr && q3.w) {
      test_leaf(r, vert, faces, q3.y, q3.w, tmin, tmax, cull, h);
      hr = false;
    }
    if (hl || hr) lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
    hl = hl && tl <= lim;
    hr = hr && tr <= lim;
    if (hl && hr) {
      const bool lfirst = tl <= tr;
      if (sp < kStack) stack[sp++] = make_uint2(lfirst ? q3.y : q3.x, __float_as_uint(lfirst ? tr : tl));
      else atomicOr(err, kErrStackOverflow);
      cur = lfirst ? q3.x : q3.y;
      continue;
    }
    if (hl || hr) {
      cur = hl ? q3.x : q3.y;
      continue;
    }
    // Pop the next subtree whose entry distance can still beat the best hit.
    bool found = false;
    while (sp > 0) {
      const uint2 e = stack[--sp];
      if (__uint_as_float(e.y) <= (h.prim == kNone ? tmax : fmul(h.t, kBestSlack))) {
        cur = e.x;
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return visits;
}

// ---- ray bundles ---------------------------------------------------------------------------------
// kTraceRayBundle (CUDAKernels.cu:240-383) traverses the tree once for a block of 64 rays: a node
// is visited when any ray of the block hits it, the nearer child first by a vote of the rays. Here
// the bundle is a warp (32 neighbouring primary rays): each lane tests its own ray against both
// children of the warp's node (the node record is one broadcast load), __any_sync decides whether
// the warp goes down a side, a majority ballot picks the near side, and the stack is warp-uniform
// (each lane keeps its own entry distance of a pushed node, +inf where its ray missed it, so a pop
// is skipped when no lane can still improve). A lane tests a leaf's triangles only where its own
// ray hits the leaf's box. Every lane thus tests a superset of what its own traversal would test,
// and the closest-hit rule (smallest t, then smallest primitive) picks the same hit; the visit
// count (intCount) is the warp's. All lanes of the warp must call it; inactive lanes pass active =
// false and get no hit. REC: traversal records (true) or the node array (false).
template <bool REC>
__device__ __forceinline__ uint32_t traverse_bundle(const RayPre &r, bool active, const bvhgb_node *__restrict__ nodes,
                                                    const TravNode *__restrict__ trav, uint32_t numNodes,
                                                    uint32_t root, const float *__restrict__ vert,
                                                    const uint32_t *__restrict__ faces, float tmin, float tmax,
                                                    bool cull, Hit &h, uint32_t *err) {
  const float kInf = __int_as_float(0x7f800000);
  uint32_t stN[kStack];
  float stT[kStack];
  int sp = 0;
  uint32_t visits = 0;
  h.prim = kNone;
  h.t = tmax;
  float4 a, b, c;
  load_node(nodes, root, a, b, c);
  float tn;
  const bool hitRoot = active && box_hit(r, a, b, tmin, tmax, tn);
  if (!__any_sync(0xFFFFFFFFu, hitRoot)) return 0;
  if (__float_as_uint(c.y) & 0xFFFFu) {
    if (hitRoot) test_leaf(r, vert, faces, __float_as_uint(b.w), __float_as_uint(c.x), tmin, tmax, cull, h);
    return 0;
  }
  uint32_t cur = root;
  for (uint32_t it = 0;; ++it) {
    if (it > numNodes) {  // each node is visited at most once per warp: a cyclic (corrupted) input
      if (active) atomicOr(err, kErrBadIndex);
      break;
    }
    ++visits;
    float4 l0, l1, r0, r1;
    uint32_t lref, rref, lcnt, rcnt;
    bool ok = true;
    if (REC) {
      const float4 *q = reinterpret_cast<const float4 *>(trav + cur);
      const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
      const uint4 q3 = __ldg(reinterpret_cast<const uint4 *>(q + 3));
      l0 = q0;
      l1 = make_float4(q1.x, q1.y, 0.0f, 0.0f);
      r0 = make_float4(q1.z, q1.w, q2.x, q2.y);
      r1 = make_float4(q2.z, q2.w, 0.0f, 0.0f);
      lref = q3.x;
      rref = q3.y;
      lcnt = q3.z;
      rcnt = q3.w;
    } else {
      float4 ca, cb, cc;
      load_node(nodes, cur, ca, cb, cc);
      const uint32_t li = __float_as_uint(cb.w), ri = __float_as_uint(cc.x);
      ok = li < numNodes && ri < numNodes;
      float4 lc, rc;
      if (ok) {
        load_node(nodes, li, l0, l1, lc);
        load_node(nodes, ri, r0, r1, rc);
        const bool ll = (__float_as_uint(lc.y) & 0xFFFFu) != 0, rl = (__float_as_uint(rc.y) & 0xFFFFu) != 0;
        lref = ll ? __float_as_uint(l1.w) : li;
        rref = rl ? __float_as_uint(r1.w) : ri;
        lcnt = ll ? __float_as_uint(lc.x) : 0u;
        rcnt = rl ? __float_as_uint(rc.x) : 0u;
      }
    }
    if (!ok) {
      if (active) atomicOr(err, kErrBadIndex);
    } else {
      float lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
      float tl = kInf, tr = kInf;
      bool hl = active && box_hit(r, l0, l1, tmin, lim, tl);
      bool hr = active && box_hit(r, r0, r1, tmin, lim, tr);
      if (hl && lcnt) {
        test_leaf(r, vert, faces, lref, lcnt, tmin, tmax, cull, h);
        hl = false;
      }
      if (hr && rcnt) {
        test_leaf(r, vert, faces, rref, rcnt, tmin, tmax, cull, h);
        hr = false;
      }
      lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
      hl = hl && tl <= lim;
      hr = hr && tr <= lim;
      const bool anyL = __any_sync(0xFFFFFFFFu, hl), anyR = __any_sync(0xFFFFFFFFu, hr);
      if (anyL && anyR) {
        const int wantL = __popc(__ballot_sync(0xFFFFFFFFu, hl && (!hr || tl <= tr)));
        const int wantR = __popc(__ballot_sync(0xFFFFFFFFu, hr && (!hl || tr < tl)));
        const bool lfirst = wantL >= wantR;
        if (sp < kStack) {
          stN[sp] = lfirst ? rref : lref;
          stT[sp] = lfirst ? (hr ? tr : kInf) : (hl ? tl : kInf);
          ++sp;
        } else if (active) {
          atomicOr(err, kErrStackOverflow);
        }
        cur = lfirst ? lref : rref;
        continue;
      }
      if (anyL || anyR) {
        cur = anyL ? lref : rref;
        continue;
      }
    }
    // Pop the next subtree that some lane can still improve on.
    bool found = false;
    while (sp > 0) {
      --sp;
      const float lim = h.prim == kNone ? tmax : fmul(h.t, kBestSlack);
      if (__any_sync(0xFFFFFFFFu, active && stT[sp] <= lim)) {
        cur = stN[sp];
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return active ? visits : 0u;
}

}  // namespace
}  // namespace bvhgb
