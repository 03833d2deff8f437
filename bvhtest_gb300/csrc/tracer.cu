// Closest-hit tracer: fused primary-ray generation + stack traversal + watertight triangle test +
// Lambert shade (lib/tracer/CUDAKernels.cu:43-223, 386-417).
//
// Differences from the reference, all deliberate:
//  * the triangle test is the watertight test of Woop, Benthin and Wald (JCGT 2013), two-sided by
//    default, with t in (tmin, tmax]; the reference's Moller-Trumbore culls back faces and has no
//    t range, so its hit IDs are not those of a brute-force search;
//  * rays are generated in registers (no 48-byte Ray round trip through HBM);
//  * a short stack replaces the 128-bit trail, and the slab test is the robust form of Ize
//    (JCGT 2013): the far distance is scaled by 1 + 2*gamma(3), so a box that holds the closest
//    hit is never culled; closest-hit ties resolve to the smallest primitive index;
//  * each hit also yields (primId, t).
#include <cmath>

#include "common.cuh"

namespace bvhgb {
namespace {

constexpr int kStack = 96;
constexpr float kFarScale = 1.0000004f;   // 1 + 2 * gamma(3), gamma(n) = n u / (1 - n u), u = 2^-24
constexpr float kBestSlack = 1.0000153f;  // relative slack on the best t when culling boxes

__device__ uint32_t g_trace_errors = 0;

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
                                             Hit &h) {
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
      atomicOr(&g_trace_errors, kErrBadIndex);
      break;
    }
    if (leaf) {
      test_leaf(r, vert, faces, left, right, tmin, tmax, cull, h);
    } else {
      ++visits;
      if (left >= numNodes || right >= numNodes) {
        atomicOr(&g_trace_errors, kErrBadIndex);
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
          else atomicOr(&g_trace_errors, kErrStackOverflow);
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

__device__ __forceinline__ void normalize3(float *v) {
  const float l2 = fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2]));
  const float inv = fdiv(1.0f, __fsqrt_rn(l2));
  v[0] = fmul(v[0], inv);
  v[1] = fmul(v[1], inv);
  v[2] = fmul(v[2], inv);
}

// CUDAKernels.cu:208-218 with glm::triangleNormal(v1, v2, v3) = normalize(cross(v1 - v2, v1 - v3)).
__device__ __forceinline__ uint8_t shade(const RayPre &r, float t, const float *v1, const float *v2, const float *v3,
                                         const float *light) {
  float a[3], b[3], n[3], l[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a[k] = fsub(v1[k], v2[k]);
    b[k] = fsub(v1[k], v3[k]);
  }
  n[0] = fsub(fmul(a[1], b[2]), fmul(a[2], b[1]));
  n[1] = fsub(fmul(a[2], b[0]), fmul(a[0], b[2]));
  n[2] = fsub(fmul(a[0], b[1]), fmul(a[1], b[0]));
  normalize3(n);
#pragma unroll
  for (int k = 0; k < 3; ++k) l[k] = fsub(light[k], fadd(r.o[k], fmul(t, r.d[k])));
  normalize3(l);
  float d = fadd(1.0f, fadd(fadd(fmul(n[0], l[0]), fmul(n[1], l[1])), fmul(n[2], l[2])));
  d = d > 0.0f ? d : 0.0f;
  return (uint8_t)fmul(d, 127.0f);
}

struct CamParams {
  float pos[3], s[3], u[3], f[3];
  float scale, ratio;
  uint32_t w, h;
};

struct TraceParams {
  float light[3];
  float tmin, tmax;
  uint32_t cull;
};

// Camera::genRays (Camera.cpp:67-88): pixel coordinates in double, the rest in float.
__device__ __forceinline__ void camera_ray(const CamParams &cam, uint32_t x, uint32_t y, RayPre &r) {
  const double qx = __ddiv_rn(__dadd_rn((double)x, 0.5), (double)cam.w);
  const double qy = __ddiv_rn(__dadd_rn((double)y, 0.5), (double)cam.h);
  const float px = (float)__dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(2.0, qx), 1.0), (double)cam.scale), (double)cam.ratio);
  const float py = (float)__dmul_rn(__dsub_rn(1.0, __dmul_rn(2.0, qy)), (double)cam.scale);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.o[k] = cam.pos[k];
    r.d[k] = fadd(fadd(fmul(cam.s[k], px), fmul(cam.u[k], py)), cam.f[k]);
  }
  normalize3(r.d);
  setup_ray(r);
}

// Counter-based uniform floats in [0, 1): SplitMix64 finaliser of (seed, index, lane).
__device__ __forceinline__ float uniform01(uint64_t seed, uint64_t idx, uint32_t lane) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (2 * idx + lane + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// One cosine-weighted diffuse bounce from every primary hit (an addition: the reference traces
// primary rays only). The bounce starts on the hit point, offset along the normal that faces the
// incoming ray; the direction follows Malley's method around that normal in the orthonormal basis
// of Duff et al. (JCGT 2017).
__global__ void __launch_bounds__(128) trace_bounce_kernel(const bvhgb_node *__restrict__ nodes, uint32_t numNodes,
                                                           uint32_t root, const float *__restrict__ vert,
                                                           const uint32_t *__restrict__ faces, CamParams cam,
                                                           TraceParams tp, uint64_t seed, float offset,
                                                           const bvhgb_hit *__restrict__ primary,
                                                           bvhgb_hit *__restrict__ out, float *__restrict__ rayOrg,
                                                           float *__restrict__ rayDir) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= cam.w || y >= cam.h) return;
  const size_t pix = (size_t)y * cam.w + x;
  const bvhgb_hit ph = primary[pix];
  bvhgb_hit o;
  o.primId = kNone;
  o.t = __int_as_float(0x7f800000);
  if (ph.primId == kNone) {
    out[pix] = o;
    if (rayOrg) {
#pragma unroll
      for (int k = 0; k < 3; ++k) rayOrg[3 * pix + k] = rayDir[3 * pix + k] = 0.0f;
    }
    return;
  }
  RayPre cr;
  camera_ray(cam, x, y, cr);
  float v0[3], v1[3], v2[3];
  load_tri(vert, faces, ph.primId, v0, v1, v2);
  float e1[3], e2[3], n[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    e1[k] = fsub(v1[k], v0[k]);
    e2[k] = fsub(v2[k], v0[k]);
  }
  n[0] = fsub(fmul(e1[1], e2[2]), fmul(e1[2], e2[1]));
  n[1] = fsub(fmul(e1[2], e2[0]), fmul(e1[0], e2[2]));
  n[2] = fsub(fmul(e1[0], e2[1]), fmul(e1[1], e2[0]));
  normalize3(n);
  const float dn = fadd(fadd(fmul(n[0], cr.d[0]), fmul(n[1], cr.d[1])), fmul(n[2], cr.d[2]));
  if (dn > 0.0f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
  // Orthonormal basis (t, b, n).
  const float sgn = copysignf(1.0f, n[2]);
  const float a = -1.0f / (sgn + n[2]);
  const float bb = n[0] * n[1] * a;
  const float tv[3] = {1.0f + sgn * n[0] * n[0] * a, sgn * bb, -sgn * n[0]};
  const float bv[3] = {bb, sgn + n[1] * n[1] * a, -n[1]};
  const float u1 = uniform01(seed, pix, 0), u2 = uniform01(seed, pix, 1);
  const float rr = sqrtf(u1), phi = 6.28318530717958647692f * u2;
  float sn, cs;
  sincosf(phi, &sn, &cs);
  const float lx = rr * cs, ly = rr * sn, lz = sqrtf(fmaxf(0.0f, 1.0f - u1));
  RayPre r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float hp = fadd(cr.o[k], fmul(ph.t, cr.d[k]));
    r.o[k] = hp + offset * n[k];
    r.d[k] = lx * tv[k] + ly * bv[k] + lz * n[k];
  }
  if (rayOrg) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      rayOrg[3 * pix + k] = r.o[k];
      rayDir[3 * pix + k] = r.d[k];
    }
  }
  setup_ray(r);
  Hit h;
  traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h);
  o.primId = h.prim;
  o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
  out[pix] = o;
}

__global__ void __launch_bounds__(128) trace_image_kernel(const bvhgb_node *__restrict__ nodes, uint32_t numNodes,
                                                          uint32_t root, const float *__restrict__ vert,
                                                          const uint32_t *__restrict__ faces, CamParams cam,
                                                          TraceParams tp, bvhgb_pixel *__restrict__ img,
                                                          bvhgb_hit *__restrict__ hits) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= cam.w || y >= cam.h) return;
  RayPre r;
  camera_ray(cam, x, y, r);
  Hit h;
  const uint32_t visits = traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h);
  bvhgb_pixel px_out;
  px_out.hit = 0;
  px_out.diffuse = 0;
  px_out.intCount = (uint16_t)visits;
  if (h.prim != kNone) {
    float v0[3], v1[3], v2[3];
    load_tri(vert, faces, h.prim, v0, v1, v2);
    px_out.hit = 1;
    px_out.diffuse = shade(r, h.t, v0, v1, v2, tp.light);
  }
  const size_t pix = (size_t)y * cam.w + x;
  img[pix] = px_out;
  if (hits) {
    bvhgb_hit o;
    o.primId = h.prim;
    o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
    hits[pix] = o;
  }
}

__global__ void __launch_bounds__(128) trace_rays_kernel(const bvhgb_node *__restrict__ nodes, uint32_t numNodes,
                                                         uint32_t root, const float *__restrict__ vert,
                                                         const uint32_t *__restrict__ faces,
                                                         const float *__restrict__ org, const float *__restrict__ dir,
                                                         uint32_t n, TraceParams tp, bvhgb_hit *__restrict__ hits) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  RayPre r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.o[k] = __ldg(org + 3 * (size_t)i + k);
    r.d[k] = __ldg(dir + 3 * (size_t)i + k);
  }
  setup_ray(r);
  Hit h;
  traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h);
  bvhgb_hit o;
  o.primId = h.prim;
  o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
  hits[i] = o;
}

// Host mirror of the device normalise (each operation rounds once; this file's host code is
// compiled with -ffp-contract=off).
void h_normalize(float *v) {
  float l2 = v[0] * v[0];
  float t1 = v[1] * v[1];
  float t2 = v[2] * v[2];
  l2 = l2 + t1;
  l2 = l2 + t2;
  float inv = 1.0f / std::sqrt(l2);
  v[0] = v[0] * inv;
  v[1] = v[1] * inv;
  v[2] = v[2] * inv;
}
void h_cross(const float *a, const float *b, float *o) {
  float x0 = a[1] * b[2], x1 = a[2] * b[1];
  float y0 = a[2] * b[0], y1 = a[0] * b[2];
  float z0 = a[0] * b[1], z1 = a[1] * b[0];
  o[0] = x0 - x1;
  o[1] = y0 - y1;
  o[2] = z0 - z1;
}

// Camera basis of inverse(lookAtRH(pos, lookAt, up)) (CUDAKernels.cu:389-391), host side.
CamParams make_cam_params(const bvhgb_camera *cam) {
  CamParams cp;
  float f[3] = {cam->lookAt[0] - cam->pos[0], cam->lookAt[1] - cam->pos[1], cam->lookAt[2] - cam->pos[2]};
  h_normalize(f);
  float s[3];
  h_cross(f, cam->up, s);
  h_normalize(s);
  float u[3];
  h_cross(s, f, u);
  for (int k = 0; k < 3; ++k) {
    cp.pos[k] = cam->pos[k];
    cp.s[k] = s[k];
    cp.u[k] = u[k];
    cp.f[k] = f[k];
  }
  cp.scale = (float)std::tan(0.5 * (double)cam->fov * 0.01745329251994329576923690768489);
  cp.ratio = (float)cam->width / (float)cam->height;
  cp.w = cam->width;
  cp.h = cam->height;
  return cp;
}

TraceParams make_trace_params(const bvhgb_trace_config *cfg) {
  TraceParams tp;
  if (cfg) {
    for (int k = 0; k < 3; ++k) tp.light[k] = cfg->light[k];
    tp.cull = cfg->faceCulling;
    tp.tmin = cfg->tmin;
    tp.tmax = cfg->tmax;
  } else {
    tp.light[0] = tp.light[1] = tp.light[2] = 2.0f;
    tp.cull = 0;
    tp.tmin = 0.0f;
    tp.tmax = INFINITY;
  }
  return tp;
}

}  // namespace
}  // namespace bvhgb

using namespace bvhgb;

extern "C" BVHGB_API int bvhgb_trace_image(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                           const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                           bvhgb_pixel *img, bvhgb_hit *hits, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || !cam || !img || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  if (cam->width == 0 || cam->height == 0) return BVHGB_OK;
  const CamParams cp = make_cam_params(cam);
  dim3 block(16, 8);
  dim3 grid(ceil_div(cam->width, 16), ceil_div(cam->height, 8));
  trace_image_kernel<<<grid, block, 0, as_stream(stream)>>>(nodes, numNodes, root, vert, faces, cp, make_trace_params(cfg),
                                                            img, hits);
  BVHGB_LAUNCH_CHECK("trace image");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_trace_rays(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                          const uint32_t *faces, const float *org, const float *dir, uint32_t n,
                                          const bvhgb_trace_config *cfg, bvhgb_hit *hits, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  if (n == 0) return BVHGB_OK;
  if (!org || !dir || !hits) return BVHGB_INVALID_ARGUMENT;
  trace_rays_kernel<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(nodes, numNodes, root, vert, faces, org, dir, n,
                                                                     make_trace_params(cfg), hits);
  BVHGB_LAUNCH_CHECK("trace rays");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_trace_bounce(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                            const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                            uint64_t seed, float offset, const bvhgb_hit *primary, bvhgb_hit *bounce,
                                            float *rayOrg, float *rayDir, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || !cam || !primary || !bounce || numNodes == 0 || root >= numNodes)
    return BVHGB_INVALID_ARGUMENT;
  if ((rayOrg == nullptr) != (rayDir == nullptr)) return BVHGB_INVALID_ARGUMENT;
  if (cam->width == 0 || cam->height == 0) return BVHGB_OK;
  const CamParams cp = make_cam_params(cam);
  dim3 block(16, 8);
  dim3 grid(ceil_div(cam->width, 16), ceil_div(cam->height, 8));
  trace_bounce_kernel<<<grid, block, 0, as_stream(stream)>>>(nodes, numNodes, root, vert, faces, cp,
                                                             make_trace_params(cfg), seed, offset, primary, bounce,
                                                             rayOrg, rayDir);
  BVHGB_LAUNCH_CHECK("trace bounce");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_trace_read_errors(uint32_t *flags, int reset) {
  if (!flags) return BVHGB_INVALID_ARGUMENT;
  BVHGB_CUDA_TRY(cudaMemcpyFromSymbol(flags, g_trace_errors, sizeof(uint32_t)));
  if (reset) {
    uint32_t z = 0;
    BVHGB_CUDA_TRY(cudaMemcpyToSymbol(g_trace_errors, &z, sizeof(uint32_t)));
  }
  return BVHGB_OK;
}
