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
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "tracer_device.cuh"

namespace bvhgb {
namespace {

__device__ uint32_t g_trace_errors = 0;

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
// Incoherent rays (bounce, random) are bound by the latency of their record and triangle loads:
// at most 48 registers keep 40 warps per SM resident instead of 36 (2.5% faster bounce phase).
template <bool REC>
__global__ void __launch_bounds__(128, 10) trace_bounce_kernel(const bvhgb_node *__restrict__ nodes,
                                                           const TravNode *__restrict__ trav, uint32_t numNodes,
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
  if (REC) traverse_records(r, nodes, trav, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h, &g_trace_errors);
  else traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h, &g_trace_errors);
  o.primId = h.prim;
  o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
  out[pix] = o;
}

// BUNDLE: the warp traverses as one bundle of rays (traverse_bundle, the reference's rayBundles);
// otherwise each ray on its own. Same hits either way.
template <bool REC, bool BUNDLE>
__global__ void __launch_bounds__(128) trace_image_kernel(const bvhgb_node *__restrict__ nodes,
                                                          const TravNode *__restrict__ trav, uint32_t numNodes,
                                                          uint32_t root, const float *__restrict__ vert,
                                                          const uint32_t *__restrict__ faces, CamParams cam,
                                                          TraceParams tp, bvhgb_pixel *__restrict__ img,
                                                          bvhgb_hit *__restrict__ hits) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  const bool active = x < cam.w && y < cam.h;
  if (!BUNDLE && !active) return;  // a bundle keeps its whole warp in the traversal
  RayPre r;
  camera_ray(cam, active ? x : 0u, active ? y : 0u, r);
  Hit h;
  const uint32_t visits =
      BUNDLE ? traverse_bundle<REC>(r, active, nodes, trav, numNodes, root, vert, faces, tp.tmin, tp.tmax,
                                    tp.cull != 0, h, &g_trace_errors)
      : REC  ? traverse_records(r, nodes, trav, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h,
                                &g_trace_errors)
             : traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h, &g_trace_errors);
  if (!active) return;
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

template <bool REC>
__global__ void __launch_bounds__(128, 10) trace_rays_kernel(const bvhgb_node *__restrict__ nodes,
                                                         const TravNode *__restrict__ trav, uint32_t numNodes,
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
  if (REC) traverse_records(r, nodes, trav, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h, &g_trace_errors);
  else traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h, &g_trace_errors);
  bvhgb_hit o;
  o.primId = h.prim;
  o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
  hits[i] = o;
}

// The reference's Ray (lib/base/Ray.hpp:38-80): origin, direction, 1 / direction, sign of the
// inverse direction per axis, pixel coordinates. 48 bytes, 16-byte aligned.
struct RefRay {
  float pos[3], dir[3], inv[3];
  uint8_t sign[3], pad;
  uint32_t px, py;
};
static_assert(sizeof(RefRay) == 48, "Ray layout");

// kGenerateRays (CUDAKernels.cu:43-59): one camera ray per pixel written as a Ray record
// (Ray::set: 1 / dir and its signs).
__global__ void gen_rays_kernel(RefRay *__restrict__ rays, CamParams cam) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= cam.w || y >= cam.h) return;
  RayPre r;
  camera_ray(cam, x, y, r);
  RefRay o;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    o.pos[k] = r.o[k];
    o.dir[k] = r.d[k];
    o.inv[k] = r.inv[k];
    o.sign[k] = r.inv[k] < 0.0f ? 1 : 0;
  }
  o.pad = 0;
  o.px = x;
  o.py = y;
  rays[(size_t)y * cam.w + x] = o;
}

// kTraceRay (CUDAKernels.cu:114-223) on caller-supplied Ray records: closest hit, the pixel
// {hit, diffuse, intCount} and (optionally) (primId, t), one ray per pixel in record order.
template <bool REC, bool BUNDLE>
__global__ void __launch_bounds__(128) trace_ray_image_kernel(const bvhgb_node *__restrict__ nodes,
                                                              const TravNode *__restrict__ trav, uint32_t numNodes,
                                                              uint32_t root, const float *__restrict__ vert,
                                                              const uint32_t *__restrict__ faces,
                                                              const RefRay *__restrict__ rays, uint32_t n,
                                                              TraceParams tp, bvhgb_pixel *__restrict__ img,
                                                              bvhgb_hit *__restrict__ hits) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  if (!BUNDLE && !active) return;  // a bundle keeps its whole warp in the traversal
  const float4 *rp = reinterpret_cast<const float4 *>(rays + (active ? i : 0u));
  const float4 a = __ldg(rp), b = __ldg(rp + 1);
  RayPre r;
  r.o[0] = a.x; r.o[1] = a.y; r.o[2] = a.z;
  r.d[0] = a.w; r.d[1] = b.x; r.d[2] = b.y;
  setup_ray(r);
  Hit h;
  const uint32_t visits =
      BUNDLE ? traverse_bundle<REC>(r, active, nodes, trav, numNodes, root, vert, faces, tp.tmin, tp.tmax,
                                    tp.cull != 0, h, &g_trace_errors)
      : REC  ? traverse_records(r, nodes, trav, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h,
                                &g_trace_errors)
             : traverse(r, nodes, numNodes, root, vert, faces, tp.tmin, tp.tmax, tp.cull != 0, h, &g_trace_errors);
  if (!active) return;
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
  img[i] = px_out;
  if (hits) {
    bvhgb_hit o;
    o.primId = h.prim;
    o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
    hits[i] = o;
  }
}

__global__ void build_trav_kernel(const bvhgb_node *__restrict__ nodes, uint32_t numNodes, TravNode *__restrict__ out) {
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < numNodes; x += gridDim.x * blockDim.x)
    build_trav(nodes, numNodes, x, out, &g_trace_errors);
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

// The three traces, on the node array (trav == nullptr) or on a prepared tracer's records.
int launch_image(const bvhgb_node *nodes, const TravNode *trav, uint32_t numNodes, uint32_t root, const float *vert,
                 const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg, bvhgb_pixel *img,
                 bvhgb_hit *hits, cudaStream_t s) {
  if (cam->width == 0 || cam->height == 0) return BVHGB_OK;
  const CamParams cp = make_cam_params(cam);
  dim3 block(16, 8);
  dim3 grid(ceil_div(cam->width, 16), ceil_div(cam->height, 8));
  const TraceParams tp = make_trace_params(cfg);
  const bool bundle = cfg && cfg->rayBundles;
  if (trav && bundle)
    trace_image_kernel<true, true><<<grid, block, 0, s>>>(nodes, trav, numNodes, root, vert, faces, cp, tp, img, hits);
  else if (trav)
    trace_image_kernel<true, false><<<grid, block, 0, s>>>(nodes, trav, numNodes, root, vert, faces, cp, tp, img, hits);
  else if (bundle)
    trace_image_kernel<false, true><<<grid, block, 0, s>>>(nodes, trav, numNodes, root, vert, faces, cp, tp, img, hits);
  else
    trace_image_kernel<false, false><<<grid, block, 0, s>>>(nodes, trav, numNodes, root, vert, faces, cp, tp, img, hits);
  BVHGB_LAUNCH_CHECK("trace image");
  return BVHGB_OK;
}

int launch_rays(const bvhgb_node *nodes, const TravNode *trav, uint32_t numNodes, uint32_t root, const float *vert,
                const uint32_t *faces, const float *org, const float *dir, uint32_t n, const bvhgb_trace_config *cfg,
                bvhgb_hit *hits, cudaStream_t s) {
  if (n == 0) return BVHGB_OK;
  if (!org || !dir || !hits) return BVHGB_INVALID_ARGUMENT;
  if (trav)
    trace_rays_kernel<true><<<ceil_div(n, 128), 128, 0, s>>>(nodes, trav, numNodes, root, vert, faces, org, dir, n,
                                                             make_trace_params(cfg), hits);
  else
    trace_rays_kernel<false><<<ceil_div(n, 128), 128, 0, s>>>(nodes, trav, numNodes, root, vert, faces, org, dir, n,
                                                              make_trace_params(cfg), hits);
  BVHGB_LAUNCH_CHECK("trace rays");
  return BVHGB_OK;
}

int launch_bounce(const bvhgb_node *nodes, const TravNode *trav, uint32_t numNodes, uint32_t root, const float *vert,
                  const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg, uint64_t seed,
                  float offset, const bvhgb_hit *primary, bvhgb_hit *bounce, float *rayOrg, float *rayDir,
                  cudaStream_t s) {
  if (!primary || !bounce || (rayOrg == nullptr) != (rayDir == nullptr)) return BVHGB_INVALID_ARGUMENT;
  if (cam->width == 0 || cam->height == 0) return BVHGB_OK;
  const CamParams cp = make_cam_params(cam);
  dim3 block(16, 8);
  dim3 grid(ceil_div(cam->width, 16), ceil_div(cam->height, 8));
  if (trav)
    trace_bounce_kernel<true><<<grid, block, 0, s>>>(nodes, trav, numNodes, root, vert, faces, cp,
                                                     make_trace_params(cfg), seed, offset, primary, bounce, rayOrg,
                                                     rayDir);
  else
    trace_bounce_kernel<false><<<grid, block, 0, s>>>(nodes, trav, numNodes, root, vert, faces, cp,
                                                      make_trace_params(cfg), seed, offset, primary, bounce, rayOrg,
                                                      rayDir);
  BVHGB_LAUNCH_CHECK("trace bounce");
  return BVHGB_OK;
}

}  // namespace
}  // namespace bvhgb

// A tracer prepared for one tree: its traversal records, rebuilt by bvhgb_tracer_update.
struct bvhgb_tracer {
  uint32_t maxNodes = 0;
  const bvhgb_node *nodes = nullptr;
  uint32_t numNodes = 0, root = 0;
  bvhgb::TravNode *trav = nullptr;
};

using namespace bvhgb;

extern "C" BVHGB_API int bvhgb_trace_image(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                           const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                           bvhgb_pixel *img, bvhgb_hit *hits, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || !cam || !img || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  return launch_image(nodes, nullptr, numNodes, root, vert, faces, cam, cfg, img, hits, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_trace_rays(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                          const uint32_t *faces, const float *org, const float *dir, uint32_t n,
                                          const bvhgb_trace_config *cfg, bvhgb_hit *hits, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  return launch_rays(nodes, nullptr, numNodes, root, vert, faces, org, dir, n, cfg, hits, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_trace_bounce(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                            const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                            uint64_t seed, float offset, const bvhgb_hit *primary, bvhgb_hit *bounce,
                                            float *rayOrg, float *rayDir, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || !cam || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  return launch_bounce(nodes, nullptr, numNodes, root, vert, faces, cam, cfg, seed, offset, primary, bounce, rayOrg,
                       rayDir, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_tracer_create(uint32_t maxNodes, bvhgb_tracer **out) {
  if (!out || maxNodes == 0) return BVHGB_INVALID_ARGUMENT;
  *out = nullptr;
  auto *tr = new bvhgb_tracer();
  tr->maxNodes = maxNodes;
  const cudaError_t e = dev_malloc(&tr->trav, sizeof(TravNode) * (size_t)maxNodes);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_tracer_create", e);
    delete tr;
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  *out = tr;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_tracer_destroy(bvhgb_tracer *tr) {
  if (!tr) return BVHGB_OK;
  cudaFree(tr->trav);
  delete tr;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_tracer_update(bvhgb_tracer *tr, const bvhgb_node *nodes, uint32_t numNodes, uint32_t root,
                                             bvhgb_stream stream) {
  if (!tr || !nodes || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  if (numNodes > tr->maxNodes) return BVHGB_TOO_LARGE;
  tr->nodes = nodes;
  tr->numNodes = numNodes;
  tr->root = root;
  build_trav_kernel<<<std::min(ceil_div(numNodes, 256), (uint32_t)sm_count() * 16), 256, 0, as_stream(stream)>>>(
      nodes, numNodes, tr->trav);
  BVHGB_LAUNCH_CHECK("tracer records");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_tracer_trace_image(const bvhgb_tracer *tr, const float *vert, const uint32_t *faces,
                                                  const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                                  bvhgb_pixel *img, bvhgb_hit *hits, bvhgb_stream stream) {
  if (!tr || !tr->nodes || !vert || !faces || !cam || !img) return BVHGB_INVALID_ARGUMENT;
  return launch_image(tr->nodes, tr->trav, tr->numNodes, tr->root, vert, faces, cam, cfg, img, hits, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_tracer_trace_rays(const bvhgb_tracer *tr, const float *vert, const uint32_t *faces,
                                                 const float *org, const float *dir, uint32_t n,
                                                 const bvhgb_trace_config *cfg, bvhgb_hit *hits, bvhgb_stream stream) {
  if (!tr || !tr->nodes || !vert || !faces) return BVHGB_INVALID_ARGUMENT;
  return launch_rays(tr->nodes, tr->trav, tr->numNodes, tr->root, vert, faces, org, dir, n, cfg, hits,
                     as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_tracer_trace_bounce(const bvhgb_tracer *tr, const float *vert, const uint32_t *faces,
                                                   const bvhgb_camera *cam, const bvhgb_trace_config *cfg, uint64_t seed,
                                                   float offset, const bvhgb_hit *primary, bvhgb_hit *bounce,
                                                   float *rayOrg, float *rayDir, bvhgb_stream stream) {
  if (!tr || !tr->nodes || !vert || !faces || !cam) return BVHGB_INVALID_ARGUMENT;
  return launch_bounce(tr->nodes, tr->trav, tr->numNodes, tr->root, vert, faces, cam, cfg, seed, offset, primary,
                       bounce, rayOrg, rayDir, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_generate_rays(void *rays, const bvhgb_camera *cam, bvhgb_stream stream) {
  if (!rays || !cam) return BVHGB_INVALID_ARGUMENT;
  if (cam->width == 0 || cam->height == 0) return BVHGB_OK;
  if (reinterpret_cast<uintptr_t>(rays) % 16) return BVHGB_INVALID_ARGUMENT;
  const CamParams cp = make_cam_params(cam);
  dim3 block(16, 8);
  dim3 grid(ceil_div(cam->width, 16), ceil_div(cam->height, 8));
  gen_rays_kernel<<<grid, block, 0, as_stream(stream)>>>(static_cast<RefRay *>(rays), cp);
  BVHGB_LAUNCH_CHECK("generate rays");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_trace_ray_image(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root,
                                              const float *vert, const uint32_t *faces, const void *rays, uint32_t n,
                                              const bvhgb_trace_config *cfg, int bundle, bvhgb_pixel *img,
                                              bvhgb_hit *hits, bvhgb_stream stream) {
  if (!nodes || !vert || !faces || !rays || !img || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  if (reinterpret_cast<uintptr_t>(rays) % 16) return BVHGB_INVALID_ARGUMENT;
  if (n == 0) return BVHGB_OK;
  const TraceParams tp = make_trace_params(cfg);
  if (bundle || (cfg && cfg->rayBundles))
    trace_ray_image_kernel<false, true><<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(
        nodes, nullptr, numNodes, root, vert, faces, static_cast<const RefRay *>(rays), n, tp, img, hits);
  else
    trace_ray_image_kernel<false, false><<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(
        nodes, nullptr, numNodes, root, vert, faces, static_cast<const RefRay *>(rays), n, tp, img, hits);
  BVHGB_LAUNCH_CHECK("trace ray image");
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
