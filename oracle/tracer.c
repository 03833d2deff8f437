/*
 * Oracle (test infrastructure only): ray generation, the watertight ray/triangle test,
 * brute-force and BVH closest hit, the reference's stackless CPU tracer (timed baseline) and
 * the Lambert shade of a hit. Parity unpinned: see oracle.h.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NONE 0xFFFFFFFFu

static float dot3(const float *a, const float *b) {
  float s = a[0] * b[0];
  float t = a[1] * b[1];
  float u = a[2] * b[2];
  s = s + t;
  return s + u;
}
static void cross3(const float *a, const float *b, float *o) {
  float x0 = a[1] * b[2], x1 = a[2] * b[1];
  float y0 = a[2] * b[0], y1 = a[0] * b[2];
  float z0 = a[0] * b[1], z1 = a[1] * b[0];
  o[0] = x0 - x1;
  o[1] = y0 - y1;
  o[2] = z0 - z1;
}
/* v * (1 / sqrt(dot(v, v))), each operation correctly rounded. */
static void normalize3(float *v) {
  float inv = 1.0f / sqrtf(dot3(v, v));
  v[0] = v[0] * inv;
  v[1] = v[1] * inv;
  v[2] = v[2] * inv;
}

/* Camera::genRays (Camera.cpp:67-88) / kGenerateRays (CUDAKernels.cu:43-59):
 * camera-to-world = inverse(lookAt) whose rotation columns are (s, u, -f); the pixel
 * coordinates are evaluated in double and rounded to float, the rest in float. */
void orc_camera_ray(const orc_camera *cam, uint32_t x, uint32_t y, float org[3], float dir[3]) {
  float f[3] = {cam->lookat[0] - cam->pos[0], cam->lookat[1] - cam->pos[1], cam->lookat[2] - cam->pos[2]};
  normalize3(f);
  float s[3];
  cross3(f, cam->up, s);
  normalize3(s);
  float u[3];
  cross3(s, f, u);
  float scale = (float)tan(0.5 * (double)cam->fov * 0.01745329251994329576923690768489);
  float ratio = (float)cam->width / (float)cam->height;
  float px = (float)((2.0 * (((double)x + 0.5) / (double)cam->width) - 1.0) * (double)scale * (double)ratio);
  float py = (float)((1.0 - 2.0 * (((double)y + 0.5) / (double)cam->height)) * (double)scale);
  for (int k = 0; k < 3; ++k) {
    float a = s[k] * px;
    float b = u[k] * py;
    float c = a + b;
    dir[k] = c + f[k];
    org[k] = cam->pos[k];
  }
  normalize3(dir);
}

void orc_camera_rays(const orc_camera *cam, float *org, float *dir) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)cam->width * cam->height; ++i)
    orc_camera_ray(cam, (uint32_t)(i % cam->width), (uint32_t)(i / cam->width), org + 3 * i, dir + 3 * i);
}

/* Watertight test (Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1),
 * 2013): shear the triangle into the ray's frame, 2D edge functions U, V, W with a
 * double-precision recomputation when one is exactly zero, then the scaled hit distance. */
int orc_ray_tri(const float org[3], const float dir[3], const float *v0, const float *v1,
                const float *v2, float tmin, float tmax, int cull, float *t_out) {
  float ax = fabsf(dir[0]), ay = fabsf(dir[1]), az = fabsf(dir[2]);
  int kz = (ax >= ay) ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  if (dir[kz] < 0.0f) { int tmp = kx; kx = ky; ky = tmp; }
  float sx = dir[kx] / dir[kz];
  float sy = dir[ky] / dir[kz];
  float sz = 1.0f / dir[kz];

  float A[3], B[3], C[3];
  for (int k = 0; k < 3; ++k) {
    A[k] = v0[k] - org[k];
    B[k] = v1[k] - org[k];
    C[k] = v2[k] - org[k];
  }
  float Ax = A[kx] - sx * A[kz], Ay = A[ky] - sy * A[kz];
  float Bx = B[kx] - sx * B[kz], By = B[ky] - sy * B[kz];
  float Cx = C[kx] - sx * C[kz], Cy = C[ky] - sy * C[kz];
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
    double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
    double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
    U = (float)(cxby - cybx);
    V = (float)(axcy - aycx);
    W = (float)(bxay - byax);
  }
  if (cull) {
    if (U < 0.0f || V < 0.0f || W < 0.0f) return 0;
  } else {
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
  }
  float det = U + V;
  det = det + W;
  if (det == 0.0f) return 0;
  float Az = sz * A[kz], Bz = sz * B[kz], Cz = sz * C[kz];
  float T = U * Az;
  float T1 = V * Bz;
  float T2 = W * Cz;
  T = T + T1;
  T = T + T2;
  float t = T / det;
  if (!(t > tmin) || !(t <= tmax)) return 0;
  *t_out = t;
  return 1;
}

void orc_trace_brute(const float *org, const float *dir, uint32_t n_rays, const float *vert,
                     const uint32_t *faces, uint32_t n_faces, float tmin, float tmax, int cull,
                     orc_hit *hits) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t r = 0; r < (int64_t)n_rays; ++r) {
    orc_hit h = {NONE, tmax};
    int any = 0;
    for (uint32_t f = 0; f < n_faces; ++f) {
      const uint32_t *fc = faces + 3 * (size_t)f;
      float t;
      if (orc_ray_tri(org + 3 * r, dir + 3 * r, vert + 3 * (size_t)fc[0], vert + 3 * (size_t)fc[1],
                      vert + 3 * (size_t)fc[2], tmin, tmax, cull, &t)) {
        if (!any || t < h.t) { h.t = t; h.prim = f; any = 1; }
      }
    }
    if (!any) { h.prim = NONE; h.t = INFINITY; }
    hits[r] = h;
  }
}

/* Slab test in double with a relative slack so that a box holding the closest hit is never
 * culled (the oracle must be conservative; visiting extra boxes changes nothing). */
static int box_hit(const orc_aabb *b, const double o[3], const double inv[3], double tmin, double tmax,
                   double *tn) {
  double t0 = tmin, t1 = tmax;
  for (int k = 0; k < 3; ++k) {
    double a = ((double)b->mn[k] - o[k]) * inv[k];
    double c = ((double)b->mx[k] - o[k]) * inv[k];
    if (isnan(a)) a = -INFINITY; /* 0 * inf: the ray lies in the slab plane */
    if (isnan(c)) c = INFINITY;
    double lo = a < c ? a : c, hi = a < c ? c : a;
    if (lo > t0) t0 = lo;
    if (hi < t1) t1 = hi;
  }
  *tn = t0;
  return t0 <= t1;
}

void orc_trace_bvh(const float *org, const float *dir, uint32_t n_rays, const orc_node *nodes,
                   uint32_t root, const float *vert, const uint32_t *faces, float tmin, float tmax,
                   int cull, orc_hit *hits) {
#pragma omp parallel
  {
    uint32_t *stack = malloc(sizeof(uint32_t) * 4096);
#pragma omp for schedule(dynamic, 64)
    for (int64_t r = 0; r < (int64_t)n_rays; ++r) {
      const float *ro = org + 3 * r, *rd = dir + 3 * r;
      double o[3] = {ro[0], ro[1], ro[2]};
      double inv[3] = {1.0 / (double)rd[0], 1.0 / (double)rd[1], 1.0 / (double)rd[2]};
      uint32_t best = NONE;
      float bt = tmax;
      uint32_t sp = 0;
      stack[sp++] = root;
      while (sp) {
        uint32_t x = stack[--sp];
        const orc_node *nd = &nodes[x];
        double tn;
        double lim = best == NONE ? (double)tmax : (double)bt * (1.0 + 1e-5) + 1e-6;
        if (!box_hit(&nd->bbox, o, inv, (double)tmin - 1e-6, lim, &tn)) continue;
        if (nd->isLeafFlag) {
          for (uint32_t f = nd->left; f < nd->left + nd->right; ++f) {
            const uint32_t *fc = faces + 3 * (size_t)f;
            float t;
            if (orc_ray_tri(ro, rd, vert + 3 * (size_t)fc[0], vert + 3 * (size_t)fc[1],
                            vert + 3 * (size_t)fc[2], tmin, tmax, cull, &t)) {
              if (best == NONE || t < bt || (t == bt && f < best)) { bt = t; best = f; }
            }
          }
        } else if (sp + 2 <= 4096) {
          stack[sp++] = nd->right;
          stack[sp++] = nd->left;
        }
      }
      hits[r].prim = best;
      hits[r].t = best == NONE ? INFINITY : bt;
    }
    free(stack);
  }
}

/* AABB::intersect (lib/base/BVH.hpp:77-101), float. */
static int ref_box(const orc_aabb *b, const float o[3], const float inv[3], const uint8_t sg[3], float t0,
                   float t1, float *tmin_out) {
  const float *lo = b->mn, *hi = b->mx;
  float tmin = ((sg[0] ? hi : lo)[0] - o[0]) * inv[0];
  float tmax = ((sg[0] ? lo : hi)[0] - o[0]) * inv[0];
  float tymin = ((sg[1] ? hi : lo)[1] - o[1]) * inv[1];
  float tymax = ((sg[1] ? lo : hi)[1] - o[1]) * inv[1];
  if ((tmin > tymax) || (tymin > tmax)) return 0;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  float tzmin = ((sg[2] ? hi : lo)[2] - o[2]) * inv[2];
  float tzmax = ((sg[2] ? lo : hi)[2] - o[2]) * inv[2];
  if ((tmin > tzmax) || (tzmin > tmax)) return 0;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  *tmin_out = tmin;
  return (tmin < t1) && (tmax > t0);
}

/* Moller-Trumbore in double, two-sided (the CPU tracers call glm::intersectRayTriangle<double>,
 * CPUTracer.cpp:115-121; glm is not available, so the textbook form is used). */
static int mt_double(const float *ro, const float *rd, const float *a, const float *b, const float *c,
                     double *t_out) {
  double e1[3], e2[3], p[3], s[3], q[3];
  for (int k = 0; k < 3; ++k) { e1[k] = (double)b[k] - a[k]; e2[k] = (double)c[k] - a[k]; s[k] = (double)ro[k] - a[k]; }
  p[0] = rd[1] * e2[2] - rd[2] * e2[1];
  p[1] = rd[2] * e2[0] - rd[0] * e2[2];
  p[2] = rd[0] * e2[1] - rd[1] * e2[0];
  double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
  if (det == 0.0) return 0;
  double f = 1.0 / det;
  double u = f * (s[0] * p[0] + s[1] * p[1] + s[2] * p[2]);
  if (u < 0.0 || u > 1.0) return 0;
  q[0] = s[1] * e1[2] - s[2] * e1[1];
  q[1] = s[2] * e1[0] - s[0] * e1[2];
  q[2] = s[0] * e1[1] - s[1] * e1[0];
  double v = f * (rd[0] * q[0] + rd[1] * q[1] + rd[2] * q[2]);
  if (v < 0.0 || u + v > 1.0) return 0;
  double t = f * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
  if (!(t > 0.0)) return 0;
  *t_out = t;
  return 1;
}

/* CPUTracer::trace (CPUTracer.cpp:56-162): stackless traversal with a 128-bit trail
 * (Afra & Szirmay-Kalos 2014), near child first, back-tracking through parent pointers. */
void orc_trace_cpu_reference(const float *org, const float *dir, uint32_t n_rays,
                             const orc_node *nodes, uint32_t root, const float *vert,
                             const uint32_t *faces, orc_hit *hits, uint16_t *int_count) {
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t r = 0; r < (int64_t)n_rays; ++r) {
    const float *ro = org + 3 * r, *rd = dir + 3 * r;
    float inv[3] = {1.0f / rd[0], 1.0f / rd[1], 1.0f / rd[2]};
    uint8_t sg[3] = {inv[0] < 0, inv[1] < 0, inv[2] < 0};
    unsigned __int128 trail = 0;
    uint32_t x = root, closest = NONE;
    float nearest = INFINITY;
    uint16_t cnt = 0;
    for (;;) {
      const orc_node *nd = &nodes[x];
      if (!nd->isLeafFlag) {
        cnt++;
        float tl, tr;
        int hl = ref_box(&nodes[nd->left].bbox, ro, inv, sg, 0.01f, nearest + 0.01f, &tl);
        int hr = ref_box(&nodes[nd->right].bbox, ro, inv, sg, 0.01f, nearest + 0.01f, &tr);
        if (hl || hr) {
          trail <<= 1;
          if (hl && hr) {
            trail |= 1;
            x = tl < tr ? nd->left : nd->right;
          } else {
            x = hl ? nd->left : nd->right;
          }
          continue;
        }
      } else {
        for (uint32_t f = nd->left; f < nd->left + nd->right; ++f) {
          const uint32_t *fc = faces + 3 * (size_t)f;
          double t;
          if (mt_double(ro, rd, vert + 3 * (size_t)fc[0], vert + 3 * (size_t)fc[1], vert + 3 * (size_t)fc[2], &t) &&
              t < nearest) {
            nearest = (float)t;
            closest = f;
          }
        }
      }
      while ((trail & 1) == 0) {
        if (trail == 0) goto done;
        x = nodes[x].parent;
        trail >>= 1;
      }
      {
        const orc_node *p = &nodes[nodes[x].parent];
        x = nodes[x].isLeft ? p->right : p->left;
      }
      trail ^= 1;
    }
  done:
    hits[r].prim = closest;
    hits[r].t = nearest;
    if (int_count) int_count[r] = cnt;
  }
}

/* Shade (CUDAKernels.cu:208-218): n = normalize(cross(v1 - v2, v1 - v3)) (glm::triangleNormal),
 * diffuse = max(1 + dot(n, normalize(light - hit)), 0) * 127 truncated to a byte. */
uint8_t orc_shade(const float org[3], const float dir[3], float t, const float *v1, const float *v2,
                  const float *v3, const float light[3]) {
  float a[3], b[3], n[3], h[3], l[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = v1[k] - v2[k];
    b[k] = v1[k] - v3[k];
  }
  cross3(a, b, n);
  normalize3(n);
  for (int k = 0; k < 3; ++k) {
    float td = t * dir[k];
    h[k] = org[k] + td;
    l[k] = light[k] - h[k];
  }
  normalize3(l);
  float d = 1.0f + dot3(n, l);
  d = d > 0.0f ? d : 0.0f;
  return (uint8_t)(d * 127.0f);
}
