// Test infrastructure only: geometric functions, view matrices, matrix inverse and the ray /
// triangle test of the vector-math interface the reference's CPU files call, written from their
// mathematical definitions (see shim_core.hpp for why this exists and what it claims).
#pragma once

#include "shim_core.hpp"

namespace glm {

template <typename T>
inline T radians(T deg) {
  return deg * static_cast<T>(0.01745329251994329576923690768489);
}

template <typename T>
inline T dot(const tvec3<T> &a, const tvec3<T> &b) {
  T x = a.x * b.x;
  T y = a.y * b.y;
  T z = a.z * b.z;
  return (x + y) + z;
}

template <typename T>
inline tvec3<T> cross(const tvec3<T> &a, const tvec3<T> &b) {
  return tvec3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

template <typename T>
inline T length(const tvec3<T> &v) {
  return std::sqrt(dot(v, v));
}

template <typename T>
inline tvec3<T> normalize(const tvec3<T> &v) {
  return v * (static_cast<T>(1) / std::sqrt(dot(v, v)));
}

// Unit normal of the triangle (a, b, c), counter-clockwise front face:
// (a - b) x (a - c) = (b - a) x (c - a).
template <typename T>
inline tvec3<T> triangleNormal(const tvec3<T> &a, const tvec3<T> &b, const tvec3<T> &c) {
  return normalize(cross(a - b, a - c));
}

// Right-handed view matrix: rows s, u, -f of the camera basis, translated by -eye.
template <typename T>
inline tmat4<T> lookAtRH(const tvec3<T> &eye, const tvec3<T> &center, const tvec3<T> &up) {
  const tvec3<T> f(normalize(center - eye));
  const tvec3<T> s(normalize(cross(f, up)));
  const tvec3<T> u(cross(s, f));
  tmat4<T> m(static_cast<T>(1));
  m[0][0] = s.x;
  m[1][0] = s.y;
  m[2][0] = s.z;
  m[0][1] = u.x;
  m[1][1] = u.y;
  m[2][1] = u.z;
  m[0][2] = -f.x;
  m[1][2] = -f.y;
  m[2][2] = -f.z;
  m[3][0] = -dot(s, eye);
  m[3][1] = -dot(u, eye);
  m[3][2] = dot(f, eye);
  return m;
}

template <typename T>
inline tmat4<T> lookAt(const tvec3<T> &eye, const tvec3<T> &center, const tvec3<T> &up) {
  return lookAtRH(eye, center, up);
}

// Right-handed perspective projection with depth mapped to [-1, 1].
template <typename T>
inline tmat4<T> perspective(T fovy, T aspect, T zNear, T zFar) {
  const T t = std::tan(fovy / static_cast<T>(2));
  tmat4<T> m(static_cast<T>(0));
  m[0][0] = static_cast<T>(1) / (aspect * t);
  m[1][1] = static_cast<T>(1) / t;
  m[2][2] = -(zFar + zNear) / (zFar - zNear);
  m[2][3] = -static_cast<T>(1);
  m[3][2] = -(static_cast<T>(2) * zFar * zNear) / (zFar - zNear);
  return m;
}

// General inverse by cofactors: inverse = adjugate / determinant. a[r][c] below is row r,
// column c of the matrix (m[c][r] in column storage).
template <typename T>
inline tmat4<T> inverse(const tmat4<T> &m) {
  T a[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) a[r][c] = m[c][r];
  // 2x2 minors of rows 2,3 and of rows 0,1 (columns i<j).
  auto minor2 = [&](int r0, int r1, int c0, int c1) { return a[r0][c0] * a[r1][c1] - a[r0][c1] * a[r1][c0]; };
  T cof[4][4];
  for (int r = 0; r < 4; ++r) {
    for (int c = 0; c < 4; ++c) {
      int rr[3], cc[3];
      for (int k = 0, n = 0; k < 4; ++k)
        if (k != r) rr[n++] = k;
      for (int k = 0, n = 0; k < 4; ++k)
        if (k != c) cc[n++] = k;
      T d = a[rr[0]][cc[0]] * minor2(rr[1], rr[2], cc[1], cc[2]) -
            a[rr[0]][cc[1]] * minor2(rr[1], rr[2], cc[0], cc[2]) +
            a[rr[0]][cc[2]] * minor2(rr[1], rr[2], cc[0], cc[1]);
      cof[r][c] = ((r + c) & 1) ? -d : d;
    }
  }
  T det = a[0][0] * cof[0][0] + a[0][1] * cof[0][1] + a[0][2] * cof[0][2] + a[0][3] * cof[0][3];
  tmat4<T> inv;
  // inverse[r][c] = cof[c][r] / det  ->  stored as inv[c][r] (column c, row r).
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) inv[c][r] = cof[c][r] / det;
  return inv;
}

// Moller & Trumbore (1997), two-sided: returns true when the ray orig + t dir meets the triangle
// (v0, v1, v2) with a determinant outside [-eps, eps]; bary = (u, v) and distance = t.
template <typename T>
inline bool intersectRayTriangle(const tvec3<T> &orig, const tvec3<T> &dir, const tvec3<T> &v0,
                                 const tvec3<T> &v1, const tvec3<T> &v2, tvec2<T> &bary, T &distance) {
  const tvec3<T> e1 = v1 - v0;
  const tvec3<T> e2 = v2 - v0;
  const tvec3<T> p = cross(dir, e2);
  const T det = dot(e1, p);
  const T eps = std::numeric_limits<T>::epsilon();
  tvec3<T> q;
  if (det > eps) {
    const tvec3<T> s = orig - v0;
    bary.x = dot(s, p);
    if (bary.x < T(0) || bary.x > det) return false;
    q = cross(s, e1);
    bary.y = dot(dir, q);
    if (bary.y < T(0) || bary.x + bary.y > det) return false;
  } else if (det < -eps) {
    const tvec3<T> s = orig - v0;
    bary.x = dot(s, p);
    if (bary.x > T(0) || bary.x < det) return false;
    q = cross(s, e1);
    bary.y = dot(dir, q);
    if (bary.y > T(0) || bary.x + bary.y < det) return false;
  } else {
    return false;
  }
  const T invDet = static_cast<T>(1) / det;
  distance = dot(e2, q) * invDet;
  bary *= invDet;
  return true;
}

}  // namespace glm
