// Test infrastructure only: the subset of the vector-math library interface that the reference's
// CPU files compile against (lib/base/BVH.hpp, Ray.hpp, lib/misc/Camera.cpp,
// lib/tracer/CPUTracer.cpp, BruteForceTracer.cpp), written here from the mathematics because the
// reference's math submodule is empty in its tree. It is used only to compile the reference's own
// sources into oracle/_ref (the parity pin of the oracle); nothing in the product includes it.
//
// Conventions restated (their published definitions):
//  * vectors are plain component structs; arithmetic is component-wise, with a scalar broadcast
//    on either side;
//  * 4x4 matrices are stored as four column vectors; M * v = sum_j column_j * v[j], summed in
//    column order;
//  * dot(a, b) = a.x*b.x + a.y*b.y + a.z*b.z summed left to right; normalize(v) =
//    v * (1 / sqrt(dot(v, v)));
//  * lookAtRH builds the right-handed view matrix from the orthonormal basis f = normalize(center -
//    eye), s = normalize(cross(f, up)), u = cross(s, f); inverse() is the general cofactor inverse.
// The library version the reference used is unknown (no pinned commit), so ties to it at the
// last bit are not claimed; the files here only make the reference's own algorithms runnable.
#pragma once

#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>

namespace glm {

template <typename T>
struct tvec4;

template <typename T>
struct tvec2 {
  T x, y;
  tvec2() {}
  explicit tvec2(T s) : x(s), y(s) {}
  template <typename A, typename B>
  tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
  T &operator[](std::size_t i) { return (&x)[i]; }
  const T &operator[](std::size_t i) const { return (&x)[i]; }
  tvec2 &operator*=(T s) {
    x *= s;
    y *= s;
    return *this;
  }
};

template <typename T>
struct tvec3 {
  T x, y, z;
  tvec3() {}
  explicit tvec3(T s) : x(s), y(s), z(s) {}
  template <typename A, typename B, typename C>
  tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
  template <typename U>
  tvec3(const tvec3<U> &v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
  template <typename U>
  tvec3(const tvec4<U> &v);  // drops w
  T &operator[](std::size_t i) { return (&x)[i]; }
  const T &operator[](std::size_t i) const { return (&x)[i]; }
  tvec3 &operator+=(const tvec3 &o) {
    x += o.x;
    y += o.y;
    z += o.z;
    return *this;
  }
  tvec3 &operator-=(const tvec3 &o) {
    x -= o.x;
    y -= o.y;
    z -= o.z;
    return *this;
  }
  tvec3 &operator*=(T s) {
    x *= s;
    y *= s;
    z *= s;
    return *this;
  }
  tvec3 &operator/=(T s) {
    x /= s;
    y /= s;
    z /= s;
    return *this;
  }
};

template <typename T>
struct tvec4 {
  T x, y, z, w;
  tvec4() {}
  explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
  template <typename A, typename B, typename C, typename D>
  tvec4(A a, B b, C c, D d) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
  template <typename U, typename D>
  tvec4(const tvec3<U> &v, D d) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(d)) {}
  T &operator[](std::size_t i) { return (&x)[i]; }
  const T &operator[](std::size_t i) const { return (&x)[i]; }
};

template <typename T>
template <typename U>
tvec3<T>::tvec3(const tvec4<U> &v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}

// ---- component-wise arithmetic -------------------------------------------------------------
#define GLM_SHIM_BINOP(OP)                                                                         \
  template <typename T>                                                                            \
  inline tvec3<T> operator OP(const tvec3<T> &a, const tvec3<T> &b) {                              \
    return tvec3<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                                           \
  }                                                                                                \
  template <typename T>                                                                            \
  inline tvec3<T> operator OP(const tvec3<T> &a, T s) {                                            \
    return tvec3<T>(a.x OP s, a.y OP s, a.z OP s);                                                 \
  }                                                                                                \
  template <typename T>                                                                            \
  inline tvec3<T> operator OP(T s, const tvec3<T> &a) {                                            \
    return tvec3<T>(s OP a.x, s OP a.y, s OP a.z);                                                 \
  }                                                                                                \
  template <typename T>                                                                            \
  inline tvec4<T> operator OP(const tvec4<T> &a, const tvec4<T> &b) {                              \
    return tvec4<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                               \
  }                                                                                                \
  template <typename T>                                                                            \
  inline tvec4<T> operator OP(const tvec4<T> &a, T s) {                                            \
    return tvec4<T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s);                                       \
  }                                                                                                \
  template <typename T>                                                                            \
  inline tvec2<T> operator OP(const tvec2<T> &a, const tvec2<T> &b) {                              \
    return tvec2<T>(a.x OP b.x, a.y OP b.y);                                                       \
  }

GLM_SHIM_BINOP(+)
GLM_SHIM_BINOP(-)
GLM_SHIM_BINOP(*)
GLM_SHIM_BINOP(/)
#undef GLM_SHIM_BINOP

template <typename T>
inline tvec3<T> operator-(const tvec3<T> &a) {
  return tvec3<T>(-a.x, -a.y, -a.z);
}
template <typename T>
inline bool operator==(const tvec3<T> &a, const tvec3<T> &b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <typename T>
inline bool operator!=(const tvec3<T> &a, const tvec3<T> &b) {
  return !(a == b);
}

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using dvec2 = tvec2<double>;
using dvec3 = tvec3<double>;
using dvec4 = tvec4<double>;
using uvec3 = tvec3<uint32_t>;
using ivec3 = tvec3<int32_t>;

// ---- 4x4 matrices, four columns -----------------------------------------------------------
template <typename T>
struct tmat4 {
  tvec4<T> c[4];
  tmat4() {}
  explicit tmat4(T d) {
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) c[j][i] = (i == j) ? d : T(0);
  }
  tvec4<T> &operator[](std::size_t j) { return c[j]; }
  const tvec4<T> &operator[](std::size_t j) const { return c[j]; }
};
using mat4 = tmat4<float>;
using dmat4 = tmat4<double>;

template <typename T>
inline tvec4<T> operator*(const tmat4<T> &m, const tvec4<T> &v) {
  tvec4<T> r;
  for (int i = 0; i < 4; ++i) {
    T a = m[0][i] * v[0];
    T b = m[1][i] * v[1];
    T c = m[2][i] * v[2];
    T d = m[3][i] * v[3];
    r[i] = ((a + b) + c) + d;
  }
  return r;
}

template <typename T>
inline tmat4<T> operator*(const tmat4<T> &a, const tmat4<T> &b) {
  tmat4<T> r;
  for (int j = 0; j < 4; ++j) r[j] = a * b[j];
  return r;
}

}  // namespace glm
