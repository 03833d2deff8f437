// Shared device helpers: node layout, exactly-rounded float helpers, gpu-scope acquire/release
// atomics, bounded waits, error reporting and launch accounting.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bvhgb.h"

namespace bvhgb {

static_assert(sizeof(bvhgb_node) == 48, "BVHNode must stay 48 bytes (lib/base/BVH.hpp:113)");
static_assert(offsetof(bvhgb_node, parent) == 24, "BVHNode.parent offset");
static_assert(offsetof(bvhgb_node, isLeafFlag) == 36, "BVHNode.isLeafFlag offset");
static_assert(offsetof(bvhgb_node, surfaceArea) == 44, "BVHNode.surfaceArea offset");
static_assert(sizeof(bvhgb_pixel) == 4, "CUDAPixel is 4 bytes");
static_assert(sizeof(bvhgb_device_bvh) == 32, "device BVH image is 32 bytes");

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kSpinLimit = 1u << 24;  // bounded device-side waits

// Device-side error word layout (bitwise OR of these).
enum DeviceError : uint32_t {
  kErrTimeout = 1u,        // a bounded wait gave up
  kErrStackOverflow = 2u,  // traversal stack exhausted
  kErrBadIndex = 4u,       // an index outside its array was found and skipped
};

// ---- float helpers: each operation rounds once, no FMA contraction ---------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

struct Box {
  float mn[3];
  float mx[3];
};

// AABB::surfaceArea (lib/base/BVH.hpp:62-65) without contraction.
__device__ __forceinline__ float surface_area(const Box &b) {
  float dx = fsub(b.mx[0], b.mn[0]);
  float dy = fsub(b.mx[1], b.mn[1]);
  float dz = fsub(b.mx[2], b.mn[2]);
  float s = fadd(fmul(dx, dy), fmul(dx, dz));
  s = fadd(s, fmul(dy, dz));
  return fmul(2.0f, s);
}

// AABB::mergeWith (BVH.hpp:67-74): a keeps its value unless b is strictly smaller / larger.
__device__ __forceinline__ void merge_into(Box &a, const Box &b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a.mn[k] = a.mn[k] < b.mn[k] ? a.mn[k] : b.mn[k];
    a.mx[k] = a.mx[k] > b.mx[k] ? a.mx[k] : b.mx[k];
  }
}

// ---- node access ---------------------------------------------------------------------------
// The 48-byte node as three 16-byte words: [mn.xyz mx.x] [mx.yz parent left] [right flags level|pad sa]
__device__ __forceinline__ void load_node(const bvhgb_node *nodes, uint32_t i, float4 &a, float4 &b, float4 &c) {
  const float4 *p = reinterpret_cast<const float4 *>(nodes + i);
  a = __ldg(p);
  b = __ldg(p + 1);
  c = __ldg(p + 2);
}

// L2-coherent loads (bypass L1) for data written by other threads of the same launch.
__device__ __forceinline__ float4 ld_cg4(const void *p) { return __ldcg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ float2 ld_cg2(const void *p) { return __ldcg(reinterpret_cast<const float2 *>(p)); }
__device__ __forceinline__ uint32_t ld_cg(const uint32_t *p) { return __ldcg(p); }

__device__ __forceinline__ Box load_box_cg(const bvhgb_node *n) {
  float4 a = ld_cg4(n);
  float2 b = ld_cg2(reinterpret_cast<const char *>(n) + 16);
  Box r;
  r.mn[0] = a.x; r.mn[1] = a.y; r.mn[2] = a.z;
  r.mx[0] = a.w; r.mx[1] = b.x; r.mx[2] = b.y;
  return r;
}

// ---- gpu-scope atomics with explicit ordering (PTX memory model) ------------------------------
__device__ __forceinline__ uint32_t atom_exch_acq_rel(uint32_t *p, uint32_t v) {
  uint32_t r;
  asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(r) : "l"(p), "r"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t *p, uint32_t v) {
  uint32_t r;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "r"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t r;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(r) : "l"(p) : "memory");
  return r;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Order-preserving float <-> uint32 mapping for atomicMin/atomicMax on floats.
__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

}  // namespace bvhgb

// ---- host-side helpers shared by the translation units ---------------------------------------
namespace bvhgb {
void set_last_error(const char *what, cudaError_t e);
int check_launch(const char *what);
void count_launch(uint32_t n = 1);
void uncount_launches(uint64_t n);
inline cudaStream_t as_stream(bvhgb_stream s) { return reinterpret_cast<cudaStream_t>(s); }
inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }
int sm_count();
uint64_t context_id();
// cudaMalloc through the library's allocation-failure injection (bvhgb_debug_fail_allocations).
cudaError_t dev_malloc(void **p, size_t bytes);
template <typename T>
inline cudaError_t dev_malloc(T **p, size_t bytes) {
  return dev_malloc(reinterpret_cast<void **>(p), bytes);
}
}  // namespace bvhgb

#define BVHGB_CUDA_TRY(call)                          \
  do {                                                \
    cudaError_t e__ = (call);                         \
    if (e__ != cudaSuccess) {                         \
      ::bvhgb::set_last_error(#call, e__);            \
      return e__ == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR; \
    }                                                 \
  } while (0)

#define BVHGB_LAUNCH_CHECK(name)                      \
  do {                                                \
    ::bvhgb::count_launch();                          \
    int s__ = ::bvhgb::check_launch(name);            \
    if (s__ != BVHGB_OK) return s__;                  \
  } while (0)
