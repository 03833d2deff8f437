// Learned reinsertion scorer: node features, the 24 -> 64 -> 64 -> 1 GELU MLP (BF16 weights,
// inputs and activations, FP32 accumulation) and its training kernels. The reference has no learned
// part; its node selection is the inefficiency of lib/builder/Bittner13CUDA.cu:480-500, which stays
// the default (bittner.cu) and evaluates the scorer by the SAH it reaches.
//
// Layout in HBM: feature rows are 24 BF16 values (48 bytes, three 16-byte words) per inner node in
// the order of the optimizer's ascending inner-node list; parameters are one FP32 master array of
// 5825 values plus its BF16 copy, AdamW moments beside them.
//
// GELU is the tanh approximation of Hendrycks and Gimpel, 0.5 z (1 + tanh(sqrt(2/pi)(z + 0.044715 z^3))).
// Backward passes the BF16 rounding of weights and activations through as identity; the gradients
// of the pre-activations are rounded to BF16 where they enter the tensor-core products.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "learned.cuh"

namespace bvhgb {
namespace {

constexpr int kIn = kMlpIn, kH = kMlpHidden;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH, oB3 = oW3 + kH;
static_assert(oB3 + 1 == kMlpParams, "parameter layout");
constexpr int kWPad = (kMlpParams + 3) & ~3;

constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float gelu(float z) {
  const float u = kGeluC * (z + kGeluA * z * z * z);
  return 0.5f * z * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float u = kGeluC * (z + kGeluA * z * z * z);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * kGeluC * (1.0f + 3.0f * kGeluA * z * z);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Inference GELU: tanh(u) = 1 - 2 / (1 + e^(2u)), e^(2u) = 2^(2u / ln 2) from the hardware's
// approximate base-2 exponential and 1 / (1 + e^(2u)) from its approximate reciprocal (relative
// errors near 2^-22 each), which leaves an absolute error of about 2e-7, far below the BF16 step
// the activations are rounded to; the infinite or zero exponential saturates it to +-1. Training
// keeps tanhf (its gradients are checked against float64).
__device__ __forceinline__ float tanh_fast(float u) {
  float e, r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(u * 2.8853900817779268f));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
  return fmaf(-2.0f, r, 1.0f);
}
__device__ __forceinline__ float gelu_fast(float z) {
  const float u = kGeluC * (z + kGeluA * z * z * z);
  return 0.5f * z * (1.0f + tanh_fast(u));
}
// Two values to BF16 in one conversion, packed low | high << 16.
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&p);
}

__device__ __forceinline__ void load_row(const uint16_t *__restrict__ x, size_t row, float in[kIn]) {
  const uint4 *p = reinterpret_cast<const uint4 *>(x + row * kIn);
#pragma unroll
  for (int w = 0; w < 3; ++w) {
    const uint4 v = __ldg(p + w);
    const uint32_t u[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      in[w * 8 + h * 2 + 0] = __uint_as_float(u[h] << 16);
      in[w * 8 + h * 2 + 1] = __uint_as_float(u[h] & 0xFFFF0000u);
    }
  }
}

__device__ __forceinline__ void load_weights(const __nv_bfloat16 *__restrict__ w, float *W) {
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) W[i] = __bfloat162float(w[i]);
}

// ---- inference on the 5th-generation tensor cores (tcgen05) ----------------------------------------
// Persistent CTAs of 4 warps; a tile is 128 rows. Layer 1: D1[128 x 64] = X[128 x 32] * W1^T (the 24
// features padded to K = 32), layer 2: D2[128 x 64] = A1[128 x 64] * W2^T, both BF16 operands in
// shared memory and FP32 accumulators in tensor memory (columns 0-63 and 64-127 of a 128-column
// allocation). Thread 0 issues the MMAs and commits them to an mbarrier; each warp then reads its 32
// accumulator rows (TMEM lanes 32w .. 32w + 31) with tcgen05.ld, adds the bias, applies GELU and
// rounds to BF16 (layer 1 into the next A operand, layer 2 straight into the 64 -> 1 dot product).
// Operand layout: the no-swizzle K-major canonical layout of 8-row x 16-byte core matrices, core
// (r8, k8) at r8 * SBO + k8 * LBO with LBO = 128 bytes (next 8 K-elements) and SBO = K * 16 bytes
// (next 8 rows); an MMA consumes K = 16, so its descriptors advance by 2 * LBO per step.
constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 128;        // tensor-memory columns per CTA
constexpr int kTcK1 = 32;                // layer-1 K (24 features + zero padding)
constexpr uint32_t kTcWaitLimit = 1u << 22;

struct TcSmem {
  alignas(128) uint8_t a1[kTcRows * kTcK1 * 2];  // X tile, 8 KB
  alignas(128) uint8_t b1[kH * kTcK1 * 2];       // W1 (N = 64 rows x K = 32), 4 KB
  alignas(128) uint8_t a2[kTcRows * kH * 2];     // layer-1 activations, 16 KB
  alignas(128) uint8_t b2[kH * kH * 2];          // W2 (64 x 64), 8 KB
  float b1f[kH], b2f[kH], w3f[kH], b3f;
  alignas(8) uint64_t bar;
  uint32_t tmem;
  uint32_t fail;
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a K-major operand with K columns in the core-matrix layout
__device__ __forceinline__ uint32_t core_off(uint32_t row, uint32_t k, uint32_t K) {
  return (row >> 3) * (K * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;  // descriptor version 0b001 (bits 46-48); base offset 0; no swizzle (bits 61-63 = 0)
  return d;
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N = 64, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kH >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(kTcIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase 'parity' of the barrier; false (and the CTA's fail flag) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *fail) {
  for (uint32_t i = 0; i < kTcWaitLimit; ++i) {
    if (mbar_try(bar, parity)) return true;
    if (i > 64) __nanosleep(64);
  }
  atomicOr(fail, 1u);
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <bool KEYS>
__global__ void __launch_bounds__(128, 4) mlp_forward_tc_kernel(const __nv_bfloat16 *__restrict__ w,
                                                                const uint16_t *__restrict__ x, uint32_t n,
                                                                float *__restrict__ y,
                                                                const uint32_t *__restrict__ inner,
                                                                uint32_t *__restrict__ keys,
                                                                uint32_t *__restrict__ vals, uint32_t *err) {
  __shared__ TcSmem sm;
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  const uint16_t *wb = reinterpret_cast<const uint16_t *>(w);
  // weights -> B operands (zero K padding for layer 1) and FP32 epilogue constants
  for (uint32_t i = tid; i < (uint32_t)(kH * kTcK1); i += blockDim.x) {
    const uint32_t j = i / kTcK1, k = i % kTcK1;
    *reinterpret_cast<uint16_t *>(sm.b1 + core_off(j, k, kTcK1)) = k < (uint32_t)kIn ? wb[oW1 + j * kIn + k] : 0;
  }
  for (uint32_t i = tid; i < (uint32_t)(kH * kH); i += blockDim.x) {
    const uint32_t j = i / kH, k = i % kH;
    *reinterpret_cast<uint16_t *>(sm.b2 + core_off(j, k, kH)) = wb[oW2 + j * kH + k];
  }
  for (uint32_t i = tid; i < (uint32_t)kH; i += blockDim.x) {
    sm.b1f[i] = __bfloat162float(w[oB1 + i]);
    sm.b2f[i] = __bfloat162float(w[oB2 + i]);
    sm.w3f[i] = __bfloat162float(w[oW3 + i]);
  }
  if (tid == 0) {
    sm.b3f = __bfloat162float(w[oB3]);
    sm.fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&sm.bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&sm.tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem;
  const uint32_t lanebase = (warp * 32u) << 16;  // this warp's TMEM lanes
  const uint32_t a1 = smem_addr(sm.a1), b1 = smem_addr(sm.b1), a2 = smem_addr(sm.a2), b2 = smem_addr(sm.b2);
  uint32_t phase = 0;
  bool failed = false;  // block-uniform: decided by __syncthreads_or after every wait
  const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t row = tile * kTcRows + tid;  // this thread's row (= its TMEM lane)
    const bool live = row < n;
    {  // feature row -> A1 (3 x 16 bytes of features, one 16-byte chunk of zero padding)
      uint4 q[3] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
      if (live) {
        const uint4 *src = reinterpret_cast<const uint4 *>(x + (size_t)row * kIn);
        q[0] = __ldg(src);
        q[1] = __ldg(src + 1);
        q[2] = __ldg(src + 2);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) *reinterpret_cast<uint4 *>(sm.a1 + core_off(tid, 8 * c, kTcK1)) = q[c];
      *reinterpret_cast<uint4 *>(sm.a1 + core_off(tid, 24, kTcK1)) = make_uint4(0, 0, 0, 0);
    }
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < kTcK1 / 16; ++k)
        tc_mma(tmem, tc_smem_desc(a1 + 256u * k, 128u, kTcK1 * 16u), tc_smem_desc(b1 + 256u * k, 128u, kTcK1 * 16u),
               k > 0);
      tc_commit(&sm.bar);
    }
    if (__syncthreads_or(!mbar_wait(&sm.bar, phase, &sm.fail))) {
      failed = true;
      break;
    }
    phase ^= 1u;
    tc_fence_after();
    // layer-1 epilogue: bias, GELU, BF16 -> A2 (this thread's row)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tc_ld32(tmem + lanebase + 32u * half, v);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        uint32_t u[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int j0 = 32 * half + 8 * c + 2 * h;
          const float g0 = gelu_fast(v[8 * c + 2 * h] + sm.b1f[j0]);
          const float g1 = gelu_fast(v[8 * c + 2 * h + 1] + sm.b1f[j0 + 1]);
          u[h] = bf16x2_bits(g0, g1);
        }
        *reinterpret_cast<uint4 *>(sm.a2 + core_off(tid, 32 * half + 8 * c, kH)) = make_uint4(u[0], u[1], u[2], u[3]);
      }
    }
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < kH / 16; ++k)
        tc_mma(tmem + 64u, tc_smem_desc(a2 + 256u * k, 128u, kH * 16u), tc_smem_desc(b2 + 256u * k, 128u, kH * 16u),
               k > 0);
      tc_commit(&sm.bar);
    }
    if (__syncthreads_or(!mbar_wait(&sm.bar, phase, &sm.fail))) {
      failed = true;
      break;
    }
    phase ^= 1u;
    tc_fence_after();
    // layer-2 epilogue and layer 3: y = b3 + sum_j W3[j] * bf16(gelu(D2[j] + b2[j]))
    float out = sm.b3f;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float v[32];
      tc_ld32(tmem + lanebase + 64u + 32u * half, v);
#pragma unroll
      for (int i = 0; i < 32; i += 2) {
        const uint32_t u = bf16x2_bits(gelu_fast(v[i] + sm.b2f[32 * half + i]),
                                       gelu_fast(v[i + 1] + sm.b2f[32 * half + i + 1]));
        out += sm.w3f[32 * half + i] * __uint_as_float(u << 16);
        out += sm.w3f[32 * half + i + 1] * __uint_as_float(u & 0xFFFF0000u);
      }
    }
    if (live) {
      y[row] = out;
      if (KEYS) {
        keys[row] = ~f2ord(out);
        vals[row] = __ldg(inner + row);
      }
    }
    tc_fence_before();  // the next tile's MMAs overwrite the accumulators these loads read
  }
  // Release the tensor memory on every path. After a timeout an MMA may still be in flight: wait
  // (bounded) for the last commit before freeing its columns.
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (failed) {
    if (tid == 0) {
      atomicOr(err, kErrTimeout);
      mbar_wait(&sm.bar, phase, &sm.fail);
    }
    __syncthreads();
  }
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

// Forward + backward of one tile of kTile samples per block, every contraction on the tensor cores
// (mma.sync m16n8k16, BF16 operands, FP32 accumulation). Gradients of loss = sum (y - t)^2 / scaleN
// are stored as the tile's row of part (FP32); the tile's loss is added to loss[slot].
//   forward   Z1[q][j] = b1 + X[q][:] . W1[j][:]    (q = sample, K = 24 features padded to 32)
//             Z2[q][j] = b2 + A1[q][:] . W2[j][:]   (A1 = bf16(gelu(Z1)), K = 64)
//             y[q]     = b3 + sum_j W3[j] bf16(gelu(Z2[q][j]))
//   backward  dZ2[q][j] = bf16(dY[q] W3[j] gelu'(Z2[q][j])),  dZ1[q][i] = bf16(sum_j dZ2[q][j] W2[j][i] gelu'(Z1[q][i]))
//             dW2[j][i] = sum_q dZ2[q][j] A1[q][i],  dW1[j][f] = sum_q dZ1[q][j] X[q][f]  (K = the 128 samples)
// The two gradient rounding points (dZ2, dZ1 to BF16) are the tensor cores' operand type; the FP64
// oracle (oracle/mlp.py) rounds at the same places. Sums over the tile run in a fixed order, so a
// training step repeats bit for bit.
constexpr int kTile = 128;                 // samples per block, 4 warps
constexpr int kK1 = 32;                    // layer-1 K: 24 features + 8 zeros
constexpr int kSX = 40;                    // bf16 row strides chosen so fragment loads hit distinct banks
constexpr int kSH = 72;
constexpr int kSZ = 68;                    // fp32 row stride of the pre-activations
constexpr size_t kTrainSmem = sizeof(float) * (kWPad + 2 * kTile * kSZ + kTile) +
                              sizeof(uint16_t) * (kH * kSX + 2 * kH * kSH + kTile * kSX + 3 * kTile * kSH);

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ uint32_t ld32(const uint16_t *p) { return *reinterpret_cast<const uint32_t *>(p); }
__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }
__device__ __forceinline__ uint16_t bf16_u16(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// A fragment of a 16 x 16 tile at (r0, k0) of a row-major [row][k] array (g = lane / 4, t = lane % 4).
__device__ __forceinline__ void frag_a(const uint16_t *m, int stride, int r0, int k0, int g, int t, uint32_t a[4]) {
  const uint16_t *p = m + (r0 + g) * stride + k0 + 2 * t;
  a[0] = ld32(p);
  a[1] = ld32(p + 8 * stride);
  a[2] = ld32(p + 8);
  a[3] = ld32(p + 8 * stride + 8);
}
// A fragment of the transpose: element (r, k) of the tile is m[k][r].
__device__ __forceinline__ void frag_a_t(const uint16_t *m, int stride, int r0, int k0, int g, int t, uint32_t a[4]) {
  const uint16_t *p = m + (k0 + 2 * t) * stride + r0 + g;
  a[0] = pack2(p[0], p[stride]);
  a[1] = pack2(p[8], p[stride + 8]);
  a[2] = pack2(p[8 * stride], p[9 * stride]);
  a[3] = pack2(p[8 * stride + 8], p[9 * stride + 8]);
}
// B fragment (16 x 8 at (k0, n0)) of an array stored [n][k] (so element (k, n) = m[n][k]).
__device__ __forceinline__ void frag_b(const uint16_t *m, int stride, int k0, int n0, int g, int t, uint32_t b[2]) {
  const uint16_t *p = m + (n0 + g) * stride + k0 + 2 * t;
  b[0] = ld32(p);
  b[1] = ld32(p + 8);
}
// B fragment of an array stored [k][n].
__device__ __forceinline__ void frag_b_t(const uint16_t *m, int stride, int k0, int n0, int g, int t, uint32_t b[2]) {
  const uint16_t *p = m + (k0 + 2 * t) * stride + n0 + g;
  b[0] = pack2(p[0], p[stride]);
  b[1] = pack2(p[8 * stride], p[9 * stride]);
}

__global__ void __launch_bounds__(kTile) mlp_train_kernel(const __nv_bfloat16 *__restrict__ w,
                                                          const uint16_t *__restrict__ x, const float *__restrict__ tgt,
                                                          const uint32_t *__restrict__ index, uint32_t n, float scaleN,
                                                          float *__restrict__ part, float *__restrict__ lossBase,
                                                          const uint32_t *__restrict__ stepDev, uint32_t step0,
                                                          uint32_t lossCap) {
  extern __shared__ __align__(16) float sm[];
  float *grad = part + (size_t)blockIdx.x * kMlpParams;
  float *W = sm;                       // fp32 copy of the (BF16) parameters: biases and W3
  float *Z1 = W + kWPad;               // [q][j] pre-activations
  float *Z2 = Z1 + kTile * kSZ;
  float *dY = Z2 + kTile * kSZ;
  uint16_t *sW1 = reinterpret_cast<uint16_t *>(dY + kTile);  // [j][f], f padded to 32
  uint16_t *sW2 = sW1 + kH * kSX;                             // [j][i]
  uint16_t *sW2T = sW2 + kH * kSH;                            // [i][j]
  uint16_t *sX = sW2T + kH * kSH;                             // [q][f]
  uint16_t *sA1 = sX + kTile * kSX;                           // [q][i] = bf16(gelu(Z1))
  uint16_t *sD2 = sA1 + kTile * kSH;                          // [q][j] = dZ2
  uint16_t *sD1 = sD2 + kTile * kSH;                          // [q][i] = dZ1; first the layer-2 activations
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const int g = (int)(lane >> 2), t = (int)(lane & 3u);
  const uint16_t *wb = reinterpret_cast<const uint16_t *>(w);
  for (int i = tid; i < kMlpParams; i += kTile) W[i] = bf16_val(__ldg(wb + i));
  for (int i = tid; i < kH * kK1; i += kTile) {
    const int j = i / kK1, f = i % kK1;
    sW1[j * kSX + f] = f < kIn ? __ldg(wb + oW1 + j * kIn + f) : (uint16_t)0;
  }
  for (int i = tid; i < kH * kH; i += kTile) {
    const int j = i / kH, k = i % kH;
    const uint16_t v = __ldg(wb + oW2 + i);
    sW2[j * kSH + k] = v;
    sW2T[k * kSH + j] = v;
  }
  {
    const uint32_t s = blockIdx.x * kTile + tid;
    const bool live = s < n;
    const uint32_t row = live ? (index ? __ldg(index + s) : s) : 0u;
    const uint4 *p = reinterpret_cast<const uint4 *>(x + (size_t)row * kIn);
    uint32_t *dst = reinterpret_cast<uint32_t *>(sX + tid * kSX);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const uint4 v = live ? __ldg(p + c) : make_uint4(0u, 0u, 0u, 0u);
      dst[4 * c + 0] = v.x;
      dst[4 * c + 1] = v.y;
      dst[4 * c + 2] = v.z;
      dst[4 * c + 3] = v.w;
    }
#pragma unroll
    for (int c = 12; c < kK1 / 2; ++c) dst[c] = 0u;
  }
  __syncthreads();

  // ---- forward: warp w owns samples [32w, 32w + 32), two 16-row tiles ----
  const int q0 = 32 * (int)warp;
  float yPart[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};  // [tile][row g / g + 8]
  for (int mt = 0; mt < 2; ++mt) {
    const int r0 = q0 + 16 * mt;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float b0 = W[oB1 + 8 * nt + 2 * t], b1v = W[oB1 + 8 * nt + 2 * t + 1];
      acc[nt][0] = b0;
      acc[nt][1] = b1v;
      acc[nt][2] = b0;
      acc[nt][3] = b1v;
    }
#pragma unroll
    for (int k0 = 0; k0 < kK1; k0 += 16) {
      uint32_t a[4];
      frag_a(sX, kSX, r0, k0, g, t, a);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b[2];
        frag_b(sW1, kSX, k0, 8 * nt, g, t, b);
        mma16816(acc[nt], a, b);
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = r0 + g + 8 * h, j = 8 * nt + 2 * t;
        Z1[q * kSZ + j] = acc[nt][2 * h];
        Z1[q * kSZ + j + 1] = acc[nt][2 * h + 1];
        sA1[q * kSH + j] = bf16_u16(gelu(acc[nt][2 * h]));
        sA1[q * kSH + j + 1] = bf16_u16(gelu(acc[nt][2 * h + 1]));
      }
    }
  }
  __syncwarp();
  for (int mt = 0; mt < 2; ++mt) {
    const int r0 = q0 + 16 * mt;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float b0 = W[oB2 + 8 * nt + 2 * t], b1v = W[oB2 + 8 * nt + 2 * t + 1];
      acc[nt][0] = b0;
      acc[nt][1] = b1v;
      acc[nt][2] = b0;
      acc[nt][3] = b1v;
    }
#pragma unroll
    for (int k0 = 0; k0 < kH; k0 += 16) {
      uint32_t a[4];
      frag_a(sA1, kSH, r0, k0, g, t, a);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b[2];
        frag_b(sW2, kSH, k0, 8 * nt, g, t, b);
        mma16816(acc[nt], a, b);
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = r0 + g + 8 * h, j = 8 * nt + 2 * t;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const float z = acc[nt][2 * h + e];
          Z2[q * kSZ + j + e] = z;
          const uint16_t a2 = bf16_u16(gelu(z));
          sD1[q * kSH + j + e] = a2;  // the layer-2 activations, until dZ1 takes the buffer
          yPart[mt][h] += W[oW3 + j + e] * bf16_val(a2);
        }
      }
    }
  }
  // y of each row: the four lanes of a quad hold its 64 columns
  float lsum = 0.0f;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float v = yPart[mt][h];
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 1);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 2);
      const int q = q0 + 16 * mt + g + 8 * h;
      const uint32_t s = blockIdx.x * kTile + q;
      const bool live = s < n;
      const uint32_t row = live ? (index ? __ldg(index + s) : s) : 0u;
      const float yv = W[oB3] + v;
      const float diff = live ? yv - __ldg(tgt + row) : 0.0f;
      if (t == 0) {
        dY[q] = 2.0f * diff / scaleN;
        lsum += diff * diff / scaleN;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, o);
  if (lane == 0) {
    uint32_t slot = 0;
    if (stepDev) slot = *stepDev - step0;
    if (slot < lossCap) atomicAdd(lossBase + slot, lsum);
  }
  __syncwarp();
  // dZ2 of the warp's rows
  for (int i = lane; i < 32 * kH; i += 32) {
    const int q = q0 + i / kH, j = i % kH;
    sD2[q * kSH + j] = bf16_u16(dY[q] * W[oW3 + j] * gelu_grad(Z2[q * kSZ + j]));
  }
  __syncthreads();
  // dW3[j] = sum_q dY[q] A2[q][j], db3 = sum_q dY[q]: a warp per unit, lanes over samples
  for (int j = warp; j < kH; j += kTile / 32) {
    float gsum = 0.0f;
    for (int q = lane; q < kTile; q += 32) gsum += dY[q] * bf16_val(sD1[q * kSH + j]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gsum += __shfl_xor_sync(0xFFFFFFFFu, gsum, o);
    if (lane == 0) grad[oW3 + j] = gsum;
  }
  if (warp == 0) {
    float gsum = 0.0f;
    for (int q = lane; q < kTile; q += 32) gsum += dY[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gsum += __shfl_xor_sync(0xFFFFFFFFu, gsum, o);
    if (lane == 0) grad[oB3] = gsum;
  }
  // dA1 = dZ2 . W2 for the warp's rows (registers), then dZ1 once every warp has read the
  // activations out of sD1
  float dacc[2][8][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const int r0 = q0 + 16 * mt;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) dacc[mt][nt][0] = dacc[mt][nt][1] = dacc[mt][nt][2] = dacc[mt][nt][3] = 0.0f;
#pragma unroll
    for (int k0 = 0; k0 < kH; k0 += 16) {
      uint32_t a[4];
      frag_a(sD2, kSH, r0, k0, g, t, a);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b[2];
        frag_b(sW2T, kSH, k0, 8 * nt, g, t, b);
        mma16816(dacc[mt][nt], a, b);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = q0 + 16 * mt + g + 8 * h, i = 8 * nt + 2 * t;
#pragma unroll
        for (int e = 0; e < 2; ++e)
          sD1[q * kSH + i + e] = bf16_u16(dacc[mt][nt][2 * h + e] * gelu_grad(Z1[q * kSZ + i + e]));
      }
    }
  }
  __syncthreads();
  // ---- weight gradients: warp w owns units [16w, 16w + 16), K = the tile's samples ----
  {
    const int j0 = 16 * (int)warp;
    float g2[8][4], g1[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) g2[nt][0] = g2[nt][1] = g2[nt][2] = g2[nt][3] = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) g1[nt][0] = g1[nt][1] = g1[nt][2] = g1[nt][3] = 0.0f;
#pragma unroll 2
    for (int k0 = 0; k0 < kTile; k0 += 16) {
      uint32_t a2[4], a1[4];
      frag_a_t(sD2, kSH, j0, k0, g, t, a2);
      frag_a_t(sD1, kSH, j0, k0, g, t, a1);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b[2];
        frag_b_t(sA1, kSH, k0, 8 * nt, g, t, b);
        mma16816(g2[nt], a2, b);
      }
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        uint32_t b[2];
        frag_b_t(sX, kSX, k0, 8 * nt, g, t, b);
        mma16816(g1[nt], a1, b);
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = j0 + g + 8 * h;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        grad[oW2 + j * kH + 8 * nt + 2 * t] = g2[nt][2 * h];
        grad[oW2 + j * kH + 8 * nt + 2 * t + 1] = g2[nt][2 * h + 1];
      }
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int f = 8 * nt + 2 * t + e;
          if (f < kIn) grad[oW1 + j * kIn + f] = g1[nt][2 * h + e];
        }
      }
    }
  }
  // bias gradients: a warp per unit, lanes over samples
  for (int j = warp; j < kH; j += kTile / 32) {
    float b2 = 0.0f, b1 = 0.0f;
    for (int q = lane; q < kTile; q += 32) {
      b2 += bf16_val(sD2[q * kSH + j]);
      b1 += bf16_val(sD1[q * kSH + j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      b2 += __shfl_xor_sync(0xFFFFFFFFu, b2, o);
      b1 += __shfl_xor_sync(0xFFFFFFFFu, b1, o);
    }
    if (lane == 0) {
      grad[oB2 + j] = b2;
      grad[oB1 + j] = b1;
    }
  }
}

// g = the sum of the tiles' gradient rows, in tile order.
__global__ void grad_reduce_kernel(const float *__restrict__ part, uint32_t tiles, float *__restrict__ g) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)kMlpParams) return;
  float acc = 0.0f;
  for (uint32_t b = 0; b < tiles; ++b) acc += part[(size_t)b * kMlpParams + i];
  g[i] = acc;
}

// AdamW (Loshchilov and Hutter) on all parameters in one block: moments, bias correction with the
// step count t = *stepDev + 1, decoupled weight decay on weights only; refreshes the BF16 copy,
// clears the gradient and advances the device step counter.
__global__ void __launch_bounds__(1024) adamw_kernel(float *__restrict__ p, __nv_bfloat16 *__restrict__ pb,
                                                     float *__restrict__ g, float *__restrict__ m,
                                                     float *__restrict__ v, uint32_t *stepDev, float lr, float wd) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float t = (float)(*stepDev + 1u);
  const float c1 = 1.0f - powf(b1, t), c2 = 1.0f - powf(b2, t);
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const bool bias = (i >= oB1 && i < oW2) || (i >= oB2 && i < oW3) || i == oB3;
    float pi = p[i];
    if (!bias) pi -= lr * wd * pi;
    pi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
    g[i] = 0.0f;
  }
  __syncthreads();
  if (threadIdx.x == 0) *stepDev += 1u;
}

__global__ void to_bf16_kernel(const float *__restrict__ p, __nv_bfloat16 *__restrict__ pb, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pb[i] = __float2bfloat16_rn(p[i]);
}

// Batch rows for step t = *stepDev + 1: SplitMix64 of (seed, t, i), reduced modulo numSamples.
__global__ void batch_index_kernel(uint32_t *__restrict__ idx, uint32_t batch, uint32_t numSamples, uint64_t seed,
                                   const uint32_t *__restrict__ stepDev) {
  const uint64_t t = (uint64_t)*stepDev + 1u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < batch; i += gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (t * (uint64_t)batch + i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    idx[i] = (uint32_t)(z % numSamples);
  }
}

// ---- features ----------------------------------------------------------------------------------

__device__ __forceinline__ float clamp64(float v) { return fminf(fmaxf(v, -64.0f), 64.0f); }
__device__ __forceinline__ float nan0(float v) { return isnan(v) ? 0.0f : v; }
__device__ __forceinline__ uint32_t rank_bin(float v) { return f2ord(v) >> 16; }

// Depth by pointer jumping on ad[x] = distance << 32 | ancestor: each round replaces a node's
// ancestor a by a's own (ad[a] read whole, so the pair is always an ancestor and its distance,
// whichever round wrote it). A round follows kDepthHops pointers beyond the node's own: if every
// pointer reached R levels when the round began, the node now reaches at least (kDepthHops + 1) R,
// so after kDepthLaunches rounds it is the root or 4^4 = 256 levels up, and the features get
// min(depth, 2^kDepthRounds) exactly. Only inner nodes jump (a leaf is nobody's ancestor and its
// depth is not a feature); a node whose ancestor is the root is done.
constexpr int kDepthHops = 3, kDepthLaunches = 4;
static_assert(kDepthHops == 3 && kDepthLaunches == 4 && kDepthRounds == 8, "(hops + 1)^launches >= 2^rounds");
// One coalesced pass over the nodes: the depth recursion's start, and compact copies of every
// node's surface area and parent (bit 31: the node is a leaf) that the leaf counts and the feature
// rows gather from (33 MB per 8M nodes each, so they stay in L2 where the 48-byte records do not).
constexpr uint32_t kLeafBit = 0x80000000u;
__global__ void depth_init_kernel(const bvhgb_node *__restrict__ t, uint32_t n, uint32_t root,
                                  unsigned long long *__restrict__ ad, float *__restrict__ sa,
                                  uint32_t *__restrict__ par) {
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
    const float4 w1 = __ldg(reinterpret_cast<const float4 *>(t + x) + 1);  // mx.y mx.z parent left
    const float4 w2 = __ldg(reinterpret_cast<const float4 *>(t + x) + 2);  // right flags level sa
    const uint32_t p = __float_as_uint(w1.z);
    const uint32_t a = (x == root || p >= n) ? root : p;
    ad[x] = ((unsigned long long)(x == root ? 0u : 1u) << 32) | a;
    sa[x] = w2.w;
    par[x] = (p & ~kLeafBit) | ((__float_as_uint(w2.y) & 0xFFFFu) ? kLeafBit : 0u);
  }
}
__global__ void depth_jump_kernel(const uint32_t *__restrict__ inner, uint32_t numInner, uint32_t n, uint32_t root,
                                  unsigned long long *ad) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < numInner; i += gridDim.x * blockDim.x) {
    const uint32_t x = __ldg(inner + i);
    if (x >= n) continue;  // flagged by the feature rows
    const unsigned long long v = __ldcg(ad + x);
    uint32_t a = (uint32_t)v, d = (uint32_t)(v >> 32);
    if (a == root || a >= n) continue;
#pragma unroll
    for (int h = 0; h < kDepthHops; ++h) {
      const unsigned long long w = __ldcg(ad + a);
      d += (uint32_t)(w >> 32);
      a = (uint32_t)w;
      if (a == root || a >= n) break;
    }
    __stcg(ad + x, ((unsigned long long)d << 32) | a);
  }
}
// Leaf counts bottom-up. A leaf starts a climb with count 1; at each parent the two arrivals add
// 2^40 + their count to the parent's 64-bit accumulator: the first sees 0 and stops, the second
// receives the first's count in the same atomic, writes the parent's count and goes on. The count
// travels in the atomic itself, so no fence or sibling load is needed; the next parent is loaded
// before the atomic.
__global__ void leaf_count_kernel(const uint32_t *__restrict__ par, uint32_t n, uint32_t root, uint32_t *cnt,
                                  unsigned long long *acc, uint32_t *err) {
  constexpr unsigned long long kArrival = 1ull << 40;
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
    const uint32_t pv = __ldg(par + x);
    if (!(pv & kLeafBit)) continue;
    __stcg(cnt + x, 1u);
    if (x == root) continue;
    uint32_t c = 1;
    uint32_t y = pv & ~kLeafBit;
    for (uint32_t steps = 0;; ++steps) {
      if (y >= n || steps > n) {
        atomicOr(err, kErrBadIndex);
        break;
      }
      const uint32_t next = y == root ? root : (__ldg(par + y) & ~kLeafBit);
      const unsigned long long old = atomicAdd(acc + y, kArrival | c);
      if (old == 0ull) break;  // first arrival: the sibling's climb continues
      c += (uint32_t)(old & (kArrival - 1ull));
      __stcg(cnt + y, c);
      if (y == root) break;
      y = next;
    }
  }
}

__device__ __forceinline__ uint32_t bf16_bits(float v) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ uint32_t bf16_pair(float lo, float hi) { return bf16_bits(lo) | (bf16_bits(hi) << 16); }

// The rank histograms: kHistCopies copies of the four count histograms (a block adds into copy
// blockIdx % kHistCopies, so that the few hot bins are not one address for the whole grid), summed
// into copy 0 before the scan, then the four exclusive prefixes.
constexpr uint32_t kHistCopies = 16;
constexpr size_t kHistPrefix = (size_t)kHistCopies * 4 * kRankBins;  // offset of the prefixes
constexpr size_t kHistWords = kHistPrefix + 4 * kRankBins;

// Raw features and the four rank histograms. A feature row is three 16-byte blocks: features 0-7 and
// the zero padding 16-23 are final here and stored at once; the middle block (features 8-9 and
// the four ranks) waits for the histograms, so features 8-9 and the rank bins go to pend[i]. The
// loop is warp-uniform so that the lanes of a warp that fall into the same histogram bin add their
// count with one atomic (the values of neighbouring nodes are alike, so a few bins are hot).
__global__ void features_raw_kernel(const bvhgb_node *__restrict__ t, const uint32_t *__restrict__ inner,
                                    uint32_t numInner, uint32_t numNodes, uint32_t root,
                                    const unsigned long long *__restrict__ depth, const uint32_t *__restrict__ leafCount,
                                    const float *__restrict__ saOf, const uint32_t *__restrict__ par,
                                    float invLog2Leaves, uint16_t *__restrict__ rows, uint4 *__restrict__ pend,
                                    uint32_t *__restrict__ hist, uint32_t *__restrict__ err) {
  const float sroot = __ldg(saOf + root);
  uint32_t *hc = hist + (size_t)(blockIdx.x % kHistCopies) * 4 * kRankBins;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < numInner; base += stride) {
    const uint32_t i = base + threadIdx.x;
    const bool live = i < numInner;
    float s4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (live) {
      float f[kMlpRaw];
#pragma unroll
      for (int k = 0; k < kMlpRaw; ++k) f[k] = 0.0f;
      const uint32_t x = __ldg(inner + i);
      if (x >= numNodes) {  // not a node: a zero row, flagged
        atomicOr(err, kErrBadIndex);
      } else {
        const float4 w1 = __ldg(reinterpret_cast<const float4 *>(t + x) + 1);  // mx.y mx.z parent left
        const float4 w2 = __ldg(reinterpret_cast<const float4 *>(t + x) + 2);  // right flags level sa
        const float sa = w2.w;
        const uint32_t l = min(__float_as_uint(w1.w), numNodes - 1), r = min(__float_as_uint(w2.x), numNodes - 1);
        const float sl = __ldg(saOf + l), sr = __ldg(saOf + r);
        const uint32_t p = x == root ? root : min(__float_as_uint(w1.z), numNodes - 1);
        const uint32_t g = p == root ? root : min(__ldg(par + p) & ~kLeafBit, numNodes - 1);
        const float mn = sl < sr ? sl : sr;
        const float sum = fadd(sl, sr);
        const float cost = fdiv(fmul(fmul(fmul(sa, sa), sa), 2.0f), fmul(sum, mn));  // kCalcCost
        const uint32_t d = (uint32_t)min(depth[x] >> 32, 1ull << kDepthRounds);
        f[0] = log2f(sa);
        f[1] = fdiv(sa, __ldg(saOf + p));
        f[2] = fdiv(sa, __ldg(saOf + g));
        f[3] = fdiv(sa, sum);
        f[4] = fmul((float)d, invLog2Leaves);
        f[5] = log2f((float)__ldcg(leafCount + l));
        f[6] = log2f((float)__ldcg(leafCount + r));
        f[7] = log2f(fdiv(sa, sroot));
        f[8] = log2f(fdiv(sa, mn));
        f[9] = log2f(cost);
#pragma unroll
        for (int k = 0; k < kMlpRaw; ++k) f[k] = clamp64(f[k]);
        s4[0] = nan0(cost);
        s4[1] = nan0(fdiv(sa, mn));
        s4[2] = nan0(fdiv(sa, sum));
        s4[3] = nan0(sa);
      }
      static_assert(kMlpRaw == 10 && kIn == 24, "row blocks: features 0-7, 8-15 (8-9 raw, 10-13 ranks), 16-23");
      uint4 *o = reinterpret_cast<uint4 *>(rows + (size_t)i * kIn);
      o[0] = make_uint4(bf16_pair(f[0], f[1]), bf16_pair(f[2], f[3]), bf16_pair(f[4], f[5]), bf16_pair(f[6], f[7]));
      o[2] = make_uint4(0u, 0u, 0u, 0u);
      pend[i] = make_uint4(rank_bin(s4[0]) | (rank_bin(s4[1]) << 16), rank_bin(s4[2]) | (rank_bin(s4[3]) << 16),
                           bf16_pair(f[8], f[9]), 0u);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t bin = live ? rank_bin(s4[q]) : 0xFFFFFFFFu;
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, bin);
      if (live && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(hc + q * kRankBins + bin, (uint32_t)__popc(peers));
    }
  }
}

// Copy 0 of the count histograms += the other copies.
__global__ void hist_reduce_kernel(uint32_t *hist) {
  constexpr uint32_t n4 = kRankBins;  // 16-byte vectors per copy (4 histograms)
  uint4 *h = reinterpret_cast<uint4 *>(hist);
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n4; j += gridDim.x * blockDim.x) {
    uint4 a = h[j];
#pragma unroll
    for (uint32_t c = 1; c < kHistCopies; ++c) {
      const uint4 b = h[(size_t)c * n4 + j];
      a.x += b.x;
      a.y += b.y;
      a.z += b.z;
      a.w += b.w;
    }
    h[j] = a;
  }
}

// Exclusive prefix of each of the four histograms (copy 0) into the prefix area (one block each).
__global__ void __launch_bounds__(1024) hist_scan_kernel(uint32_t *hist) {
  constexpr uint32_t kPer = kRankBins / 1024;
  __shared__ uint32_t warpSum[32];
  const uint32_t *h = hist + blockIdx.x * kRankBins;
  uint32_t *pre = hist + kHistPrefix + blockIdx.x * kRankBins;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  // Each thread owns kPer consecutive bins, read (and written) as 16-byte vectors.
  static_assert(kPer % 16 == 0, "vector access");
  const uint4 *h4 = reinterpret_cast<const uint4 *>(h + tid * kPer);
  uint32_t local = 0;
  for (uint32_t k0 = 0; k0 < kPer / 4; k0 += 4) {
    uint4 v[4];
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) v[k] = h4[k0 + k];
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) local += v[k].x + v[k].y + v[k].z + v[k].w;
  }
  uint32_t inc = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= (uint32_t)o) inc += v;
  }
  if (lane == 31) warpSum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = warpSum[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= (uint32_t)o) wi += v;
    }
    warpSum[lane] = wi - w;
  }
  __syncthreads();
  uint32_t run = warpSum[warp] + inc - local;
  uint4 *p4 = reinterpret_cast<uint4 *>(pre + tid * kPer);
  for (uint32_t k0 = 0; k0 < kPer / 4; k0 += 4) {
    uint4 v[4];
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) v[k] = h4[k0 + k];
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
      uint4 o;
      o.x = run; run += v[k].x;
      o.y = run; run += v[k].y;
      o.z = run; run += v[k].z;
      o.w = run; run += v[k].w;
      p4[k0 + k] = o;
    }
  }
}

// The middle block of each row: features 8-9 (from pend) and the four ranks (mid-rank of the row's
// bin: the values below it plus half of those in it, over the row count).
__global__ void features_pack_kernel(const uint4 *__restrict__ pend, const uint32_t *__restrict__ hist,
                                     uint32_t numInner, uint16_t *__restrict__ x) {
  const float fn = (float)numInner;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < numInner; i += gridDim.x * blockDim.x) {
    const uint4 pd = pend[i];
    const uint32_t bins[4] = {pd.x & 0xFFFFu, pd.x >> 16, pd.y & 0xFFFFu, pd.y >> 16};
    float r[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float below = (float)hist[kHistPrefix + q * kRankBins + bins[q]];
      const float own = (float)hist[q * kRankBins + bins[q]];
      r[q] = fdiv(fadd(below, fmul(0.5f, own)), fn);
    }
    reinterpret_cast<uint4 *>(x + (size_t)i * kIn)[1] = make_uint4(pd.z, bf16_pair(r[0], r[1]), bf16_pair(r[2], r[3]), 0u);
  }
}

// Persistent tensor-core CTAs: up to four per SM (4 x 128 of the 512 tensor-memory columns).
uint32_t tc_grid(uint32_t rows) {
  return std::max(1u, std::min(ceil_div(rows, kTcRows), (uint32_t)sm_count() * 4));
}

uint32_t grid_for(uint32_t n, uint32_t block) {
  return std::max(1u, std::min(ceil_div(n, block), (uint32_t)sm_count() * 8));
}

}  // namespace

float lr_inv_log2_leaves(uint32_t numLeaves) { return 1.0f / std::log2((float)std::max(numLeaves, 2u)); }

int lr_scratch_alloc(LrScratch &s, uint32_t numNodes) {
  lr_scratch_free(s);
  const size_t n = std::max(numNodes, 1u), ni = n / 2 + 1;
  cudaError_t e = cudaSuccess;
  e = dev_malloc(&s.ad, 8 * n);
  if (e == cudaSuccess) e = dev_malloc(&s.leafCount, 4 * n);
  if (e == cudaSuccess) e = dev_malloc(&s.sa, 4 * n);
  if (e == cudaSuccess) e = dev_malloc(&s.par, 4 * n);
  if (e == cudaSuccess) e = dev_malloc(&s.acc, 8 * n);
  if (e == cudaSuccess) e = dev_malloc(&s.err, 4);
  if (e == cudaSuccess) e = dev_malloc(&s.hist, 4 * kHistWords);
  if (e == cudaSuccess) e = dev_malloc(&s.pend, 16 * ni);
  if (e == cudaSuccess) e = dev_malloc(&s.x, 2ull * kIn * ni);
  if (e == cudaSuccess) e = dev_malloc(&s.y, 4 * ni);
  if (e == cudaSuccess) e = cudaMemset(s.err, 0, 4);
  if (e != cudaSuccess) {
    set_last_error("lr_scratch_alloc", e);
    lr_scratch_free(s);
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  s.numNodes = (uint32_t)n;
  return BVHGB_OK;
}

void lr_scratch_free(LrScratch &s) {
  cudaFree(s.ad);
  s.ad = nullptr;
  cudaFree(s.leafCount);
  cudaFree(s.sa);
  cudaFree(s.par);
  s.sa = nullptr;
  s.par = nullptr;
  cudaFree(s.acc);
  cudaFree(s.err);
  cudaFree(s.hist);
  cudaFree(s.pend);
  cudaFree(s.x);
  cudaFree(s.y);
  s.leafCount = s.hist = s.err = nullptr;
  s.acc = nullptr;
  s.pend = nullptr;
  s.y = nullptr;
  s.x = nullptr;
  s.numNodes = 0;
}

uint32_t *lr_error_word(LrScratch &s) { return s.err; }

int lr_features(LrScratch &s, const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const uint32_t *inner,
                uint32_t numInner, float invLog2Leaves, cudaStream_t st) {
  if (numNodes > s.numNodes || numInner > s.numNodes / 2 + 1) return BVHGB_TOO_LARGE;
  if (numInner == 0) return BVHGB_OK;
  const uint32_t g = grid_for(numNodes, 256);
  depth_init_kernel<<<g, 256, 0, st>>>(nodes, numNodes, root, s.ad, s.sa, s.par);
  BVHGB_LAUNCH_CHECK("lr depth init");
  const uint32_t gi = grid_for(numInner, 256);
  for (int r = 0; r < kDepthLaunches; ++r) {
    depth_jump_kernel<<<gi, 256, 0, st>>>(inner, numInner, numNodes, root, s.ad);
    BVHGB_LAUNCH_CHECK("lr depth jump");
  }
  BVHGB_CUDA_TRY(cudaMemsetAsync(s.acc, 0, 8ull * numNodes, st));
  leaf_count_kernel<<<g, 256, 0, st>>>(s.par, numNodes, root, s.leafCount, s.acc, lr_error_word(s));
  BVHGB_LAUNCH_CHECK("lr leaf count");
  BVHGB_CUDA_TRY(cudaMemsetAsync(s.hist, 0, 4 * kHistPrefix, st));
  features_raw_kernel<<<gi, 256, 0, st>>>(nodes, inner, numInner, numNodes, root, s.ad, s.leafCount, s.sa, s.par,
                                          invLog2Leaves, s.x, s.pend, s.hist, lr_error_word(s));
  BVHGB_LAUNCH_CHECK("lr features");
  hist_reduce_kernel<<<grid_for(kRankBins, 256), 256, 0, st>>>(s.hist);
  BVHGB_LAUNCH_CHECK("lr rank reduce");
  hist_scan_kernel<<<4, 1024, 0, st>>>(s.hist);
  BVHGB_LAUNCH_CHECK("lr rank scan");
  features_pack_kernel<<<gi, 256, 0, st>>>(s.pend, s.hist, numInner, s.x);
  BVHGB_LAUNCH_CHECK("lr features pack");
  return BVHGB_OK;
}

}  // namespace bvhgb

// ---- MLP object and C ABI -----------------------------------------------------------------------

struct bvhgb_mlp {
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  __nv_bfloat16 *pb = nullptr;
  uint32_t *stepDev = nullptr;
  uint32_t *err = nullptr;  // error bits of the inference kernel (kErrTimeout)
  uint32_t *idx = nullptr;
  uint32_t idxCap = 0, lossCap = 0;
  float *part = nullptr;  // per-tile gradient rows [partCap][kMlpParams]
  uint32_t partCap = 0;
};

struct bvhgb_lr_features_ctx {
  bvhgb::LrScratch s;
};

namespace bvhgb {

int lr_score_keys(const bvhgb_mlp *m, LrScratch &s, const bvhgb_node *nodes, uint32_t root, const uint32_t *inner,
                  uint32_t numInner, uint32_t *keys, uint32_t *vals, cudaStream_t st) {
  if (numInner == 0) return BVHGB_OK;
  mlp_forward_tc_kernel<true><<<tc_grid(numInner), 128, 0, st>>>(m->pb, s.x, numInner, s.y, inner, keys, vals, m->err);
  BVHGB_LAUNCH_CHECK("lr score");
  return BVHGB_OK;
}

namespace {
// The shared-memory opt-in belongs to the context: set once per context (another device, or the
// context after a device reset, sets it again). Thread-safe.
int ensure_train_attr() {
  static std::mutex mu;
  static std::vector<uint64_t> done;
  const uint64_t ctx = context_id();
  std::lock_guard<std::mutex> lock(mu);
  if (ctx != 0 && std::find(done.begin(), done.end(), ctx) != done.end()) return BVHGB_OK;
  BVHGB_CUDA_TRY(cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
  if (ctx != 0) done.push_back(ctx);
  return BVHGB_OK;
}

int ensure_part(bvhgb_mlp *m, uint32_t tiles) {
  if (m->partCap >= tiles && m->part) return BVHGB_OK;
  cudaFree(m->part);
  m->part = nullptr;
  m->partCap = 0;
  BVHGB_CUDA_TRY(dev_malloc(&m->part, 4ull * kMlpParams * std::max(tiles, 1u)));
  m->partCap = std::max(tiles, 1u);
  return BVHGB_OK;
}

int ensure_loss(bvhgb_mlp *m, uint32_t n) {
  if (m->lossCap >= n && m->loss) return BVHGB_OK;
  cudaFree(m->loss);
  m->loss = nullptr;
  m->lossCap = 0;
  BVHGB_CUDA_TRY(dev_malloc(&m->loss, 4ull * std::max(n, 1u)));
  m->lossCap = std::max(n, 1u);
  return BVHGB_OK;
}
}  // namespace
}  // namespace bvhgb

using namespace bvhgb;

extern "C" BVHGB_API int bvhgb_mlp_create(uint64_t seed, bvhgb_mlp **out) {
  if (!out) return BVHGB_INVALID_ARGUMENT;
  *out = nullptr;
  auto *m = new bvhgb_mlp();
  cudaError_t e = dev_malloc(&m->p, 4 * kMlpParams);
  if (e == cudaSuccess) e = dev_malloc(&m->g, 4 * kMlpParams);
  if (e == cudaSuccess) e = dev_malloc(&m->m, 4 * kMlpParams);
  if (e == cudaSuccess) e = dev_malloc(&m->v, 4 * kMlpParams);
  if (e == cudaSuccess) e = dev_malloc(&m->pb, 2 * kMlpParams);
  if (e == cudaSuccess) e = dev_malloc(&m->stepDev, 4);
  if (e == cudaSuccess) e = dev_malloc(&m->err, 4);
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, 4);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_mlp_create", e);
    bvhgb_mlp_destroy(m);
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  std::vector<float> h(kMlpParams, 0.0f);
  uint64_t state = seed;
  auto uni = [&]() {  // SplitMix64 -> uniform in [-1, 1)
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((double)(z >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
  };
  for (int i = 0; i < kH * kIn; ++i) h[oW1 + i] = uni() * std::sqrt(6.0f / kIn);
  for (int i = 0; i < kH * kH; ++i) h[oW2 + i] = uni() * std::sqrt(6.0f / kH);
  for (int i = 0; i < kH; ++i) h[oW3 + i] = uni() * std::sqrt(6.0f / kH) * 0.1f;
  const int st = bvhgb_mlp_set_params(m, h.data());
  if (st) {
    bvhgb_mlp_destroy(m);
    return st;
  }
  *out = m;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_destroy(bvhgb_mlp *m) {
  if (!m) return BVHGB_OK;
  cudaFree(m->p);
  cudaFree(m->g);
  cudaFree(m->part);
  cudaFree(m->m);
  cudaFree(m->v);
  cudaFree(m->loss);
  cudaFree(m->pb);
  cudaFree(m->stepDev);
  cudaFree(m->err);
  cudaFree(m->idx);
  delete m;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_set_params(bvhgb_mlp *m, const float *params) {
  if (!m || !params) return BVHGB_INVALID_ARGUMENT;
  BVHGB_CUDA_TRY(cudaMemcpy(m->p, params, 4 * kMlpParams, cudaMemcpyHostToDevice));
  BVHGB_CUDA_TRY(cudaMemset(m->g, 0, 4 * kMlpParams));
  BVHGB_CUDA_TRY(cudaMemset(m->m, 0, 4 * kMlpParams));
  BVHGB_CUDA_TRY(cudaMemset(m->v, 0, 4 * kMlpParams));
  BVHGB_CUDA_TRY(cudaMemset(m->stepDev, 0, 4));
  to_bf16_kernel<<<ceil_div(kMlpParams, 256), 256>>>(m->p, m->pb, kMlpParams);
  BVHGB_LAUNCH_CHECK("mlp bf16 copy");
  BVHGB_CUDA_TRY(cudaDeviceSynchronize());
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_get_params(const bvhgb_mlp *m, float *params) {
  if (!m || !params) return BVHGB_INVALID_ARGUMENT;
  BVHGB_CUDA_TRY(cudaMemcpy(params, m->p, 4 * kMlpParams, cudaMemcpyDeviceToHost));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_forward(const bvhgb_mlp *m, const uint16_t *x, uint32_t n, float *y,
                                           bvhgb_stream stream) {
  if (!m || (n && (!x || !y))) return BVHGB_INVALID_ARGUMENT;
  if (n == 0) return BVHGB_OK;
  mlp_forward_tc_kernel<false><<<tc_grid(n), 128, 0, as_stream(stream)>>>(m->pb, x, n, y, nullptr, nullptr, nullptr,
                                                                         m->err);
  BVHGB_LAUNCH_CHECK("mlp forward");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_gradient(bvhgb_mlp *m, const uint16_t *x, const float *t, uint32_t n,
                                            float *gradHost, float *lossHost, bvhgb_stream stream) {
  if (!m || !x || !t || n == 0) return BVHGB_INVALID_ARGUMENT;
  const uint32_t tiles = ceil_div(n, kTile);
  int st = ensure_train_attr();
  if (!st) st = ensure_loss(m, 1);
  if (!st) st = ensure_part(m, tiles);
  if (st) return st;
  cudaStream_t s = as_stream(stream);
  BVHGB_CUDA_TRY(cudaMemsetAsync(m->loss, 0, 4, s));
  mlp_train_kernel<<<tiles, kTile, kTrainSmem, s>>>(m->pb, x, t, nullptr, n, (float)n, m->part, m->loss, nullptr, 0, 1);
  BVHGB_LAUNCH_CHECK("mlp gradient");
  grad_reduce_kernel<<<ceil_div((uint32_t)kMlpParams, 256u), 256, 0, s>>>(m->part, tiles, m->g);
  BVHGB_LAUNCH_CHECK("mlp gradient reduce");
  if (gradHost) BVHGB_CUDA_TRY(cudaMemcpyAsync(gradHost, m->g, 4 * kMlpParams, cudaMemcpyDeviceToHost, s));
  if (lossHost) BVHGB_CUDA_TRY(cudaMemcpyAsync(lossHost, m->loss, 4, cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaMemsetAsync(m->g, 0, 4 * kMlpParams, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_train(bvhgb_mlp *m, const uint16_t *x, const float *t, uint32_t numSamples,
                                         uint32_t batch, uint32_t steps, float lr, float weightDecay, uint64_t seed,
                                         float *lossHistory, bvhgb_stream stream) {
  if (!m || !x || !t || numSamples == 0 || batch == 0) return BVHGB_INVALID_ARGUMENT;
  if (steps == 0) return BVHGB_OK;
  const uint32_t tiles = ceil_div(batch, kTile);
  int st = ensure_train_attr();
  if (!st) st = ensure_loss(m, steps);
  if (!st) st = ensure_part(m, tiles);
  if (st) return st;
  cudaStream_t s = as_stream(stream);
  if (m->idxCap < batch) {
    cudaFree(m->idx);
    m->idx = nullptr;
    m->idxCap = 0;
    BVHGB_CUDA_TRY(dev_malloc(&m->idx, 4ull * batch));
    m->idxCap = batch;
  }
  uint32_t step0 = 0;
  BVHGB_CUDA_TRY(cudaMemcpyAsync(&step0, m->stepDev, 4, cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  BVHGB_CUDA_TRY(cudaMemsetAsync(m->loss, 0, 4ull * steps, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  // Capture one step (batch rows, forward + backward, AdamW) and replay it; the kernels read the
  // step number from device memory so every replay is the next step.
  cudaStream_t cap = nullptr;
  BVHGB_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    batch_index_kernel<<<ceil_div(batch, 256), 256, 0, cap>>>(m->idx, batch, numSamples, seed, m->stepDev);
    mlp_train_kernel<<<tiles, kTile, kTrainSmem, cap>>>(m->pb, x, t, m->idx, batch, (float)batch, m->part, m->loss,
                                                         m->stepDev, step0, steps);
    grad_reduce_kernel<<<ceil_div((uint32_t)kMlpParams, 256u), 256, 0, cap>>>(m->part, tiles, m->g);
    adamw_kernel<<<1, 1024, 0, cap>>>(m->p, m->pb, m->g, m->m, m->v, m->stepDev, lr, weightDecay);
    e = cudaStreamEndCapture(cap, &graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cap);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_mlp_train capture", e);
    if (exec) cudaGraphExecDestroy(exec);
    return BVHGB_CUDA_ERROR;
  }
  for (uint32_t k = 0; k < steps && e == cudaSuccess; ++k) e = cudaGraphLaunch(exec, s);
  count_launch(4u * steps);  // (the capture itself recorded none: its launches are not counted)
  if (e == cudaSuccess && lossHistory) e = cudaMemcpyAsync(lossHistory, m->loss, 4ull * steps, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaGraphExecDestroy(exec);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_mlp_train", e);
    return BVHGB_CUDA_ERROR;
  }
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lr_features_create(uint32_t maxNodes, bvhgb_lr_features_ctx **out) {
  if (!out || maxNodes == 0) return BVHGB_INVALID_ARGUMENT;
  *out = nullptr;
  auto *c = new bvhgb_lr_features_ctx();
  const int st = lr_scratch_alloc(c->s, maxNodes);
  if (st) {
    delete c;
    return st;
  }
  *out = c;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lr_features_destroy(bvhgb_lr_features_ctx *ctx) {
  if (!ctx) return BVHGB_OK;
  lr_scratch_free(ctx->s);
  delete ctx;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lr_features(bvhgb_lr_features_ctx *ctx, const bvhgb_node *nodes, uint32_t numNodes,
                                           uint32_t root, const uint32_t *inner, uint32_t numInner, uint32_t numLeaves,
                                           uint16_t *x, bvhgb_stream stream) {
  if (!ctx || !nodes || !inner || !x || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  cudaStream_t s = as_stream(stream);
  const int st = lr_features(ctx->s, nodes, numNodes, root, inner, numInner, lr_inv_log2_leaves(numLeaves), s);
  if (st) return st;
  if (numInner) BVHGB_CUDA_TRY(cudaMemcpyAsync(x, ctx->s.x, 2ull * kIn * numInner, cudaMemcpyDeviceToDevice, s));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_mlp_read_errors(bvhgb_mlp *m, uint32_t *flags, int reset) {
  if (!m || !flags) return BVHGB_INVALID_ARGUMENT;
  BVHGB_CUDA_TRY(cudaMemcpy(flags, m->err, 4, cudaMemcpyDeviceToHost));
  if (reset) BVHGB_CUDA_TRY(cudaMemset(m->err, 0, 4));
  return BVHGB_OK;
}
