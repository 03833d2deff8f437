// LBVH build: scene box, Morton codes, onesweep sort, and a fused bottom-up topology + refit.
//
// Reference: lib/builder/LBVH_CUDA.cu. Kernel plan (HBM-bound, no tensor cores):
//   lbvh_bounds  : per-triangle box (+-FLT_EPSILON) reduced into the scene box, whose initial value
//                  is the origin box (LBVH_CUDA.cu:60-119). Reads faces + vertices once.
//   lbvh_morton  : re-reads the triangle, centroid -> 30- or 63-bit Morton key + index
//                  (LBVH_CUDA.cu:132-183); also resets the build's exchange slots and, when the
//                  workspace has them, writes each triangle's box as a 32-byte record in face order
//                  (the build then gathers one sector per leaf instead of a face and three vertices).
//   sort         : sort.cu (replaces cub::DeviceRadixSort, LBVH_CUDA.cu:185-193).
//   lbvh_build   : one thread per sorted leaf writes the leaf and climbs (Apetrei 2014 style): at each
//                  step it picks the parent from the two neighbouring key deltas, meets its sibling
//                  at the split, and the second thread to arrive merges the boxes and writes the
//                  parent with the Karras node index the reference assigns (kGenLeafNodes +
//                  kBuildTree + kFixAABBTree, LBVH_CUDA.cu:273-374), meeting its sibling through one
//                  acq_rel exchange on the split's slot.
#include <cstring>

#include "common.cuh"
#include "lbvh_device.cuh"
#include "sort.cuh"

struct bvhgb_lbvh_workspace {
  uint32_t maxFaces = 0;
  bvhgb_lbvh_config cfg{};
  uint32_t keyBytes = 4;
  uint32_t *scene = nullptr;  // 6 order-mapped floats + error word
  void *keys = nullptr;
  void *keysSorted = nullptr;
  uint32_t *vals = nullptr;
  uint32_t *valsSorted = nullptr;
  uint32_t *slots = nullptr;
  float4 *triBoxes = nullptr;  // 2 x float4 per face (mn.xyz mx.x | mx.yz 0 0); null: gather the triangle
  bool slotsArmed = false;  // slots hold kNone (set by the Morton kernel)
  void *sortTemp = nullptr;
  size_t sortTempBytes = 0;
};

namespace bvhgb {
namespace {

constexpr int kBoundsThreads = 256;
constexpr int kMortonThreads = 256;
constexpr int kBuildThreads = 128;

__global__ void lbvh_init_kernel(uint32_t *scene) {
  if (threadIdx.x < 6) scene[threadIdx.x] = f2ord(0.0f);  // origin box [(0,0,0),(0,0,0)]
  if (threadIdx.x == 6) scene[6] = 0;                     // error word
}

__global__ void __launch_bounds__(kBoundsThreads) lbvh_bounds_kernel(const float *__restrict__ vert,
                                                                     const uint32_t *__restrict__ faces, uint32_t n,
                                                                     uint32_t *scene) {
  // Starting the local box at the origin is the same as merging the reduction's initial value.
  float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f};
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    Box b;
    tri_box(vert, faces, (uint32_t)i, b, nullptr);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      mn[k] = fminf(mn[k], b.mn[k]);
      mx[k] = fmaxf(mx[k], b.mx[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
    }
  }
  __shared__ float red[kBoundsThreads / 32][6];
  const uint32_t warp = threadIdx.x >> 5;
  if (lane_id() == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) { red[warp][k] = mn[k]; red[warp][3 + k] = mx[k]; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    float v = red[0][threadIdx.x];
    for (int w = 1; w < kBoundsThreads / 32; ++w)
      v = threadIdx.x < 3 ? fminf(v, red[w][threadIdx.x]) : fmaxf(v, red[w][threadIdx.x]);
    if (threadIdx.x < 3) atomicMin(&scene[threadIdx.x], f2ord(v));
    else atomicMax(&scene[threadIdx.x], f2ord(v));
  }
}

template <int BITS>
__global__ void __launch_bounds__(kMortonThreads) lbvh_morton_kernel(const float *__restrict__ vert,
                                                                     const uint32_t *__restrict__ faces, uint32_t n,
                                                                     const uint32_t *__restrict__ scene, void *keysOut,
                                                                     uint32_t *__restrict__ vals,
                                                                     uint32_t *__restrict__ slots,
                                                                     float4 *__restrict__ boxes) {
  float off[3], sc[3];
  morton_params(scene, off, sc);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    Box b;
    float c[3];
    tri_box(vert, faces, (uint32_t)i, b, c);
    if (BITS == 30) static_cast<uint32_t *>(keysOut)[i] = (uint32_t)morton_key<30>(c, off, sc);
    else static_cast<uint64_t *>(keysOut)[i] = morton_key<63>(c, off, sc);
    vals[i] = (uint32_t)i;
    if (i + 1 < n) slots[i] = kNone;
    if (boxes) {
      boxes[2 * i] = make_float4(b.mn[0], b.mn[1], b.mn[2], b.mx[0]);
      boxes[2 * i + 1] = make_float4(b.mx[1], b.mx[2], 0.0f, 0.0f);
    }
  }
}

template <int MODE, typename K>
__global__ void __launch_bounds__(kBuildThreads) lbvh_build_kernel(const float *__restrict__ vert,
                                                                   const uint32_t *__restrict__ faces,
                                                                   const K *__restrict__ keys,
                                                                   const uint32_t *__restrict__ idx, uint32_t n,
                                                                   const float4 *__restrict__ boxes,
                                                                   bvhgb_node *nodes, uint32_t *slots,
                                                                   uint32_t *err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t face = __ldg(idx + i);
  Box box;
  if (boxes) {
    const float4 a = __ldg(boxes + 2 * (size_t)face), c = __ldg(boxes + 2 * (size_t)face + 1);
    box.mn[0] = a.x; box.mn[1] = a.y; box.mn[2] = a.z;
    box.mx[0] = a.w; box.mx[1] = c.x; box.mx[2] = c.y;
  } else {
    tri_box(vert, faces, face, box, nullptr);
  }
  lbvh_climb<MODE, K>(i, n, keys, face, box, nodes, slots, err);
}

template <int MODE>
int launch_build(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces, uint32_t n,
                 bvhgb_node *nodes, cudaStream_t s) {
  // The exchange slots are re-armed by the Morton kernel; a second build from the same sorted keys
  // re-arms them here.
  if (!ws->slotsArmed) BVHGB_CUDA_TRY(cudaMemsetAsync(ws->slots, 0xFF, 4ull * n, s));
  ws->slotsArmed = false;
  dim3 grid(ceil_div(n, kBuildThreads));
  if (ws->keyBytes == 4)
    lbvh_build_kernel<MODE, uint32_t><<<grid, kBuildThreads, 0, s>>>(
        vert, faces, static_cast<const uint32_t *>(ws->keysSorted), ws->valsSorted, n, ws->triBoxes, nodes, ws->slots,
        ws->scene + 6);
  else
    lbvh_build_kernel<MODE, uint64_t><<<grid, kBuildThreads, 0, s>>>(
        vert, faces, static_cast<const uint64_t *>(ws->keysSorted), ws->valsSorted, n, ws->triBoxes, nodes, ws->slots,
        ws->scene + 6);
  BVHGB_LAUNCH_CHECK("lbvh build");
  return BVHGB_OK;
}

int check_ws(const bvhgb_lbvh_workspace *ws, uint32_t n) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  if (n > ws->maxFaces) return BVHGB_TOO_LARGE;
  return BVHGB_OK;
}

}  // namespace
}  // namespace bvhgb

using namespace bvhgb;

extern "C" BVHGB_API int bvhgb_lbvh_create(uint32_t maxFaces, const bvhgb_lbvh_config *cfg, bvhgb_lbvh_workspace **out) {
  if (!out) return BVHGB_INVALID_ARGUMENT;
  *out = nullptr;
  bvhgb_lbvh_config c = cfg ? *cfg : bvhgb_lbvh_config{30u, BVHGB_TOPO_REFCOMPAT};
  if ((c.mortonBits != 30 && c.mortonBits != 63) || c.topology > BVHGB_TOPO_KARRAS) return BVHGB_INVALID_ARGUMENT;
  if (maxFaces >= (1u << 30)) return BVHGB_TOO_LARGE;
  int pst = sort_prepare();
  if (pst) return pst;
  auto *ws = new bvhgb_lbvh_workspace();
  ws->maxFaces = maxFaces;
  ws->cfg = c;
  ws->keyBytes = c.mortonBits == 30 ? 4u : 8u;
  const size_t m = maxFaces ? maxFaces : 1;
  ws->sortTempBytes = sort_temp_bytes(maxFaces, ws->keyBytes, 0, c.mortonBits);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = dev_malloc(&ws->scene, 256);
  if (e == cudaSuccess) e = dev_malloc(&ws->keys, ws->keyBytes * m);
  if (e == cudaSuccess) e = dev_malloc(&ws->keysSorted, ws->keyBytes * m);
  if (e == cudaSuccess) e = dev_malloc(&ws->vals, 4 * m);
  if (e == cudaSuccess) e = dev_malloc(&ws->valsSorted, 4 * m);
  if (e == cudaSuccess) e = dev_malloc(&ws->slots, 4 * m);
  if (e == cudaSuccess) e = dev_malloc(&ws->triBoxes, 32 * m);
  if (e == cudaSuccess) e = dev_malloc(&ws->sortTemp, ws->sortTempBytes ? ws->sortTempBytes : 256);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_lbvh_create", e);
    bvhgb_lbvh_destroy(ws);
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  *out = ws;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_destroy(bvhgb_lbvh_workspace *ws) {
  if (!ws) return BVHGB_OK;
  cudaFree(ws->scene);
  cudaFree(ws->keys);
  cudaFree(ws->keysSorted);
  cudaFree(ws->vals);
  cudaFree(ws->valsSorted);
  cudaFree(ws->slots);
  cudaFree(ws->triBoxes);
  cudaFree(ws->sortTemp);
  delete ws;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_init_tri_data(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                                  uint32_t n, bvhgb_stream stream) {
  int st = check_ws(ws, n);
  if (st) return st;
  cudaStream_t s = as_stream(stream);
  lbvh_init_kernel<<<1, 32, 0, s>>>(ws->scene);
  BVHGB_LAUNCH_CHECK("lbvh init");
  if (n == 0) return BVHGB_OK;
  if (!vert || !faces) return BVHGB_INVALID_ARGUMENT;
  uint32_t grid = min(ceil_div(n, kBoundsThreads * 4), (uint32_t)sm_count() * 8);
  lbvh_bounds_kernel<<<grid, kBoundsThreads, 0, s>>>(vert, faces, n, ws->scene);
  BVHGB_LAUNCH_CHECK("lbvh bounds");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_calc_morton(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                                uint32_t n, bvhgb_stream stream) {
  int st = check_ws(ws, n);
  if (st) return st;
  if (n == 0) return BVHGB_OK;
  if (!vert || !faces) return BVHGB_INVALID_ARGUMENT;
  cudaStream_t s = as_stream(stream);
  uint32_t grid = ceil_div(n, kMortonThreads * 2);
  if (ws->cfg.mortonBits == 30)
    lbvh_morton_kernel<30><<<grid, kMortonThreads, 0, s>>>(vert, faces, n, ws->scene, ws->keys, ws->vals, ws->slots,
                                                           ws->triBoxes);
  else
    lbvh_morton_kernel<63><<<grid, kMortonThreads, 0, s>>>(vert, faces, n, ws->scene, ws->keys, ws->vals, ws->slots,
                                                           ws->triBoxes);
  BVHGB_LAUNCH_CHECK("lbvh morton");
  ws->slotsArmed = true;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_sort(bvhgb_lbvh_workspace *ws, uint32_t n, bvhgb_stream stream) {
  int st = check_ws(ws, n);
  if (st) return st;
  return sort_pairs(ws->sortTemp, ws->keys, ws->keysSorted, ws->vals, ws->valsSorted, n, ws->keyBytes, 0,
                    ws->cfg.mortonBits, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_lbvh_build_tree(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                               uint32_t n, bvhgb_node *nodes, bvhgb_stream stream) {
  int st = check_ws(ws, n);
  if (st) return st;
  if (n == 0) return BVHGB_OK;
  if (!vert || !faces || !nodes) return BVHGB_INVALID_ARGUMENT;
  if (ws->cfg.topology == BVHGB_TOPO_REFCOMPAT)
    return launch_build<BVHGB_TOPO_REFCOMPAT>(ws, vert, faces, n, nodes, as_stream(stream));
  return launch_build<BVHGB_TOPO_KARRAS>(ws, vert, faces, n, nodes, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_lbvh_build(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                          uint32_t n, bvhgb_node *nodes, bvhgb_stream stream) {
  int st = check_ws(ws, n);
  if (st) return st;
  if (n == 0) return BVHGB_OK;
  if (!vert || !faces || !nodes) return BVHGB_INVALID_ARGUMENT;
  if ((st = bvhgb_lbvh_init_tri_data(ws, vert, faces, n, stream))) return st;
  if ((st = bvhgb_lbvh_calc_morton(ws, vert, faces, n, stream))) return st;
  if ((st = bvhgb_lbvh_sort(ws, n, stream))) return st;
  return bvhgb_lbvh_build_tree(ws, vert, faces, n, nodes, stream);
}

extern "C" BVHGB_API int bvhgb_lbvh_read_scene_box(bvhgb_lbvh_workspace *ws, bvhgb_aabb *scene, bvhgb_stream stream) {
  if (!ws || !scene) return BVHGB_INVALID_ARGUMENT;
  uint32_t h[6];
  cudaStream_t s = as_stream(stream);
  BVHGB_CUDA_TRY(cudaMemcpyAsync(h, ws->scene, sizeof(h), cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  float f[6];
  for (int k = 0; k < 6; ++k) {
    uint32_t u = h[k];
    uint32_t bits = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    std::memcpy(&f[k], &bits, 4);
  }
  scene->minMax[0] = {f[0], f[1], f[2]};
  scene->minMax[1] = {f[3], f[4], f[5]};
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_set_scene_box(bvhgb_lbvh_workspace *ws, const bvhgb_aabb *scene,
                                                  bvhgb_stream stream) {
  if (!ws || !scene) return BVHGB_INVALID_ARGUMENT;
  // The order-preserving integer image of each float, as the bounds kernel's atomics keep it.
  const float f[6] = {scene->minMax[0].x, scene->minMax[0].y, scene->minMax[0].z,
                      scene->minMax[1].x, scene->minMax[1].y, scene->minMax[1].z};
  uint32_t h[6];
  for (int k = 0; k < 6; ++k) {
    uint32_t u;
    std::memcpy(&u, &f[k], 4);
    h[k] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  }
  cudaStream_t s = as_stream(stream);
  BVHGB_CUDA_TRY(cudaMemcpyAsync(ws->scene, h, sizeof(h), cudaMemcpyHostToDevice, s));
  // The copy reads pageable host memory, so it is staged before the call returns.
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_read_keys(bvhgb_lbvh_workspace *ws, int sorted, void *keys_host, uint32_t *idx_host,
                                              uint32_t n, bvhgb_stream stream) {
  int st = check_ws(ws, n);
  if (st) return st;
  cudaStream_t s = as_stream(stream);
  if (keys_host)
    BVHGB_CUDA_TRY(cudaMemcpyAsync(keys_host, sorted ? ws->keysSorted : ws->keys, (size_t)ws->keyBytes * n,
                                   cudaMemcpyDeviceToHost, s));
  if (idx_host)
    BVHGB_CUDA_TRY(cudaMemcpyAsync(idx_host, sorted ? ws->valsSorted : ws->vals, 4ull * n, cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_lbvh_read_errors(bvhgb_lbvh_workspace *ws, uint32_t *flags, bvhgb_stream stream) {
  if (!ws || !flags) return BVHGB_INVALID_ARGUMENT;
  uint32_t a = 0, b = 0;
  cudaStream_t s = as_stream(stream);
  BVHGB_CUDA_TRY(cudaMemcpyAsync(&a, ws->scene + 6, 4, cudaMemcpyDeviceToHost, s));
  const uint32_t *se = sort_error_word(ws->sortTemp, ws->maxFaces, ws->keyBytes, 0, ws->cfg.mortonBits);
  BVHGB_CUDA_TRY(cudaMemcpyAsync(&b, se, 4, cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  *flags = a | b;
  return BVHGB_OK;
}

// ---- allocation-free build -------------------------------------------------------------------
//
// Some callers cannot allocate device memory while they build: a per-frame rebuild inside a render
// or simulation loop (cudaMalloc synchronises the whole device and stalls the frame), host
// applications whose device memory is owned by their own pool and that forbid driver allocations,
// and code that must not fail for lack of memory once started. For them the build below takes its
// working memory from one array in this file, sized for BVHGB_STATIC_MAX_FACES triangles and
// reserved on every GPU that loads the library until the process exits.
#include <mutex>
#include <vector>

namespace bvhgb {
namespace {

constexpr size_t kStaticScratchBytes = 12ull << 20;  // covers keys, values, slots and sort scratch
__device__ __align__(256) unsigned char g_lbvh_static_scratch[kStaticScratchBytes];

struct StaticBase {
  uint64_t context;  // context_id() of the context the address belongs to
  unsigned char *base;
};
std::mutex g_static_mutex;
std::vector<StaticBase> g_static_base;

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of the array in the current context, looked up once per context: every device
// has its own copy, and a device reset (cudaDeviceReset, bvhgb_reset_device) makes a new context
// whose copy may sit elsewhere, so an address is never reused across contexts.
int static_scratch(unsigned char **out) {
  const uint64_t ctx = context_id();
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (ctx != 0) {
    for (const StaticBase &b : g_static_base)
      if (b.context == ctx) {
        *out = b.base;
        return BVHGB_OK;
      }
  }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_lbvh_static_scratch);
  if (e != cudaSuccess) {
    set_last_error("cudaGetSymbolAddress(g_lbvh_static_scratch)", e);
    return BVHGB_CUDA_ERROR;
  }
  if (ctx != 0) g_static_base.push_back({ctx, static_cast<unsigned char *>(p)});
  *out = static_cast<unsigned char *>(p);
  return BVHGB_OK;
}

// The working memory of one build carved out of the array for the largest size: the same layout
// for a build and for the read-back of its error bits.
int static_workspace(const bvhgb_lbvh_config &c, bvhgb_lbvh_workspace &ws) {
  unsigned char *base = nullptr;
  int st = static_scratch(&base);
  if (st) return st;
  ws.maxFaces = BVHGB_STATIC_MAX_FACES;
  ws.cfg = c;
  ws.keyBytes = c.mortonBits == 30 ? 4u : 8u;
  const size_t m = BVHGB_STATIC_MAX_FACES;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *p = base + off;
    off += round256(bytes);
    return p;
  };
  ws.scene = reinterpret_cast<uint32_t *>(take(256));
  ws.keys = take(ws.keyBytes * m);
  ws.keysSorted = take(ws.keyBytes * m);
  ws.vals = reinterpret_cast<uint32_t *>(take(4 * m));
  ws.valsSorted = reinterpret_cast<uint32_t *>(take(4 * m));
  ws.slots = reinterpret_cast<uint32_t *>(take(4 * m));
  ws.sortTempBytes = sort_temp_bytes(BVHGB_STATIC_MAX_FACES, ws.keyBytes, 0, c.mortonBits);
  ws.sortTemp = take(ws.sortTempBytes);
  if (off > kStaticScratchBytes) return BVHGB_GENERIC_ERROR;  // the array is sized for the worst case
  return BVHGB_OK;
}

bool static_cfg_valid(const bvhgb_lbvh_config &c) {
  return (c.mortonBits == 30 || c.mortonBits == 63) && c.topology <= BVHGB_TOPO_KARRAS;
}

}  // namespace
}  // namespace bvhgb

extern "C" BVHGB_API int bvhgb_lbvh_build_static(const float *vert, const uint32_t *faces, uint32_t numFaces,
                                                 const bvhgb_lbvh_config *cfg, bvhgb_node *nodes,
                                                 bvhgb_stream stream) {
  const bvhgb_lbvh_config c = cfg ? *cfg : bvhgb_lbvh_config{30u, BVHGB_TOPO_REFCOMPAT};
  if (!static_cfg_valid(c)) return BVHGB_INVALID_ARGUMENT;
  if (numFaces > BVHGB_STATIC_MAX_FACES) return BVHGB_TOO_LARGE;
  if (numFaces == 0) return BVHGB_OK;
  if (!vert || !faces || !nodes) return BVHGB_INVALID_ARGUMENT;
  bvhgb_lbvh_workspace ws;
  int st = static_workspace(c, ws);
  if (st) return st;
  st = sort_prepare();  // a function attribute, not an allocation
  if (st) return st;
  // The same phases as bvhgb_lbvh_build; every scratch word that must start at a known value is
  // written by the phase that uses it (scene box init kernel, which also clears the build's error
  // word; slot reset in the Morton kernel; the sort's memset of its counters and error word), so
  // the previous call's contents do not matter.
  if ((st = bvhgb_lbvh_init_tri_data(&ws, vert, faces, numFaces, stream))) return st;
  if ((st = bvhgb_lbvh_calc_morton(&ws, vert, faces, numFaces, stream))) return st;
  if ((st = bvhgb_lbvh_sort(&ws, numFaces, stream))) return st;
  return bvhgb_lbvh_build_tree(&ws, vert, faces, numFaces, nodes, stream);
}

extern "C" BVHGB_API int bvhgb_lbvh_static_read_errors(const bvhgb_lbvh_config *cfg, uint32_t *flags,
                                                       bvhgb_stream stream) {
  const bvhgb_lbvh_config c = cfg ? *cfg : bvhgb_lbvh_config{30u, BVHGB_TOPO_REFCOMPAT};
  if (!flags || !static_cfg_valid(c)) return BVHGB_INVALID_ARGUMENT;
  bvhgb_lbvh_workspace ws;
  int st = static_workspace(c, ws);
  if (st) return st;
  return bvhgb_lbvh_read_errors(&ws, flags, stream);
}

