// Batched multi-mesh pipeline: many independent meshes of uneven size built, optimised and traced
// together, one launch per phase for the whole batch, the whole pipeline captured as one CUDA graph.
// The reference runs one mesh per command (LBVH.cpp, Bittner13GPU.cpp, CUDATracer.cpp); each mesh's
// result here is byte-identical to that single-mesh pipeline on the same mesh:
//   - bounds : per-mesh scene boxes (atomic min/max of the order-mapped floats, origin box start);
//   - Morton : key = mesh << 30 | 30-bit Morton code, so one stable sort of the whole batch is the
//              per-mesh sort by (code, face) (the mesh id only separates the segments);
//   - build  : the single-mesh leaf climb on each sorted segment (node arrays at per-mesh offsets,
//              leaves store the face index within their mesh);
//   - Bittner13 : per iteration, one sort of (mesh << 32 | ~order(inefficiency)) gives every mesh's
//              selection; chunk c of every mesh runs in the same four launches (meshes share nothing,
//              so this equals running each mesh's chunks one after another);
//   - trace  : random rays per mesh (origins uniform in the mesh box grown 1.5x about its centre,
//              directions uniform on the sphere), closest hit in that mesh's tree.
// Mesh-level indices are found by binary search over the offset arrays held in shared memory.
#include <algorithm>
#include <cmath>
#include <vector>

#include "bn13_device.cuh"
#include "common.cuh"
#include "lbvh_device.cuh"
#include "sort.cuh"
#include "tracer_device.cuh"

struct bvhgb_batch_workspace {
  bvhgb_batch_config cfg{};
  uint32_t numMeshes = 0, meshBits = 1, totalFaces = 0, totalNodes = 0, totalInner = 0, items = 0;
  std::vector<uint32_t> hFaceOff, hNodeOff, hInnerOff, hChunk, hItemOff;
  uint32_t *faceOff = nullptr, *nodeOff = nullptr, *innerOff = nullptr, *chunk = nullptr, *itemOff = nullptr;
  uint32_t *itemMesh = nullptr;
  uint32_t *scene = nullptr;  // 6 order-mapped floats per mesh
  uint32_t *err = nullptr;
  uint64_t *keys = nullptr, *keysSorted = nullptr;
  uint32_t *vals = nullptr, *valsSorted = nullptr, *slots = nullptr;
  float4 *triBoxes = nullptr;
  void *sortTemp = nullptr;
  // optimizer
  uint32_t *todo = nullptr, *valid = nullptr, *toFix = nullptr, *owner = nullptr, *counter = nullptr;
  unsigned long long *mail = nullptr;  // refit mail slots, three words per node, empty between launches
  bvhgb::PatchOut *patches = nullptr;
  unsigned long long *stats = nullptr;
  // captured whole pipeline
  cudaGraphExec_t graph = nullptr;
  const void *gVert = nullptr, *gFaces = nullptr, *gNodes = nullptr, *gHits = nullptr;
  uint32_t gIterations = 0, gRays = 0;
  uint64_t gSeed = 0, graphKernels = 0;
};

namespace bvhgb {
namespace {

constexpr uint32_t kMaxMeshes = 4096;
constexpr int kBatchThreads = 256;

// Largest m with off[m] <= x over the numMeshes + 1 offsets (off[0] = 0); x < off[numMeshes].
__device__ __forceinline__ uint32_t segment_of(const uint32_t *off, uint32_t numMeshes, uint32_t x) {
  uint32_t lo = 0, hi = numMeshes;  // invariant: off[lo] <= x < off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Copies numMeshes + 1 offsets into shared memory (the block's threads together).
__device__ __forceinline__ void stage_offsets(uint32_t *sh, const uint32_t *off, uint32_t numMeshes) {
  for (uint32_t k = threadIdx.x; k <= numMeshes; k += blockDim.x) sh[k] = off[k];
  __syncthreads();
}

__global__ void batch_init_kernel(uint32_t *scene, uint32_t numMeshes, uint32_t *err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 6 * numMeshes) scene[i] = f2ord(0.0f);  // origin box [(0,0,0),(0,0,0)] per mesh
  if (i == 0) *err = 0;
}

__global__ void __launch_bounds__(kBatchThreads) batch_bounds_kernel(const float *__restrict__ vert,
                                                                     const uint32_t *__restrict__ faces,
                                                                     const uint32_t *__restrict__ faceOff,
                                                                     uint32_t numMeshes, uint32_t totalFaces,
                                                                     uint32_t *scene) {
  extern __shared__ uint32_t shOff[];
  stage_offsets(shOff, faceOff, numMeshes);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  // every lane of a warp runs the same number of iterations (the loop bound is rounded up)
  const uint32_t rounds = (totalFaces + stride - 1) / stride;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t g = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = g < totalFaces;
    const uint32_t m = live ? segment_of(shOff, numMeshes, g) : 0xFFFFFFFFu;
    float v[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // the origin box merges as the identity here
    if (live) {
      Box b;
      tri_box(vert, faces, g, b, nullptr);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        v[k] = fminf(0.0f, b.mn[k]);
        v[3 + k] = fmaxf(0.0f, b.mx[k]);
      }
    }
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, m);
    if (peers == 0xFFFFFFFFu) {  // the whole warp is in one mesh: reduce, one lane updates
#pragma unroll
      for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          v[k] = fminf(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
          v[3 + k] = fmaxf(v[3 + k], __shfl_xor_sync(0xFFFFFFFFu, v[3 + k], o));
        }
      }
      if (lane == 0 && live) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          atomicMin(&scene[6 * m + k], f2ord(v[k]));
          atomicMax(&scene[6 * m + 3 + k], f2ord(v[3 + k]));
        }
      }
    } else if (live) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        atomicMin(&scene[6 * m + k], f2ord(v[k]));
        atomicMax(&scene[6 * m + 3 + k], f2ord(v[3 + k]));
      }
    }
  }
}

__global__ void __launch_bounds__(kBatchThreads) batch_morton_kernel(const float *__restrict__ vert,
                                                                     const uint32_t *__restrict__ faces,
                                                                     const uint32_t *__restrict__ faceOff,
                                                                     uint32_t numMeshes, uint32_t totalFaces,
                                                                     const uint32_t *__restrict__ scene,
                                                                     uint64_t *__restrict__ keys,
                                                                     uint32_t *__restrict__ vals,
                                                                     uint32_t *__restrict__ slots,
                                                                     float4 *__restrict__ boxes) {
  extern __shared__ uint32_t shOff[];
  stage_offsets(shOff, faceOff, numMeshes);
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < totalFaces; g += gridDim.x * blockDim.x) {
    const uint32_t m = segment_of(shOff, numMeshes, g);
    float off[3], sc[3];
    morton_params(scene + 6 * m, off, sc);
    Box b;
    float c[3];
    tri_box(vert, faces, g, b, c);
    keys[g] = ((uint64_t)m << 30) | morton_key<30>(c, off, sc);
    vals[g] = g;
    slots[g] = kNone;
    boxes[2 * (size_t)g] = make_float4(b.mn[0], b.mn[1], b.mn[2], b.mx[0]);
    boxes[2 * (size_t)g + 1] = make_float4(b.mx[1], b.mx[2], 0.0f, 0.0f);
  }
}

template <int MODE>
__global__ void __launch_bounds__(128) batch_build_kernel(const uint64_t *__restrict__ keys,
                                                          const uint32_t *__restrict__ idx,
                                                          const float4 *__restrict__ boxes,
                                                          const uint32_t *__restrict__ faceOff,
                                                          const uint32_t *__restrict__ nodeOff, uint32_t numMeshes,
                                                          uint32_t totalFaces, bvhgb_node *nodes, uint32_t *slots,
                                                          uint32_t *err) {
  extern __shared__ uint32_t shOff[];
  stage_offsets(shOff, faceOff, numMeshes);
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= totalFaces) return;
  const uint32_t m = segment_of(shOff, numMeshes, g);
  const uint32_t base = shOff[m], n = shOff[m + 1] - base, i = g - base;
  const uint32_t face = __ldg(idx + g);
  if (face < base || face - base >= n) {  // a sorted face outside its mesh: keys were corrupted
    atomicOr(err, kErrBadIndex);
    return;
  }
  const float4 a = __ldg(boxes + 2 * (size_t)face), c = __ldg(boxes + 2 * (size_t)face + 1);
  Box box;
  box.mn[0] = a.x; box.mn[1] = a.y; box.mn[2] = a.z;
  box.mx[0] = a.w; box.mx[1] = c.x; box.mx[2] = c.y;
  lbvh_climb<MODE, uint64_t>(i, n, keys + base, face - base, box, nodes + __ldg(nodeOff + m), slots + base, err);
}

// Selection keys of every mesh's inner nodes: mesh << 32 | ~order(inefficiency); values = local ids.
__global__ void __launch_bounds__(kBatchThreads) batch_cost_kernel(const bvhgb_node *__restrict__ nodes,
                                                                   const uint32_t *__restrict__ innerOff,
                                                                   const uint32_t *__restrict__ nodeOff,
                                                                   uint32_t numMeshes, uint32_t totalInner,
                                                                   uint64_t *__restrict__ keys,
                                                                   uint32_t *__restrict__ vals) {
  extern __shared__ uint32_t shOff[];
  stage_offsets(shOff, innerOff, numMeshes);
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < totalInner; q += gridDim.x * blockDim.x) {
    const uint32_t m = segment_of(shOff, numMeshes, q);
    const uint32_t x = q - shOff[m];  // LBVH inner nodes are [0, N - 1) and stay inner
    keys[q] = ((uint64_t)m << 32) | ~f2ord(inefficiency(nodes + __ldg(nodeOff + m), x));
    vals[q] = x;
  }
}

struct MeshItem {
  uint32_t m, k;  // mesh, rank of the item within the mesh's chunk
};
__device__ __forceinline__ MeshItem item_of(const uint32_t *__restrict__ itemMesh, const uint32_t *__restrict__ itemOff,
                                            uint32_t q) {
  const uint32_t m = __ldg(itemMesh + q);
  return {m, q - __ldg(itemOff + m)};
}

__global__ void __launch_bounds__(kWarpItemsPerBlock * 32, 5) batch_patch_kernel(
    const bvhgb_node *__restrict__ nodes, const uint32_t *__restrict__ todo, const uint32_t *__restrict__ itemMesh,
    const uint32_t *__restrict__ itemOff, const uint32_t *__restrict__ chunkSize,
    const uint32_t *__restrict__ faceOff, const uint32_t *__restrict__ nodeOff,
    const uint32_t *__restrict__ innerOff, uint32_t items, uint32_t chunk, PatchOut *__restrict__ out,
    uint32_t *__restrict__ valid, uint32_t *__restrict__ toFix, uint32_t *__restrict__ owner,
    unsigned long long *__restrict__ stats, uint32_t *__restrict__ err) {
  const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= items) return;  // whole warps leave together
  const MeshItem it = item_of(itemMesh, itemOff, q);
  const uint32_t n = __ldg(faceOff + it.m + 1) - __ldg(faceOff + it.m);
  const uint32_t numNodes = 2 * n - 1, numInner = n - 1, nb = __ldg(nodeOff + it.m);
  const uint32_t pos = chunk * __ldg(chunkSize + it.m) + it.k;
  const bool ok = pos < numInner;
  const uint32_t node = ok ? __ldg(todo + __ldg(innerOff + it.m) + pos) : kNone;
  warp_patch_item(nodes + nb, 0u, numNodes, node, ok, it.k, out + q, valid + q, toFix + 3 * (size_t)q, owner + nb,
                  stats, err);
}

__global__ void batch_apply_kernel(bvhgb_node *nodes, const PatchOut *__restrict__ in, uint32_t *__restrict__ valid,
                                   uint32_t *__restrict__ toFix, const uint32_t *__restrict__ owner,
                                   const uint32_t *__restrict__ itemMesh, const uint32_t *__restrict__ itemOff,
                                   const uint32_t *__restrict__ nodeOff, uint32_t items,
                                   unsigned long long *__restrict__ stats) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= items) return;
  const MeshItem it = item_of(itemMesh, itemOff, q);
  const uint32_t nb = __ldg(nodeOff + it.m);
  apply_item(nodes + nb, in[q], valid + q, toFix + 3 * (size_t)q, owner + nb, it.k, stats);
}

// The count and refit climbs run a few per warp (lanes 0 .. perWarp - 1): climbs sharing a warp
// each wait, level by level, for the slowest lane's level, so a launch uses as few per warp as keep
// it within one wave of resident warps.
__device__ __forceinline__ uint32_t batch_path_index(uint32_t perWarp) {
  const uint32_t lane = threadIdx.x & 31u;
  if (lane >= perWarp) return 0xFFFFFFFFu;
  return ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * perWarp + lane;
}

__global__ void batch_count_kernel(const bvhgb_node *__restrict__ nodes, const PatchOut *__restrict__ in,
                                   const uint32_t *__restrict__ toFix, uint32_t *__restrict__ owner,
                                   uint32_t *__restrict__ counter, const uint32_t *__restrict__ itemMesh,
                                   const uint32_t *__restrict__ itemOff, const uint32_t *__restrict__ faceOff,
                                   const uint32_t *__restrict__ nodeOff, uint32_t items, uint32_t perWarp,
                                   uint32_t *__restrict__ err) {
  const uint32_t i = batch_path_index(perWarp);
  if (i >= 3 * items) return;
  const uint32_t q = i / 3;
  const MeshItem it = item_of(itemMesh, itemOff, q);
  const uint32_t n = __ldg(faceOff + it.m + 1) - __ldg(faceOff + it.m), nb = __ldg(nodeOff + it.m);
  count_path(nodes + nb, 0u, 2 * n - 1, in[q], i - 3 * q, toFix[i], owner + nb, counter + nb, err);
}

__global__ void batch_refit_kernel(bvhgb_node *nodes, const uint32_t *__restrict__ toFix,
                                   uint32_t *__restrict__ counter, unsigned long long *__restrict__ mail,
                                   const uint32_t *__restrict__ itemMesh,
                                   const uint32_t *__restrict__ itemOff, const uint32_t *__restrict__ faceOff,
                                   const uint32_t *__restrict__ nodeOff, uint32_t items, uint32_t perWarp,
                                   uint32_t *__restrict__ err) {
  const uint32_t i = batch_path_index(perWarp);
  if (i >= 3 * items) return;
  const MeshItem it = item_of(itemMesh, itemOff, i / 3);
  const uint32_t n = __ldg(faceOff + it.m + 1) - __ldg(faceOff + it.m), nb = __ldg(nodeOff + it.m);
  refit_path(nodes + nb, 0u, 2 * n - 1, toFix[i], counter + nb, mail + 3ull * nb, err);
}

// SplitMix64 of (seed, index, lane) -> uniform in [0, 1) with 24 bits.
__device__ __forceinline__ float batch_uniform(uint64_t seed, uint64_t idx, uint32_t lane) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (4 * idx + lane + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}

__global__ void batch_trace_kernel(const bvhgb_node *__restrict__ nodes, const float *__restrict__ vert,
                                   const uint32_t *__restrict__ faces, const uint32_t *__restrict__ faceOff,
                                   const uint32_t *__restrict__ nodeOff, uint32_t numMeshes, uint32_t raysPerMesh,
                                   uint64_t seed, bvhgb_hit *__restrict__ hits, float *__restrict__ rayOrg,
                                   float *__restrict__ rayDir, uint32_t *__restrict__ err) {
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (uint64_t)numMeshes * raysPerMesh) return;
  const uint32_t m = (uint32_t)(r / raysPerMesh);
  const uint32_t fb = __ldg(faceOff + m), n = __ldg(faceOff + m + 1) - fb;
  const bvhgb_node *t = nodes + __ldg(nodeOff + m);
  // mesh box = the root's box, grown 1.5x about its centre
  float4 a, b, c;
  load_node(t, 0, a, b, c);
  const float mn[3] = {a.x, a.y, a.z}, mx[3] = {a.w, b.x, b.y};
  RayPre ray;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float ctr = 0.5f * (mn[k] + mx[k]), half = 0.75f * (mx[k] - mn[k]);
    ray.o[k] = ctr + (2.0f * batch_uniform(seed, r, k) - 1.0f) * half;
  }
  const float z = 1.0f - 2.0f * batch_uniform(seed, r, 3);
  const float phi = 6.283185307179586f * batch_uniform(seed ^ 0x5DEECE66Dull, r, 0);
  const float s = sqrtf(fmaxf(0.0f, 1.0f - z * z));
  ray.d[0] = s * cosf(phi);
  ray.d[1] = s * sinf(phi);
  ray.d[2] = z;
  if (rayOrg) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      rayOrg[3 * r + k] = ray.o[k];
      rayDir[3 * r + k] = ray.d[k];
    }
  }
  setup_ray(ray);
  Hit h;
  traverse(ray, t, 2 * n - 1, 0u, vert, faces + 3 * (size_t)fb, 0.0f, __int_as_float(0x7f800000), false, h, err);
  bvhgb_hit o;
  o.primId = h.prim;
  o.t = h.prim == kNone ? __int_as_float(0x7f800000) : h.t;
  hits[r] = o;
}

uint32_t grid_of(uint64_t n, uint32_t block) {
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + block - 1) / block, (uint64_t)sm_count() * 16));
}

size_t off_smem(uint32_t numMeshes) { return sizeof(uint32_t) * (numMeshes + 1); }

int batch_build(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces, bvhgb_node *nodes,
                cudaStream_t s) {
  const uint32_t M = ws->numMeshes, F = ws->totalFaces;
  batch_init_kernel<<<ceil_div(6ull * M + 1, 256), 256, 0, s>>>(ws->scene, M, ws->err);
  BVHGB_LAUNCH_CHECK("batch init");
  if (F == 0) return BVHGB_OK;
  batch_bounds_kernel<<<grid_of(F, kBatchThreads), kBatchThreads, off_smem(M), s>>>(vert, faces, ws->faceOff, M, F,
                                                                                     ws->scene);
  BVHGB_LAUNCH_CHECK("batch bounds");
  batch_morton_kernel<<<grid_of(F, kBatchThreads), kBatchThreads, off_smem(M), s>>>(
      vert, faces, ws->faceOff, M, F, ws->scene, ws->keys, ws->vals, ws->slots, ws->triBoxes);
  BVHGB_LAUNCH_CHECK("batch morton");
  int st = sort_pairs(ws->sortTemp, ws->keys, ws->keysSorted, ws->vals, ws->valsSorted, F, 8, 0, 30 + ws->meshBits, s,
                      ws->cfg.sortTileKeys);
  if (st) return st;
  if (ws->cfg.topology == BVHGB_TOPO_KARRAS)
    batch_build_kernel<BVHGB_TOPO_KARRAS><<<ceil_div(F, 128), 128, off_smem(M), s>>>(
        ws->keysSorted, ws->valsSorted, ws->triBoxes, ws->faceOff, ws->nodeOff, M, F, nodes, ws->slots, ws->err);
  else
    batch_build_kernel<BVHGB_TOPO_REFCOMPAT><<<ceil_div(F, 128), 128, off_smem(M), s>>>(
        ws->keysSorted, ws->valsSorted, ws->triBoxes, ws->faceOff, ws->nodeOff, M, F, nodes, ws->slots, ws->err);
  BVHGB_LAUNCH_CHECK("batch build");
  return BVHGB_OK;
}

int batch_iteration(bvhgb_batch_workspace *ws, bvhgb_node *nodes, cudaStream_t s) {
  const uint32_t M = ws->numMeshes, I = ws->totalInner, T = ws->items;
  if (I == 0) return BVHGB_OK;
  batch_cost_kernel<<<grid_of(I, kBatchThreads), kBatchThreads, off_smem(M), s>>>(nodes, ws->innerOff, ws->nodeOff, M,
                                                                                   I, ws->keys, ws->vals);
  BVHGB_LAUNCH_CHECK("batch cost");
  int st = sort_pairs(ws->sortTemp, ws->keys, ws->keysSorted, ws->vals, ws->todo, I, 8, 0, 32 + ws->meshBits, s,
                      ws->cfg.sortTileKeys);
  if (st) return st;
  if (T == 0) return BVHGB_OK;
  const uint32_t bs = ws->cfg.refitBlock;
  // climbs per warp: the fewest that fit in one wave of resident warps
  auto perWarp = [&](const void *kernel) {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, (int)bs, 0) != cudaSuccess || blocks <= 0)
      blocks = 1;
    const uint64_t slots = (uint64_t)blocks * (bs / 32) * (uint64_t)sm_count();
    return (uint32_t)std::min<uint64_t>(std::max<uint64_t>((3ull * T + slots - 1) / slots, 1), 32);
  };
  const uint32_t pc = perWarp((const void *)batch_count_kernel), pr = perWarp((const void *)batch_refit_kernel);
  for (uint32_t c = 0; c < ws->cfg.numChunks; ++c) {
    batch_patch_kernel<<<ceil_div(T, kWarpItemsPerBlock), kWarpItemsPerBlock * 32, 0, s>>>(
        nodes, ws->todo, ws->itemMesh, ws->itemOff, ws->chunk, ws->faceOff, ws->nodeOff, ws->innerOff, T, c,
        ws->patches, ws->valid, ws->toFix, ws->owner, ws->stats, ws->err);
    BVHGB_LAUNCH_CHECK("batch patch");
    batch_apply_kernel<<<ceil_div(T, bs), bs, 0, s>>>(nodes, ws->patches, ws->valid, ws->toFix, ws->owner,
                                                      ws->itemMesh, ws->itemOff, ws->nodeOff, T, ws->stats);
    BVHGB_LAUNCH_CHECK("batch apply");
    batch_count_kernel<<<ceil_div(3ull * T, (uint64_t)pc * (bs / 32)), bs, 0, s>>>(
        nodes, ws->patches, ws->toFix, ws->owner, ws->counter, ws->itemMesh, ws->itemOff, ws->faceOff, ws->nodeOff, T,
        pc, ws->err);
    BVHGB_LAUNCH_CHECK("batch count");
    batch_refit_kernel<<<ceil_div(3ull * T, (uint64_t)pr * (bs / 32)), bs, 0, s>>>(
        nodes, ws->toFix, ws->counter, ws->mail, ws->itemMesh, ws->itemOff, ws->faceOff, ws->nodeOff, T, pr, ws->err);
    BVHGB_LAUNCH_CHECK("batch refit");
  }
  return BVHGB_OK;
}

int batch_trace(bvhgb_batch_workspace *ws, const bvhgb_node *nodes, const float *vert, const uint32_t *faces,
                uint32_t raysPerMesh, uint64_t seed, bvhgb_hit *hits, float *rayOrg, float *rayDir, cudaStream_t s) {
  const uint64_t R = (uint64_t)ws->numMeshes * raysPerMesh;
  if (R == 0) return BVHGB_OK;
  const uint32_t bs = ws->cfg.traceBlock;
  batch_trace_kernel<<<(uint32_t)((R + bs - 1) / bs), bs, 0, s>>>(nodes, vert, faces, ws->faceOff, ws->nodeOff,
                                                                  ws->numMeshes, raysPerMesh, seed, hits, rayOrg,
                                                                  rayDir, ws->err);
  BVHGB_LAUNCH_CHECK("batch trace");
  return BVHGB_OK;
}

bool valid_config(const bvhgb_batch_config &c) {
  const bool tile = c.sortTileKeys == 2048 || c.sortTileKeys == 4096 || c.sortTileKeys == 8192;
  const bool refit = c.refitBlock >= 32 && c.refitBlock <= 1024 && c.refitBlock % 32 == 0;
  const bool trace = c.traceBlock >= 32 && c.traceBlock <= 1024 && c.traceBlock % 32 == 0;
  return tile && refit && trace && c.numChunks > 0 && c.topology <= BVHGB_TOPO_KARRAS && c.mortonBits == 30;
}

void drop_graph(bvhgb_batch_workspace *ws) {
  if (ws->graph) cudaGraphExecDestroy(ws->graph);
  ws->graph = nullptr;
}

}  // namespace
}  // namespace bvhgb

using namespace bvhgb;

extern "C" BVHGB_API int bvhgb_batch_create(uint32_t numMeshes, const uint32_t *faceCounts,
                                            const bvhgb_batch_config *cfg, bvhgb_batch_workspace **out) {
  if (!out || !faceCounts || numMeshes == 0) return BVHGB_INVALID_ARGUMENT;
  *out = nullptr;
  if (numMeshes > kMaxMeshes) return BVHGB_TOO_LARGE;
  bvhgb_batch_config c = cfg ? *cfg
                             : bvhgb_batch_config{30u, BVHGB_TOPO_REFCOMPAT, 32u, 1.0f, kSortTileDefault, 128u, 128u};
  if (c.batchPercent <= 0.01f) c.batchPercent = 0.01f;  // Bittner13GPU.cpp:59-60
  if (c.batchPercent >= 75.0f) c.batchPercent = 75.0f;
  if (!valid_config(c)) return BVHGB_INVALID_ARGUMENT;
  int pst = sort_prepare();
  if (pst) return pst;
  auto *ws = new bvhgb_batch_workspace();
  ws->cfg = c;
  ws->numMeshes = numMeshes;
  while ((1u << ws->meshBits) < numMeshes) ++ws->meshBits;
  ws->hFaceOff.assign(numMeshes + 1, 0);
  ws->hNodeOff.assign(numMeshes + 1, 0);
  ws->hInnerOff.assign(numMeshes + 1, 0);
  ws->hItemOff.assign(numMeshes + 1, 0);
  ws->hChunk.assign(numMeshes, 0);
  uint64_t faces = 0, nodes = 0, inner = 0, items = 0;
  for (uint32_t m = 0; m < numMeshes; ++m) {
    const uint32_t n = faceCounts[m];
    ws->hFaceOff[m] = (uint32_t)faces;
    ws->hNodeOff[m] = (uint32_t)nodes;
    ws->hInnerOff[m] = (uint32_t)inner;
    ws->hItemOff[m] = (uint32_t)items;
    const uint32_t numNodes = n ? 2 * n - 1 : 0;
    // Bittner13GPU.cpp:79-80: the batch is batchPercent of the node count, split into chunks
    const uint32_t lNum = (uint32_t)((c.batchPercent / 100.0f) * (float)numNodes);
    ws->hChunk[m] = lNum / c.numChunks;
    faces += n;
    nodes += numNodes;
    inner += n ? n - 1 : 0;
    items += ws->hChunk[m];
  }
  if (faces >= (1ull << 30) || nodes >= (1ull << 31)) {
    delete ws;
    return BVHGB_TOO_LARGE;
  }
  ws->hFaceOff[numMeshes] = (uint32_t)faces;
  ws->hNodeOff[numMeshes] = (uint32_t)nodes;
  ws->hInnerOff[numMeshes] = (uint32_t)inner;
  ws->hItemOff[numMeshes] = (uint32_t)items;
  ws->totalFaces = (uint32_t)faces;
  ws->totalNodes = (uint32_t)nodes;
  ws->totalInner = (uint32_t)inner;
  ws->items = (uint32_t)items;
  std::vector<uint32_t> itemMesh(std::max<uint64_t>(items, 1), 0);
  for (uint32_t m = 0; m < numMeshes; ++m)
    for (uint32_t k = 0; k < ws->hChunk[m]; ++k) itemMesh[ws->hItemOff[m] + k] = m;

  const size_t F = std::max<size_t>(faces, 1), N = std::max<size_t>(nodes, 1), T = std::max<size_t>(items, 1);
  const size_t sortN = std::max<size_t>(faces, inner);
  const size_t sortBytes = sort_temp_bytes((uint32_t)sortN, 8, 0, 32 + ws->meshBits);
  cudaError_t e = cudaSuccess;
  auto alloc = [&](auto **p, size_t bytes) {
    if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void **>(p), std::max<size_t>(bytes, 16));
  };
  alloc(&ws->faceOff, 4 * (numMeshes + 1));
  alloc(&ws->nodeOff, 4 * (numMeshes + 1));
  alloc(&ws->innerOff, 4 * (numMeshes + 1));
  alloc(&ws->itemOff, 4 * (numMeshes + 1));
  alloc(&ws->chunk, 4 * numMeshes);
  alloc(&ws->itemMesh, 4 * T);
  alloc(&ws->scene, 4 * 6 * (size_t)numMeshes);
  alloc(&ws->err, 4);
  alloc(&ws->keys, 8 * F);
  alloc(&ws->keysSorted, 8 * F);
  alloc(&ws->vals, 4 * F);
  alloc(&ws->valsSorted, 4 * F);
  alloc(&ws->slots, 4 * F);
  alloc(&ws->triBoxes, 32 * F);
  alloc(&ws->sortTemp, sortBytes);
  alloc(&ws->todo, 4 * F);
  alloc(&ws->valid, 4 * T);
  alloc(&ws->toFix, 12 * T);
  alloc(&ws->patches, sizeof(PatchOut) * T);
  alloc(&ws->owner, 4 * N);
  alloc(&ws->counter, 4 * N);
  alloc(&ws->mail, 24 * N);
  alloc(&ws->stats, sizeof(unsigned long long) * S_COUNT);
  if (e == cudaSuccess) e = cudaMemcpy(ws->faceOff, ws->hFaceOff.data(), 4 * (numMeshes + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ws->nodeOff, ws->hNodeOff.data(), 4 * (numMeshes + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ws->innerOff, ws->hInnerOff.data(), 4 * (numMeshes + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ws->itemOff, ws->hItemOff.data(), 4 * (numMeshes + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ws->chunk, ws->hChunk.data(), 4 * numMeshes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ws->itemMesh, itemMesh.data(), 4 * itemMesh.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(ws->owner, 0xFF, 4 * N);
  if (e == cudaSuccess) e = cudaMemset(ws->counter, 0, 4 * N);
  if (e == cudaSuccess) e = cudaMemset(ws->mail, 0xFF, 24 * N);
  if (e == cudaSuccess) e = cudaMemset(ws->stats, 0, sizeof(unsigned long long) * S_COUNT);
  if (e == cudaSuccess) e = cudaMemset(ws->err, 0, 4);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_batch_create", e);
    bvhgb_batch_destroy(ws);
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  *out = ws;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_destroy(bvhgb_batch_workspace *ws) {
  if (!ws) return BVHGB_OK;
  drop_graph(ws);
  for (void *p : {(void *)ws->faceOff, (void *)ws->nodeOff, (void *)ws->innerOff, (void *)ws->itemOff, (void *)ws->chunk,
                  (void *)ws->itemMesh, (void *)ws->scene, (void *)ws->err, (void *)ws->keys, (void *)ws->keysSorted,
                  (void *)ws->vals, (void *)ws->valsSorted, (void *)ws->slots, (void *)ws->triBoxes, ws->sortTemp,
                  (void *)ws->todo, (void *)ws->valid, (void *)ws->toFix, (void *)ws->patches, (void *)ws->owner,
                  (void *)ws->counter, (void *)ws->mail, (void *)ws->stats})
    cudaFree(p);
  delete ws;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_offsets(const bvhgb_batch_workspace *ws, uint32_t *faceOffsets,
                                             uint32_t *nodeOffsets) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  if (faceOffsets) std::copy(ws->hFaceOff.begin(), ws->hFaceOff.end(), faceOffsets);
  if (nodeOffsets) std::copy(ws->hNodeOff.begin(), ws->hNodeOff.end(), nodeOffsets);
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_get_config(const bvhgb_batch_workspace *ws, bvhgb_batch_config *cfg) {
  if (!ws || !cfg) return BVHGB_INVALID_ARGUMENT;
  *cfg = ws->cfg;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_set_config(bvhgb_batch_workspace *ws, const bvhgb_batch_config *cfg) {
  if (!ws || !cfg) return BVHGB_INVALID_ARGUMENT;
  bvhgb_batch_config c = *cfg;
  // only the tuning knobs may change: the sizes below were fixed when the workspace was made
  if (c.mortonBits != ws->cfg.mortonBits || c.numChunks != ws->cfg.numChunks ||
      c.batchPercent != ws->cfg.batchPercent || !valid_config(c))
    return BVHGB_INVALID_ARGUMENT;
  if (c.sortTileKeys != ws->cfg.sortTileKeys || c.refitBlock != ws->cfg.refitBlock ||
      c.traceBlock != ws->cfg.traceBlock || c.topology != ws->cfg.topology)
    drop_graph(ws);
  ws->cfg = c;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_build(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces,
                                           bvhgb_node *nodes, bvhgb_stream stream) {
  if (!ws || (ws->totalFaces && (!vert || !faces || !nodes))) return BVHGB_INVALID_ARGUMENT;
  return batch_build(ws, vert, faces, nodes, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_batch_optimize(bvhgb_batch_workspace *ws, bvhgb_node *nodes, uint32_t iterations,
                                              bvhgb_stream stream) {
  if (!ws || (ws->totalFaces && !nodes)) return BVHGB_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < iterations; ++i) {
    const int st = batch_iteration(ws, nodes, as_stream(stream));
    if (st) return st;
  }
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_trace_random(bvhgb_batch_workspace *ws, const bvhgb_node *nodes,
                                                  const float *vert, const uint32_t *faces, uint32_t raysPerMesh,
                                                  uint64_t seed, bvhgb_hit *hits, float *rayOrg, float *rayDir,
                                                  bvhgb_stream stream) {
  if (!ws || (raysPerMesh && (!nodes || !vert || !faces || !hits))) return BVHGB_INVALID_ARGUMENT;
  if ((rayOrg == nullptr) != (rayDir == nullptr)) return BVHGB_INVALID_ARGUMENT;
  for (uint32_t m = 0; m < ws->numMeshes; ++m)
    if (raysPerMesh && ws->hFaceOff[m + 1] == ws->hFaceOff[m]) return BVHGB_INVALID_ARGUMENT;  // an empty mesh
  return batch_trace(ws, nodes, vert, faces, raysPerMesh, seed, hits, rayOrg, rayDir, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_batch_run(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces,
                                         bvhgb_node *nodes, uint32_t iterations, uint32_t raysPerMesh, uint64_t seed,
                                         bvhgb_hit *hits, bvhgb_stream stream) {
  if (!ws || (ws->totalFaces && (!vert || !faces || !nodes)) || (raysPerMesh && !hits)) return BVHGB_INVALID_ARGUMENT;
  for (uint32_t m = 0; m < ws->numMeshes; ++m)
    if (raysPerMesh && ws->hFaceOff[m + 1] == ws->hFaceOff[m]) return BVHGB_INVALID_ARGUMENT;
  cudaStream_t s = as_stream(stream);
  const bool same = ws->graph && ws->gVert == vert && ws->gFaces == faces && ws->gNodes == nodes && ws->gHits == hits &&
                    ws->gIterations == iterations && ws->gRays == raysPerMesh && ws->gSeed == seed;
  if (!same) {
    drop_graph(ws);
    int pst = sort_prepare();
    if (pst) return pst;
    cudaStream_t cap = nullptr;
    BVHGB_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    const uint64_t before = bvhgb_launch_count();
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int st = BVHGB_OK;
    if (e == cudaSuccess) {
      st = batch_build(ws, vert, faces, nodes, cap);
      for (uint32_t i = 0; i < iterations && st == BVHGB_OK; ++i) st = batch_iteration(ws, nodes, cap);
      if (st == BVHGB_OK) st = batch_trace(ws, nodes, vert, faces, raysPerMesh, seed, hits, nullptr, nullptr, cap);
      e = cudaStreamEndCapture(cap, &g);
    }
    const uint64_t kernels = bvhgb_launch_count() - before;
    uncount_launches(kernels);
    if (e == cudaSuccess && st == BVHGB_OK) e = cudaGraphInstantiate(&ws->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cap);
    if (st) return st;
    if (e != cudaSuccess) {
      set_last_error("bvhgb_batch_run capture", e);
      ws->graph = nullptr;
      return BVHGB_CUDA_ERROR;
    }
    ws->gVert = vert;
    ws->gFaces = faces;
    ws->gNodes = nodes;
    ws->gHits = hits;
    ws->gIterations = iterations;
    ws->gRays = raysPerMesh;
    ws->gSeed = seed;
    ws->graphKernels = kernels;
  }
  BVHGB_CUDA_TRY(cudaGraphLaunch(ws->graph, s));
  count_launch((uint32_t)ws->graphKernels);
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_batch_get_stats(bvhgb_batch_workspace *ws, bvhgb_bn13_stats *stats, uint32_t *errors,
                                               bvhgb_stream stream) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  unsigned long long h[S_COUNT];
  uint32_t err = 0;
  cudaStream_t s = as_stream(stream);
  BVHGB_CUDA_TRY(cudaMemcpyAsync(h, ws->stats, sizeof(h), cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaMemcpyAsync(&err, ws->err, 4, cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  if (stats) {
    stats->items = h[S_ITEMS];
    stats->applied = h[S_APPLIED];
    stats->skippedConflict = h[S_CONFLICT];
    stats->skippedInvalid = h[S_INVALID];
    stats->heapOverflow = h[S_OVERFLOW];
    stats->nodesVisited = h[S_VISITS];
  }
  if (errors) *errors = err;
  return BVHGB_OK;
}

// ---- autotuner ------------------------------------------------------------------------------------
// Coordinate search over the three knobs, each timed with CUDA events on the caller's stream on
// the caller's data (the results do not depend on them): the sort tile on the build, the refit block
// on one optimizer iteration, the trace block on the random rays. Each candidate runs twice, the
// faster run counts. The workspace keeps the best; the report lists every measurement.

extern "C" BVHGB_API int bvhgb_batch_autotune(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces,
                                              bvhgb_node *nodes, uint32_t raysPerMesh, uint64_t seed, bvhgb_hit *hits,
                                              bvhgb_batch_tune_report *report, bvhgb_stream stream) {
  if (!ws || !report || (ws->totalFaces && (!vert || !faces || !nodes)) || (raysPerMesh && !hits))
    return BVHGB_INVALID_ARGUMENT;
  cudaStream_t s = as_stream(stream);
  *report = bvhgb_batch_tune_report{};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BVHGB_CUDA_TRY(cudaEventCreate(&e0));
  BVHGB_CUDA_TRY(cudaEventCreate(&e1));
  auto timed = [&](auto &&fn, float &ms) -> int {
    float best = 3.4e38f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaError_t e = cudaEventRecord(e0, s);
      int st = e == cudaSuccess ? fn() : BVHGB_CUDA_ERROR;
      if (st) return st;
      if ((e = cudaEventRecord(e1, s)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess) {
        set_last_error("bvhgb_batch_autotune", e);
        return BVHGB_CUDA_ERROR;
      }
      float t = 0.0f;
      cudaEventElapsedTime(&t, e0, e1);
      best = std::min(best, t);
    }
    ms = best;
    return BVHGB_OK;
  };
  int st = BVHGB_OK;
  const uint32_t tiles[3] = {2048, 4096, 8192}, blocks[3] = {128, 256, 512}, traces[3] = {64, 128, 256};
  bvhgb_batch_config best = ws->cfg;
  float bestMs = 3.4e38f;
  for (int i = 0; i < 3 && !st; ++i) {
    ws->cfg.sortTileKeys = tiles[i];
    st = timed([&] { return batch_build(ws, vert, faces, nodes, s); }, report->sortTileMs[i]);
    report->sortTileKeys[i] = tiles[i];
    if (!st && report->sortTileMs[i] < bestMs) {
      bestMs = report->sortTileMs[i];
      best.sortTileKeys = tiles[i];
    }
  }
  ws->cfg.sortTileKeys = best.sortTileKeys;
  bestMs = 3.4e38f;
  for (int i = 0; i < 3 && !st; ++i) {
    ws->cfg.refitBlock = blocks[i];
    st = batch_build(ws, vert, faces, nodes, s);  // the same starting tree for every candidate
    if (!st) st = timed([&] { return batch_iteration(ws, nodes, s); }, report->refitBlockMs[i]);
    report->refitBlock[i] = blocks[i];
    if (!st && report->refitBlockMs[i] < bestMs) {
      bestMs = report->refitBlockMs[i];
      best.refitBlock = blocks[i];
    }
  }
  ws->cfg.refitBlock = best.refitBlock;
  bestMs = 3.4e38f;
  for (int i = 0; i < 3 && !st && raysPerMesh; ++i) {
    ws->cfg.traceBlock = traces[i];
    st = timed([&] { return batch_trace(ws, nodes, vert, faces, raysPerMesh, seed, hits, nullptr, nullptr, s); },
               report->traceBlockMs[i]);
    report->traceBlock[i] = traces[i];
    if (!st && report->traceBlockMs[i] < bestMs) {
      bestMs = report->traceBlockMs[i];
      best.traceBlock = traces[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  drop_graph(ws);
  ws->cfg = best;
  report->chosen = best;
  return st;
}
