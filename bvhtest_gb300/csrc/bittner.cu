// Parallel Bittner13 SAH optimizer (lib/builder/Bittner13CUDA.cu, lib/base/BVHPatch.hpp).
//
// One iteration = select + numChunks chunks. Selection: inefficiency of every inner node, then the
// onesweep sort on (~order(cost), node) gives the stable descending order of the reference's
// SortPairsDescending. Each chunk runs four kernels:
//   patch  : one thread per batch item removes its node and reinserts both children into a private
//            10-slot copy-on-write patch, finding each position by branch and bound over the induced
//            cost (findNode1 with the standard-library heap discipline), then claims every node it
//            patched with atomicMin(owner, rank);
//   apply  : an item whose every node is still owned by its own rank writes its patch; all others
//            count as skipped. Lower rank = higher cost wins, so the result does not depend on
//            scheduling (the reference locks first-come and is not deterministic);
//   count  : owners are released and each dirty path (grand parent, both reused nodes) counts its
//            arrivals on the way to the root (kFixTree3_1);
//   refit  : the last arrival at a node recomputes its box from its children (kFixTree3_2); the
//            counters are relaxed and a rewritten child box reaches the last arrival through a
//            self-validating mail slot, so no box is read before it is final.
// bvhgb_bn13_run captures one iteration into a CUDA graph and replays it. With a learned scorer
// set, iteration i selects by the scorer unless plainEvery > 0 and i % plainEvery == plainEvery - 1,
// in which case it selects by the inefficiency (one graph per kind of iteration).
#include <algorithm>
#include <vector>

#include "bn13_device.cuh"
#include "common.cuh"
#include "learned.cuh"
#include "sort.cuh"

namespace bvhgb {
namespace {

// ---- kernels ------------------------------------------------------------------------------

__global__ void cost_kernel(const bvhgb_node *__restrict__ t, const uint32_t *__restrict__ inner, uint32_t numInner,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < numInner; i += gridDim.x * blockDim.x) {
    const uint32_t x = __ldg(inner + i);
    keys[i] = ~f2ord(inefficiency(t, x));  // ascending key order = descending cost
    vals[i] = x;
  }
}

// One thread per batch item: the reference's per-thread searches, findNode1 (HEAP) or findNode2 (ALT).
template <int MODE>
__global__ void patch_kernel(const bvhgb_node *__restrict__ t, uint32_t root, const uint32_t *__restrict__ todo,
                             uint32_t numTodo, uint32_t chunk, uint32_t numChunks, uint32_t chunkSize,
                             uint32_t offsetAccess, PatchOut *__restrict__ out, uint32_t *__restrict__ valid,
                             uint32_t *__restrict__ toFix, uint32_t *__restrict__ owner, HeapItem *__restrict__ heaps,
                             uint32_t cap, unsigned long long *__restrict__ stats, uint32_t numNodes,
                             uint32_t *__restrict__ err) {
  __shared__ HeapItem heapTop[kHeapShared * kSearchThreads];
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= chunkSize) return;
  const uint32_t pos = offsetAccess ? k * numChunks + chunk : chunk * chunkSize + k;
  PatchData pd;
  Patch p;
  p.d = &pd;
  p.t = t;
  p.root = root;
  p.numNodes = numNodes;
  p.bad = false;
  p.clear();
  SearchCounters ctr = {0u, 0u};
  uint32_t ins[2], un[2], g = kNone;
  bool ok = pos < numTodo;
  const uint32_t node = ok ? __ldg(todo + pos) : kNone;
  const Heap pq{heapTop + (threadIdx.x & (kSearchThreads - 1)), heaps + (size_t)k * cap};
  ok = ok && remove_node(p, node, ins, un, g);
  ok = ok && reinsert<MODE>(p, ins[0], un[0], true, pq, cap, ctr);
  ok = ok && reinsert<MODE>(p, ins[1], un[1], false, pq, cap, ctr);
  if (p.bad) {
    atomicOr(err, kErrBadIndex);
    ok = false;
  }
  valid[k] = ok ? 1u : 0u;
  toFix[3 * k + 0] = ok ? g : kNone;
  toFix[3 * k + 1] = ok ? un[0] : kNone;
  toFix[3 * k + 2] = ok ? un[1] : kNone;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    out[k].nd[s] = p.d->nd[s];
    out[k].idx[s] = ok ? p.d->idx[s] : kNone;
    if (ok && p.d->idx[s] != kNone) atomicMin(&owner[p.d->idx[s]], k);
  }
  if (!ok) atomicAdd(&stats[S_INVALID], 1ull);
  if (ctr.overflow) atomicAdd(&stats[S_OVERFLOW], (unsigned long long)ctr.overflow);
  atomicAdd(&stats[S_VISITS], (unsigned long long)ctr.visits);
  atomicAdd(&stats[S_ITEMS], 1ull);
}

// One warp per batch item: the patch logic runs redundantly on every lane (same data, no
// divergence) and the two searches are the warp-cooperative batched search; lane 0 publishes.
__global__ void __launch_bounds__(kWarpItemsPerBlock * 32, 5) patch_warp_kernel(
    const bvhgb_node *__restrict__ t, uint32_t root, const uint32_t *__restrict__ todo, uint32_t numTodo,
    uint32_t chunk, uint32_t numChunks, uint32_t chunkSize, uint32_t offsetAccess, PatchOut *__restrict__ out,
    uint32_t *__restrict__ valid, uint32_t *__restrict__ toFix, uint32_t *__restrict__ owner,
    unsigned long long *__restrict__ stats, uint32_t numNodes, uint32_t *__restrict__ err) {
  const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (k >= chunkSize) return;  // whole warps leave together
  const uint32_t pos = offsetAccess ? k * numChunks + chunk : chunk * chunkSize + k;
  const bool ok = pos < numTodo;
  const uint32_t node = ok ? __ldg(todo + pos) : kNone;
  warp_patch_item(t, root, numNodes, node, ok, k, out + k, valid + k, toFix + 3 * k, owner, stats, err);
}

// The climbs of the chunk tail run a few per warp, climbsPerWarp (lanes 0.. of each warp; the other
// lanes leave at once). The paths of one item, or of neighbouring items, have nothing in common: in
// a shared warp every level of every path waits for the slowest lane's level, so few per warp is
// better, but a second wave of warps starts its climbs late: the chunk packs just enough per warp
// to fit in one wave of resident warps (4.19M triangles: 7,863 paths, 2 per warp; 33.5M: 62,913
// paths, 12 per warp). Measured (20 plain iterations of the 4.19M-triangle scene): 1 per warp
// 52.8 ms, 2: 51.8, 4: 52.8; (5 of the 33.5M scene) 4: 73.1, 6: 71.3, 12: 70.7, 16: 70.5.
constexpr uint32_t kTailWarpsPerBlock = 4;
constexpr uint32_t kTailMaxWaves = 1;

__device__ __forceinline__ uint32_t tail_path_index(uint32_t climbsPerWarp) {
  const uint32_t lane = threadIdx.x & 31u;
  if (lane >= climbsPerWarp) return 0xFFFFFFFFu;
  return ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * climbsPerWarp + lane;
}

// Apply + count (apply_count_path): three climbs per item.
__global__ void __launch_bounds__(kTailWarpsPerBlock * 32) apply_count_kernel(
    bvhgb_node *t, uint32_t root, const PatchOut *__restrict__ in, const uint32_t *__restrict__ valid,
    uint32_t *__restrict__ toFix, const uint32_t *__restrict__ owner, uint32_t *__restrict__ counter,
    uint32_t chunkSize, uint32_t climbsPerWarp, uint32_t numNodes, unsigned long long *__restrict__ stats,
    uint32_t *__restrict__ err) {
  const uint32_t i = tail_path_index(climbsPerWarp);
  if (i >= 3 * chunkSize) return;
  const uint32_t k = i / 3;
  apply_count_path(t, root, numNodes, in, k, i - 3 * k, valid, toFix, owner, counter, stats, err);
}

// Release the claims of the chunk, then refit the dirty paths (refit_path).
__global__ void __launch_bounds__(kTailWarpsPerBlock * 32) release_refit_kernel(
    bvhgb_node *t, uint32_t root, const PatchOut *__restrict__ in, const uint32_t *__restrict__ toFix,
    uint32_t *__restrict__ owner, uint32_t *__restrict__ counter, unsigned long long *__restrict__ mail,
    uint32_t chunkSize, uint32_t climbsPerWarp, uint32_t numNodes, uint32_t *__restrict__ err) {
  const uint32_t i = tail_path_index(climbsPerWarp);
  if (i >= 3 * chunkSize) return;
  const uint32_t k = i / 3;
  release_claims(in[k], i - 3 * k, owner);
  refit_path(t, root, numNodes, toFix[i], counter, mail, err);
}

// Climbs per warp for 'paths' climbs of 'kernel' (blocks of kTailWarpsPerBlock warps): the fewest
// that fit in kTailMaxWaves waves of resident warps.
uint32_t climbs_per_warp(const void *kernel, uint64_t paths) {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, kTailWarpsPerBlock * 32, 0) != cudaSuccess ||
      blocks <= 0)
    blocks = 1;
  const uint64_t slots = (uint64_t)blocks * kTailWarpsPerBlock * (uint64_t)sm_count() * kTailMaxWaves;
  const uint64_t per = (paths + slots - 1) / slots;
  return (uint32_t)std::min<uint64_t>(std::max<uint64_t>(per, 1), 32);
}

// Full bottom-up refit (kFixTree1, Bittner13CUDA.cu:372-404): every leaf starts a climb; at each
// inner node the first arrival stops and the second recomputes the box from both children and goes
// on. The arrival counter is acq_rel, so the second arrival sees the first one's child box; child
// boxes are read past L1. The last arrival resets the counter (the workspace keeps them at 0).
__global__ void refit_full_kernel(bvhgb_node *t, uint32_t root, uint32_t numNodes, uint32_t *__restrict__ counter,
                                  uint32_t *__restrict__ err) {
  const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= numNodes || leaf == root || !__ldg(&t[leaf].isLeafFlag)) return;
  uint32_t x = __ldg(&t[leaf].parent);
  for (uint32_t steps = 0;; ++steps) {
    if (x >= numNodes || steps > numNodes) {
      atomicOr(err, kErrBadIndex);
      return;
    }
    if (atom_add_acq_rel(&counter[x], 1u) == 0u) return;  // the sibling's climb is still on its way
    counter[x] = 0u;
    const uint32_t l = __ldcg(&t[x].left), r = __ldcg(&t[x].right);
    if (l >= numNodes || r >= numNodes) {
      atomicOr(err, kErrBadIndex);
      return;
    }
    Box b = load_box_cg(t + l);
    merge_into(b, load_box_cg(t + r));
    float4 *p = reinterpret_cast<float4 *>(t + x);
    const float4 w1 = __ldcg(p + 1);
    p[0] = make_float4(b.mn[0], b.mn[1], b.mn[2], b.mx[0]);
    p[1] = make_float4(b.mx[1], b.mx[2], w1.z, w1.w);
    t[x].surfaceArea = surface_area(b);
    if (x == root) return;
    x = __ldcg(&t[x].parent);
  }
}

// ---- isolated realised gain of one reinsertion (the learned scorer's training label) -----------
// The patch changes the children of three nodes: the grand parent (its child becomes the sibling)
// and the two reused nodes. A box changes iff its node lies on a path from one of them to the root
// in the patched tree, so the SAH reduction (cInner = 1) is the sum of old minus new surface area
// over the union of the three paths, over the root's area. Path 1 (first reused node) meets path 0
// (grand parent) at J1 = lca(s1, s0); path 2 meets path 0 or the private part of path 1 at J2, the
// deeper of lca(s2, s0) and lca(s2, s1). Boxes are rebuilt bottom-up in the order: private part of
// path 2, private part of path 1, path 0 through the root; a child's new box is the running box of
// the walk, the last box of a private part at its join node, or its unchanged box. Sums in double
// in that order.
struct GainWalk {
  uint32_t prev, last1, j1, last2, j2;
  Box prevbox, box1, box2;
};

__device__ __forceinline__ uint32_t new_parent(const Patch &p, uint32_t x) { return p.get(x).parent; }

__device__ bool new_depth(const Patch &p, uint32_t x, uint32_t &d) {
  uint32_t k = 0;
  while (x != p.root) {
    if (x >= p.numNodes || k > p.numNodes) return false;
    x = new_parent(p, x);
    ++k;
  }
  d = k;
  return true;
}

__device__ uint32_t new_lca(const Patch &p, uint32_t a, uint32_t da, uint32_t b, uint32_t db, uint32_t &dout) {
  while (da > db) { a = new_parent(p, a); --da; }
  while (db > da) { b = new_parent(p, b); --db; }
  while (a != b && da > 0) { a = new_parent(p, a); b = new_parent(p, b); --da; }
  dout = da;
  return a;
}

__device__ __forceinline__ Box child_box(const Patch &p, const GainWalk &w, uint32_t x, uint32_t c) {
  if (c == w.prev) return w.prevbox;
  if (x == w.j1 && c == w.last1) return w.box1;
  if (x == w.j2 && c == w.last2) return w.box2;
  return tree_box(p.t, c);
}

__device__ void gain_walk(const Patch &p, GainWalk &w, uint32_t x, uint32_t stop, double &acc, bool &ok) {
  w.prev = kNone;
  for (uint32_t k = 0; x != stop; ++k) {
    if (x >= p.numNodes || k > p.numNodes) {
      ok = false;
      return;
    }
    const NodeP n = p.get(x);
    if (n.left >= p.numNodes || n.right >= p.numNodes) {
      ok = false;
      return;
    }
    Box b = child_box(p, w, x, n.left);
    const Box rb = child_box(p, w, x, n.right);
    merge_into(b, rb);
    acc = __dadd_rn(acc, __dsub_rn((double)tree_sa(p.t, x), (double)surface_area(b)));
    w.prev = x;
    w.prevbox = b;
    if (x == p.root) return;
    x = n.parent;
  }
}

__device__ float isolated_gain(const Patch &p, uint32_t s0, uint32_t s1, uint32_t s2, bool &ok) {
  uint32_t d0, d1, d2, dj1, d20, d21;
  if (!new_depth(p, s0, d0) || !new_depth(p, s1, d1) || !new_depth(p, s2, d2)) {
    ok = false;
    return 0.0f;
  }
  const uint32_t j1 = new_lca(p, s1, d1, s0, d0, dj1);
  const uint32_t l20 = new_lca(p, s2, d2, s0, d0, d20);
  const uint32_t l21 = new_lca(p, s2, d2, s1, d1, d21);
  const uint32_t j2 = d20 >= d21 ? l20 : l21;
  GainWalk w;
  w.last1 = w.j1 = w.last2 = w.j2 = kNone;
  w.prevbox = w.box1 = w.box2 = Box{};
  double acc = 0.0;
  gain_walk(p, w, s2, j2, acc, ok);
  w.last2 = w.prev;
  w.box2 = w.prevbox;
  w.j2 = j2;
  gain_walk(p, w, s1, j1, acc, ok);
  w.last1 = w.prev;
  w.box1 = w.prevbox;
  w.j1 = j1;
  gain_walk(p, w, s0, kNone, acc, ok);
  if (!ok) return 0.0f;
  return __double2float_rn(__ddiv_rn(acc, (double)tree_sa(p.t, p.root)));
}

// One warp per candidate: the optimizer's removal and batched reinsertion searches against the
// unmodified tree, then the isolated gain; lane 0 writes. Nothing is applied.
__global__ void __launch_bounds__(kWarpItemsPerBlock * 32) gain_warp_kernel(
    const bvhgb_node *__restrict__ t, uint32_t root, const uint32_t *__restrict__ cand, uint32_t n, uint32_t numNodes,
    float targetScale, float *__restrict__ gain, float *__restrict__ target, uint32_t *__restrict__ err) {
  const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31u;
  if (k >= n) return;  // whole warps leave together
  Patch p;
  p.d = warp_patch_data();
  p.t = t;
  p.root = root;
  p.numNodes = numNodes;
  p.bad = false;
  p.clear();
  SearchCounters ctr = {0u, 0u};
  uint32_t ins[2], un[2], g = kNone;
  const uint32_t x = __ldg(cand + k);
  const Heap unused{nullptr, nullptr};
  bool ok = x < numNodes;
  ok = ok && remove_node(p, x, ins, un, g);
  ok = ok && reinsert<BVHGB_SEARCH_BATCHED>(p, ins[0], un[0], true, unused, 0, ctr);
  ok = ok && reinsert<BVHGB_SEARCH_BATCHED>(p, ins[1], un[1], false, unused, 0, ctr);
  if (p.bad) ok = false;
  float v = 0.0f;
  if (ok) v = isolated_gain(p, g, un[0], un[1], ok);
  if (p.bad) ok = false;
  if (lane != 0) return;
  if (p.bad) atomicOr(err, kErrBadIndex);
  if (!ok) v = 0.0f;
  gain[k] = v;
  if (target) target[k] = copysignf(log1pf(fmul(fabsf(v), targetScale)), v);
}

__global__ void init_inner_kernel(const bvhgb_node *__restrict__ t, uint32_t n, uint32_t *__restrict__ flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flag[i] = __ldg(&t[i].isLeafFlag) == 0 ? 1u : 0u;
}

}  // namespace
}  // namespace bvhgb

using namespace bvhgb;

struct bvhgb_bn13_workspace {
  bvhgb_bn13_config cfg{};
  uint32_t numNodes = 0, root = 0, numInner = 0, numChunks = 0, chunkSize = 0;
  uint32_t *inner = nullptr, *keys = nullptr, *vals = nullptr, *todo = nullptr;
  void *sortTemp = nullptr;
  PatchOut *patches = nullptr;
  uint32_t *valid = nullptr, *toFix = nullptr, *owner = nullptr, *counter = nullptr, *err = nullptr;
  unsigned long long *mail = nullptr;  // three words per node, empty between launches
  HeapItem *heaps = nullptr;
  unsigned long long *stats = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [0] plain iteration, [1] learned iteration
  bvhgb_node *graphNodes = nullptr;
  uint32_t launchesPerIteration = 0;
  uint32_t countClimbsPerWarp = 1, refitClimbsPerWarp = 1;  // chunk-tail climbs per warp
  uint32_t launchesKind[2] = {0, 0};  // kernels in each captured graph
  uint64_t iteration = 0;  // iterations run so far (selects the kind of the next one)
  uint32_t plainEvery = 0;
  std::vector<cudaEvent_t> evStart, evStop;  // per chunk, profileKernels only
  const bvhgb_mlp *scorer = nullptr;         // learned selection when set
  LrScratch lr;                              // feature scratch, allocated with the first scorer
};

namespace {

bool learned_iteration(const bvhgb_bn13_workspace *ws, uint64_t it) {
  if (!ws->scorer) return false;
  return ws->plainEvery == 0 || it % ws->plainEvery != ws->plainEvery - 1;
}

// Entries of the selection the chunks read: position chunk * chunkSize + k (or k * numChunks +
// chunk) for k < chunkSize, so the first numChunks * chunkSize (at most every inner node).
uint32_t selection_count(const bvhgb_bn13_workspace *ws) {
  return (uint32_t)std::min<uint64_t>((uint64_t)ws->numChunks * ws->chunkSize, ws->numInner);
}

void drop_graphs(bvhgb_bn13_workspace *ws) {
  for (auto &g : ws->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  ws->graphNodes = nullptr;
}

int select_kind(bvhgb_bn13_workspace *ws, const bvhgb_node *nodes, bool learned, cudaStream_t s) {
  if (ws->numInner == 0) return BVHGB_OK;
  if (learned) {
    const uint32_t numLeaves = ws->numNodes - ws->numInner;
    int st = lr_features(ws->lr, nodes, ws->numNodes, ws->root, ws->inner, ws->numInner, lr_inv_log2_leaves(numLeaves), s);
    if (!st) st = lr_score_keys(ws->scorer, ws->lr, nodes, ws->root, ws->inner, ws->numInner, ws->keys, ws->vals, s);
    if (st) return st;
  } else {
    const uint32_t grid = min(ceil_div(ws->numInner, 256), (uint32_t)sm_count() * 8);
    cost_kernel<<<grid, 256, 0, s>>>(nodes, ws->inner, ws->numInner, ws->keys, ws->vals);
    BVHGB_LAUNCH_CHECK("bn13 cost");
  }
  // bn13_selectNodes sorts every inner node (Bittner13CUDA.cu:659-726); the chunks read only the
  // first selection_count entries, which a stable selection gives in the same order.
  return select_smallest(ws->sortTemp, ws->keys, ws->vals, ws->numInner, selection_count(ws), ws->todo, s);
}

int select_nodes(bvhgb_bn13_workspace *ws, const bvhgb_node *nodes, cudaStream_t s) {
  return select_kind(ws, nodes, learned_iteration(ws, ws->iteration), s);
}

// Inside a stream capture the record must become an event node of the graph (external record);
// outside it is an ordinary record.
cudaError_t record_event(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return e;
  return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                             : cudaEventRecord(ev, s);
}

int run_chunk(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, uint32_t c, cudaStream_t s) {
  const uint32_t cs = ws->chunkSize;
  if (cs == 0) return BVHGB_OK;
  const bool prof = !ws->evStart.empty();
  if (prof) BVHGB_CUDA_TRY(record_event(ws->evStart[c], s));
  if (ws->cfg.searchMode == BVHGB_SEARCH_BATCHED) {
    patch_warp_kernel<<<ceil_div(cs, kWarpItemsPerBlock), kWarpItemsPerBlock * 32, 0, s>>>(
        nodes, ws->root, ws->todo, ws->numInner, c, ws->numChunks, cs, ws->cfg.offsetAccess, ws->patches, ws->valid,
        ws->toFix, ws->owner, ws->stats, ws->numNodes, ws->err);
  } else {
    // One warp per block: these searches are latency-bound, so spreading them over more SMs beats
    // packing them. Every chunk kernel sizes its own blocks: CUDABlockSize is accepted and kept in
    // the configuration, and results never depend on it.
    if (ws->cfg.searchMode == BVHGB_SEARCH_ALT)
      patch_kernel<BVHGB_SEARCH_ALT><<<ceil_div(cs, kSearchThreads), kSearchThreads, 0, s>>>(
          nodes, ws->root, ws->todo, ws->numInner, c, ws->numChunks, cs, ws->cfg.offsetAccess, ws->patches,
          ws->valid, ws->toFix, ws->owner, ws->heaps, ws->cfg.heapCapacity, ws->stats, ws->numNodes, ws->err);
    else
      patch_kernel<BVHGB_SEARCH_HEAP><<<ceil_div(cs, kSearchThreads), kSearchThreads, 0, s>>>(
          nodes, ws->root, ws->todo, ws->numInner, c, ws->numChunks, cs, ws->cfg.offsetAccess, ws->patches,
          ws->valid, ws->toFix, ws->owner, ws->heaps, ws->cfg.heapCapacity, ws->stats, ws->numNodes, ws->err);
  }
  BVHGB_LAUNCH_CHECK("bn13 patch");
  if (prof) BVHGB_CUDA_TRY(record_event(ws->evStop[c], s));
  // apply + count in one launch (the count reads the winners' new parents from their patches),
  // then the release of the claims and the refit
  const uint32_t pc = ws->countClimbsPerWarp, pr = ws->refitClimbsPerWarp;
  apply_count_kernel<<<ceil_div(3ull * cs, (uint64_t)pc * kTailWarpsPerBlock), kTailWarpsPerBlock * 32, 0, s>>>(
      nodes, ws->root, ws->patches, ws->valid, ws->toFix, ws->owner, ws->counter, cs, pc, ws->numNodes, ws->stats,
      ws->err);
  BVHGB_LAUNCH_CHECK("bn13 apply+count");
  release_refit_kernel<<<ceil_div(3ull * cs, (uint64_t)pr * kTailWarpsPerBlock), kTailWarpsPerBlock * 32, 0, s>>>(
      nodes, ws->root, ws->patches, ws->toFix, ws->owner, ws->counter, ws->mail, cs, pr, ws->numNodes, ws->err);
  BVHGB_LAUNCH_CHECK("bn13 refit");
  return BVHGB_OK;
}

int step_kind(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, bool learned, cudaStream_t s) {
  int st = select_kind(ws, nodes, learned, s);
  if (st) return st;
  for (uint32_t c = 0; c < ws->numChunks; ++c)
    if ((st = run_chunk(ws, nodes, c, s))) return st;
  return BVHGB_OK;
}

int do_step(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, cudaStream_t s) {
  const int st = step_kind(ws, nodes, learned_iteration(ws, ws->iteration), s);
  if (st == BVHGB_OK) ++ws->iteration;
  return st;
}

// One iteration of the given kind captured on a private stream.
int capture_step(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, bool learned, cudaGraphExec_t *out) {
  int pst = sort_prepare();
  if (pst) return pst;
  cudaStream_t cap = nullptr;
  BVHGB_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  int st = BVHGB_OK;
  const uint64_t before = bvhgb_launch_count();
  if (e == cudaSuccess) {
    st = step_kind(ws, nodes, learned, cap);
    e = cudaStreamEndCapture(cap, &g);
  }
  ws->launchesPerIteration = ws->launchesKind[learned ? 1 : 0] = (uint32_t)(bvhgb_launch_count() - before);
  uncount_launches(ws->launchesPerIteration);
  if (e == cudaSuccess && st == BVHGB_OK) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cap);
  if (st) return st;
  if (e != cudaSuccess) {
    set_last_error("bvhgb_bn13_run capture", e);
    *out = nullptr;
    return BVHGB_CUDA_ERROR;
  }
  return BVHGB_OK;
}

}  // namespace

extern "C" BVHGB_API int bvhgb_bn13_create(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root,
                                           const bvhgb_bn13_config *cfg, bvhgb_bn13_workspace **out,
                                           bvhgb_stream stream) {
  if (!out || !nodes || numNodes == 0 || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  *out = nullptr;
  auto *ws = new bvhgb_bn13_workspace();
  ws->cfg = cfg ? *cfg : bvhgb_bn13_config{32u, 128u, 1.0f, 0u, 4096u, 0u, BVHGB_SEARCH_BATCHED};
  if (ws->cfg.searchMode > BVHGB_SEARCH_ALT) {
    delete ws;
    return BVHGB_INVALID_ARGUMENT;
  }
  if (ws->cfg.numChunks == 0) ws->cfg.numChunks = 1;
  if (ws->cfg.heapCapacity < 4) ws->cfg.heapCapacity = 4096;
  if (ws->cfg.blockSize == 0 || ws->cfg.blockSize > 1024) ws->cfg.blockSize = 128;
  float bp = ws->cfg.batchPercent;
  if (bp <= 0.01f) bp = 0.01f;  // Bittner13GPU.cpp:59-60
  if (bp >= 75.0f) bp = 75.0f;
  ws->cfg.batchPercent = bp;
  int pst = sort_prepare();
  if (pst) {
    delete ws;
    return pst;
  }
  ws->numNodes = numNodes;
  ws->root = root;
  ws->numChunks = ws->cfg.numChunks;
  const uint32_t lNum = (uint32_t)((bp / 100.0f) * (float)numNodes);  // Bittner13GPU.cpp:79-80
  ws->chunkSize = ws->cfg.chunkSize ? ws->cfg.chunkSize : lNum / ws->numChunks;
  cudaStream_t s = as_stream(stream);

  // initData (Bittner13CUDA.cu:939-987): inner nodes in ascending index order.
  std::vector<uint32_t> hflags(numNodes);
  uint32_t *dflag = nullptr;
  cudaError_t e = dev_malloc(&dflag, 4ull * numNodes);
  if (e == cudaSuccess) {
    init_inner_kernel<<<min(ceil_div(numNodes, 256), 4096u), 256, 0, s>>>(nodes, numNodes, dflag);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hflags.data(), dflag, 4ull * numNodes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dflag);
  std::vector<uint32_t> inner;
  inner.reserve(numNodes / 2 + 1);
  for (uint32_t i = 0; i < numNodes; ++i)
    if (hflags[i]) inner.push_back(i);
  ws->numInner = (uint32_t)inner.size();
  const size_t ni = inner.size() ? inner.size() : 1;
  const size_t cs = ws->chunkSize ? ws->chunkSize : 1;
  const size_t sortBytes = select_temp_bytes(ws->numInner, selection_count(ws));
  if (e == cudaSuccess) e = dev_malloc(&ws->inner, 4 * ni);
  if (e == cudaSuccess) e = dev_malloc(&ws->keys, 4 * ni);
  if (e == cudaSuccess) e = dev_malloc(&ws->vals, 4 * ni);
  if (e == cudaSuccess) e = dev_malloc(&ws->todo, 4 * ni);
  if (e == cudaSuccess) e = dev_malloc(&ws->sortTemp, sortBytes ? sortBytes : 256);
  if (e == cudaSuccess) e = dev_malloc(&ws->patches, sizeof(PatchOut) * cs);
  if (e == cudaSuccess) e = dev_malloc(&ws->valid, 4 * cs);
  if (e == cudaSuccess) e = dev_malloc(&ws->toFix, 12 * cs);
  if (e == cudaSuccess) e = dev_malloc(&ws->owner, 4ull * numNodes);
  if (e == cudaSuccess) e = dev_malloc(&ws->counter, 4ull * numNodes);
  if (e == cudaSuccess) e = dev_malloc(&ws->mail, 24ull * numNodes);
  if (e == cudaSuccess) e = dev_malloc(&ws->err, 4);
  // Only the heap search keeps a queue in global memory (entries beyond the shared-memory top).
  const size_t heapItems = ws->cfg.searchMode == BVHGB_SEARCH_HEAP ? cs * ws->cfg.heapCapacity : 1;
  if (e == cudaSuccess) e = dev_malloc(&ws->heaps, sizeof(HeapItem) * heapItems);
  if (e == cudaSuccess) e = dev_malloc(&ws->stats, sizeof(unsigned long long) * S_COUNT);
  if (e == cudaSuccess && inner.size())
    e = cudaMemcpyAsync(ws->inner, inner.data(), 4 * inner.size(), cudaMemcpyHostToDevice, s);
  ws->countClimbsPerWarp = climbs_per_warp((const void *)apply_count_kernel, 3ull * cs);
  ws->refitClimbsPerWarp = climbs_per_warp((const void *)release_refit_kernel, 3ull * cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->counter, 0, 4ull * numNodes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->mail, 0xFF, 24ull * numNodes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->owner, 0xFF, 4ull * numNodes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->err, 0, 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->stats, 0, sizeof(unsigned long long) * S_COUNT, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && ws->cfg.profileKernels) {
    ws->evStart.assign(ws->numChunks, nullptr);
    ws->evStop.assign(ws->numChunks, nullptr);
    for (uint32_t c = 0; c < ws->numChunks && e == cudaSuccess; ++c) {
      e = cudaEventCreate(&ws->evStart[c]);
      if (e == cudaSuccess) e = cudaEventCreate(&ws->evStop[c]);
    }
  }
  if (e != cudaSuccess) {
    set_last_error("bvhgb_bn13_create", e);
    bvhgb_bn13_destroy(ws);
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  *out = ws;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_destroy(bvhgb_bn13_workspace *ws) {
  if (!ws) return BVHGB_OK;
  drop_graphs(ws);
  for (cudaEvent_t ev : ws->evStart)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : ws->evStop)
    if (ev) cudaEventDestroy(ev);
  cudaFree(ws->inner);
  cudaFree(ws->keys);
  cudaFree(ws->vals);
  cudaFree(ws->todo);
  cudaFree(ws->sortTemp);
  cudaFree(ws->patches);
  cudaFree(ws->valid);
  cudaFree(ws->toFix);
  cudaFree(ws->owner);
  cudaFree(ws->counter);
  cudaFree(ws->mail);
  cudaFree(ws->err);
  cudaFree(ws->heaps);
  cudaFree(ws->stats);
  lr_scratch_free(ws->lr);
  delete ws;
  return BVHGB_OK;
}

extern "C" BVHGB_API uint32_t bvhgb_bn13_launches_per_iteration(const bvhgb_bn13_workspace *ws) {
  return ws ? ws->launchesPerIteration : 0;
}

extern "C" BVHGB_API int bvhgb_bn13_search_time(bvhgb_bn13_workspace *ws, float *ms, uint32_t *launches) {
  if (!ws || !ms) return BVHGB_INVALID_ARGUMENT;
  *ms = 0.0f;
  if (launches) *launches = 0;
  if (ws->evStart.empty()) return BVHGB_INVALID_ARGUMENT;
  float total = 0.0f;
  for (uint32_t c = 0; c < ws->numChunks; ++c) {
    BVHGB_CUDA_TRY(cudaEventSynchronize(ws->evStop[c]));
    float t = 0.0f;
    BVHGB_CUDA_TRY(cudaEventElapsedTime(&t, ws->evStart[c], ws->evStop[c]));
    total += t;
  }
  *ms = total;
  if (launches) *launches = ws->numChunks;
  return BVHGB_OK;
}

extern "C" BVHGB_API uint32_t bvhgb_bn13_batch_size(const bvhgb_bn13_workspace *ws) {
  return ws ? ws->chunkSize * ws->numChunks : 0;
}

extern "C" BVHGB_API int bvhgb_bn13_select_nodes(bvhgb_bn13_workspace *ws, const bvhgb_node *nodes, bvhgb_stream stream) {
  if (!ws || !nodes) return BVHGB_INVALID_ARGUMENT;
  return select_nodes(ws, nodes, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_bn13_chunk(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, uint32_t chunk, bvhgb_stream stream) {
  if (!ws || !nodes || chunk >= ws->numChunks) return BVHGB_INVALID_ARGUMENT;
  return run_chunk(ws, nodes, chunk, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_bn13_step(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, bvhgb_stream stream) {
  if (!ws || !nodes) return BVHGB_INVALID_ARGUMENT;
  return do_step(ws, nodes, as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_bn13_run(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, uint32_t iterations,
                                        bvhgb_stream stream) {
  if (!ws || !nodes) return BVHGB_INVALID_ARGUMENT;
  if (iterations == 0) return BVHGB_OK;
  cudaStream_t s = as_stream(stream);
  // Each kind of iteration is captured once on a private stream, then replayed on the caller's.
  if (ws->graphNodes != nodes) drop_graphs(ws);
  ws->graphNodes = nodes;
  for (uint32_t i = 0; i < iterations; ++i) {
    const int kind = learned_iteration(ws, ws->iteration) ? 1 : 0;
    if (!ws->graph[kind]) {
      const int st = capture_step(ws, nodes, kind == 1, &ws->graph[kind]);
      if (st) return st;
    }
    BVHGB_CUDA_TRY(cudaGraphLaunch(ws->graph[kind], s));
    count_launch(ws->launchesKind[kind]);
    ++ws->iteration;
  }
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_refit(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, bvhgb_stream stream) {
  if (!ws || !nodes) return BVHGB_INVALID_ARGUMENT;
  const uint32_t n = ws->numNodes;
  refit_full_kernel<<<ceil_div(n, 256u), 256, 0, as_stream(stream)>>>(nodes, ws->root, n, ws->counter, ws->err);
  BVHGB_LAUNCH_CHECK("bn13 full refit");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_get_stats(bvhgb_bn13_workspace *ws, bvhgb_bn13_stats *stats, bvhgb_stream stream) {
  if (!ws || !stats) return BVHGB_INVALID_ARGUMENT;
  unsigned long long h[S_COUNT];
  uint32_t err = 0;
  cudaStream_t s = as_stream(stream);
  BVHGB_CUDA_TRY(cudaMemcpyAsync(h, ws->stats, sizeof(h), cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaMemcpyAsync(&err, ws->err, 4, cudaMemcpyDeviceToHost, s));
  BVHGB_CUDA_TRY(cudaStreamSynchronize(s));
  stats->items = h[S_ITEMS];
  stats->applied = h[S_APPLIED];
  stats->skippedConflict = h[S_CONFLICT];
  stats->skippedInvalid = h[S_INVALID];
  stats->heapOverflow = h[S_OVERFLOW];
  stats->nodesVisited = h[S_VISITS];
  return err ? BVHGB_BVH_ERROR : BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_gains(bvhgb_bn13_workspace *ws, const bvhgb_node *nodes, const uint32_t *cand,
                                         uint32_t n, float *gain, float *target, bvhgb_stream stream) {
  if (!ws || !nodes || (n && (!cand || !gain))) return BVHGB_INVALID_ARGUMENT;
  if (n == 0) return BVHGB_OK;
  gain_warp_kernel<<<ceil_div(n, kWarpItemsPerBlock), kWarpItemsPerBlock * 32, 0, as_stream(stream)>>>(
      nodes, ws->root, cand, n, ws->numNodes, (float)(ws->numNodes - ws->numInner) / kTargetEps, gain, target, ws->err);
  BVHGB_LAUNCH_CHECK("bn13 gains");
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_read_inner(const bvhgb_bn13_workspace *ws, uint32_t *out, uint32_t capacity,
                                              uint32_t *numInner, bvhgb_stream stream) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  if (numInner) *numInner = ws->numInner;
  if (!out) return BVHGB_OK;
  if (capacity < ws->numInner) return BVHGB_TOO_LARGE;
  if (ws->numInner)
    BVHGB_CUDA_TRY(cudaMemcpyAsync(out, ws->inner, 4ull * ws->numInner, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_set_scorer(bvhgb_bn13_workspace *ws, const bvhgb_mlp *scorer,
                                               uint32_t plainEvery) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  if (scorer && ws->lr.numNodes < ws->numNodes) {
    const int st = lr_scratch_alloc(ws->lr, ws->numNodes);
    if (st) return st;
  }
  if (ws->scorer != scorer) drop_graphs(ws);
  ws->scorer = scorer;
  ws->plainEvery = plainEvery;
  return BVHGB_OK;
}

extern "C" BVHGB_API uint64_t bvhgb_bn13_iteration(const bvhgb_bn13_workspace *ws) { return ws ? ws->iteration : 0; }

extern "C" BVHGB_API int bvhgb_bn13_set_tail_packing(bvhgb_bn13_workspace *ws, uint32_t climbsPerWarp) {
  if (!ws || climbsPerWarp > 32) return BVHGB_INVALID_ARGUMENT;
  const uint64_t paths = 3ull * ws->chunkSize;
  ws->countClimbsPerWarp = climbsPerWarp ? climbsPerWarp : climbs_per_warp((const void *)apply_count_kernel, paths);
  ws->refitClimbsPerWarp = climbsPerWarp ? climbsPerWarp : climbs_per_warp((const void *)release_refit_kernel, paths);
  drop_graphs(ws);
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_set_iteration(bvhgb_bn13_workspace *ws, uint64_t iteration) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  ws->iteration = iteration;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_read_selection(const bvhgb_bn13_workspace *ws, uint32_t *out, uint32_t capacity,
                                                  bvhgb_stream stream) {
  if (!ws || !out) return BVHGB_INVALID_ARGUMENT;
  const uint32_t n = selection_count(ws);
  if (capacity < n) return BVHGB_TOO_LARGE;
  if (n) BVHGB_CUDA_TRY(cudaMemcpyAsync(out, ws->todo, 4ull * n, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_set_selection(bvhgb_bn13_workspace *ws, const uint32_t *order, uint32_t n,
                                                 bvhgb_stream stream) {
  if (!ws || (n && !order) || n != ws->numInner) return BVHGB_INVALID_ARGUMENT;
  if (n) BVHGB_CUDA_TRY(cudaMemcpyAsync(ws->todo, order, 4ull * n, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return BVHGB_OK;
}
