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
//   refit  : the last arrival at a node recomputes its box from its children (kFixTree3_2) with
//            acq_rel counters, so no box is read before it is final.
// bvhgb_bn13_run captures one iteration into a CUDA graph and replays it. With a learned scorer
// set, iteration i selects by the scorer unless plainEvery > 0 and i % plainEvery == plainEvery - 1,
// in which case it selects by the inefficiency (one graph per kind of iteration).
#include <vector>

#include "common.cuh"
#include "learned.cuh"
#include "sort.cuh"

namespace bvhgb {
namespace {

constexpr int NSLOT = 10;
enum : uint32_t {
  P_GRAND_PARENT = 0, P_1ST_ROOT = 1, P_1ST_BEST = 2, P_NODE = 3, P_1ST_INSERT = 4,
  P_2ND_ROOT = 5, P_2ND_BEST = 6, P_2ND_INSERT = 7, P_SIBLING = 8, P_PARENT = 9
};
enum StatIdx { S_ITEMS = 0, S_APPLIED = 1, S_CONFLICT = 2, S_INVALID = 3, S_OVERFLOW = 4, S_VISITS = 5, S_COUNT = 6 };

struct SearchCounters {
  uint32_t overflow;  // queue pushes dropped at capacity
  uint32_t visits;    // nodes evaluated by the branch and bound
};

struct NodeP {
  uint32_t parent, left, right;
  uint16_t isLeafFlag, isLeft;
};

struct HeapItem {
  uint32_t node;
  float cost;
};

struct PatchOut {  // what the apply kernel needs
  NodeP nd[NSLOT];
  uint32_t idx[NSLOT];
};

// Read-only view of the tree during the patch kernel (nothing writes the tree in that launch).
__device__ __forceinline__ NodeP tree_node(const bvhgb_node *t, uint32_t x) {
  const float4 *p = reinterpret_cast<const float4 *>(t + x);
  const float4 b = __ldg(p + 1), c = __ldg(p + 2);
  NodeP r;
  r.parent = __float_as_uint(b.z);
  r.left = __float_as_uint(b.w);
  r.right = __float_as_uint(c.x);
  const uint32_t fl = __float_as_uint(c.y);
  r.isLeafFlag = (uint16_t)(fl & 0xFFFFu);
  r.isLeft = (uint16_t)(fl >> 16);
  return r;
}
__device__ __forceinline__ Box tree_box(const bvhgb_node *t, uint32_t x) {
  const float4 *p = reinterpret_cast<const float4 *>(t + x);
  const float4 a = __ldg(p), b = __ldg(p + 1);
  Box r;
  r.mn[0] = a.x; r.mn[1] = a.y; r.mn[2] = a.z;
  r.mx[0] = a.w; r.mx[1] = b.x; r.mx[2] = b.y;
  return r;
}
__device__ __forceinline__ float tree_sa(const bvhgb_node *t, uint32_t x) { return __ldg(&t[x].surfaceArea); }
__device__ __forceinline__ bool tree_leaf(const bvhgb_node *t, uint32_t x) { return __ldg(&t[x].isLeafFlag) != 0; }

// BVHPatch (BVHPatch.hpp:87-335), ENABLE_AABB_PATH = 0.
struct Patch {
  NodeP nd[NSLOT];
  uint32_t idx[NSLOT];
  uint32_t apath[4];
  Box abox[4];
  const bvhgb_node *t;
  uint32_t root;
  uint32_t numNodes;
  mutable bool bad;  // an index outside the node array was met (corrupted input); item is dropped

  __device__ uint32_t chk(uint32_t x) const {
    if (x < numNodes) return x;
    bad = true;
    return root;
  }

  __device__ void clear() {
#pragma unroll
    for (int i = 0; i < NSLOT; ++i) idx[i] = kNone;
#pragma unroll
    for (int i = 0; i < 4; ++i) apath[i] = kNone;
  }
  __device__ uint32_t index_subset(uint32_t x) const {
    if (idx[0] == x) return 0;
    if (idx[1] == kNone) return kNone;
    if (idx[1] == x) return 1;
    if (idx[2] == x) return 2;
    if (idx[3] == x) return 3;
    return kNone;
  }
  __device__ uint32_t index(uint32_t x) const {
    for (uint32_t i = 0; i < NSLOT; ++i)
      if (idx[i] == x) return i;
    return kNone;
  }
  __device__ NodeP get(uint32_t x) const {
    uint32_t i = index(x);
    return i == kNone ? tree_node(t, chk(x)) : nd[i];
  }
  __device__ NodeP get_subset(uint32_t x) const {
    uint32_t i = index_subset(x);
    return i == kNone ? tree_node(t, chk(x)) : nd[i];
  }
  __device__ uint32_t patch_node(uint32_t x, uint32_t slot) {
    idx[slot] = x;
    nd[slot] = tree_node(t, chk(x));
    return slot;
  }
  __device__ uint32_t move(uint32_t from, uint32_t to) {
    idx[to] = idx[from];
    idx[from] = kNone;
    nd[to] = nd[from];
    return to;
  }
  __device__ uint32_t sibling(const NodeP &n) const {
    NodeP p = get(n.parent);
    return n.isLeft == 0 ? p.left : p.right;
  }
  __device__ Box get_aabb(uint32_t x) const {
    for (int i = 0; i < 4; ++i)
      if (apath[i] == x) return abox[i];
    return tree_box(t, chk(x));
  }
  // patchAABBFrom (BVHPatch.hpp:293-316)
  __device__ void patch_aabb_from(uint32_t x, uint32_t pidx) {
    uint32_t ni = x;
    NodeP n = get_subset(ni);
    Box b = get_aabb(n.left);
    bool lastLeft = true;
    for (uint32_t i = 0; i < 2; ++i) {
      uint32_t sib = lastLeft ? n.right : n.left;
      Box sb = get_aabb(sib);
      merge_into(b, sb);
      abox[pidx * 2 + i] = b;
      apath[pidx * 2 + i] = ni;
      lastLeft = n.isLeft != 0;
      if (ni == root) break;
      ni = n.parent;
      n = get_subset(ni);
    }
  }
};

// Heap with the hole-based sift of the standard library heap algorithms (CUDAHeap.hpp:33-112);
// "less(a, b)" is a.cost > b.cost, so h[0] holds the smallest induced cost.
__device__ __forceinline__ bool hless(const HeapItem &a, const HeapItem &b) { return a.cost > b.cost; }

// Two-level storage: the first kHeapShared entries of each search live in shared memory,
// interleaved across the warp's lanes (entry i of lane l at i * 32 + l, conflict-free when lanes
// touch the same depth); deeper entries spill to the item's global region. The index space and
// the capacity are unchanged, so the pop order is exactly that of a flat array.
constexpr int kSearchThreads = 32;
constexpr int kHeapShared = 128;

struct Heap {
  HeapItem *sm;  // this lane's entry 0 in shared memory (stride kSearchThreads)
  HeapItem *gm;  // this item's global region (cap entries)
  __device__ __forceinline__ HeapItem &at(long i) const { return i < kHeapShared ? sm[i * kSearchThreads] : gm[i]; }
};

__device__ __forceinline__ void sift_up(const Heap &h, long hole, long top, HeapItem v) {
  long parent = (hole - 1) / 2;
  while (hole > top && hless(h.at(parent), v)) {
    h.at(hole) = h.at(parent);
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h.at(hole) = v;
}
__device__ __forceinline__ void heap_push(const Heap &h, long lenAfter) { sift_up(h, lenAfter - 1, 0, h.at(lenAfter - 1)); }
__device__ __forceinline__ void heap_pop(const Heap &h, long len) {
  if (len <= 1) return;
  const long last = len - 1;
  const HeapItem v = h.at(last);
  h.at(last) = h.at(0);
  const long n = last;
  long hole = 0, second = 0;
  while (second < (n - 1) / 2) {
    second = 2 * (second + 1);
    if (hless(h.at(second), h.at(second - 1))) second--;
    h.at(hole) = h.at(second);
    hole = second;
  }
  if ((n & 1) == 0 && second == (n - 2) / 2) {
    second = 2 * (second + 1);
    h.at(hole) = h.at(second - 1);
    hole = second - 1;
  }
  sift_up(h, hole, 0, v);
}

// Starts fetching a node's 48-byte record into L2 while the search keeps working.
__device__ __forceinline__ void prefetch_node(const bvhgb_node *t, uint32_t x) {
  const char *p = reinterpret_cast<const char *>(t + x);
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p + 32));
}

// findNode1 (Bittner13CUDA.cu:141-191).
__device__ uint32_t find_node(const Patch &p, uint32_t n, const Heap &pq, uint32_t cap, SearchCounters &ctr) {
  float best_cost = __int_as_float(0x7f800000);
  uint32_t best = 0;
  const Box nbox = tree_box(p.t, p.chk(n));
  const float sarea = tree_sa(p.t, p.chk(n));
  long size = 1;
  pq.at(0).node = p.root;
  pq.at(0).cost = 0.0f;
  // A tree pops each node at most once; the bound only matters for corrupted input.
  for (uint32_t it = 0; size > 0; ++it) {
    if (it > p.numNodes) {
      p.bad = true;
      break;
    }
    const HeapItem cur = pq.at(0);
    if (fadd(cur.cost, sarea) >= best_cost) break;
    heap_pop(pq, size);
    size--;
    ctr.visits++;
    const NodeP cn = p.get_subset(cur.node);
    Box b = p.get_aabb(cur.node);
    float induced = fmul(-1.0f, surface_area(b));
    merge_into(b, nbox);
    const float direct = surface_area(b);
    const float total = fadd(cur.cost, direct);
    if (total < best_cost) {
      best_cost = total;
      best = cur.node;
    }
    induced = fadd(induced, total);
    if (fadd(induced, sarea) < best_cost && !cn.isLeafFlag) {
      if ((uint32_t)size + 2 <= cap) {
        if (cn.left < p.numNodes) prefetch_node(p.t, cn.left);
        if (cn.right < p.numNodes) prefetch_node(p.t, cn.right);
        pq.at(size).node = cn.left;
        pq.at(size).cost = induced;
        pq.at(size + 1).node = cn.right;
        pq.at(size + 1).cost = induced;
        heap_push(pq, size + 1);
        heap_push(pq, size + 2);
        size += 2;
      } else {
        ctr.overflow++;
      }
    }
  }
  return best;
}

// removeNode (Bittner13CUDA.cu:267-305).
__device__ bool remove_node(Patch &p, uint32_t x, uint32_t ins[2], uint32_t un[2], uint32_t &g_out) {
  if (tree_leaf(p.t, p.chk(x)) || x == p.root) return false;
  const uint32_t sn = p.patch_node(x, P_NODE);
  const uint32_t s = p.sibling(p.nd[sn]);
  const uint32_t pi = p.nd[sn].parent;
  if (pi == p.root) return false;
  const uint32_t ss = p.patch_node(s, P_SIBLING);
  const uint32_t sp = p.patch_node(pi, P_PARENT);
  const uint32_t gi = p.nd[sp].parent;
  const uint32_t sg = p.patch_node(gi, P_GRAND_PARENT);
  if (p.nd[sp].isLeft) {
    p.nd[sg].left = s;
    p.nd[ss].isLeft = 1;
  } else {
    p.nd[sg].right = s;
    p.nd[ss].isLeft = 0;
  }
  p.nd[ss].parent = gi;
  p.patch_aabb_from(gi, 0);
  const uint32_t l = p.nd[sn].left, r = p.nd[sn].right;
  if (tree_sa(p.t, p.chk(l)) > tree_sa(p.t, p.chk(r))) { ins[0] = l; ins[1] = r; }
  else { ins[0] = r; ins[1] = l; }
  un[0] = x;
  un[1] = pi;
  g_out = gi;
  return true;
}

// ---- batched best-first search: one warp per item -------------------------------------------
//
// The frontier (up to 128 entries) lives in registers, 4 slots per lane, entry e = slot * 32 + lane,
// kept sorted by (cost, node). Each round the warp evaluates slot 0 (the 32 lowest-bound entries)
// in parallel, reduces the best total, sorts the up-to-64 children with a bitonic network and
// merges them into slots 1..3 with a bitonic merge; entries past 128 are dropped and counted.
// oracle/bittner.c (gpu_find_node_batched) restates the same rounds.
constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr int kFrontier = 4;  // slots per lane (128 entries)

__device__ __forceinline__ bool fe_gt(float ca, uint32_t na, float cb, uint32_t nb) {
  return ca > cb || (ca == cb && na > nb);
}

// One compare-exchange stage of a bitonic network over S slots x 32 lanes.
template <int S>
__device__ __forceinline__ void bitonic_stage(float (&c)[S], uint32_t (&n)[S], int j, int k, bool descending,
                                              uint32_t lane) {
  if (j >= 32) {
    const int d = j >> 5;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      if (s & d) continue;
      const int t = s + d;
      const uint32_t e = (uint32_t)s * 32u + lane;
      const bool asc = ((e & (uint32_t)k) == 0) != descending;
      const bool swap = asc ? fe_gt(c[s], n[s], c[t], n[t]) : fe_gt(c[t], n[t], c[s], n[s]);
      if (swap) {
        const float tc = c[s]; c[s] = c[t]; c[t] = tc;
        const uint32_t tn = n[s]; n[s] = n[t]; n[t] = tn;
      }
    }
  } else {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const float oc = __shfl_xor_sync(kFull, c[s], j);
      const uint32_t on = __shfl_xor_sync(kFull, n[s], j);
      const uint32_t e = (uint32_t)s * 32u + lane;
      const bool asc = ((e & (uint32_t)k) == 0) != descending;
      const bool keepMin = ((lane & (uint32_t)j) == 0) == asc;
      if (keepMin ? fe_gt(c[s], n[s], oc, on) : fe_gt(oc, on, c[s], n[s])) {
        c[s] = oc;
        n[s] = on;
      }
    }
  }
}

template <int S>
__device__ __forceinline__ void bitonic_sort(float (&c)[S], uint32_t (&n)[S], bool descending, uint32_t lane) {
#pragma unroll
  for (int k = 2; k <= S * 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) bitonic_stage<S>(c, n, j, k, descending, lane);
  }
}

template <int S>
__device__ __forceinline__ void bitonic_merge(float (&c)[S], uint32_t (&n)[S], uint32_t lane) {
#pragma unroll
  for (int j = S * 16; j > 0; j >>= 1) bitonic_stage<S>(c, n, j, S * 32, false, lane);
}

// findNode1's cost model in batched rounds (every lane of the warp calls it with the same patch).
__device__ uint32_t find_node_batched(const Patch &p, uint32_t n, SearchCounters &ctr) {
  const uint32_t lane = threadIdx.x & 31u;
  const float kInf = __int_as_float(0x7f800000);
  float best_cost = kInf;
  uint32_t best = 0;
  const Box nbox = tree_box(p.t, p.chk(n));
  const float sarea = tree_sa(p.t, p.chk(n));
  float fc[kFrontier];
  uint32_t fn[kFrontier];
#pragma unroll
  for (int s = 0; s < kFrontier; ++s) {
    fc[s] = kInf;
    fn[s] = kNone;
  }
  if (lane == 0) {
    fc[0] = 0.0f;
    fn[0] = p.root;
  }
  uint32_t fsize = 1;  // finite frontier entries (warp-uniform)
  for (uint32_t round = 0;; ++round) {
    if (round > p.numNodes) {  // bounded: every round evaluates at least one node
      p.bad = true;
      break;
    }
    const bool cand = fc[0] != kInf && fadd(fc[0], sarea) < best_cost;
    const uint32_t vmask = __ballot_sync(kFull, cand);
    if (vmask == 0) break;
    ctr.visits += __popc(vmask);
    NodeP cn;
    float total = kInf, induced = kInf;
    if (cand) {
      cn = p.get_subset(fn[0]);
      Box b = p.get_aabb(fn[0]);
      induced = fmul(-1.0f, surface_area(b));
      merge_into(b, nbox);
      total = fadd(fc[0], surface_area(b));
      induced = fadd(induced, total);
    }
    // Best of the round: smallest total, first in frontier order on ties.
    const uint32_t key = cand ? f2ord(total) : 0xFFFFFFFFu;
    const uint32_t kmin = __reduce_min_sync(kFull, key);
    const uint32_t first = __ffs(__ballot_sync(kFull, cand && key == kmin)) - 1;
    const float rbest = __shfl_sync(kFull, total, first);
    const uint32_t rnode = __shfl_sync(kFull, fn[0], first);
    if (rbest < best_cost) {
      best_cost = rbest;
      best = rnode;
    }
    const bool kids = cand && !cn.isLeafFlag && fadd(induced, sarea) < best_cost;
    if (kids) {
      if (cn.left < p.numNodes) prefetch_node(p.t, cn.left);
      if (cn.right < p.numNodes) prefetch_node(p.t, cn.right);
    }
    const uint32_t kmask = __ballot_sync(kFull, kids);
    const uint32_t m = 2u * __popc(kmask);                 // children this round
    const uint32_t rest = fsize - min(fsize, 32u);        // frontier entries left in slots 1..3
    if (m == 0) {
      // Nothing to insert: the remaining frontier is already in order, shift it down a slot.
#pragma unroll
      for (int s = 0; s + 1 < kFrontier; ++s) {
        fc[s] = fc[s + 1];
        fn[s] = fn[s + 1];
      }
      fc[kFrontier - 1] = kInf;
      fn[kFrontier - 1] = kNone;
      fsize = rest;
    } else if (m <= 32) {
      // Common case: gather the children into one slot (lane j takes child j), sort it
      // descending and merge it with the remaining frontier; at most 128 entries, no overflow.
      const uint32_t src = lane < m ? __fns(kmask, 0, (lane >> 1) + 1) : lane;
      const float sc = __shfl_sync(kFull, induced, src);
      const uint32_t sl = __shfl_sync(kFull, cn.left, src), sr = __shfl_sync(kFull, cn.right, src);
      float c1[1] = {lane < m ? sc : kInf};
      uint32_t n1[1] = {lane < m ? ((lane & 1) ? sr : sl) : kNone};
      bitonic_sort<1>(c1, n1, true, lane);
      if (rest <= 32) {
        float mc[2] = {fc[1], c1[0]};
        uint32_t mn[2] = {fn[1], n1[0]};
        bitonic_merge<2>(mc, mn, lane);
        fc[0] = mc[0]; fn[0] = mn[0];
        fc[1] = mc[1]; fn[1] = mn[1];
        fc[2] = fc[3] = kInf;
        fn[2] = fn[3] = kNone;
      } else {
        float mc[4] = {fc[1], fc[2], fc[3], c1[0]};
        uint32_t mn[4] = {fn[1], fn[2], fn[3], n1[0]};
        bitonic_merge<4>(mc, mn, lane);
#pragma unroll
        for (int s = 0; s < kFrontier; ++s) {
          fc[s] = mc[s];
          fn[s] = mn[s];
        }
      }
      fsize = rest + m;
    } else {
      // Wide round: sort all children (two slots) and merge into 256, keeping the lowest 128.
      float cc[2] = {kids ? induced : kInf, kids ? induced : kInf};
      uint32_t cnn[2] = {kids ? cn.left : kNone, kids ? cn.right : kNone};
      bitonic_sort<2>(cc, cnn, true, lane);
      float mc[8] = {fc[1], fc[2], fc[3], kInf, kInf, kInf, cc[0], cc[1]};
      uint32_t mn[8] = {fn[1], fn[2], fn[3], kNone, kNone, kNone, cnn[0], cnn[1]};
      bitonic_merge<8>(mc, mn, lane);
#pragma unroll
      for (int s = 0; s < kFrontier; ++s) {
        fc[s] = mc[s];
        fn[s] = mn[s];
      }
      const uint32_t total = rest + m;
      ctr.overflow += total > 128u ? total - 128u : 0u;
      fsize = min(total, 128u);
    }
  }
  p.bad = __any_sync(kFull, p.bad);
  return best;
}

// reinsert (Bittner13CUDA.cu:308-358).
template <bool BATCHED>
__device__ bool reinsert(Patch &p, uint32_t x, uint32_t unused, bool update, const Heap &pq, uint32_t cap,
                         SearchCounters &ctr) {
  const uint32_t best = BATCHED ? find_node_batched(p, x, ctr) : find_node(p, x, pq, cap, ctr);
  if (best == p.root) return false;
  const uint32_t bpi = p.index(best);
  uint32_t sb;
  if (bpi == kNone) sb = p.patch_node(best, update ? P_1ST_BEST : P_2ND_BEST);
  else if (bpi == P_GRAND_PARENT) sb = P_GRAND_PARENT;
  else sb = p.move(bpi, update ? P_1ST_BEST : P_2ND_BEST);
  const uint32_t sx = p.patch_node(x, update ? P_1ST_INSERT : P_2ND_INSERT);
  const uint32_t su = update ? P_NODE : P_PARENT;
  const uint32_t ri = p.nd[sb].parent;
  const uint32_t rpi = p.index(ri);
  const uint32_t sr = rpi == kNone ? p.patch_node(ri, update ? P_1ST_ROOT : P_2ND_ROOT)
                                   : p.move(rpi, update ? P_1ST_ROOT : P_2ND_ROOT);
  if (p.nd[sb].isLeft) {
    p.nd[sr].left = unused;
    p.nd[su].isLeft = 1;
  } else {
    p.nd[sr].right = unused;
    p.nd[su].isLeft = 0;
  }
  p.nd[su].parent = ri;
  p.nd[su].left = best;
  p.nd[su].right = x;
  p.nd[sb].parent = unused;
  p.nd[sb].isLeft = 1;
  p.nd[sx].parent = unused;
  p.nd[sx].isLeft = 0;
  if (update) p.patch_aabb_from(unused, 1);
  return true;
}

// ---- kernels ------------------------------------------------------------------------------

__global__ void cost_kernel(const bvhgb_node *__restrict__ t, const uint32_t *__restrict__ inner, uint32_t numInner,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < numInner; i += gridDim.x * blockDim.x) {
    const uint32_t x = __ldg(inner + i);
    const float4 *p = reinterpret_cast<const float4 *>(t + x);
    const float4 b = __ldg(p + 1), c = __ldg(p + 2);
    float cost = 0.0f;
    if ((__float_as_uint(c.y) & 0xFFFFu) == 0) {
      const float sa = c.w;
      const float l = __ldg(&t[__float_as_uint(b.w)].surfaceArea);
      const float r = __ldg(&t[__float_as_uint(c.x)].surfaceArea);
      const float num = fmul(fmul(fmul(sa, sa), sa), 2.0f);
      const float den = fmul(fadd(l, r), l < r ? l : r);
      cost = fdiv(num, den);
    }
    keys[i] = ~f2ord(cost);  // ascending key order = descending cost
    vals[i] = x;
  }
}

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
  Patch p;
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
  ok = ok && reinsert<false>(p, ins[0], un[0], true, pq, cap, ctr);
  ok = ok && reinsert<false>(p, ins[1], un[1], false, pq, cap, ctr);
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
    out[k].nd[s] = p.nd[s];
    out[k].idx[s] = ok ? p.idx[s] : kNone;
    if (ok && p.idx[s] != kNone) atomicMin(&owner[p.idx[s]], k);
  }
  if (!ok) atomicAdd(&stats[S_INVALID], 1ull);
  if (ctr.overflow) atomicAdd(&stats[S_OVERFLOW], (unsigned long long)ctr.overflow);
  atomicAdd(&stats[S_VISITS], (unsigned long long)ctr.visits);
  atomicAdd(&stats[S_ITEMS], 1ull);
}

// One warp per batch item: the patch logic runs redundantly on every lane (same data, no
// divergence) and the two searches are the warp-cooperative batched search; lane 0 publishes.
constexpr int kWarpItemsPerBlock = 4;

__global__ void __launch_bounds__(kWarpItemsPerBlock * 32) patch_warp_kernel(
    const bvhgb_node *__restrict__ t, uint32_t root, const uint32_t *__restrict__ todo, uint32_t numTodo,
    uint32_t chunk, uint32_t numChunks, uint32_t chunkSize, uint32_t offsetAccess, PatchOut *__restrict__ out,
    uint32_t *__restrict__ valid, uint32_t *__restrict__ toFix, uint32_t *__restrict__ owner,
    unsigned long long *__restrict__ stats, uint32_t numNodes, uint32_t *__restrict__ err) {
  const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31u;
  if (k >= chunkSize) return;  // whole warps leave together
  const uint32_t pos = offsetAccess ? k * numChunks + chunk : chunk * chunkSize + k;
  Patch p;
  p.t = t;
  p.root = root;
  p.numNodes = numNodes;
  p.bad = false;
  p.clear();
  SearchCounters ctr = {0u, 0u};
  uint32_t ins[2], un[2], g = kNone;
  bool ok = pos < numTodo;
  const uint32_t node = ok ? __ldg(todo + pos) : kNone;
  const Heap unused{nullptr, nullptr};
  ok = ok && remove_node(p, node, ins, un, g);
  ok = ok && reinsert<true>(p, ins[0], un[0], true, unused, 0, ctr);
  ok = ok && reinsert<true>(p, ins[1], un[1], false, unused, 0, ctr);
  if (p.bad) ok = false;
  if (lane != 0) return;
  if (p.bad) atomicOr(err, kErrBadIndex);
  valid[k] = ok ? 1u : 0u;
  toFix[3 * k + 0] = ok ? g : kNone;
  toFix[3 * k + 1] = ok ? un[0] : kNone;
  toFix[3 * k + 2] = ok ? un[1] : kNone;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    out[k].nd[s] = p.nd[s];
    out[k].idx[s] = ok ? p.idx[s] : kNone;
    if (ok && p.idx[s] != kNone) atomicMin(&owner[p.idx[s]], k);
  }
  if (!ok) atomicAdd(&stats[S_INVALID], 1ull);
  if (ctr.overflow) atomicAdd(&stats[S_OVERFLOW], (unsigned long long)ctr.overflow);
  atomicAdd(&stats[S_VISITS], (unsigned long long)ctr.visits);
  atomicAdd(&stats[S_ITEMS], 1ull);
}

__global__ void apply_kernel(bvhgb_node *t, const PatchOut *__restrict__ in, uint32_t *__restrict__ valid,
                             uint32_t *__restrict__ toFix, const uint32_t *__restrict__ owner, uint32_t chunkSize,
                             unsigned long long *__restrict__ stats) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= chunkSize || !valid[k]) return;
  bool win = true;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const uint32_t x = in[k].idx[s];
    if (x != kNone && owner[x] != k) win = false;
  }
  if (!win) {
    valid[k] = 0;
    toFix[3 * k + 0] = toFix[3 * k + 1] = toFix[3 * k + 2] = kNone;
    atomicAdd(&stats[S_CONFLICT], 1ull);
    return;
  }
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const uint32_t x = in[k].idx[s];
    if (x == kNone) continue;
    const NodeP n = in[k].nd[s];
    t[x].parent = n.parent;
    t[x].left = n.left;
    t[x].right = n.right;
    t[x].isLeft = n.isLeft;
  }
  atomicAdd(&stats[S_APPLIED], 1ull);
}

// Release the claims and count, per node, how many dirty paths arrive (kFixTree3_1). One thread
// per dirty path (3 per item); the parent link is loaded together with the counter update, so a
// level costs one round trip.
__global__ void count_kernel(const bvhgb_node *__restrict__ t, uint32_t root, const PatchOut *__restrict__ in,
                             const uint32_t *__restrict__ toFix, uint32_t *__restrict__ owner,
                             uint32_t *__restrict__ counter, uint32_t chunkSize, uint32_t numNodes,
                             uint32_t *__restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * chunkSize) return;
  const uint32_t k = i / 3, j = i - 3 * k;
  for (uint32_t s = j; s < (uint32_t)NSLOT; s += 3) {
    const uint32_t x = in[k].idx[s];
    if (x != kNone) owner[x] = kNone;
  }
  uint32_t x = toFix[i];
  if (x == kNone) return;
  for (uint32_t steps = 0;; ++steps) {
    if (x >= numNodes || steps > numNodes) {
      atomicOr(err, kErrBadIndex);
      break;
    }
    const uint32_t px = t[x].parent;  // issued before the update; the links are final here
    if (atomicAdd(&counter[x], 1u) != 0u) break;
    if (x == root) break;
    x = px;
  }
}

// The last path to arrive at a node recomputes its box (kFixTree3_2). A node's links do not change
// in this launch, so they are read before its counter; after the acq_rel update only the other
// child's box is loaded (the box of the child the path came from is still in registers).
__global__ void refit_kernel(bvhgb_node *t, uint32_t root, const uint32_t *__restrict__ toFix,
                             uint32_t *__restrict__ counter, uint32_t chunkSize, uint32_t numNodes,
                             uint32_t *__restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * chunkSize) return;
  uint32_t x = toFix[i];
  if (x == kNone) return;
  uint32_t from = kNone;  // child the path came from, whose box is 'cur'
  Box cur;
  for (uint32_t steps = 0;; ++steps) {
    if (x >= numNodes || steps > numNodes) {
      atomicOr(err, kErrBadIndex);
      return;
    }
    const float4 w1 = __ldcg(reinterpret_cast<const float4 *>(t + x) + 1);  // mx.y mx.z parent left
    const float4 w2 = __ldcg(reinterpret_cast<const float4 *>(t + x) + 2);  // right flags level sa
    if (atom_add_acq_rel(&counter[x], 0xFFFFFFFFu) != 1u) return;  // not the last arrival
    const uint32_t parent = __float_as_uint(w1.z), l = __float_as_uint(w1.w), r = __float_as_uint(w2.x);
    if ((__float_as_uint(w2.y) & 0xFFFFu) || l >= numNodes || r >= numNodes) {
      if (!(__float_as_uint(w2.y) & 0xFFFFu)) atomicOr(err, kErrBadIndex);
      return;
    }
    Box b = from == l ? cur : load_box_cg(t + l);
    const Box rb = from == r ? cur : load_box_cg(t + r);
    merge_into(b, rb);
    float4 *p = reinterpret_cast<float4 *>(t + x);
    p[0] = make_float4(b.mn[0], b.mn[1], b.mn[2], b.mx[0]);
    p[1] = make_float4(b.mx[1], b.mx[2], w1.z, w1.w);
    t[x].surfaceArea = surface_area(b);
    if (x == root) return;
    from = x;
    cur = b;
    x = parent;
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
  ok = ok && reinsert<true>(p, ins[0], un[0], true, unused, 0, ctr);
  ok = ok && reinsert<true>(p, ins[1], un[1], false, unused, 0, ctr);
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
  uint32_t *inner = nullptr, *keys = nullptr, *vals = nullptr, *keysSorted = nullptr, *todo = nullptr;
  void *sortTemp = nullptr;
  PatchOut *patches = nullptr;
  uint32_t *valid = nullptr, *toFix = nullptr, *owner = nullptr, *counter = nullptr, *err = nullptr;
  HeapItem *heaps = nullptr;
  unsigned long long *stats = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [0] plain iteration, [1] learned iteration
  bvhgb_node *graphNodes = nullptr;
  uint32_t launchesPerIteration = 0;
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
  return sort_pairs(ws->sortTemp, ws->keys, ws->keysSorted, ws->vals, ws->todo, ws->numInner, 4, 0, 32, s);
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
  const uint32_t bs = ws->cfg.blockSize ? ws->cfg.blockSize : 128;
  const uint32_t grid = ceil_div(cs, bs);
  const bool prof = !ws->evStart.empty();
  if (prof) BVHGB_CUDA_TRY(record_event(ws->evStart[c], s));
  if (ws->cfg.searchMode == BVHGB_SEARCH_BATCHED) {
    patch_warp_kernel<<<ceil_div(cs, kWarpItemsPerBlock), kWarpItemsPerBlock * 32, 0, s>>>(
        nodes, ws->root, ws->todo, ws->numInner, c, ws->numChunks, cs, ws->cfg.offsetAccess, ws->patches, ws->valid,
        ws->toFix, ws->owner, ws->stats, ws->numNodes, ws->err);
  } else {
    // One warp per block: these searches are latency-bound, so spreading them over more SMs beats
    // packing them (CUDABlockSize only sizes the other kernels; results do not depend on it).
    patch_kernel<<<ceil_div(cs, kSearchThreads), kSearchThreads, 0, s>>>(
        nodes, ws->root, ws->todo, ws->numInner, c, ws->numChunks, cs, ws->cfg.offsetAccess, ws->patches, ws->valid,
        ws->toFix, ws->owner, ws->heaps, ws->cfg.heapCapacity, ws->stats, ws->numNodes, ws->err);
  }
  BVHGB_LAUNCH_CHECK("bn13 patch");
  if (prof) BVHGB_CUDA_TRY(record_event(ws->evStop[c], s));
  apply_kernel<<<grid, bs, 0, s>>>(nodes, ws->patches, ws->valid, ws->toFix, ws->owner, cs, ws->stats);
  BVHGB_LAUNCH_CHECK("bn13 apply");
  count_kernel<<<ceil_div(3ull * cs, bs), bs, 0, s>>>(nodes, ws->root, ws->patches, ws->toFix, ws->owner, ws->counter,
                                                      cs, ws->numNodes,
                                   ws->err);
  BVHGB_LAUNCH_CHECK("bn13 count");
  refit_kernel<<<ceil_div(3ull * cs, bs), bs, 0, s>>>(nodes, ws->root, ws->toFix, ws->counter, cs, ws->numNodes, ws->err);
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
  if (ws->cfg.searchMode > BVHGB_SEARCH_HEAP) {
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
  ws->chunkSize = lNum / ws->numChunks;
  cudaStream_t s = as_stream(stream);

  // initData (Bittner13CUDA.cu:939-987): inner nodes in ascending index order.
  std::vector<uint32_t> hflags(numNodes);
  uint32_t *dflag = nullptr;
  cudaError_t e = cudaMalloc(&dflag, 4ull * numNodes);
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
  const size_t sortBytes = sort_temp_bytes(ws->numInner, 4, 0, 32);
  if (e == cudaSuccess) e = cudaMalloc(&ws->inner, 4 * ni);
  if (e == cudaSuccess) e = cudaMalloc(&ws->keys, 4 * ni);
  if (e == cudaSuccess) e = cudaMalloc(&ws->vals, 4 * ni);
  if (e == cudaSuccess) e = cudaMalloc(&ws->keysSorted, 4 * ni);
  if (e == cudaSuccess) e = cudaMalloc(&ws->todo, 4 * ni);
  if (e == cudaSuccess) e = cudaMalloc(&ws->sortTemp, sortBytes ? sortBytes : 256);
  if (e == cudaSuccess) e = cudaMalloc(&ws->patches, sizeof(PatchOut) * cs);
  if (e == cudaSuccess) e = cudaMalloc(&ws->valid, 4 * cs);
  if (e == cudaSuccess) e = cudaMalloc(&ws->toFix, 12 * cs);
  if (e == cudaSuccess) e = cudaMalloc(&ws->owner, 4ull * numNodes);
  if (e == cudaSuccess) e = cudaMalloc(&ws->counter, 4ull * numNodes);
  if (e == cudaSuccess) e = cudaMalloc(&ws->err, 4);
  if (e == cudaSuccess) e = cudaMalloc(&ws->heaps, sizeof(HeapItem) * cs * ws->cfg.heapCapacity);
  if (e == cudaSuccess) e = cudaMalloc(&ws->stats, sizeof(unsigned long long) * S_COUNT);
  if (e == cudaSuccess && inner.size())
    e = cudaMemcpyAsync(ws->inner, inner.data(), 4 * inner.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->counter, 0, 4ull * numNodes, s);
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
  cudaFree(ws->keysSorted);
  cudaFree(ws->todo);
  cudaFree(ws->sortTemp);
  cudaFree(ws->patches);
  cudaFree(ws->valid);
  cudaFree(ws->toFix);
  cudaFree(ws->owner);
  cudaFree(ws->counter);
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

extern "C" BVHGB_API int bvhgb_bn13_set_iteration(bvhgb_bn13_workspace *ws, uint64_t iteration) {
  if (!ws) return BVHGB_INVALID_ARGUMENT;
  ws->iteration = iteration;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_read_selection(const bvhgb_bn13_workspace *ws, uint32_t *out, uint32_t capacity,
                                                  bvhgb_stream stream) {
  if (!ws || !out) return BVHGB_INVALID_ARGUMENT;
  if (capacity < ws->numInner) return BVHGB_TOO_LARGE;
  if (ws->numInner)
    BVHGB_CUDA_TRY(cudaMemcpyAsync(out, ws->todo, 4ull * ws->numInner, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_bn13_set_selection(bvhgb_bn13_workspace *ws, const uint32_t *order, uint32_t n,
                                                 bvhgb_stream stream) {
  if (!ws || (n && !order) || n != ws->numInner) return BVHGB_INVALID_ARGUMENT;
  if (n) BVHGB_CUDA_TRY(cudaMemcpyAsync(ws->todo, order, 4ull * n, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return BVHGB_OK;
}
