// Device side of the parallel Bittner13 optimizer (lib/builder/Bittner13CUDA.cu,
// lib/base/BVHPatch.hpp), shared by the single-tree kernels (bittner.cu) and the batched ones
// (batch.cu): node views, the 10-slot patch, both reinsertion searches, removal / reinsertion,
// and the per-item steps of a chunk.
#pragma once

#include "common.cuh"

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

// The storage of a BVHPatch: its node slots and patched boxes. Every lane of a warp that runs one
// item holds the same patch, so the warp kernels keep one copy per warp in shared memory (a copy
// per lane would not fit L1); the thread-per-item kernel keeps its own.
struct PatchData {
  NodeP nd[NSLOT];
  uint32_t idx[NSLOT];
  uint32_t apath[4];
  Box abox[4];
};

// BVHPatch (BVHPatch.hpp:87-335), ENABLE_AABB_PATH = 0.
struct Patch {
  PatchData *d;
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
    for (int i = 0; i < NSLOT; ++i) d->idx[i] = kNone;
#pragma unroll
    for (int i = 0; i < 4; ++i) d->apath[i] = kNone;
  }
  __device__ uint32_t index_subset(uint32_t x) const {
    if (d->idx[0] == x) return 0;
    if (d->idx[1] == kNone) return kNone;
    if (d->idx[1] == x) return 1;
    if (d->idx[2] == x) return 2;
    if (d->idx[3] == x) return 3;
    return kNone;
  }
  __device__ uint32_t index(uint32_t x) const {
    for (uint32_t i = 0; i < NSLOT; ++i)
      if (d->idx[i] == x) return i;
    return kNone;
  }
  __device__ NodeP get(uint32_t x) const {
    uint32_t i = index(x);
    return i == kNone ? tree_node(t, chk(x)) : d->nd[i];
  }
  __device__ NodeP get_subset(uint32_t x) const {
    uint32_t i = index_subset(x);
    return i == kNone ? tree_node(t, chk(x)) : d->nd[i];
  }
  __device__ uint32_t patch_node(uint32_t x, uint32_t slot) {
    d->idx[slot] = x;
    d->nd[slot] = tree_node(t, chk(x));
    return slot;
  }
  __device__ uint32_t move(uint32_t from, uint32_t to) {
    d->idx[to] = d->idx[from];
    d->idx[from] = kNone;
    d->nd[to] = d->nd[from];
    return to;
  }
  __device__ uint32_t sibling(const NodeP &n) const {
    NodeP p = get(n.parent);
    return n.isLeft == 0 ? p.left : p.right;
  }
  // get_subset(x) and get_aabb(x) given the tree's 48-byte record of x (a, m, c: its three float4).
  __device__ void subset_aabb_from(uint32_t x, const float4 &a, const float4 &m, const float4 &c, NodeP &n,
                                   Box &b) const {
    const uint32_t i = index_subset(x);
    if (i != kNone) {
      n = d->nd[i];
    } else {
      n.parent = __float_as_uint(m.z);
      n.left = __float_as_uint(m.w);
      n.right = __float_as_uint(c.x);
      const uint32_t fl = __float_as_uint(c.y);
      n.isLeafFlag = (uint16_t)(fl & 0xFFFFu);
      n.isLeft = (uint16_t)(fl >> 16);
    }
    for (int k = 0; k < 4; ++k) {
      if (d->apath[k] == x) {
        b = d->abox[k];
        return;
      }
    }
    b.mn[0] = a.x; b.mn[1] = a.y; b.mn[2] = a.z;
    b.mx[0] = a.w; b.mx[1] = m.x; b.mx[2] = m.y;
  }
  __device__ Box get_aabb(uint32_t x) const {
    for (int i = 0; i < 4; ++i)
      if (d->apath[i] == x) return d->abox[i];
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
      d->abox[pidx * 2 + i] = b;
      d->apath[pidx * 2 + i] = ni;
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

// findNode2 (Bittner13CUDA.cu:194-264), the approximate search of altFindNode: kAltQueue (cost,
// node) slots, empty = +inf. Each step pops the first slot of smallest cost; an expanded node's
// left child takes the popped slot and its right child the slot the previous scan found to hold
// the largest cost (the first empty one while there is one, else the worst entry, which is lost);
// a scan in which no cost exceeds 0 keeps the previous max slot. One thread per item; the slots
// live in registers (the scans are unrolled, the two writes select by index).
constexpr uint32_t kAltQueue = 16;  // CUDA_ALT_QUEUE_SIZE (Bittner13CUDA.hpp:30)

__device__ uint32_t find_node2(const Patch &p, uint32_t n, SearchCounters &ctr) {
  const float kInf = __int_as_float(0x7f800000);
  float best_cost = kInf;
  uint32_t best = 0;
  const Box nbox = tree_box(p.t, p.chk(n));
  const float sarea = tree_sa(p.t, p.chk(n));
  float co[kAltQueue];
  uint32_t nl[kAltQueue];
#pragma unroll
  for (uint32_t i = 0; i < kAltQueue; ++i) {
    co[i] = kInf;
    nl[i] = 0;
  }
  uint32_t mnI = 0, mxI = 1;
  float mn = 0.0f;
  nl[0] = p.root;
  co[0] = 0.0f;
  for (uint32_t it = 0; mn < kInf; ++it) {
    if (it > p.numNodes) {  // only a corrupted tree gets here
      p.bad = true;
      break;
    }
    uint32_t cur = 0;
    float cc = 0.0f;
#pragma unroll
    for (uint32_t i = 0; i < kAltQueue; ++i)
      if (i == mnI) {
        cur = nl[i];
        cc = co[i];
        co[i] = kInf;
      }
    if (fadd(cc, sarea) >= best_cost) break;
    ctr.visits++;
    const NodeP cn = p.get_subset(cur);
    Box b = p.get_aabb(cur);
    float induced = fmul(-1.0f, surface_area(b));
    merge_into(b, nbox);
    const float direct = surface_area(b);
    const float total = fadd(cc, direct);
    if (total < best_cost) {
      best_cost = total;
      best = cur;
    }
    induced = fadd(induced, total);
    if (fadd(induced, sarea) < best_cost && !cn.isLeafFlag) {
#pragma unroll
      for (uint32_t i = 0; i < kAltQueue; ++i) {
        if (i == mnI) {
          nl[i] = cn.left;
          co[i] = induced;
        }
        if (i == mxI) {  // after the left child: the same slot takes the right one
          nl[i] = cn.right;
          co[i] = induced;
        }
      }
    }
    mn = kInf;
    float mx = 0.0f;
#pragma unroll
    for (uint32_t i = 0; i < kAltQueue; ++i) {
      if (co[i] < mn) {
        mn = co[i];
        mnI = i;
      }
      if (co[i] > mx) {
        mx = co[i];
        mxI = i;
      }
    }
  }
  return best;
}

// removeNode (Bittner13CUDA.cu:267-305).
__device__ bool remove_node(Patch &p, uint32_t x, uint32_t ins[2], uint32_t un[2], uint32_t &g_out) {
  if (tree_leaf(p.t, p.chk(x)) || x == p.root) return false;
  const uint32_t sn = p.patch_node(x, P_NODE);
  const uint32_t s = p.sibling(p.d->nd[sn]);
  const uint32_t pi = p.d->nd[sn].parent;
  if (pi == p.root) return false;
  const uint32_t ss = p.patch_node(s, P_SIBLING);
  const uint32_t sp = p.patch_node(pi, P_PARENT);
  const uint32_t gi = p.d->nd[sp].parent;
  const uint32_t sg = p.patch_node(gi, P_GRAND_PARENT);
  if (p.d->nd[sp].isLeft) {
    p.d->nd[sg].left = s;
    p.d->nd[ss].isLeft = 1;
  } else {
    p.d->nd[sg].right = s;
    p.d->nd[ss].isLeft = 0;
  }
  p.d->nd[ss].parent = gi;
  p.patch_aabb_from(gi, 0);
  const uint32_t l = p.d->nd[sn].left, r = p.d->nd[sn].right;
  if (tree_sa(p.t, p.chk(l)) > tree_sa(p.t, p.chk(r))) { ins[0] = l; ins[1] = r; }
  else { ins[0] = r; ins[1] = l; }
  un[0] = x;
  un[1] = pi;
  g_out = gi;
  return true;
}

// ---- batched best-first search: one warp per item -------------------------------------------
//
// The frontier (up to 128 entries, unordered) lives in registers, 4 slots per lane, entry
// e = slot * 32 + lane; slots at or past `used` are empty. Each round the warp evaluates every
// entry whose bound passes (up to four per lane, their loads issued together), reduces the best
// total (ties: the entry first in (cost, node) order) and gathers the children of the expanded
// entries into the warp's shared buffer, which becomes the next frontier. Only when more than 128
// children arrive are the 128 lowest in (cost, node) order selected (a radix selection by warp
// ballots) and kept, the rest counted as overflow. The records of the next round's slot 0 are loaded as soon as it is known.
// oracle/bittner.c (gpu_find_node_batched) restates the same rounds.
constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr int kFrontier = 4;  // slots per lane (128 entries)
constexpr uint32_t kFrontierCap = 32u * kFrontier;

// The k-th smallest (1 <= k <= number of flagged entries) of the 32-bit keys of the slots flagged
// in 'in' (bit s: this lane's slot s), S slots per lane: a most-significant-first radix selection
// over 2-bit digits, one warp sum per digit, starting below the bits that all flagged keys share.
template <int S>
__device__ __forceinline__ uint32_t warp_select_kth(const uint32_t (&key)[S], uint32_t in, uint32_t k) {
  uint32_t lo = 0xFFFFFFFFu, hi = 0u;
#pragma unroll
  for (int s = 0; s < S; ++s)
    if ((in >> s) & 1u) {
      lo = min(lo, key[s]);
      hi = max(hi, key[s]);
    }
  lo = __reduce_min_sync(kFull, lo);
  hi = __reduce_max_sync(kFull, hi);
  if (lo == hi) return lo;
  const int top = 31 - __clz(lo ^ hi);
  uint32_t res = lo & ~((2u << top) - 1u);  // 2u << 31 wraps to 0: no common bits
  uint32_t alive = in;
  int bit = top;
  // two bits per step: the counts of the digits 00, 01 and 10 (at most 1,023 each) travel packed
  // 10 bits apart in one warp sum
  for (; bit >= 1; bit -= 2) {
    uint32_t hi1 = 0, lo1 = 0;  // this lane's slots whose key has bit / bit - 1 set
#pragma unroll
    for (int s = 0; s < S; ++s) {
      hi1 |= ((key[s] >> bit) & 1u) << s;
      lo1 |= ((key[s] >> (bit - 1)) & 1u) << s;
    }
    const uint32_t m00 = alive & ~hi1 & ~lo1, m01 = alive & ~hi1 & lo1, m10 = alive & hi1 & ~lo1;
    const uint32_t c = __reduce_add_sync(kFull, (uint32_t)__popc(m00) | ((uint32_t)__popc(m01) << 10) |
                                                    ((uint32_t)__popc(m10) << 20));
    const uint32_t c00 = c & 1023u, c01 = (c >> 10) & 1023u, c10 = c >> 20;
    if (k <= c00) {
      alive = m00;
    } else if (k <= c00 + c01) {
      k -= c00;
      alive = m01;
      res |= 1u << (bit - 1);
    } else if (k <= c00 + c01 + c10) {
      k -= c00 + c01;
      alive = m10;
      res |= 1u << bit;
    } else {
      k -= c00 + c01 + c10;
      alive &= hi1 & lo1;
      res |= 3u << (bit - 1);
    }
  }
  if (bit == 0) {
    uint32_t ones = 0;
#pragma unroll
    for (int s = 0; s < S; ++s) ones |= (key[s] & 1u) << s;
    const uint32_t zeros = __reduce_add_sync(kFull, (uint32_t)__popc(alive & ~ones));
    if (k > zeros) res |= 1u;
  }
  return res;
}

// Per-warp buffer of a round's children (up to 256 entries; blocks of up to kRankWarps warps).
constexpr int kRankWarps = 8;
__device__ __forceinline__ uint2 *child_buffer() {
  __shared__ uint2 buf[kRankWarps][2 * kFrontierCap];
  return buf[(threadIdx.x >> 5) & (kRankWarps - 1)];
}

// State of one batched search (warp-uniform except the per-lane frontier entries and records).
struct BatchedSearch {
  float fc[kFrontier];
  uint32_t fn[kFrontier];
  uint32_t used;     // slots holding entries
  bool haveRec;      // slot 0's tree records are already in rec[]
  float4 rec[3];
  float bestCost;
  uint32_t best;
};

// One round over the first S slots (S >= used). Returns false when no entry passed the bound.
template <int S>
__device__ __forceinline__ bool batched_round(const Patch &p, BatchedSearch &st, const Box &nbox, float sarea,
                                              uint2 *buf, SearchCounters &ctr) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t ltMask = (1u << lane) - 1u;
  const float kInf = __int_as_float(0x7f800000);
  bool cand[S];
  uint32_t nc = 0;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    cand[s] = st.fc[s] != kInf && fadd(st.fc[s], sarea) < st.bestCost;
    nc += __popc(__ballot_sync(kFull, cand[s]));
  }
  if (nc == 0) return false;
  ctr.visits += nc;
  NodeP cn[S];
  float total[S], induced[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    total[s] = induced[s] = kInf;
    if (!cand[s]) continue;
    const uint32_t xs = p.chk(st.fn[s]);
    float4 q0, q1, q2;
    if (s == 0 && st.haveRec) {
      q0 = st.rec[0]; q1 = st.rec[1]; q2 = st.rec[2];
    } else {
      const float4 *q = reinterpret_cast<const float4 *>(p.t + xs);
      q0 = __ldg(q); q1 = __ldg(q + 1); q2 = __ldg(q + 2);
    }
    Box b;
    p.subset_aabb_from(st.fn[s], q0, q1, q2, cn[s], b);
    const float ind = fmul(-1.0f, surface_area(b));
    merge_into(b, nbox);
    total[s] = fadd(st.fc[s], surface_area(b));
    induced[s] = fadd(ind, total[s]);
  }
  // Best of the round: smallest total, then smallest (cost, node) of the entry.
  uint32_t kl = 0xFFFFFFFFu;
#pragma unroll
  for (int s = 0; s < S; ++s)
    if (cand[s]) kl = min(kl, f2ord(total[s]));
  const uint32_t kmin = __reduce_min_sync(kFull, kl);
  uint32_t rnode;
  uint32_t tieMask = 0;  // this lane's slots that reach kmin
#pragma unroll
  for (int s = 0; s < S; ++s)
    if (cand[s] && f2ord(total[s]) == kmin) tieMask |= 1u << s;
  const uint32_t tieLanes = __ballot_sync(kFull, tieMask != 0);
  if (__popc(tieLanes) == 1 && (S == 1 || __popc(__shfl_sync(kFull, tieMask, __ffs(tieLanes) - 1)) == 1)) {
    uint32_t mine = kNone;
#pragma unroll
    for (int s = 0; s < S; ++s)
      if (tieMask & (1u << s)) mine = st.fn[s];
    rnode = __shfl_sync(kFull, mine, __ffs(tieLanes) - 1);
  } else {
    uint32_t cl = 0xFFFFFFFFu;
#pragma unroll
    for (int s = 0; s < S; ++s)
      if (tieMask & (1u << s)) cl = min(cl, f2ord(st.fc[s]));
    const uint32_t cmin = __reduce_min_sync(kFull, cl);
    uint32_t nl = 0xFFFFFFFFu;
#pragma unroll
    for (int s = 0; s < S; ++s)
      if ((tieMask & (1u << s)) && f2ord(st.fc[s]) == cmin) nl = min(nl, st.fn[s]);
    rnode = __reduce_min_sync(kFull, nl);
  }
  const float rbest = ord2f(kmin);
  if (rbest < st.bestCost) {
    st.bestCost = rbest;
    st.best = rnode;
  }
  // Children of the expanded entries: the k-th expanded entry (slot-major, then lane) writes
  // children 2k and 2k + 1 to the warp's buffer.
  uint32_t m = 0;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const bool kids = cand[s] && !cn[s].isLeafFlag && fadd(induced[s], sarea) < st.bestCost;
    const uint32_t kmask = __ballot_sync(kFull, kids);
    const uint32_t mk = 2u * __popc(kmask);
    if (kids) {
      const uint32_t k = m / 2 + __popc(kmask & ltMask);
      buf[2 * k] = make_uint2(__float_as_uint(induced[s]), cn[s].left);
      buf[2 * k + 1] = make_uint2(__float_as_uint(induced[s]), cn[s].right);
      if (m + mk > 32u) {  // children past slot 0: warm their records in L2
        if (cn[s].left < p.numNodes) prefetch_node(p.t, cn[s].left);
        if (cn[s].right < p.numNodes) prefetch_node(p.t, cn[s].right);
      }
    }
    m += mk;
  }
  __syncwarp();
  st.haveRec = false;
  if (m <= kFrontierCap) {
    st.used = (m + 31u) / 32u;
#pragma unroll
    for (int s = 0; s < kFrontier; ++s) {
      const uint32_t e = (uint32_t)s * 32u + lane;
      if ((uint32_t)s < st.used) {
        const uint2 v = e < m ? buf[e] : make_uint2(__float_as_uint(kInf), kNone);
        st.fc[s] = __uint_as_float(v.x);
        st.fn[s] = v.y;
      } else {
        st.fc[s] = kInf;
        st.fn[s] = kNone;
      }
    }
    if (lane < m) {  // slot 0's records for the next round (an index out of range: the root's)
      const float4 *q = reinterpret_cast<const float4 *>(p.t + (st.fn[0] < p.numNodes ? st.fn[0] : p.root));
      st.rec[0] = __ldg(q);
      st.rec[1] = __ldg(q + 1);
      st.rec[2] = __ldg(q + 2);
    }
    st.haveRec = true;
  } else {
    // Overflow: keep the 128 lowest children in (cost, node) order. The frontier is unordered, so
    // only that set matters: select the 128th smallest cost, then, among the children at that cost
    // (siblings share their parent's), the lowest nodes up to 128 entries; the kept entries are
    // compacted to the front of the buffer.
    uint32_t key[2 * kFrontier], nd[2 * kFrontier];
    uint32_t in = 0;  // bit s: slot s holds a child
#pragma unroll
    for (int s = 0; s < 2 * kFrontier; ++s) {
      const uint32_t e = (uint32_t)s * 32u + lane;
      const uint2 v = e < m ? buf[e] : make_uint2(0u, kNone);
      in |= (e < m ? 1u : 0u) << s;
      key[s] = f2ord(__uint_as_float(v.x));
      nd[s] = v.y;
    }
    __syncwarp();
    const uint32_t tc = warp_select_kth<2 * kFrontier>(key, in, kFrontierCap);
    uint32_t below = 0, tie = 0;
#pragma unroll
    for (int s = 0; s < 2 * kFrontier; ++s) {
      below += __popc(__ballot_sync(kFull, ((in >> s) & 1u) && key[s] < tc));
      tie |= (((in >> s) & 1u) && key[s] == tc ? 1u : 0u) << s;
    }
    uint32_t ties = 0;
#pragma unroll
    for (int s = 0; s < 2 * kFrontier; ++s) ties += __popc(__ballot_sync(kFull, (tie >> s) & 1u));
    const uint32_t need = kFrontierCap - below;  // 1 <= need <= ties
    uint32_t tn = 0xFFFFFFFFu;                    // largest node kept at cost tc
    if (need < ties) {
      if (need == 1u) {
        uint32_t nl = 0xFFFFFFFFu;
#pragma unroll
        for (int s = 0; s < 2 * kFrontier; ++s)
          if ((tie >> s) & 1u) nl = min(nl, nd[s]);
        tn = __reduce_min_sync(kFull, nl);
      } else {
        tn = warp_select_kth<2 * kFrontier>(nd, tie, need);
      }
    }
    uint32_t pos = 0;
#pragma unroll
    for (int s = 0; s < 2 * kFrontier; ++s) {
      const bool keep = ((in >> s) & 1u) && (key[s] < tc || (((tie >> s) & 1u) && nd[s] <= tn));
      const uint32_t km = __ballot_sync(kFull, keep);
      if (keep) buf[pos + __popc(km & ltMask)] = make_uint2(__float_as_uint(ord2f(key[s])), nd[s]);
      pos += __popc(km);
    }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < kFrontier; ++s) {
      const uint2 v = buf[(uint32_t)s * 32u + lane];
      st.fc[s] = __uint_as_float(v.x);
      st.fn[s] = v.y;
    }
    ctr.overflow += m - kFrontierCap;
    st.used = kFrontier;
  }
  __syncwarp();
  return true;
}

// findNode1's cost model in batched rounds (every lane of the warp calls it with the same patch).
__device__ uint32_t find_node_batched(const Patch &p, uint32_t n, SearchCounters &ctr) {
  const uint32_t lane = threadIdx.x & 31u;
  __syncwarp();  // the warp's patch writes are visible to every lane
  const float kInf = __int_as_float(0x7f800000);
  const Box nbox = tree_box(p.t, p.chk(n));
  const float sarea = tree_sa(p.t, p.chk(n));
  BatchedSearch st;
#pragma unroll
  for (int s = 0; s < kFrontier; ++s) {
    st.fc[s] = kInf;
    st.fn[s] = kNone;
  }
  if (lane == 0) {
    st.fc[0] = 0.0f;
    st.fn[0] = p.root;
  }
  st.used = 1;
  st.haveRec = false;
  st.bestCost = kInf;
  st.best = 0;
  uint2 *buf = child_buffer();
  for (uint32_t round = 0;; ++round) {
    if (round > p.numNodes) {  // bounded: every round evaluates at least one node
      p.bad = true;
      break;
    }
    const bool more = st.used <= 1   ? batched_round<1>(p, st, nbox, sarea, buf, ctr)
                      : st.used <= 2 ? batched_round<2>(p, st, nbox, sarea, buf, ctr)
                                     : batched_round<kFrontier>(p, st, nbox, sarea, buf, ctr);
    if (!more) break;
  }
  __syncwarp();  // every lane is done reading the patch before it changes again
  p.bad = __any_sync(kFull, p.bad);
  return st.best;
}

// reinsert (Bittner13CUDA.cu:308-358).
// MODE: BVHGB_SEARCH_BATCHED (warp-cooperative), BVHGB_SEARCH_HEAP (findNode1) or
// BVHGB_SEARCH_ALT (findNode2).
template <int MODE>
__device__ bool reinsert(Patch &p, uint32_t x, uint32_t unused, bool update, const Heap &pq, uint32_t cap,
                         SearchCounters &ctr) {
  const uint32_t best = MODE == BVHGB_SEARCH_BATCHED ? find_node_batched(p, x, ctr)
                        : MODE == BVHGB_SEARCH_ALT   ? find_node2(p, x, ctr)
                                                     : find_node(p, x, pq, cap, ctr);
  if (best == p.root) return false;
  const uint32_t bpi = p.index(best);
  uint32_t sb;
  if (bpi == kNone) sb = p.patch_node(best, update ? P_1ST_BEST : P_2ND_BEST);
  else if (bpi == P_GRAND_PARENT) sb = P_GRAND_PARENT;
  else sb = p.move(bpi, update ? P_1ST_BEST : P_2ND_BEST);
  const uint32_t sx = p.patch_node(x, update ? P_1ST_INSERT : P_2ND_INSERT);
  const uint32_t su = update ? P_NODE : P_PARENT;
  const uint32_t ri = p.d->nd[sb].parent;
  const uint32_t rpi = p.index(ri);
  const uint32_t sr = rpi == kNone ? p.patch_node(ri, update ? P_1ST_ROOT : P_2ND_ROOT)
                                   : p.move(rpi, update ? P_1ST_ROOT : P_2ND_ROOT);
  if (p.d->nd[sb].isLeft) {
    p.d->nd[sr].left = unused;
    p.d->nd[su].isLeft = 1;
  } else {
    p.d->nd[sr].right = unused;
    p.d->nd[su].isLeft = 0;
  }
  p.d->nd[su].parent = ri;
  p.d->nd[su].left = best;
  p.d->nd[su].right = x;
  p.d->nd[sb].parent = unused;
  p.d->nd[sb].isLeft = 1;
  p.d->nd[sx].parent = unused;
  p.d->nd[sx].isLeft = 0;
  if (update) p.patch_aabb_from(unused, 1);
  return true;
}


// ---- per-item steps shared by the single-tree and the batched kernels ---------------------------
// (t, root, numNodes) describe one tree; owner / counter point at that tree's entries; rank is the
// item's position in its tree's chunk (lower rank wins a conflict).

constexpr int kWarpItemsPerBlock = 4;

// The patch storage of this warp (blocks of kWarpItemsPerBlock warps).
__device__ __forceinline__ PatchData *warp_patch_data() {
  __shared__ PatchData pd[kWarpItemsPerBlock];
  return &pd[(threadIdx.x >> 5) & (kWarpItemsPerBlock - 1)];
}

// kRemoveAndReinsert for one item on a whole warp (batched search); lane 0 publishes.
__device__ __forceinline__ void warp_patch_item(const bvhgb_node *__restrict__ t, uint32_t root, uint32_t numNodes,
                                                uint32_t node, bool ok, uint32_t rank, PatchOut *__restrict__ out,
                                                uint32_t *__restrict__ valid, uint32_t *__restrict__ toFix3,
                                                uint32_t *__restrict__ owner, unsigned long long *__restrict__ stats,
                                                uint32_t *__restrict__ err) {
  const uint32_t lane = threadIdx.x & 31u;
  Patch p;
  p.d = warp_patch_data();
  p.t = t;
  p.root = root;
  p.numNodes = numNodes;
  p.bad = false;
  p.clear();
  SearchCounters ctr = {0u, 0u};
  uint32_t ins[2], un[2], g = kNone;
  const Heap unused{nullptr, nullptr};
  ok = ok && remove_node(p, node, ins, un, g);
  ok = ok && reinsert<BVHGB_SEARCH_BATCHED>(p, ins[0], un[0], true, unused, 0, ctr);
  ok = ok && reinsert<BVHGB_SEARCH_BATCHED>(p, ins[1], un[1], false, unused, 0, ctr);
  if (p.bad) ok = false;
  __syncwarp();
  if (lane != 0) return;
  if (p.bad) atomicOr(err, kErrBadIndex);
  *valid = ok ? 1u : 0u;
  toFix3[0] = ok ? g : kNone;
  toFix3[1] = ok ? un[0] : kNone;
  toFix3[2] = ok ? un[1] : kNone;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    out->nd[s] = p.d->nd[s];
    out->idx[s] = ok ? p.d->idx[s] : kNone;
    if (ok && p.d->idx[s] != kNone) atomicMin(&owner[p.d->idx[s]], rank);
  }
  if (!ok) atomicAdd(&stats[S_INVALID], 1ull);
  if (ctr.overflow) atomicAdd(&stats[S_OVERFLOW], (unsigned long long)ctr.overflow);
  atomicAdd(&stats[S_VISITS], (unsigned long long)ctr.visits);
  atomicAdd(&stats[S_ITEMS], 1ull);
}

// kCheckConflicts + kApplyPatches for one item.
__device__ __forceinline__ void apply_item(bvhgb_node *t, const PatchOut &in, uint32_t *__restrict__ valid,
                                           uint32_t *__restrict__ toFix3, const uint32_t *__restrict__ owner,
                                           uint32_t rank, unsigned long long *__restrict__ stats) {
  if (!*valid) return;
  bool win = true;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const uint32_t x = in.idx[s];
    if (x != kNone && owner[x] != rank) win = false;
  }
  if (!win) {
    *valid = 0;
    toFix3[0] = toFix3[1] = toFix3[2] = kNone;
    atomicAdd(&stats[S_CONFLICT], 1ull);
    return;
  }
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const uint32_t x = in.idx[s];
    if (x == kNone) continue;
    const NodeP n = in.nd[s];
    t[x].parent = n.parent;
    t[x].left = n.left;
    t[x].right = n.right;
    t[x].isLeft = n.isLeft;
  }
  atomicAdd(&stats[S_APPLIED], 1ull);
}

// Apply and count in one launch, three climbs per item. The count climbs the new tree while the
// winners' patches are still being written: a node that a winning item patched takes its new parent
// from that item's patch record, every other node keeps its parent (its record is not written in
// this launch). A node y is patched by a winner iff its owner o (the lowest rank that claimed it;
// the claims are final before this launch) wins, i.e. owns every node of its own patch: a higher
// rank that also claimed y does not own y, so it cannot win. The claims are released later, by
// the refit launch.
__device__ __forceinline__ bool item_wins(const PatchOut &in, const uint32_t *__restrict__ owner, uint32_t rank) {
  bool win = true;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const uint32_t x = in.idx[s];
    if (x != kNone && owner[x] != rank) win = false;
  }
  return win;
}

// The parent of y in the tree being patched, given y's owner o and its parent p before the patch.
__device__ __forceinline__ uint32_t new_parent(const PatchOut *__restrict__ in, const uint32_t *__restrict__ owner,
                                               uint32_t y, uint32_t o, uint32_t p) {
  if (o == kNone) return p;
  const PatchOut &po = in[o];
  if (!item_wins(po, owner, o)) return p;
#pragma unroll
  for (int s = 0; s < NSLOT; ++s)
    if (po.idx[s] == y) return po.nd[s].parent;
  return p;
}

// Climb j of item k: all three decide the item's outcome (the owner array is final; valid[k], the
// patch kernel's decision, is only read here, so the three climbs see the same value); climb 0
// writes the patch and the statistics, climb j counts the arrivals along the item's j-th dirty
// path (kFixTree3_1) in the new tree. The start node gets bit 31 as in count_path.
__device__ __forceinline__ void apply_count_path(bvhgb_node *t, uint32_t root, uint32_t numNodes,
                                                 const PatchOut *__restrict__ in, uint32_t k, uint32_t j,
                                                 const uint32_t *__restrict__ valid, uint32_t *__restrict__ toFix,
                                                 const uint32_t *__restrict__ owner, uint32_t *__restrict__ counter,
                                                 unsigned long long *__restrict__ stats, uint32_t *__restrict__ err) {
  if (!valid[k]) return;  // refused by removeNode or the search: it claimed nothing
  uint32_t x = toFix[3 * k + j];
  const PatchOut &me = in[k];
  const bool win = item_wins(me, owner, k);
  if (!win) {
    toFix[3 * k + j] = kNone;  // the refit skips a lost item's paths
    if (j == 0) atomicAdd(&stats[S_CONFLICT], 1ull);
    return;
  }
  if (j == 0) {
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) {
      const uint32_t y = me.idx[s];
      if (y == kNone) continue;
      const NodeP n = me.nd[s];
      t[y].parent = n.parent;
      t[y].left = n.left;
      t[y].right = n.right;
      t[y].isLeft = n.isLeft;
    }
    atomicAdd(&stats[S_APPLIED], 1ull);
  }
  if (x == kNone) return;
  uint32_t add = 0x80000001u;
  for (uint32_t steps = 0;; ++steps) {
    if (x >= numNodes || steps > numNodes) {
      atomicOr(err, kErrBadIndex);
      break;
    }
    // owner, old parent and the counter update go out together: one round trip per level where
    // no patch touched the node
    const uint32_t o = owner[x];
    const uint32_t p = __ldcg(&t[x].parent);  // discarded if a winner rewrites it in this launch
    if (atomicAdd(&counter[x], add) != 0u) break;
    if (x == root) break;
    add = 1u;
    x = new_parent(in, owner, x, o, p);
  }
}

// Release a third of an item's claims (after the launch that counted with them).
__device__ __forceinline__ void release_claims(const PatchOut &in, uint32_t j, uint32_t *__restrict__ owner) {
  for (uint32_t s = j; s < (uint32_t)NSLOT; s += 3) {
    const uint32_t y = in.idx[s];
    if (y != kNone) owner[y] = kNone;
  }
}

// Release a third of an item's claims and count the arrivals along one dirty path (kFixTree3_1);
// the parent link is loaded together with the counter update, so a level costs one round trip.
// The path's own start node gets bit 31 as well (the refit below must know its start nodes).
__device__ __forceinline__ void count_path(const bvhgb_node *__restrict__ t, uint32_t root, uint32_t numNodes,
                                          const PatchOut &in, uint32_t j, uint32_t x, uint32_t *__restrict__ owner,
                                          uint32_t *__restrict__ counter, uint32_t *__restrict__ err) {
  for (uint32_t s = j; s < (uint32_t)NSLOT; s += 3) {
    const uint32_t y = in.idx[s];
    if (y != kNone) owner[y] = kNone;
  }
  if (x == kNone) return;
  uint32_t add = 0x80000001u;
  for (uint32_t steps = 0;; ++steps) {
    if (x >= numNodes || steps > numNodes) {
      atomicOr(err, kErrBadIndex);
      break;
    }
    const uint32_t px = t[x].parent;  // issued before the update; the links are final here
    if (atomicAdd(&counter[x], add) != 0u) break;
    if (x == root) break;
    add = 1u;
    x = px;
  }
}

// ---- dirty-path refit (kFixTree3_2) ------------------------------------------------------------
// The last path to arrive at a node recomputes its box. A node's counter (set by the count pass)
// holds the arrivals still expected in its low 16 bits and bit 31 for a start node (grand parent or
// reused node: its children were relinked, so it is always recomputed). Each arrival subtracts one
// and, for the child it comes from (side 0 left, 1 right), sets bit 16 + side if it rewrote that
// child's box in this launch and bit 18 + side if the child changed (rewritten, or a start node,
// which may have moved under a new parent). A side arrives at most once, so the bits never carry.
//
// Every counter update is relaxed: a rewritten box does not travel through the node record, whose
// visibility would need a release by the writer and an acquire by the reader (fences that cost
// several L2 round trips each), but through a mail slot of three 64-bit words per child that
// carries its own validity. A path that may not be the last at a node posts its child's new box
// there before its update; the last arrival finds the posting side in the counter bits and reads
// the slot until all three words differ from the empty pattern (each 64-bit word is written and
// read whole), then empties it again; a path that posted and turned out last empties its own. A
// child whose box was not rewritten in this launch is read from its record, loaded speculatively
// together with the counter update. (Two coordinates of a box that both hold the bit pattern
// 0xFFFFFFFF would read as empty: the wait then ends at its limit with kErrTimeout.)
//
// Links do not change in this launch and a node's box is written only by its last arrival, so the
// climb reads one level ahead: while it handles node x it loads the parent's record and counter. A
// node whose counter already shows this path as the only arrival left needs no update at all.
constexpr unsigned long long kMailEmpty = 0xFFFFFFFFFFFFFFFFull;

__device__ __forceinline__ unsigned long long pack2(float a, float b) {
  return (unsigned long long)__float_as_uint(a) | ((unsigned long long)__float_as_uint(b) << 32);
}

__device__ __forceinline__ void mail_post(unsigned long long *mail, uint32_t child, const Box &b) {
  unsigned long long *m = mail + 3ull * child;
  __stcg(m, pack2(b.mn[0], b.mn[1]));
  __stcg(m + 1, pack2(b.mn[2], b.mx[0]));
  __stcg(m + 2, pack2(b.mx[1], b.mx[2]));
}

__device__ __forceinline__ void mail_clear(unsigned long long *mail, uint32_t child) {
  unsigned long long *m = mail + 3ull * child;
  __stcg(m, kMailEmpty);
  __stcg(m + 1, kMailEmpty);
  __stcg(m + 2, kMailEmpty);
}

// Takes the box posted for 'child' (bounded wait per word) and empties the slot.
__device__ __forceinline__ Box mail_take(unsigned long long *mail, uint32_t child, uint32_t *__restrict__ err) {
  unsigned long long *m = mail + 3ull * child;
  unsigned long long w[3] = {__ldcg(m), __ldcg(m + 1), __ldcg(m + 2)};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    for (uint32_t spins = 0; w[q] == kMailEmpty; ++spins) {
      if (spins > kSpinLimit) {
        atomicOr(err, kErrTimeout);
        break;
      }
      __nanosleep(32);
      w[q] = __ldcg(m + q);
    }
  }
  mail_clear(mail, child);
  Box b;
  b.mn[0] = __uint_as_float((uint32_t)w[0]); b.mn[1] = __uint_as_float((uint32_t)(w[0] >> 32));
  b.mn[2] = __uint_as_float((uint32_t)w[1]); b.mx[0] = __uint_as_float((uint32_t)(w[1] >> 32));
  b.mx[1] = __uint_as_float((uint32_t)w[2]); b.mx[2] = __uint_as_float((uint32_t)(w[2] >> 32));
  return b;
}

__device__ __forceinline__ void refit_path(bvhgb_node *t, uint32_t root, uint32_t numNodes, uint32_t x,
                                          uint32_t *__restrict__ counter, unsigned long long *__restrict__ mail,
                                          uint32_t *__restrict__ err) {
  if (x == kNone) return;
  if (x >= numNodes) {
    atomicOr(err, kErrBadIndex);
    return;
  }
  const float4 *q = reinterpret_cast<const float4 *>(t + x);
  float4 w0 = __ldcg(q), w1 = __ldcg(q + 1), w2 = __ldcg(q + 2);  // [mn.xyz mx.x] [mx.yz parent left] [right flags . sa]
  uint32_t cnt = __ldcg(&counter[x]);
  uint32_t from = kNone;  // child the path came from, whose box is 'cur'
  Box cur;
  bool written = false;   // cur was rewritten in this launch
  bool changed = true;    // the start node's children were relinked
  for (uint32_t steps = 0;; ++steps) {
    const uint32_t parent = __float_as_uint(w1.z), l = __float_as_uint(w1.w), r = __float_as_uint(w2.x);
    if ((__float_as_uint(w2.y) & 0xFFFFu) || l >= numNodes || r >= numNodes || steps > numNodes ||
        (from != kNone && from != l && from != r)) {
      if (!(__float_as_uint(w2.y) & 0xFFFFu)) atomicOr(err, kErrBadIndex);
      return;
    }
    const bool top = x == root;
    if (!top && parent >= numNodes) {
      atomicOr(err, kErrBadIndex);
      return;
    }
    const uint32_t side = from == r ? 1u : 0u;  // meaningful only when from != kNone
    // this level's child boxes from their records (valid unless rewritten in this launch) and the
    // next level's record and counter
    Box lb = from == l ? cur : load_box_cg(t + l);
    Box rb = from == r ? cur : load_box_cg(t + r);
    float4 n0 = w0, n1 = w1, n2 = w2;
    uint32_t ncnt = 0u;
    if (!top) {
      const float4 *pq = reinterpret_cast<const float4 *>(t + parent);
      n0 = __ldcg(pq);
      n1 = __ldcg(pq + 1);
      n2 = __ldcg(pq + 2);
      ncnt = __ldcg(&counter[parent]);
    }
    uint32_t old = cnt;
    if ((cnt & 0x7FFFFFFFu) != 1u) {  // other arrivals are (or were) expected here
      const bool post = from != kNone && written;
      if (post) mail_post(mail, from, cur);
      uint32_t add = 0xFFFFFFFFu;  // one arrival less
      if (from != kNone) add += (written ? (1u << (16 + side)) : 0u) + (changed ? (1u << (18 + side)) : 0u);
      old = atomicAdd(&counter[x], add);
      if ((old & 0xFFFFu) != 1u) return;  // not the last arrival
      if (post) mail_clear(mail, from);   // posted for nobody
      if (from != l && ((old >> 16) & 1u)) lb = mail_take(mail, l, err);
      if (from != r && ((old >> 17) & 1u)) rb = mail_take(mail, r, err);
    }
    counter[x] = 0u;
    const bool start = (old >> 31) != 0u;  // x started a path (this one or an earlier arrival)
    const bool anyChanged = changed || start || ((old >> 18) & 3u) != 0u;
    Box b;
    b.mn[0] = w0.x; b.mn[1] = w0.y; b.mn[2] = w0.z;
    b.mx[0] = w0.w; b.mx[1] = w1.x; b.mx[2] = w1.y;
    bool upChanged = false;
    if (anyChanged) {
      merge_into(lb, rb);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        upChanged |= __float_as_uint(lb.mn[k]) != __float_as_uint(b.mn[k]) ||
                     __float_as_uint(lb.mx[k]) != __float_as_uint(b.mx[k]);
      if (upChanged) {
        float4 *p = reinterpret_cast<float4 *>(t + x);
        p[0] = make_float4(lb.mn[0], lb.mn[1], lb.mn[2], lb.mx[0]);
        p[1] = make_float4(lb.mx[1], lb.mx[2], w1.z, w1.w);
        t[x].surfaceArea = surface_area(lb);
        b = lb;
      }
    }
    if (top) return;
    // A start node may have moved (a reused node now hangs under a new parent), so its parent
    // cannot compare against the old box: it always counts as changed.
    written = upChanged;
    changed = upChanged || start;
    from = x;
    cur = b;
    x = parent;
    w0 = n0;
    w1 = n1;
    w2 = n2;
    cnt = ncnt;
  }
}

// kCalcCost for one inner node (0 for a leaf).
__device__ __forceinline__ float inefficiency(const bvhgb_node *__restrict__ t, uint32_t x) {
  const float4 *p = reinterpret_cast<const float4 *>(t + x);
  const float4 b = __ldg(p + 1), c = __ldg(p + 2);
  if ((__float_as_uint(c.y) & 0xFFFFu) != 0) return 0.0f;
  const float sa = c.w;
  const float l = __ldg(&t[__float_as_uint(b.w)].surfaceArea);
  const float r = __ldg(&t[__float_as_uint(c.x)].surfaceArea);
  const float num = fmul(fmul(fmul(sa, sa), sa), 2.0f);
  const float den = fmul(fadd(l, r), l < r ? l : r);
  return fdiv(num, den);
}

}  // namespace
}  // namespace bvhgb
