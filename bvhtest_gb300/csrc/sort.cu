// Onesweep-style stable LSD radix sort of (key, uint32 value) pairs, 8-bit digits.
//
// Replaces cub::DeviceRadixSort::SortPairs (lib/builder/LBVH_CUDA.cu:185-193) and
// SortPairsDescending (lib/builder/Bittner13CUDA.cu:674-680). Design (Adinets & Merrill 2022):
//   1. one read of all keys builds the digit histograms of every pass;
//   2. a tiny scan turns them into global digit offsets;
//   3. per pass, one kernel: each CTA takes the next tile index from an atomic counter (so the
//      tiles it looks back on are already running), ranks its 8192 keys stably (per item, the lanes
//      holding the same digit are found with 9 ballots and a warp-private counter per digit is
//      advanced by one shared-memory atomic of the lowest such lane; the atomics of all items are
//      issued before any result is used), publishes per-digit counts, resolves its exclusive prefix
//      by decoupled look-back (kLook predecessors per round trip, bounded spin), stages the tile in
//      shared memory in digit order and writes it out in runs, so each digit's run is a contiguous
//      store.
// A status word holds a flag and a count together and nothing else is read through it, so it is
// published and polled with relaxed gpu-scope accesses (no fences); the next pass reads the keys
// this pass wrote only after the kernel boundary.
#include <atomic>

#include "common.cuh"
#include "sort.cuh"

#include <algorithm>
#include <mutex>
#include <vector>

namespace bvhgb {

namespace {

constexpr int kThreads = 512;  // histogram blocks; the onesweep tile shape is a template parameter
constexpr int kMinTile = 2048;  // smallest tile: the status arrays are sized for it
constexpr int kRadix = 256;
constexpr int kBins = kRadix + 1;  // + a bin for padding keys of the last tile
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;
// Predecessors read per look-back round trip. The tiles of a wave start together, so a tile k
// places behind the last finished one needs about k / kLook round trips.
constexpr int kLook = 16;
// Polls of an unpublished predecessor before a tile gives up and raises kErrTimeout (the tile then
// scatters with the partial prefix it has: positions below the true ones, so every write stays in
// bounds). Adjustable for tests of that path (bvhgb_sort_set_spin_limit).
__constant__ uint32_t g_lookback_spin_limit = kSpinLimit;

// The last digit may be narrower than 8 bits when (endBit - beginBit) is not a multiple of 8.
__host__ __device__ __forceinline__ uint32_t digit_mask(uint32_t shift, uint32_t endBit) {
  const uint32_t w = endBit - shift;
  return w >= 8 ? 0xFFu : ((1u << w) - 1u);
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
  size_t hist, counters, err, status, altKeys, altVals, total;
  uint32_t passes, tiles;
};

Layout make_layout(uint32_t n, uint32_t keyBytes, uint32_t beginBit, uint32_t endBit, uint32_t tile = kMinTile) {
  Layout L{};
  L.passes = (endBit > beginBit) ? (endBit - beginBit + 7) / 8 : 0;
  L.tiles = n ? (uint32_t)((n + tile - 1) / tile) : 0;
  size_t off = 0;
  L.hist = off;     off = align256(off + sizeof(uint32_t) * kRadix * (L.passes ? L.passes : 1));
  L.counters = off; off = align256(off + sizeof(uint32_t) * (L.passes ? L.passes : 1));
  L.err = off;      off = align256(off + sizeof(uint32_t));
  L.status = off;   off = align256(off + sizeof(uint32_t) * kRadix * (size_t)L.tiles * (L.passes ? L.passes : 1));
  L.altKeys = off;  off = align256(off + (size_t)keyBytes * n);
  L.altVals = off;  off = align256(off + sizeof(uint32_t) * (size_t)n);
  L.total = off;
  return L;
}

template <typename K>
__global__ void __launch_bounds__(kThreads) histogram_kernel(const K *__restrict__ keys, uint32_t n,
                                                             uint32_t beginBit, uint32_t endBit, uint32_t passes,
                                                             uint32_t *__restrict__ hist) {
  extern __shared__ uint32_t sh[];  // passes * 256
  for (uint32_t i = threadIdx.x; i < passes * kRadix; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    K k = keys[i];
    for (uint32_t p = 0; p < passes; ++p) {
      const uint32_t sh0 = beginBit + 8 * p;
      uint32_t d = (uint32_t)(k >> sh0) & digit_mask(sh0, endBit);
      atomicAdd(&sh[p * kRadix + d], 1u);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Exclusive scan of each pass's 256 counts, in place. One CTA per pass.
__global__ void __launch_bounds__(kRadix) scan_kernel(uint32_t *hist) {
  __shared__ uint32_t s[kRadix];
  uint32_t *h = hist + blockIdx.x * kRadix;
  uint32_t v = h[threadIdx.x];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < kRadix; off <<= 1) {
    uint32_t t = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0u;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  h[threadIdx.x] = s[threadIdx.x] - v;
}

template <typename K, int THREADS, int ITEMS>
struct OnesweepSmem {
  static constexpr int kWarps = THREADS / 32;
  static constexpr int kTile = THREADS * ITEMS;
  uint32_t warpHist[kWarps][kBins];
  uint32_t tileStart[kRadix];
  uint32_t globalBase[kRadix];
  uint32_t scanTot[kRadix / 32];
  uint32_t tileIdx;
  K keys[kTile];
  uint32_t vals[kTile];
};

template <typename K, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, THREADS <= 256 ? 2 : 1) onesweep_kernel(const K *__restrict__ keysIn, K *__restrict__ keysOut,
                                                            const uint32_t *__restrict__ valsIn,
                                                            uint32_t *__restrict__ valsOut, uint32_t n,
                                                            uint32_t shift, uint32_t mask,
                                                            const uint32_t *__restrict__ offsets,
                                                            uint32_t *tileCounter, uint32_t *status, uint32_t *err) {
  using Smem = OnesweepSmem<K, THREADS, ITEMS>;
  constexpr int kWarps = Smem::kWarps, kTile = Smem::kTile, kItems = ITEMS, kThreads = THREADS;
  static_assert(THREADS >= kRadix, "one thread per digit in the look-back");
  extern __shared__ __align__(16) unsigned char smraw[];
  Smem &sm = *reinterpret_cast<Smem *>(smraw);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) sm.tileIdx = atomicAdd(tileCounter, 1u);
  for (uint32_t i = lane; i < kBins; i += 32) sm.warpHist[warp][i] = 0;
  __syncthreads();
  const uint32_t tile = sm.tileIdx;
  const uint64_t base = (uint64_t)tile * kTile;
  const uint32_t valid = (uint32_t)min((uint64_t)kTile, (uint64_t)n - base);

  // Warp-striped load: warp w owns keys [w*kItems*32, (w+1)*kItems*32) of the tile.
  K key[kItems];
  uint32_t val[kItems], dig[kItems], loc[kItems];
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    uint32_t t = warp * (kItems * 32) + j * 32 + lane;
    if (t < valid) {
      key[j] = keysIn[base + t];
      val[j] = valsIn[base + t];
      dig[j] = (uint32_t)(key[j] >> shift) & mask;
    } else {
      key[j] = 0;
      val[j] = 0;
      dig[j] = kRadix;  // padding bin
    }
  }
  // Stable rank within the warp: items in order, lanes in order. Peers of an item are the lanes
  // with the same digit (9 ballots: 8 digit bits + the padding bin); the lowest of them advances
  // the warp's counter for that digit by their number. All atomics are issued first, in item
  // order (__syncwarp orders them), and their results are used afterwards.
  const uint32_t ltMask = (1u << lane) - 1u;
  uint32_t old[kItems], peersOf[kItems];
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    uint32_t peers = 0xFFFFFFFFu;
#pragma unroll
    for (int bit = 0; bit < 9; ++bit) {
      const bool on = (dig[j] >> bit) & 1u;
      const uint32_t bal = __ballot_sync(0xFFFFFFFFu, on);
      peers &= on ? bal : ~bal;
    }
    peersOf[j] = peers;
    old[j] = 0;
    if ((peers & ltMask) == 0) old[j] = atomicAdd(&sm.warpHist[warp][dig[j]], (uint32_t)__popc(peers));
    __syncwarp();
  }
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const uint32_t leader = __ffs(peersOf[j]) - 1u;
    loc[j] = __shfl_sync(0xFFFFFFFFu, old[j], leader) + __popc(peersOf[j] & ltMask);
  }
  __syncthreads();

  // Per digit (one thread each): exclusive over warps, tile count, publish, look back; the tile's
  // exclusive scan over digits runs at the same time (a warp scan per 32 digits).
  uint32_t count = 0, incl = 0;
  if (threadIdx.x < kRadix) {
    const uint32_t d = threadIdx.x;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      uint32_t c = sm.warpHist[w][d];
      sm.warpHist[w][d] = count;
      count += c;
    }
    uint32_t *st = status + (size_t)tile * kRadix + d;
    st_relaxed(st, (tile == 0 ? kFlagInc : kFlagAgg) | count);
    incl = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) sm.scanTot[warp] = incl;
    uint32_t excl = 0;
    if (tile > 0) {
      int64_t pred = (int64_t)tile - 1;
      bool done = false;
      while (!done) {
        uint32_t v[kLook];
#pragma unroll
        for (int q = 0; q < kLook; ++q) v[q] = pred - q >= 0 ? ld_relaxed(status + (size_t)(pred - q) * kRadix + d) : kFlagInc;
#pragma unroll
        for (int q = 0; q < kLook; ++q) {
          if (done) break;
          if (pred - q < 0) {
            done = true;
            break;
          }
          const uint32_t *ps = status + (size_t)(pred - q) * kRadix + d;
          uint32_t spins = 0;
          while ((v[q] & kFlagMask) == 0u) {
            if (++spins > g_lookback_spin_limit) {
              atomicOr(err, kErrTimeout);
              break;
            }
            __nanosleep(32);
            v[q] = ld_relaxed(ps);
          }
          if ((v[q] & kFlagMask) == 0u) {
            done = true;
            break;
          }
          excl += v[q] & kValMask;
          if (v[q] & kFlagInc) done = true;
        }
        pred -= kLook;
      }
      st_relaxed(st, kFlagInc | (excl + count));
    }
    sm.globalBase[d] = offsets[d] + excl;
  }
  __syncthreads();
  if (threadIdx.x < kRadix) {
    uint32_t prefix = 0;
    for (uint32_t w = 0; w < warp; ++w) prefix += sm.scanTot[w];
    sm.tileStart[threadIdx.x] = prefix + incl - count;
  }
  __syncthreads();
  // Stage the tile in digit order.
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    if (dig[j] < kRadix) {
      uint32_t pos = sm.tileStart[dig[j]] + sm.warpHist[warp][dig[j]] + loc[j];
      sm.keys[pos] = key[j];
      sm.vals[pos] = val[j];
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < valid; i += kThreads) {
    K k = sm.keys[i];
    uint32_t d = (uint32_t)(k >> shift) & mask;
    uint32_t dst = sm.globalBase[d] + (i - sm.tileStart[d]);
    // Always true for a consistent sort; after a look-back timeout (err set) a later pass reads a
    // permuted, partly stale key array whose digits no longer match the histogram, and this keeps
    // its writes inside the arrays.
    if (dst < n) {
      keysOut[dst] = k;
      valsOut[dst] = sm.vals[i];
    }
  }
}

template <typename K, int THREADS, int ITEMS>
int onesweep_passes(const Layout &L, const K *keysIn, K *keysOut, const uint32_t *valsIn, uint32_t *valsOut, K *altK,
                    uint32_t *altV, uint32_t *hist, uint32_t *counters, uint32_t *status, uint32_t *err, uint32_t n,
                    uint32_t beginBit, uint32_t endBit, cudaStream_t s) {
  const size_t smem = sizeof(OnesweepSmem<K, THREADS, ITEMS>);
  // Ping-pong so that the last pass lands in keysOut/valsOut.
  const K *srcK = keysIn;
  const uint32_t *srcV = valsIn;
  for (uint32_t p = 0; p < L.passes; ++p) {
    const bool toOut = ((L.passes - 1 - p) % 2) == 0;
    K *dstK = toOut ? keysOut : altK;
    uint32_t *dstV = toOut ? valsOut : altV;
    const uint32_t shift = beginBit + 8 * p;
    onesweep_kernel<K, THREADS, ITEMS><<<L.tiles, THREADS, smem, s>>>(
        srcK, dstK, srcV, dstV, n, shift, digit_mask(shift, endBit), hist + p * kRadix, counters + p,
        status + (size_t)p * L.tiles * kRadix, err);
    BVHGB_LAUNCH_CHECK("radix onesweep");
    srcK = dstK;
    srcV = dstV;
  }
  return BVHGB_OK;
}

std::atomic<uint32_t> g_default_tile{kSortTileDefault};

template <typename K>
int sort_impl(void *temp, uint32_t tileKeys, const K *keysIn, K *keysOut, const uint32_t *valsIn, uint32_t *valsOut,
              uint32_t n, uint32_t beginBit, uint32_t endBit, cudaStream_t s) {
  if (tileKeys == 0) tileKeys = g_default_tile.load(std::memory_order_relaxed);
  const Layout L = make_layout(n, sizeof(K), beginBit, endBit, tileKeys);
  const Layout Lmax = make_layout(n, sizeof(K), beginBit, endBit, kMinTile);  // the temp space's layout
  char *t = static_cast<char *>(temp);
  uint32_t *hist = reinterpret_cast<uint32_t *>(t + Lmax.hist);
  uint32_t *counters = reinterpret_cast<uint32_t *>(t + Lmax.counters);
  uint32_t *err = reinterpret_cast<uint32_t *>(t + Lmax.err);
  uint32_t *status = reinterpret_cast<uint32_t *>(t + Lmax.status);
  K *altK = reinterpret_cast<K *>(t + Lmax.altKeys);
  uint32_t *altV = reinterpret_cast<uint32_t *>(t + Lmax.altVals);
  if (n == 0) return BVHGB_OK;
  if (L.passes == 0) {
    BVHGB_CUDA_TRY(cudaMemcpyAsync(keysOut, keysIn, sizeof(K) * n, cudaMemcpyDeviceToDevice, s));
    BVHGB_CUDA_TRY(cudaMemcpyAsync(valsOut, valsIn, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    return BVHGB_OK;
  }
  // hist, counters, err and the status words this tile size uses start at zero
  BVHGB_CUDA_TRY(cudaMemsetAsync(t, 0, Lmax.status + sizeof(uint32_t) * kRadix * (size_t)L.tiles * L.passes, s));
  uint32_t hgrid = min(ceil_div(n, kThreads * 8), (uint32_t)sm_count() * 4);
  histogram_kernel<K><<<hgrid, kThreads, sizeof(uint32_t) * kRadix * L.passes, s>>>(keysIn, n, beginBit, endBit,
                                                                                      L.passes, hist);
  BVHGB_LAUNCH_CHECK("radix histogram");
  scan_kernel<<<L.passes, kRadix, 0, s>>>(hist);
  BVHGB_LAUNCH_CHECK("radix scan");
  int st = sort_prepare();
  if (st) return st;
  switch (tileKeys) {
    case 2048:
      return onesweep_passes<K, 256, 8>(L, keysIn, keysOut, valsIn, valsOut, altK, altV, hist, counters, status, err, n,
                                        beginBit, endBit, s);
    case 4096:
      return onesweep_passes<K, 256, 16>(L, keysIn, keysOut, valsIn, valsOut, altK, altV, hist, counters, status, err,
                                         n, beginBit, endBit, s);
    default:
      return onesweep_passes<K, 512, 16>(L, keysIn, keysOut, valsIn, valsOut, altK, altV, hist, counters, status, err,
                                         n, beginBit, endBit, s);
  }
}

template <typename K, int THREADS, int ITEMS>
cudaError_t set_smem_attr() {
  return cudaFuncSetAttribute(onesweep_kernel<K, THREADS, ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(OnesweepSmem<K, THREADS, ITEMS>));
}

}  // namespace

int sort_prepare() {
  // Opt in to more than 48 KB of dynamic shared memory. The attribute belongs to the context, so it
  // is set once per context (another device, or the context after a device reset, sets it again);
  // the first call on a context must come before any stream capture. Thread-safe.
  static std::mutex m;
  static std::vector<uint64_t> done;
  const uint64_t ctx = context_id();
  std::lock_guard<std::mutex> lock(m);
  if (ctx != 0 && std::find(done.begin(), done.end(), ctx) != done.end()) return BVHGB_OK;
  BVHGB_CUDA_TRY((set_smem_attr<uint32_t, 256, 8>()));
  BVHGB_CUDA_TRY((set_smem_attr<uint32_t, 256, 16>()));
  BVHGB_CUDA_TRY((set_smem_attr<uint32_t, 512, 16>()));
  BVHGB_CUDA_TRY((set_smem_attr<uint64_t, 256, 8>()));
  BVHGB_CUDA_TRY((set_smem_attr<uint64_t, 256, 16>()));
  BVHGB_CUDA_TRY((set_smem_attr<uint64_t, 512, 16>()));
  if (ctx != 0) done.push_back(ctx);
  return BVHGB_OK;
}

int sort_set_spin_limit(uint32_t limit, uint32_t *previous) {
  uint32_t old = 0;
  BVHGB_CUDA_TRY(cudaMemcpyFromSymbol(&old, g_lookback_spin_limit, sizeof(old)));
  const uint32_t v = limit == 0xFFFFFFFFu ? kSpinLimit : limit;
  BVHGB_CUDA_TRY(cudaMemcpyToSymbol(g_lookback_spin_limit, &v, sizeof(v)));
  if (previous) *previous = old;
  return BVHGB_OK;
}

bool sort_tile_valid(uint32_t tileKeys) { return tileKeys == 2048 || tileKeys == 4096 || tileKeys == 8192; }

size_t sort_temp_bytes(uint32_t n, uint32_t keyBytes, uint32_t beginBit, uint32_t endBit) {
  return make_layout(n, keyBytes, beginBit, endBit).total;
}

uint32_t *sort_error_word(void *temp, uint32_t n, uint32_t keyBytes, uint32_t beginBit, uint32_t endBit) {
  Layout L = make_layout(n, keyBytes, beginBit, endBit);
  return reinterpret_cast<uint32_t *>(static_cast<char *>(temp) + L.err);
}

int sort_pairs(void *temp, const void *keysIn, void *keysOut, const uint32_t *valsIn, uint32_t *valsOut, uint32_t n,
               uint32_t keyBytes, uint32_t beginBit, uint32_t endBit, cudaStream_t s, uint32_t tileKeys) {
  if (keyBytes == 4)
    return sort_impl<uint32_t>(temp, tileKeys, static_cast<const uint32_t *>(keysIn), static_cast<uint32_t *>(keysOut),
                               valsIn, valsOut, n, beginBit, endBit, s);
  return sort_impl<uint64_t>(temp, tileKeys, static_cast<const uint64_t *>(keysIn), static_cast<uint64_t *>(keysOut),
                             valsIn, valsOut, n, beginBit, endBit, s);
}


// ---- stable selection of the k smallest keys ------------------------------------------------------
//
// The first k pairs of a stable ascending sort of (keys, vals), without sorting all n: a radix
// selection finds the k-th smallest key T (three histogram passes over 11, 11 and 10 bits, each
// counting only the keys that match the digits found so far), a stable compaction keeps the keys
// below T and, of those equal to T, the first ones in index order up to k in all, and the k kept
// pairs are sorted. The compaction keeps index order, so the stable sort of the kept pairs is the
// prefix of the stable sort of all pairs.
namespace {

constexpr uint32_t kSelBins = 2048;
constexpr uint32_t kSelTile = 4096;        // keys per compaction tile (256 threads x 16)
__host__ __device__ constexpr uint32_t sel_shift(int pass) { return pass == 0 ? 21u : pass == 1 ? 10u : 0u; }
__host__ __device__ constexpr uint32_t sel_bits(int pass) { return pass == 2 ? 10u : 11u; }

struct SelState {
  uint32_t prefix;  // the digits of T found so far
  uint32_t below;   // keys below every key with that prefix
};

struct SelLayout {
  size_t state, hist, tileLt, tileEq, keys, vals, keysOut, sortTemp, total;
  uint32_t tiles;
};

SelLayout make_sel_layout(uint32_t n, uint32_t k) {
  SelLayout L{};
  auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
  L.tiles = ceil_div(max(n, 1u), kSelTile);
  size_t o = 0;
  L.state = o; o = up(o + sizeof(SelState));
  L.hist = o; o = up(o + 4ull * kSelBins);
  L.tileLt = o; o = up(o + 4ull * L.tiles);
  L.tileEq = o; o = up(o + 4ull * L.tiles);
  L.keys = o; o = up(o + 4ull * k);
  L.vals = o; o = up(o + 4ull * k);
  L.keysOut = o; o = up(o + 4ull * k);
  L.sortTemp = o; o = up(o + sort_temp_bytes(k, 4, 0, 32));
  L.total = o;
  return L;
}

// Histogram of digit 'pass' of the keys whose higher digits equal the prefix found so far (the lanes
// of a warp with the same bin add together; the block's counts go out once).
__global__ void __launch_bounds__(512) select_hist_kernel(const uint32_t *__restrict__ keys, uint32_t n,
                                                          const SelState *__restrict__ st, uint32_t *__restrict__ hist,
                                                          int pass, bool vec) {
  __shared__ uint32_t sh[kSelBins];
  for (uint32_t b = threadIdx.x; b < kSelBins; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const uint32_t shift = sel_shift(pass), mask = (1u << sel_bits(pass)) - 1u, hi = shift + sel_bits(pass);
  const uint32_t prefix = pass ? st->prefix : 0u;
  const uint32_t lane = threadIdx.x & 31u;
  // Four keys per thread and trip (one 16-byte load when the keys are 16-byte aligned).
  for (size_t base = (size_t)blockIdx.x * blockDim.x * 4; base < n; base += (size_t)gridDim.x * blockDim.x * 4) {
    const size_t i0 = base + 4 * (size_t)threadIdx.x;  // warp-uniform loop
    uint32_t k4[4];
    if (vec && i0 + 4 <= n) {
      const uint4 q = __ldg(reinterpret_cast<const uint4 *>(keys + i0));
      k4[0] = q.x;
      k4[1] = q.y;
      k4[2] = q.z;
      k4[3] = q.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) k4[j] = i0 + j < n ? __ldg(keys + i0 + j) : 0u;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint32_t bin = 0xFFFFFFFFu;
      if (i0 + j < n && (pass == 0 || (k4[j] >> hi) == prefix)) bin = (k4[j] >> shift) & mask;
      if (__ballot_sync(0xFFFFFFFFu, bin != 0xFFFFFFFFu) == 0u) continue;  // after the first pass, most warps
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, bin);
      if (bin != 0xFFFFFFFFu && (peers & ((1u << lane) - 1u)) == 0u) atomicAdd(&sh[bin], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < kSelBins; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// Block-wide exclusive sum (blocks of up to 1024 threads); *total receives the sum.
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t v, uint32_t *warpSums, uint32_t &total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, warps = (blockDim.x + 31u) >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31u) warpSums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < warps ? warpSums[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= (uint32_t)o) wi += t;
    }
    warpSums[lane] = wi - w;
    if (lane == 31u) warpSums[32] = wi;
  }
  __syncthreads();
  total = warpSums[32];
  const uint32_t r = warpSums[warp] + inc - v;
  __syncthreads();  // warpSums may be reused
  return r;
}

// The bin of digit 'pass' that holds the k-th smallest key: the prefix and the count below it
// advance; the histogram is cleared for the next pass. One block of 1024 threads, 2 bins each.
__global__ void __launch_bounds__(1024) select_find_kernel(SelState *st, uint32_t *hist, uint32_t k, int pass) {
  __shared__ uint32_t warpSums[33];
  const uint32_t b0 = 2u * threadIdx.x;
  const uint32_t h0 = hist[b0], h1 = hist[b0 + 1];
  const uint32_t below = pass ? st->below : 0u, prefix = pass ? st->prefix : 0u;
  uint32_t total;
  const uint32_t ex = block_exclusive_sum(h0 + h1, warpSums, total);
  const uint32_t need = k - below;  // rank (from 1) of the wanted key among those with the prefix
  int bin = -1;
  uint32_t exb = 0;
  if (ex < need && need <= ex + h0) {
    bin = (int)b0;
    exb = ex;
  } else if (ex + h0 < need && need <= ex + h0 + h1) {
    bin = (int)b0 + 1;
    exb = ex + h0;
  }
  __syncthreads();  // every thread has read the state
  if (bin >= 0) {
    st->prefix = (prefix << sel_bits(pass)) | (uint32_t)bin;
    st->below = below + exb;
  }
  hist[b0] = 0u;
  hist[b0 + 1] = 0u;
}

// Per tile: keys below T and keys equal to T.
__global__ void __launch_bounds__(256) select_count_kernel(const uint32_t *__restrict__ keys, uint32_t n,
                                                           const SelState *__restrict__ st, uint32_t *__restrict__ tileLt,
                                                           uint32_t *__restrict__ tileEq) {
  __shared__ uint32_t warpSums[33];
  const uint32_t T = st->prefix;
  const size_t base = (size_t)blockIdx.x * kSelTile;
  uint32_t lt = 0, eq = 0;
  for (uint32_t j = threadIdx.x; j < kSelTile; j += blockDim.x) {
    const size_t i = base + j;
    if (i < n) {
      const uint32_t key = __ldg(keys + i);
      lt += key < T ? 1u : 0u;
      eq += key == T ? 1u : 0u;
    }
  }
  uint32_t totLt, totEq;
  block_exclusive_sum(lt, warpSums, totLt);
  block_exclusive_sum(eq, warpSums, totEq);
  if (threadIdx.x == 0) {
    tileLt[blockIdx.x] = totLt;
    tileEq[blockIdx.x] = totEq;
  }
}

// Exclusive prefix of both tile counts, in place (one block, any number of tiles).
__global__ void __launch_bounds__(1024) select_scan_kernel(uint32_t *tileLt, uint32_t *tileEq, uint32_t tiles) {
  __shared__ uint32_t warpSums[33];
  uint32_t carryLt = 0, carryEq = 0;
  for (uint32_t c = 0; c < tiles; c += blockDim.x) {
    const uint32_t t = c + threadIdx.x;
    const uint32_t lt = t < tiles ? tileLt[t] : 0u, eq = t < tiles ? tileEq[t] : 0u;
    uint32_t sumLt, sumEq;
    const uint32_t exLt = block_exclusive_sum(lt, warpSums, sumLt);
    const uint32_t exEq = block_exclusive_sum(eq, warpSums, sumEq);
    if (t < tiles) {
      tileLt[t] = carryLt + exLt;
      tileEq[t] = carryEq + exEq;
    }
    carryLt += sumLt;
    carryEq += sumEq;
  }
}

// The kept pairs in index order: key < T, or key == T among the first (k - below) such keys. Each
// thread walks 16 consecutive keys; a key's place is (keys below T before it) + min(keys equal to
// T before it, k - below).
__global__ void __launch_bounds__(256) select_scatter_kernel(const uint32_t *__restrict__ keys,
                                                             const uint32_t *__restrict__ vals, uint32_t n, uint32_t k,
                                                             const SelState *__restrict__ st,
                                                             const uint32_t *__restrict__ offLt,
                                                             const uint32_t *__restrict__ offEq,
                                                             uint32_t *__restrict__ outKeys,
                                                             uint32_t *__restrict__ outVals, bool vec) {
  __shared__ uint32_t warpSums[33];
  constexpr uint32_t kPer = kSelTile / 256;
  const uint32_t T = st->prefix, need = k - st->below;
  const size_t first = (size_t)blockIdx.x * kSelTile + (size_t)threadIdx.x * kPer;
  uint32_t key[kPer];
  if (vec && first + kPer <= n) {  // 16-byte loads: keys 16-byte aligned, first a multiple of 16 keys
#pragma unroll
    for (uint32_t j = 0; j < kPer; j += 4) {
      const uint4 q = __ldg(reinterpret_cast<const uint4 *>(keys + first + j));
      key[j] = q.x;
      key[j + 1] = q.y;
      key[j + 2] = q.z;
      key[j + 3] = q.w;
    }
  } else {
#pragma unroll
    for (uint32_t j = 0; j < kPer; ++j) key[j] = first + j < n ? __ldg(keys + first + j) : 0xFFFFFFFFu;
  }
  uint32_t lt = 0, eq = 0;
#pragma unroll
  for (uint32_t j = 0; j < kPer; ++j) {
    const bool live = first + j < n;
    lt += live && key[j] < T ? 1u : 0u;
    eq += live && key[j] == T ? 1u : 0u;
  }
  uint32_t totLt, totEq;
  uint32_t ltBefore = offLt[blockIdx.x] + block_exclusive_sum(lt, warpSums, totLt);
  uint32_t eqBefore = offEq[blockIdx.x] + block_exclusive_sum(eq, warpSums, totEq);
#pragma unroll
  for (uint32_t j = 0; j < kPer; ++j) {
    if (first + j >= n) break;
    if (key[j] < T) {
      const uint32_t pos = ltBefore + min(eqBefore, need);
      if (pos < k) {  // always, unless the keys changed between the passes
        outKeys[pos] = key[j];
        outVals[pos] = __ldg(vals + first + j);
      }
      ++ltBefore;
    } else if (key[j] == T) {
      const uint32_t pos = ltBefore + eqBefore;
      if (eqBefore < need && pos < k) {
        outKeys[pos] = key[j];
        outVals[pos] = __ldg(vals + first + j);
      }
      ++eqBefore;
    }
  }
}

}  // namespace

size_t select_temp_bytes(uint32_t n, uint32_t k) { return make_sel_layout(n, min(k, n)).total; }

int select_smallest(void *temp, const uint32_t *keys, const uint32_t *vals, uint32_t n, uint32_t k, uint32_t *valsOut,
                    cudaStream_t s, uint32_t tileKeys) {
  k = min(k, n);
  if (k == 0) return BVHGB_OK;
  const SelLayout L = make_sel_layout(n, k);
  char *t = static_cast<char *>(temp);
  SelState *st = reinterpret_cast<SelState *>(t + L.state);
  uint32_t *hist = reinterpret_cast<uint32_t *>(t + L.hist);
  uint32_t *tileLt = reinterpret_cast<uint32_t *>(t + L.tileLt);
  uint32_t *tileEq = reinterpret_cast<uint32_t *>(t + L.tileEq);
  uint32_t *ck = reinterpret_cast<uint32_t *>(t + L.keys);
  uint32_t *cv = reinterpret_cast<uint32_t *>(t + L.vals);
  uint32_t *ko = reinterpret_cast<uint32_t *>(t + L.keysOut);
  if (k == n) return sort_pairs(t + L.sortTemp, keys, ko, vals, valsOut, n, 4, 0, 32, s, tileKeys);
  BVHGB_CUDA_TRY(cudaMemsetAsync(hist, 0, 4ull * kSelBins, s));
  const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0u;
  const uint32_t hgrid = min(ceil_div(n, 512u * 4u), (uint32_t)sm_count() * 4);
  for (int pass = 0; pass < 3; ++pass) {
    select_hist_kernel<<<hgrid, 512, 0, s>>>(keys, n, st, hist, pass, vec);
    BVHGB_LAUNCH_CHECK("select histogram");
    select_find_kernel<<<1, kSelBins / 2, 0, s>>>(st, hist, k, pass);
    BVHGB_LAUNCH_CHECK("select find");
  }
  select_count_kernel<<<L.tiles, 256, 0, s>>>(keys, n, st, tileLt, tileEq);
  BVHGB_LAUNCH_CHECK("select count");
  select_scan_kernel<<<1, 1024, 0, s>>>(tileLt, tileEq, L.tiles);
  BVHGB_LAUNCH_CHECK("select scan");
  select_scatter_kernel<<<L.tiles, 256, 0, s>>>(keys, vals, n, k, st, tileLt, tileEq, ck, cv, vec);
  BVHGB_LAUNCH_CHECK("select scatter");
  // A few hundred thousand kept pairs fill few CTAs at the large tiles: the smallest tile spreads
  // them wider (the order does not depend on the tile).
  if (tileKeys == 0 && k <= (1u << 18)) tileKeys = 2048;
  return sort_pairs(t + L.sortTemp, ck, ko, cv, valsOut, k, 4, 0, 32, s, tileKeys);
}

}  // namespace bvhgb

extern "C" BVHGB_API int bvhgb_radix_sort_pairs(void *temp, size_t *tempBytes, const void *keysIn, void *keysOut,
                                                const uint32_t *valsIn, uint32_t *valsOut, uint32_t n,
                                                uint32_t keyBytes, uint32_t beginBit, uint32_t endBit,
                                                bvhgb_stream stream) {
  if (!tempBytes || (keyBytes != 4 && keyBytes != 8) || beginBit > endBit || endBit > 8 * keyBytes)
    return BVHGB_INVALID_ARGUMENT;
  if (n >= (1u << 30)) return BVHGB_TOO_LARGE;
  size_t need = bvhgb::sort_temp_bytes(n, keyBytes, beginBit, endBit);
  if (!temp) {
    *tempBytes = need;
    return BVHGB_OK;
  }
  if (*tempBytes < need || (n && (!keysIn || !keysOut || !valsIn || !valsOut))) return BVHGB_INVALID_ARGUMENT;
  return bvhgb::sort_pairs(temp, keysIn, keysOut, valsIn, valsOut, n, keyBytes, beginBit, endBit,
                           bvhgb::as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_select_smallest_pairs(void *temp, size_t *tempBytes, const uint32_t *keys,
                                                     const uint32_t *vals, uint32_t *valsOut, uint32_t n, uint32_t k,
                                                     bvhgb_stream stream) {
  if (!tempBytes || k > n) return BVHGB_INVALID_ARGUMENT;
  if (n >= (1u << 30)) return BVHGB_TOO_LARGE;
  const size_t need = bvhgb::select_temp_bytes(n, k);
  if (!temp) {
    *tempBytes = need;
    return BVHGB_OK;
  }
  if (*tempBytes < need || (k && (!keys || !vals || !valsOut))) return BVHGB_INVALID_ARGUMENT;
  return bvhgb::select_smallest(temp, keys, vals, n, k, valsOut, bvhgb::as_stream(stream));
}

extern "C" BVHGB_API int bvhgb_sort_set_default_tile(uint32_t tileKeys, uint32_t *previous) {
  if (tileKeys != 0 && !bvhgb::sort_tile_valid(tileKeys)) return BVHGB_INVALID_ARGUMENT;
  const uint32_t old = tileKeys ? bvhgb::g_default_tile.exchange(tileKeys) : bvhgb::g_default_tile.load();
  if (previous) *previous = old;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_sort_set_spin_limit(uint32_t limit, uint32_t *previous) {
  return bvhgb::sort_set_spin_limit(limit, previous);
}
