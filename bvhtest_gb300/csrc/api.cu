// Library-wide host helpers, SAH reduction and the transfer entry points
// (lib/cuda/cudaFN.cu:32-187, lib/builder/Bittner13CUDA.cu:776-803, lib/base/BVH.cpp:23-70).
#include <atomic>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace bvhgb {

namespace {
thread_local char g_last_error[512] = "";
std::atomic<uint64_t> g_launches{0};
}  // namespace

void set_last_error(const char *what, cudaError_t e) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(what, e);
    return BVHGB_CUDA_ERROR;
  }
  return BVHGB_OK;
}

void count_launch(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
// Launches recorded while a stream was being captured did not run; the capture takes them back and
// every replay of the graph adds its kernel count instead.
void uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

// Identity of the CUDA context current on this thread: the driver's context ID, unique within the
// process, so a context made after a cudaDeviceReset never matches one cached before it. 0 when
// there is no current context or the driver does not report one.
uint64_t context_id() {
  typedef int (*CtxGetCurrent)(void **);
  typedef int (*CtxGetId)(void *, unsigned long long *);
  static CtxGetCurrent getCurrent = nullptr;
  static CtxGetId getId = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess)
      getCurrent = reinterpret_cast<CtxGetCurrent>(a);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess)
      getId = reinterpret_cast<CtxGetId>(b);
    cudaGetLastError();
  });
  if (!getCurrent || !getId) return 0;
  void *ctx = nullptr;
  if (getCurrent(&ctx) != 0) return 0;
  if (!ctx) {
    // No context on this thread yet (so no stream capture either): let the runtime make its
    // context current, then ask again.
    cudaFree(nullptr);
    if (getCurrent(&ctx) != 0 || !ctx) return 0;
  }
  unsigned long long id = 0;
  if (getId(ctx, &id) != 0) return 0;
  return (uint64_t)id;
}

// Allocation-failure injection for tests of the error paths: after g_alloc_budget more successful
// allocations the next one fails as if the device were out of memory (-1: off).
std::atomic<int64_t> g_alloc_budget{-1};

cudaError_t dev_malloc(void **p, size_t bytes) {
  int64_t b = g_alloc_budget.load(std::memory_order_relaxed);
  while (b >= 0) {
    if (b == 0) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
    if (g_alloc_budget.compare_exchange_weak(b, b - 1, std::memory_order_relaxed)) break;
  }
  return cudaMalloc(p, bytes);
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 148;
  return n;
}

namespace {
constexpr int kSahThreads = 256;
constexpr int kSahBlocks = 304;

// Deterministic SAH: fixed grid, fixed per-block tree order, fixed final order, all in double.
__global__ void __launch_bounds__(kSahThreads) sah_partial_kernel(const bvhgb_node *__restrict__ nodes, uint32_t n,
                                                                  uint32_t root, double *partial) {
  double s = 0.0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (i != root) s += (double)__ldg(&nodes[i].surfaceArea);
  __shared__ double red[kSahThreads];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = kSahThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < (unsigned)o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void sah_final_kernel(const bvhgb_node *nodes, uint32_t root, const double *partial, int np, double *out) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < np; ++i) s += partial[i];
  out[0] = s / (double)nodes[root].surfaceArea;
}
}  // namespace

}  // namespace bvhgb

using namespace bvhgb;

extern "C" BVHGB_API const char *bvhgb_version(void) { return "bvhgb 0.1 (sm_103a)"; }

extern "C" BVHGB_API const char *bvhgb_status_string(int s) {
  switch (s) {
    case BVHGB_OK: return "OK";
    case BVHGB_WARNING: return "WARNING";
    case BVHGB_IO_ERROR: return "IO_ERROR";
    case BVHGB_PARSE_ERROR: return "PARSE_ERROR";
    case BVHGB_BVH_ERROR: return "BVH_ERROR";
    case BVHGB_GL_ERROR: return "GL_ERROR";
    case BVHGB_CUDA_ERROR: return "CUDA_ERROR";
    case BVHGB_GENERIC_ERROR: return "GENERIC_ERROR";
    case BVHGB_INVALID_ARGUMENT: return "INVALID_ARGUMENT";
    case BVHGB_DEVICE_TIMEOUT: return "DEVICE_TIMEOUT";
    case BVHGB_OUT_OF_MEMORY: return "OUT_OF_MEMORY";
    case BVHGB_TOO_LARGE: return "TOO_LARGE";
    default: return "UNKNOWN";
  }
}

extern "C" BVHGB_API const char *bvhgb_last_error(void) { return g_last_error; }
extern "C" BVHGB_API uint64_t bvhgb_launch_count(void) { return g_launches.load(); }

extern "C" BVHGB_API int bvhgb_debug_fail_allocations(int64_t after, int64_t *previous) {
  const int64_t old = g_alloc_budget.exchange(after < 0 ? -1 : after, std::memory_order_relaxed);
  if (previous) *previous = old;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_reset_device(void) {
  // Cached per-context state (shared-memory opt-ins, symbol addresses) is keyed by context_id(),
  // so the context made after this reset looks it all up again.
  BVHGB_CUDA_TRY(cudaDeviceReset());
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_device_sync(void) {
  BVHGB_CUDA_TRY(cudaDeviceSynchronize());
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_calc_sah(const bvhgb_node *nodes, uint32_t n, uint32_t root, double *sah,
                                       bvhgb_stream stream) {
  if (!nodes || !sah || n == 0 || root >= n) return BVHGB_INVALID_ARGUMENT;
  cudaStream_t s = as_stream(stream);
  double *buf = nullptr;
  BVHGB_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * (kSahBlocks + 1), s));
  sah_partial_kernel<<<kSahBlocks, kSahThreads, 0, s>>>(nodes, n, root, buf);
  count_launch();
  sah_final_kernel<<<1, 32, 0, s>>>(nodes, root, buf, kSahBlocks, buf + kSahBlocks);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(sah, buf + kSahBlocks, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(buf, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_calc_sah", e);
    return BVHGB_CUDA_ERROR;
  }
  return BVHGB_OK;
}

// ---- transfer (cudaFN.cu) -------------------------------------------------------------------

extern "C" BVHGB_API int bvhgb_copy_mesh_to_gpu(const float *vert, uint32_t numVert, const float *norm, uint32_t numNorm,
                                                const uint32_t *faces, uint32_t numFaces, bvhgb_mesh_raw *out) {
  if (!out || (numVert && !vert) || (numNorm && !norm) || (numFaces && !faces)) return BVHGB_INVALID_ARGUMENT;
  bvhgb_mesh_raw m{};
  cudaError_t e = cudaSuccess;
  size_t vb = 12ull * numVert, nb = 12ull * numNorm, fb = 12ull * numFaces;
  if (e == cudaSuccess) e = dev_malloc(&m.vert, vb ? vb : 16);
  if (e == cudaSuccess) e = dev_malloc(&m.norm, nb ? nb : 16);
  if (e == cudaSuccess) e = dev_malloc(&m.faces, fb ? fb : 16);
  if (e == cudaSuccess && vb) e = cudaMemcpy(m.vert, vert, vb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nb) e = cudaMemcpy(m.norm, norm, nb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && fb) e = cudaMemcpy(m.faces, faces, fb, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_copy_mesh_to_gpu", e);
    cudaFree(m.vert);
    cudaFree(m.norm);
    cudaFree(m.faces);
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  m.numVert = numVert;
  m.numNorm = numNorm;
  m.numFaces = numFaces;
  *out = m;
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_free_mesh(bvhgb_mesh_raw *mesh) {
  if (!mesh) return BVHGB_INVALID_ARGUMENT;
  cudaFree(mesh->vert);
  cudaFree(mesh->norm);
  cudaFree(mesh->faces);
  *mesh = bvhgb_mesh_raw{};
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_copy_mesh_to_host(bvhgb_mesh_raw *mesh, float *vert, float *norm, uint32_t *faces) {
  if (!mesh || !mesh->vert || !mesh->faces) return BVHGB_INVALID_ARGUMENT;
  cudaError_t e = cudaSuccess;
  if (vert && mesh->numVert) e = cudaMemcpy(vert, mesh->vert, 12ull * mesh->numVert, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && norm && mesh->numNorm) e = cudaMemcpy(norm, mesh->norm, 12ull * mesh->numNorm, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && faces && mesh->numFaces) e = cudaMemcpy(faces, mesh->faces, 12ull * mesh->numFaces, cudaMemcpyDeviceToHost);
  bvhgb_free_mesh(mesh);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_copy_mesh_to_host", e);
    return BVHGB_CUDA_ERROR;
  }
  return BVHGB_OK;
}

static int make_device_bvh(bvhgb_bvh_pointer *out, uint32_t numNodes, uint32_t root, uint16_t maxLevel) {
  bvhgb_device_bvh img{};
  img.bvh = out->nodes;
  img.vSize = numNodes;
  img.vCapacity = numNodes;
  img.vRootIndex = root;
  img.vMaxLevel = maxLevel;
  BVHGB_CUDA_TRY(dev_malloc(&out->bvh, sizeof(bvhgb_device_bvh)));
  BVHGB_CUDA_TRY(cudaMemcpy(out->bvh, &img, sizeof(img), cudaMemcpyHostToDevice));
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_free_bvh(bvhgb_bvh_pointer *ptr) {
  if (!ptr) return BVHGB_INVALID_ARGUMENT;
  cudaFree(ptr->nodes);
  cudaFree(ptr->bvh);
  *ptr = bvhgb_bvh_pointer{};
  return BVHGB_OK;
}

extern "C" BVHGB_API int bvhgb_copy_bvh_to_gpu(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, uint16_t maxLevel,
                                               bvhgb_bvh_pointer *out) {
  if (!out) return BVHGB_INVALID_ARGUMENT;
  *out = bvhgb_bvh_pointer{};
  if (numNodes == 0) return BVHGB_OK;
  if (!nodes || root >= numNodes) return BVHGB_INVALID_ARGUMENT;
  cudaError_t e = dev_malloc(&out->nodes, sizeof(bvhgb_node) * (size_t)numNodes);
  if (e == cudaSuccess) e = cudaMemcpy(out->nodes, nodes, sizeof(bvhgb_node) * (size_t)numNodes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_copy_bvh_to_gpu", e);
    bvhgb_free_bvh(out);
    return BVHGB_CUDA_ERROR;
  }
  out->numNodes = numNodes;
  int st = make_device_bvh(out, numNodes, root, maxLevel);
  if (st) bvhgb_free_bvh(out);
  return st;
}

extern "C" BVHGB_API int bvhgb_allocate_bvh(bvhgb_bvh_pointer *out, uint32_t numFaces) {
  if (!out || numFaces == 0) return BVHGB_INVALID_ARGUMENT;
  if (out->bvh || out->nodes) return BVHGB_BVH_ERROR;  // LBVH_CUDA.cu:400
  if (numFaces >= (1u << 30)) return BVHGB_TOO_LARGE;
  uint32_t numNodes = 2 * numFaces - 1;
  cudaError_t e = dev_malloc(&out->nodes, sizeof(bvhgb_node) * (size_t)numNodes);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_allocate_bvh", e);
    out->nodes = nullptr;
    return e == cudaErrorMemoryAllocation ? BVHGB_OUT_OF_MEMORY : BVHGB_CUDA_ERROR;
  }
  out->numNodes = numNodes;
  int st = make_device_bvh(out, numNodes, 0, 0);
  if (st) bvhgb_free_bvh(out);
  return st;
}

extern "C" BVHGB_API int bvhgb_copy_bvh_to_host(bvhgb_bvh_pointer *ptr, bvhgb_node *nodes, uint32_t capacity,
                                                uint32_t *root, uint16_t *maxLevel) {
  if (!ptr || !ptr->bvh || !ptr->nodes || !nodes) return BVHGB_INVALID_ARGUMENT;
  if (capacity < ptr->numNodes) return BVHGB_INVALID_ARGUMENT;
  bvhgb_device_bvh img{};
  cudaError_t e = cudaMemcpy(&img, ptr->bvh, sizeof(img), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nodes, ptr->nodes, sizeof(bvhgb_node) * (size_t)ptr->numNodes, cudaMemcpyDeviceToHost);
  if (root) *root = img.vRootIndex;
  if (maxLevel) *maxLevel = img.vMaxLevel;
  bvhgb_free_bvh(ptr);
  if (e != cudaSuccess) {
    set_last_error("bvhgb_copy_bvh_to_host", e);
    return BVHGB_CUDA_ERROR;
  }
  return BVHGB_OK;
}

// BVH::fixLevels (lib/base/BVH.cpp:39-70), host side.
extern "C" BVHGB_API int bvhgb_fix_levels_host(bvhgb_node *nodes, uint32_t n, uint32_t root, uint16_t *maxLevel) {
  if (!nodes || n == 0 || root >= n) return BVHGB_INVALID_ARGUMENT;
  std::vector<uint32_t> st;
  st.reserve(128);
  uint16_t mx = 0;
  nodes[root].level = 0;
  st.push_back(root);
  size_t visited = 0;
  while (!st.empty()) {
    uint32_t x = st.back();
    st.pop_back();
    if (++visited > n) return BVHGB_BVH_ERROR;  // cycle
    if (nodes[x].level > mx) mx = nodes[x].level;
    if (!nodes[x].isLeafFlag) {
      uint32_t l = nodes[x].left, r = nodes[x].right;
      if (l >= n || r >= n) return BVHGB_BVH_ERROR;
      nodes[l].level = (uint16_t)(nodes[x].level + 1);
      nodes[r].level = (uint16_t)(nodes[x].level + 1);
      st.push_back(r);
      st.push_back(l);
    }
  }
  if (maxLevel) *maxLevel = mx;
  return BVHGB_OK;
}
