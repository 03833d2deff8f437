// The reference's GPU entry points under their own names (include/bvhtest_compat.h), implemented on
// the bvhgb_* C ABI. Each function cites the reference function whose contract it keeps.
#include "bvhtest_compat.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <cuda_runtime_api.h>

#include "bvhgb.h"

using BVHTest::base::AABB;
using BVHTest::base::BVH;
using BVHTest::base::BVHNode;
using BVHTest::base::CompatVec3;
using BVHTest::base::CUDAMemoryBVHPointer;
using BVHTest::base::Mesh;
using BVHTest::base::MeshRaw;
using BVHTest::base::Ray;
using BVHTest::base::Triangle;

static_assert(sizeof(BVHNode) == sizeof(bvhgb_node), "node layout");
static_assert(sizeof(MeshRaw) == sizeof(bvhgb_mesh_raw), "mesh layout");
static_assert(sizeof(CUDAMemoryBVHPointer) == sizeof(bvhgb_bvh_pointer), "bvh pointer layout");
static_assert(sizeof(BVH) == sizeof(bvhgb_device_bvh), "device BVH layout");
static_assert(sizeof(CUDAPixel) == sizeof(bvhgb_pixel), "pixel layout");
static_assert(sizeof(AlgoCFG) == 20, "AlgoCFG layout");
static_assert(sizeof(LBVH_WorkingMemory) == 80, "LBVH_WorkingMemory layout");

namespace {

// The reference reports CUDA failures on stdout and carries on (LBVH_CUDA.cu:29-34,
// Bittner13CUDA.cu:33-53); here the message goes to stderr with the library's own detail.
bool ok(int status, const char *where) {
  if (status == BVHGB_OK) return true;
  std::fprintf(stderr, "[bvhgb] %s: %s (%s)\n", where, bvhgb_status_string(status), bvhgb_last_error());
  return false;
}

struct LbvhHandle {
  bvhgb_lbvh_workspace *ws = nullptr;
  const float *vert = nullptr;
  const uint32_t *faces = nullptr;
  uint32_t numFaces = 0;
};

LbvhHandle *lbvh(LBVH_WorkingMemory *m) { return m ? static_cast<LbvhHandle *>(m->cubTempStorage) : nullptr; }

struct Bn13Handle {
  bvhgb_bn13_workspace *ws = nullptr;
  bvhgb_node *nodes = nullptr;  // the tree the workspace was made for
  uint32_t numNodes = 0;
  uint32_t chunkSize = 0;
  uint32_t numFaces = 0;
  AlgoCFG cfg{};
  bool haveCfg = false;
};

Bn13Handle *bn13(GPUWorkingMemory *m) { return m ? static_cast<Bn13Handle *>(m->cubSortTempStorage) : nullptr; }

bool same_cfg(const AlgoCFG &a, const AlgoCFG &b) {
  return a.numChunks == b.numChunks && a.chunkSize == b.chunkSize && a.blockSize == b.blockSize &&
         a.offsetAccess == b.offsetAccess && a.altFindNode == b.altFindNode;
}

uint32_t root_of(const CUDAMemoryBVHPointer *p) {
  bvhgb_device_bvh img{};
  if (!p || !p->bvh || cudaMemcpy(&img, p->bvh, sizeof(img), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
  return img.vRootIndex;
}

// The optimizer workspace for this configuration and tree, (re)made when either changed
// (allocateMemory + initData, Bittner13CUDA.cu:836-987).
bool bn13_ready(GPUWorkingMemory *data, CUDAMemoryBVHPointer *bvh, const AlgoCFG &cfg) {
  Bn13Handle *h = bn13(data);
  if (!h || !bvh || !bvh->nodes) return false;
  if (h->ws && h->haveCfg && same_cfg(h->cfg, cfg) && h->nodes == reinterpret_cast<bvhgb_node *>(bvh->nodes) &&
      h->numNodes == bvh->numNodes)
    return true;
  if (h->ws) bvhgb_bn13_destroy(h->ws);
  h->ws = nullptr;
  bvhgb_bn13_config c{};
  c.numChunks = cfg.numChunks ? cfg.numChunks : 1;
  c.blockSize = cfg.blockSize;
  c.batchPercent = 1.0f;
  c.offsetAccess = cfg.offsetAccess ? 1u : 0u;
  c.heapCapacity = 4096;  // CUDA_QUEUE_SIZE (Bittner13CUDA.hpp:29)
  c.searchMode = cfg.altFindNode ? BVHGB_SEARCH_ALT : BVHGB_SEARCH_BATCHED;  // findNode2 or the batched search
  c.chunkSize = cfg.chunkSize ? cfg.chunkSize : h->chunkSize;
  if (!ok(bvhgb_bn13_create(reinterpret_cast<bvhgb_node *>(bvh->nodes), bvh->numNodes, root_of(bvh), &c, &h->ws,
                            nullptr),
          "bn13 workspace"))
    return false;
  h->nodes = reinterpret_cast<bvhgb_node *>(bvh->nodes);
  h->numNodes = bvh->numNodes;
  h->cfg = cfg;
  h->haveCfg = true;
  return true;
}

AlgoCFG default_cfg(const Bn13Handle *h) {
  AlgoCFG c;
  c.numChunks = 32;
  c.chunkSize = h->chunkSize;
  c.blockSize = 128;
  c.offsetAccess = c.altFindNode = c.altFixTree = c.altSort = false;
  c.sort = true;
  c.localPatchCPY = true;
  return c;
}

}  // namespace

// ---- LBVH ----------------------------------------------------------------------------------

// LBVH_allocateWorkingMemory (LBVH_CUDA.cu:426-475): lRes reports success.
LBVH_WorkingMemory LBVH_allocateWorkingMemory(MeshRaw *_rawMesh) {
  LBVH_WorkingMemory m;
  if (!_rawMesh) return m;
  auto *h = new LbvhHandle();
  const bvhgb_lbvh_config cfg{30u, BVHGB_TOPO_REFCOMPAT};
  if (!ok(bvhgb_lbvh_create(_rawMesh->numFaces, &cfg, &h->ws), "LBVH_allocateWorkingMemory")) {
    delete h;
    return m;
  }
  h->vert = reinterpret_cast<const float *>(_rawMesh->vert);
  h->faces = reinterpret_cast<const uint32_t *>(_rawMesh->faces);
  h->numFaces = _rawMesh->numFaces;
  m.cubTempStorage = h;
  m.numFaces = _rawMesh->numFaces;
  m.numLocks = _rawMesh->numFaces;
  m.lRes = true;
  return m;
}

// LBVH_freeWorkingMemory (LBVH_CUDA.cu:477-488).
void LBVH_freeWorkingMemory(LBVH_WorkingMemory *_mem) {
  LbvhHandle *h = lbvh(_mem);
  if (!h) return;
  bvhgb_lbvh_destroy(h->ws);
  delete h;
  *_mem = LBVH_WorkingMemory();
}

// LBVH_allocateBVH (LBVH_CUDA.cu:396-424): fails when _bvh already holds a tree.
bool LBVH_allocateBVH(CUDAMemoryBVHPointer *_bvh, MeshRaw *_rawMesh) {
  if (!_bvh || !_rawMesh) return false;
  return ok(bvhgb_allocate_bvh(reinterpret_cast<bvhgb_bvh_pointer *>(_bvh), _rawMesh->numFaces), "LBVH_allocateBVH");
}

// LBVH_initTriData (LBVH_CUDA.cu:98-119): per-triangle boxes reduced into the scene box, which is
// returned (the call waits for it, as the reference's read-back does).
AABB LBVH_initTriData(LBVH_WorkingMemory *_mem, MeshRaw *_rawMesh) {
  AABB box{};
  LbvhHandle *h = lbvh(_mem);
  if (!h || !_rawMesh) return box;
  h->vert = reinterpret_cast<const float *>(_rawMesh->vert);
  h->faces = reinterpret_cast<const uint32_t *>(_rawMesh->faces);
  h->numFaces = _rawMesh->numFaces;
  if (!ok(bvhgb_lbvh_init_tri_data(h->ws, h->vert, h->faces, h->numFaces, nullptr), "LBVH_initTriData")) {
    _mem->lRes = false;
    return box;
  }
  bvhgb_aabb b{};
  if (!ok(bvhgb_lbvh_read_scene_box(h->ws, &b, nullptr), "LBVH_initTriData")) {
    _mem->lRes = false;
    return box;
  }
  std::memcpy(&box, &b, sizeof(box));
  return box;
}

// LBVH_calcMortonCodes (LBVH_CUDA.cu:168-183): codes normalised by the given scene box.
void LBVH_calcMortonCodes(LBVH_WorkingMemory *_mem, AABB _sceneAABB) {
  LbvhHandle *h = lbvh(_mem);
  if (!h) return;
  bvhgb_aabb b;
  std::memcpy(&b, &_sceneAABB, sizeof(b));
  if (!ok(bvhgb_lbvh_set_scene_box(h->ws, &b, nullptr), "LBVH_calcMortonCodes") ||
      !ok(bvhgb_lbvh_calc_morton(h->ws, h->vert, h->faces, h->numFaces, nullptr), "LBVH_calcMortonCodes"))
    _mem->lRes = false;
}

// LBVH_sortMortonCodes (LBVH_CUDA.cu:185-193).
void LBVH_sortMortonCodes(LBVH_WorkingMemory *_mem) {
  LbvhHandle *h = lbvh(_mem);
  if (!h) return;
  if (!ok(bvhgb_lbvh_sort(h->ws, h->numFaces, nullptr), "LBVH_sortMortonCodes")) _mem->lRes = false;
}

// LBVH_buildBVHTree (LBVH_CUDA.cu:273-329): leaves and inner nodes; the fused kernel also fits the
// boxes bottom up, which is what LBVH_fixAABB does in the reference.
void LBVH_buildBVHTree(LBVH_WorkingMemory *_mem, CUDAMemoryBVHPointer *_bvh) {
  LbvhHandle *h = lbvh(_mem);
  if (!h || !_bvh || !_bvh->nodes) return;
  if (!ok(bvhgb_lbvh_build_tree(h->ws, h->vert, h->faces, h->numFaces, reinterpret_cast<bvhgb_node *>(_bvh->nodes),
                                nullptr),
          "LBVH_buildBVHTree"))
    _mem->lRes = false;
}

// LBVH_fixAABB (LBVH_CUDA.cu:376-385): the boxes were fitted by LBVH_buildBVHTree's fused kernel.
void LBVH_fixAABB(LBVH_WorkingMemory *_mem, CUDAMemoryBVHPointer *_bvh) {
  (void)_mem;
  (void)_bvh;
}

// LBVH_doCUDASyc (LBVH_CUDA.cu:490).
void LBVH_doCUDASyc() { ok(bvhgb_device_sync(), "LBVH_doCUDASyc"); }

// ---- Bittner13 -----------------------------------------------------------------------------

// allocateMemory (Bittner13CUDA.cu:836-900): _batchSize is the chunk size. The device workspace is
// made by initData (or the first step) from the tree it is given.
GPUWorkingMemory allocateMemory(CUDAMemoryBVHPointer *_bvh, uint32_t _batchSize, uint32_t _numFaces) {
  GPUWorkingMemory m{};
  m.result = false;
  if (!_bvh || !_bvh->nodes || _bvh->numNodes == 0) return m;
  auto *h = new Bn13Handle();
  h->chunkSize = _batchSize;
  h->numFaces = _numFaces;
  m.cubSortTempStorage = h;
  m.numPatches = _batchSize;
  m.numNodesToFix = 3 * _batchSize;
  m.numFlags = _bvh->numNodes;
  m.numLeafNodes = _numFaces;
  m.numInnerNodes = _numFaces ? _numFaces - 1 : 0;
  m.result = true;
  return m;
}

// freeMemory (Bittner13CUDA.cu:902-937).
void freeMemory(GPUWorkingMemory *_data) {
  Bn13Handle *h = bn13(_data);
  if (!h) return;
  if (h->ws) bvhgb_bn13_destroy(h->ws);
  delete h;
  *_data = GPUWorkingMemory{};
}

// initData (Bittner13CUDA.cu:939-987): the inner-node list of the tree, with the default options
// until the first step brings its AlgoCFG.
void initData(GPUWorkingMemory *_data, CUDAMemoryBVHPointer *_GPUbvh, uint32_t _blockSize) {
  Bn13Handle *h = bn13(_data);
  if (!h) return;
  AlgoCFG c = default_cfg(h);
  c.blockSize = _blockSize;
  if (!bn13_ready(_data, _GPUbvh, c)) _data->result = false;
}

// fixTree1 (Bittner13CUDA.cu:641-648): refit of every inner node from the leaves.
void fixTree1(GPUWorkingMemory *_data, CUDAMemoryBVHPointer *_GPUbvh, uint32_t _blockSize) {
  (void)_blockSize;
  Bn13Handle *h = bn13(_data);
  if (!h || !_GPUbvh) return;
  if (!h->ws && !bn13_ready(_data, _GPUbvh, default_cfg(h))) return;
  ok(bvhgb_bn13_refit(h->ws, reinterpret_cast<bvhgb_node *>(_GPUbvh->nodes), nullptr), "fixTree1");
}

// fixTree3 (Bittner13CUDA.cu:650-656): the reference refits the paths above its fix list; the
// chunks here refit their own paths, so a call from outside refits the whole tree (a superset).
void fixTree3(GPUWorkingMemory *_data, CUDAMemoryBVHPointer *_GPUbvh, uint32_t _blockSize) {
  fixTree1(_data, _GPUbvh, _blockSize);
}

// bn13_selectNodes (Bittner13CUDA.cu:659-726).
void bn13_selectNodes(GPUWorkingMemory *_data, CUDAMemoryBVHPointer *_GPUbvh, AlgoCFG _cfg) {
  if (!bn13_ready(_data, _GPUbvh, _cfg)) return;
  ok(bvhgb_bn13_select_nodes(bn13(_data)->ws, reinterpret_cast<bvhgb_node *>(_GPUbvh->nodes), nullptr),
     "bn13_selectNodes");
}

// bn13_rmAndReinsChunk (Bittner13CUDA.cu:729-766): removal, reinsertion, conflicts, apply, refit.
void bn13_rmAndReinsChunk(GPUWorkingMemory *_data, CUDAMemoryBVHPointer *_GPUbvh, AlgoCFG _cfg, uint32_t _chunk) {
  if (!bn13_ready(_data, _GPUbvh, _cfg)) return;
  ok(bvhgb_bn13_chunk(bn13(_data)->ws, reinterpret_cast<bvhgb_node *>(_GPUbvh->nodes), _chunk, nullptr),
     "bn13_rmAndReinsChunk");
}

// bn13_doAlgorithmStep (Bittner13CUDA.cu:768-772): selection and every chunk of one iteration.
void bn13_doAlgorithmStep(GPUWorkingMemory *_data, CUDAMemoryBVHPointer *_GPUbvh, AlgoCFG _cfg) {
  if (!bn13_ready(_data, _GPUbvh, _cfg)) return;
  ok(bvhgb_bn13_step(bn13(_data)->ws, reinterpret_cast<bvhgb_node *>(_GPUbvh->nodes), nullptr),
     "bn13_doAlgorithmStep");
}

// CUDAcalcSAH (Bittner13CUDA.cu:776-803): cInner = cLeaf = 1, over the tree's own root.
float CUDAcalcSAH(CUDAMemoryBVHPointer *_GPUbvh) {
  if (!_GPUbvh || !_GPUbvh->nodes || _GPUbvh->numNodes == 0) return 0.0f;
  double sah = 0.0;
  if (!ok(bvhgb_calc_sah(reinterpret_cast<bvhgb_node *>(_GPUbvh->nodes), _GPUbvh->numNodes, root_of(_GPUbvh), &sah,
                         nullptr),
          "CUDAcalcSAH"))
    return 0.0f;
  return (float)sah;
}

// doCudaDevSync (Bittner13CUDA.cu:822-824).
void doCudaDevSync() { ok(bvhgb_device_sync(), "doCudaDevSync"); }

// calcNumSkipped (Bittner13CUDA.cu:806-821): batch items that were not applied.
uint32_t calcNumSkipped(GPUWorkingMemory *_data) {
  Bn13Handle *h = bn13(_data);
  if (!h || !h->ws) return 0;
  bvhgb_bn13_stats st{};
  if (!ok(bvhgb_bn13_get_stats(h->ws, &st, nullptr), "calcNumSkipped")) return 0;
  return (uint32_t)(st.skippedConflict + st.skippedInvalid);
}

// ---- tracer and transfer (C linkage) -------------------------------------------------------

extern "C" {

// allocateRays / allocateImage / freeRays / freeImage (CUDAKernels.cu:425-470).
bool allocateRays(Ray **_rays, uint32_t _num) {
  if (!_rays) return false;
  *_rays = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(_rays), sizeof(Ray) * (size_t)(_num ? _num : 1));
  if (e != cudaSuccess) {
    std::fprintf(stderr, "[bvhgb] allocateRays: %s\n", cudaGetErrorString(e));
    *_rays = nullptr;
    return false;
  }
  return true;
}

bool allocateImage(CUDAPixel **_img, uint32_t _w, uint32_t _h) {
  if (!_img) return false;
  *_img = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(_img), sizeof(CUDAPixel) * (size_t)_w * _h + 16);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "[bvhgb] allocateImage: %s\n", cudaGetErrorString(e));
    *_img = nullptr;
    return false;
  }
  return true;
}

void freeRays(Ray **_rays) {
  if (!_rays || !*_rays) return;
  cudaFree(*_rays);
  *_rays = nullptr;
}

void freeImage(CUDAPixel *_img) {
  if (_img) cudaFree(_img);
}

// generateRays (CUDAKernels.cu:386-397).
void generateRays(Ray *_rays, uint32_t _w, uint32_t _h, CompatVec3 _pos, CompatVec3 _lookAt, CompatVec3 _up,
                  float _fov) {
  if (!_rays) return;
  bvhgb_camera cam{{_pos.x, _pos.y, _pos.z}, {_lookAt.x, _lookAt.y, _lookAt.z}, {_up.x, _up.y, _up.z}, _fov, _w, _h};
  ok(bvhgb_generate_rays(_rays, &cam, nullptr), "generateRays");
}

// tracerImage (CUDAKernels.cu:399-417): front faces only when the library is asked for the
// reference's compile-time culling (CUDA_FACE_CULLING, on by default in the reference's build
// options); BVHGB_COMPAT_TWO_SIDED=1 in the environment traces both sides.
void tracerImage(Ray *_rays, CUDAPixel *_img, BVHNode *_nodes, uint32_t _rootNode, MeshRaw _mesh, CompatVec3 _light,
                 uint32_t _w, uint32_t _h, bool _bundle) {
  if (!_rays || !_img || !_nodes || _mesh.numFaces == 0) return;
  const char *two = std::getenv("BVHGB_COMPAT_TWO_SIDED");
  bvhgb_trace_config cfg{{_light.x, _light.y, _light.z}, (two && two[0] == '1') ? 0u : 1u, 0.0f, INFINITY,
                         _bundle ? 1u : 0u};
  const uint32_t numNodes = 2 * _mesh.numFaces - 1;  // the most nodes a tree over numFaces faces has
  ok(bvhgb_trace_ray_image(reinterpret_cast<bvhgb_node *>(_nodes), numNodes, _rootNode,
                           reinterpret_cast<const float *>(_mesh.vert), reinterpret_cast<const uint32_t *>(_mesh.faces),
                           _rays, _w * _h, &cfg, 0, reinterpret_cast<bvhgb_pixel *>(_img), nullptr,
                           nullptr),
     "tracerImage");
}

// copyImageToHost (CUDAKernels.cu:631-633).
void copyImageToHost(CUDAPixel *_hostPixel, CUDAPixel *_cudaImg, uint32_t _w, uint32_t _h) {
  if (!_hostPixel || !_cudaImg) return;
  cudaError_t e = cudaMemcpy(_hostPixel, _cudaImg, sizeof(CUDAPixel) * (size_t)_w * _h, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) std::fprintf(stderr, "[bvhgb] copyImageToHost: %s\n", cudaGetErrorString(e));
}

// tracerDoCudaSync (CUDAKernels.cu:644).
void tracerDoCudaSync() { ok(bvhgb_device_sync(), "tracerDoCudaSync"); }

// copyBVHToGPU (cudaFN.cu:32-74): an empty tree gives null pointers and succeeds.
bool copyBVHToGPU(BVH *_bvh, CUDAMemoryBVHPointer *_ptr) {
  if (!_bvh || !_ptr) return false;
  return ok(bvhgb_copy_bvh_to_gpu(reinterpret_cast<const bvhgb_node *>(_bvh->bvh), (uint32_t)_bvh->vSize,
                                  _bvh->vRootIndex, _bvh->vMaxLevel, reinterpret_cast<bvhgb_bvh_pointer *>(_ptr)),
            "copyBVHToGPU");
}

// copyMeshToGPU (cudaFN.cu:76-109).
bool copyMeshToGPU(Mesh *_mesh, MeshRaw *_meshOut) {
  if (!_mesh || !_meshOut) return false;
  return ok(bvhgb_copy_mesh_to_gpu(reinterpret_cast<const float *>(_mesh->vert.data()), (uint32_t)_mesh->vert.size(),
                                   reinterpret_cast<const float *>(_mesh->norm.data()), (uint32_t)_mesh->norm.size(),
                                   reinterpret_cast<const uint32_t *>(_mesh->faces.data()),
                                   (uint32_t)_mesh->faces.size(), reinterpret_cast<bvhgb_mesh_raw *>(_meshOut)),
            "copyMeshToGPU");
}

// copyBVHToHost (cudaFN.cu:113-146): the host tree takes size, root and max level of the device
// tree (its node array grows with realloc, as BVH::reserve does), then the device tree is freed.
bool copyBVHToHost(CUDAMemoryBVHPointer *_bvh, BVH *_ptr) {
  if (!_bvh || !_bvh->bvh || !_bvh->nodes || !_ptr) return false;
  if (_bvh->numNodes == 0) return true;
  const size_t n = _bvh->numNodes;
  if (n > _ptr->vCapacity) {
    void *p = std::realloc(_ptr->bvh, n * sizeof(BVHNode));
    if (!p) return false;
    _ptr->bvh = static_cast<BVHNode *>(p);
    _ptr->vCapacity = n;
  }
  _ptr->vSize = n;
  uint32_t root = 0;
  uint16_t maxLevel = 0;
  if (!ok(bvhgb_copy_bvh_to_host(reinterpret_cast<bvhgb_bvh_pointer *>(_bvh), reinterpret_cast<bvhgb_node *>(_ptr->bvh),
                                 (uint32_t)n, &root, &maxLevel),
          "copyBVHToHost"))
    return false;
  _ptr->vRootIndex = root;
  _ptr->vMaxLevel = maxLevel;
  return true;
}

// copyMeshToHost (cudaFN.cu:149-182): the host mesh takes the device arrays, which are freed.
bool copyMeshToHost(MeshRaw *_mesh, Mesh *_meshOut) {
  if (!_mesh || !_meshOut || !_mesh->vert || !_mesh->faces) return false;
  _meshOut->vert.resize(_mesh->numVert);
  _meshOut->norm.resize(_mesh->numNorm);
  _meshOut->faces.resize(_mesh->numFaces);
  return ok(bvhgb_copy_mesh_to_host(reinterpret_cast<bvhgb_mesh_raw *>(_mesh),
                                    reinterpret_cast<float *>(_meshOut->vert.data()),
                                    reinterpret_cast<float *>(_meshOut->norm.data()),
                                    reinterpret_cast<uint32_t *>(_meshOut->faces.data())),
            "copyMeshToHost");
}

// resetCUDA (cudaFN.cu:184-187): ends the device context; the library forgets what it cached for it.
void resetCUDA() { ok(bvhgb_reset_device(), "resetCUDA"); }

}  // extern "C"
