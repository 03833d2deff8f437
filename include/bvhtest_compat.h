/*
 * bvhtest_compat.h - the reference's own GPU entry points, under their own names and signatures,
 * implemented by libbvhgb.so on top of the bvhgb_* C ABI (bvhgb.h).
 *
 * BVHTest's command files (lib/builder/LBVH.cpp, Bittner13GPU.cpp, lib/tracer/CUDATracer.cpp,
 * lib/cuda/CopyToGPU.cpp, CopyToHost.cpp) call these functions. They are declared here with the
 * reference's types, names, argument lists and linkage, so that those files link against
 * libbvhgb.so unchanged in place of the reference's CUDA objects (LBVH_CUDA.cu, Bittner13CUDA.cu,
 * CUDAKernels.cu, cudaFN.cu):
 *   - C++ linkage:  LBVH_* (lib/builder/LBVH_CUDA.hpp:49-59) and allocateMemory ... calcNumSkipped
 *                   (lib/builder/Bittner13CUDA.hpp:68-83);
 *   - C linkage:    allocateRays ... tracerDoCudaSync (lib/tracer/CUDAKernels.hpp:39-77, without
 *                   the OpenGL-interop and dynamic-refit helpers of the viewer) and copyBVHToGPU ...
 *                   resetCUDA (lib/cuda/cudaFN.hpp:27-33).
 * The types below have the byte layout of the reference's (BVH.hpp, Ray.hpp, LBVH_CUDA.hpp,
 * Bittner13CUDA.hpp, CUDAKernels.hpp); code that includes the reference's own headers does not
 * include this one and links to the same symbols.
 *
 * Behaviour kept from the reference: bool / void results (failures print a message to stderr, as
 * the reference's CUDA_RUN does, and bvhgb_last_error() names the failing call); the default stream;
 * LBVH with 30-bit Morton codes and the reference's index-delta topology; allocation in the
 * allocate* calls only. What the working-memory structs hold differs: their pointer fields are not
 * the reference's device arrays (cubTempStorage / cubSortTempStorage carry this library's handle), so
 * callers must not read them, which the reference's command files do not.
 */
#ifndef BVHTEST_COMPAT_H
#define BVHTEST_COMPAT_H

#ifndef __cplusplus
#error "bvhtest_compat.h declares the reference's C++ interface"
#endif

#include <cstddef>
#include <cstdint>
#include <vector>

#if defined(__GNUC__)
#define BVHTEST_COMPAT_API __attribute__((visibility("default")))
#else
#define BVHTEST_COMPAT_API
#endif

namespace BVHTest {
namespace base {

struct CompatVec3 {  // glm::vec3
  float x, y, z;
};

struct Triangle final {  // BVH.hpp:38-42
  uint32_t v1, v2, v3;
};

struct Mesh final {  // BVH.hpp:44-48
  std::vector<CompatVec3> vert;
  std::vector<CompatVec3> norm;
  std::vector<Triangle> faces;
};

struct MeshRaw final {  // BVH.hpp:50-57
  CompatVec3 *vert = nullptr;
  CompatVec3 *norm = nullptr;
  Triangle *faces = nullptr;
  uint32_t numVert = 0;
  uint32_t numNorm = 0;
  uint32_t numFaces = 0;
};

struct AABB {  // BVH.hpp:59-60
  CompatVec3 minMax[2];
};

struct alignas(16) BVHNode {  // BVH.hpp:113-136
  AABB bbox;
  uint32_t parent;
  uint32_t left;
  uint32_t right;
  uint16_t isLeafFlag;
  uint16_t isLeft;
  uint16_t level;
  float surfaceArea;
};

// BVH.hpp:138-232: the host tree (nodes from malloc/realloc, freed with free()).
class BVH final {
 public:
  BVHNode *bvh = nullptr;
  size_t vSize = 0;
  size_t vCapacity = 0;
  uint32_t vRootIndex = 0;
  uint16_t vMaxLevel = 0;
};

struct CUDAMemoryBVHPointer {  // BVH.hpp:234-238
  BVH *bvh = nullptr;
  BVHNode *nodes = nullptr;
  uint32_t numNodes = 0;
};

class alignas(16) Ray final {  // Ray.hpp:38-80
 public:
  struct alignas(4) Sign {
    uint8_t x, y, z;
  };
  CompatVec3 vPos;
  CompatVec3 vDir;
  CompatVec3 vInvDir;
  Sign vSign;
  uint32_t vPX = UINT32_MAX;
  uint32_t vPY = UINT32_MAX;
};

class BVHPatch;
class MiniPatch;

static_assert(sizeof(BVHNode) == 48, "BVHNode layout");
static_assert(sizeof(Ray) == 48, "Ray layout");
static_assert(sizeof(AABB) == 24, "AABB layout");

}  // namespace base
}  // namespace BVHTest

// LBVH_CUDA.hpp:27-47
struct LBVH_TriData {
  BVHTest::base::AABB bbox;
  BVHTest::base::CompatVec3 centroid;
  uint32_t faceIndex;
  uint64_t __padding__;
};

struct LBVH_WorkingMemory {
  bool lRes = false;
  uint32_t *mortonCodes = nullptr;
  uint32_t *mortonCodesSorted = nullptr;
  LBVH_TriData *triData = nullptr;
  LBVH_TriData *triDataSorted = nullptr;
  void *cubTempStorage = nullptr;  // here: this library's LBVH handle
  uint32_t *atomicLocks = nullptr;
  uint32_t numFaces = 0;
  size_t cubTempStorageSize = 0;
  uint32_t numLocks = 0;
};

// Bittner13CUDA.hpp:27-64
struct TodoStruct {
  uint32_t *nodes = nullptr;
  float *costs = nullptr;
};

struct GPUWorkingMemory {
  bool result;
  TodoStruct todoNodes;
  TodoStruct todoSorted;
  uint32_t *leafNodes = nullptr;
  uint8_t *deviceSelectFlags = nullptr;
  BVHTest::base::BVHPatch *patches = nullptr;
  uint32_t *skipped = nullptr;
  uint32_t *nodesToFix = nullptr;
  uint32_t *flags = nullptr;
  void *cubSortTempStorage = nullptr;  // here: this library's optimizer handle
  uint32_t numLeafNodes = 0;
  uint32_t numInnerNodes = 0;
  uint32_t numPatches = 0;
  uint32_t numSkipped = 0;
  uint32_t numNodesToFix = 0;
  uint32_t numFlags = 0;
  size_t cubSortTempStorageSize = 0;
};

struct AlgoCFG {
  uint32_t numChunks;
  uint32_t chunkSize;
  uint32_t blockSize = 32;
  bool offsetAccess = true;
  bool altFindNode = true;
  bool altFixTree = true;
  bool altSort = true;
  bool sort = true;
  bool localPatchCPY = true;
};

// CUDAKernels.hpp:33-37
struct CUDAPixel {
  uint8_t hit;
  uint8_t diffuse;
  uint16_t intCount;
};

// ---- LBVH (LBVH_CUDA.hpp:49-59) ---------------------------------------------------------------
BVHTEST_COMPAT_API BVHTest::base::AABB LBVH_initTriData(LBVH_WorkingMemory *_mem, BVHTest::base::MeshRaw *_rawMesh);
BVHTEST_COMPAT_API void LBVH_calcMortonCodes(LBVH_WorkingMemory *_mem, BVHTest::base::AABB _sceneAABB);
BVHTEST_COMPAT_API void LBVH_sortMortonCodes(LBVH_WorkingMemory *_mem);
BVHTEST_COMPAT_API void LBVH_buildBVHTree(LBVH_WorkingMemory *_mem, BVHTest::base::CUDAMemoryBVHPointer *_bvh);
BVHTEST_COMPAT_API void LBVH_fixAABB(LBVH_WorkingMemory *_mem, BVHTest::base::CUDAMemoryBVHPointer *_bvh);
BVHTEST_COMPAT_API bool LBVH_allocateBVH(BVHTest::base::CUDAMemoryBVHPointer *_bvh, BVHTest::base::MeshRaw *_rawMesh);
BVHTEST_COMPAT_API LBVH_WorkingMemory LBVH_allocateWorkingMemory(BVHTest::base::MeshRaw *_rawMesh);
BVHTEST_COMPAT_API void LBVH_freeWorkingMemory(LBVH_WorkingMemory *_mem);
BVHTEST_COMPAT_API void LBVH_doCUDASyc();

// ---- Bittner13 (Bittner13CUDA.hpp:68-83) -------------------------------------------------------
BVHTEST_COMPAT_API GPUWorkingMemory allocateMemory(BVHTest::base::CUDAMemoryBVHPointer *_bvh, uint32_t _batchSize,
                                                   uint32_t _numFaces);
BVHTEST_COMPAT_API void freeMemory(GPUWorkingMemory *_data);
BVHTEST_COMPAT_API void initData(GPUWorkingMemory *_data, BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh,
                                 uint32_t _blockSize);
BVHTEST_COMPAT_API void fixTree1(GPUWorkingMemory *_data, BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh,
                                 uint32_t _blockSize);
BVHTEST_COMPAT_API void fixTree3(GPUWorkingMemory *_data, BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh,
                                 uint32_t _blockSize);
BVHTEST_COMPAT_API void bn13_selectNodes(GPUWorkingMemory *_data, BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh,
                                         AlgoCFG _cfg);
BVHTEST_COMPAT_API void bn13_rmAndReinsChunk(GPUWorkingMemory *_data, BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh,
                                             AlgoCFG _cfg, uint32_t _chunk);
BVHTEST_COMPAT_API void bn13_doAlgorithmStep(GPUWorkingMemory *_data, BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh,
                                             AlgoCFG _cfg);
BVHTEST_COMPAT_API float CUDAcalcSAH(BVHTest::base::CUDAMemoryBVHPointer *_GPUbvh);
BVHTEST_COMPAT_API void doCudaDevSync();
BVHTEST_COMPAT_API uint32_t calcNumSkipped(GPUWorkingMemory *_data);

// ---- tracer (CUDAKernels.hpp:39-77) and transfer (cudaFN.hpp:27-33) -----------------------------
extern "C" {
BVHTEST_COMPAT_API bool allocateRays(BVHTest::base::Ray **_rays, uint32_t _num);
BVHTEST_COMPAT_API bool allocateImage(CUDAPixel **_img, uint32_t _w, uint32_t _h);
BVHTEST_COMPAT_API void freeRays(BVHTest::base::Ray **_rays);
BVHTEST_COMPAT_API void freeImage(CUDAPixel *_img);
BVHTEST_COMPAT_API void generateRays(BVHTest::base::Ray *_rays, uint32_t _w, uint32_t _h, BVHTest::base::CompatVec3 _pos,
                                     BVHTest::base::CompatVec3 _lookAt, BVHTest::base::CompatVec3 _up, float _fov);
BVHTEST_COMPAT_API void tracerImage(BVHTest::base::Ray *_rays, CUDAPixel *_img, BVHTest::base::BVHNode *_nodes,
                                    uint32_t _rootNode, BVHTest::base::MeshRaw _mesh, BVHTest::base::CompatVec3 _light,
                                    uint32_t _w, uint32_t _h, bool _bundle);
BVHTEST_COMPAT_API void copyImageToHost(CUDAPixel *_hostPixel, CUDAPixel *_cudaImg, uint32_t _w, uint32_t _h);
BVHTEST_COMPAT_API void tracerDoCudaSync();

BVHTEST_COMPAT_API bool copyBVHToGPU(BVHTest::base::BVH *_bvh, BVHTest::base::CUDAMemoryBVHPointer *_ptr);
BVHTEST_COMPAT_API bool copyMeshToGPU(BVHTest::base::Mesh *_mesh, BVHTest::base::MeshRaw *_meshOut);
BVHTEST_COMPAT_API bool copyBVHToHost(BVHTest::base::CUDAMemoryBVHPointer *_bvh, BVHTest::base::BVH *_ptr);
BVHTEST_COMPAT_API bool copyMeshToHost(BVHTest::base::MeshRaw *_mesh, BVHTest::base::Mesh *_meshOut);
BVHTEST_COMPAT_API void resetCUDA();
}

#endif
