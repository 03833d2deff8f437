// Test driver: runs the reference's GPU pipeline through the reference's own entry points only
// (include/bvhtest_compat.h, implemented by libbvhgb.so), in the order the reference's command
// files call them:
//   CopyToGPU  (lib/cuda/CopyToGPU.cpp:33-37)        copyMeshToGPU
//   LBVH       (lib/builder/LBVH.cpp:28-55)          LBVH_allocateWorkingMemory, LBVH_allocateBVH,
//              LBVH_initTriData, LBVH_calcMortonCodes, LBVH_sortMortonCodes, LBVH_buildBVHTree,
//              LBVH_fixAABB, LBVH_doCUDASyc, LBVH_freeWorkingMemory
//   CopyToHost (lib/cuda/CopyToHost.cpp:33-39)       copyBVHToHost (then copyBVHToGPU back)
//   bittner13GPU (lib/builder/Bittner13GPU.cpp:78-133) allocateMemory, initData, CUDAcalcSAH,
//              bn13_doAlgorithmStep, doCudaDevSync, calcNumSkipped, freeMemory
//   CUDATracer (lib/tracer/CUDATracer.cpp:43-150)    allocateRays, allocateImage, generateRays,
//              tracerImage (per-ray and bundle schedules), tracerDoCudaSync, copyImageToHost,
//              freeImage, freeRays
//   CopyToHost                                       copyMeshToHost, resetCUDA
// Usage: compat_driver IN_DIR OUT_DIR ITERS WIDTH HEIGHT
//   IN_DIR/vert.bin (float32 x 3 per vertex), IN_DIR/faces.bin (uint32 x 3 per face)
//   OUT_DIR/{lbvh.bin, opt.bin, sah.bin, skipped.txt, img.bin, img_bundle.bin, mesh_vert.bin}
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bvhtest_compat.h"

using namespace BVHTest::base;

static std::vector<char> slurp(const std::string &p) {
  std::vector<char> d;
  FILE *f = std::fopen(p.c_str(), "rb");
  if (!f) return d;
  std::fseek(f, 0, SEEK_END);
  d.resize((size_t)std::ftell(f));
  std::fseek(f, 0, SEEK_SET);
  if (!d.empty() && std::fread(d.data(), 1, d.size(), f) != d.size()) d.clear();
  std::fclose(f);
  return d;
}

static bool spit(const std::string &p, const void *data, size_t n) {
  FILE *f = std::fopen(p.c_str(), "wb");
  if (!f) return false;
  bool ok = std::fwrite(data, 1, n, f) == n;
  std::fclose(f);
  return ok;
}

#define REQUIRE(c)                                            \
  do {                                                        \
    if (!(c)) {                                               \
      std::fprintf(stderr, "compat_driver: failed: %s\n", #c); \
      return 1;                                               \
    }                                                         \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: compat_driver IN_DIR OUT_DIR ITERS WIDTH HEIGHT\n");
    return 2;
  }
  const std::string in = argv[1], out = argv[2];
  const uint32_t iters = (uint32_t)std::atoi(argv[3]);
  const uint32_t w = (uint32_t)std::atoi(argv[4]), h = (uint32_t)std::atoi(argv[5]);

  Mesh mesh;
  {
    std::vector<char> v = slurp(in + "/vert.bin"), f = slurp(in + "/faces.bin");
    REQUIRE(!v.empty() && !f.empty());
    mesh.vert.resize(v.size() / sizeof(CompatVec3));
    std::memcpy(mesh.vert.data(), v.data(), mesh.vert.size() * sizeof(CompatVec3));
    mesh.faces.resize(f.size() / sizeof(Triangle));
    std::memcpy(mesh.faces.data(), f.data(), mesh.faces.size() * sizeof(Triangle));
  }

  // CopyToGPU (the mesh; the tree comes from LBVH)
  MeshRaw raw;
  REQUIRE(copyMeshToGPU(&mesh, &raw));
  CUDAMemoryBVHPointer gpuBvh;

  // LBVH::setup / runImpl / teardown
  LBVH_WorkingMemory mem = LBVH_allocateWorkingMemory(&raw);
  REQUIRE(mem.lRes);
  REQUIRE(LBVH_allocateBVH(&gpuBvh, &raw));
  REQUIRE(!LBVH_allocateBVH(&gpuBvh, &raw));  // a second allocation into the same pointer fails
  AABB box = LBVH_initTriData(&mem, &raw);
  LBVH_calcMortonCodes(&mem, box);
  LBVH_sortMortonCodes(&mem);
  LBVH_buildBVHTree(&mem, &gpuBvh);
  LBVH_fixAABB(&mem, &gpuBvh);
  LBVH_doCUDASyc();
  REQUIRE(mem.lRes);
  LBVH_freeWorkingMemory(&mem);

  // CopyToHost / CopyToGPU round trip of the tree
  BVH host;
  REQUIRE(copyBVHToHost(&gpuBvh, &host));
  REQUIRE(gpuBvh.nodes == nullptr && gpuBvh.bvh == nullptr);
  REQUIRE(host.vSize == 2 * raw.numFaces - 1);
  REQUIRE(spit(out + "/lbvh.bin", host.bvh, host.vSize * sizeof(BVHNode)));
  REQUIRE(copyBVHToGPU(&host, &gpuBvh));

  // Bittner13GPU::setup / runImpl / teardown with the reference's defaults
  const float batchPercent = 1.0f;
  const uint32_t numChunks = 32;
  uint32_t lNumNodes = (uint32_t)((batchPercent / 100.0f) * (float)gpuBvh.numNodes);
  const uint32_t chunkSize = lNumNodes / numChunks;
  GPUWorkingMemory wm = allocateMemory(&gpuBvh, chunkSize, raw.numFaces);
  REQUIRE(wm.result);
  initData(&wm, &gpuBvh, 128);
  AlgoCFG cfg;
  cfg.numChunks = numChunks;
  cfg.chunkSize = chunkSize;
  cfg.blockSize = 128;
  cfg.offsetAccess = false;
  cfg.altFindNode = false;
  cfg.altFixTree = false;
  cfg.altSort = false;
  cfg.sort = true;
  cfg.localPatchCPY = false;
  std::vector<float> sah;
  sah.push_back(CUDAcalcSAH(&gpuBvh));
  for (uint32_t i = 0; i < iters; ++i) {
    doCudaDevSync();
    bn13_doAlgorithmStep(&wm, &gpuBvh, cfg);
    sah.push_back(CUDAcalcSAH(&gpuBvh));
  }
  doCudaDevSync();
  const uint32_t skipped = calcNumSkipped(&wm);
  freeMemory(&wm);
  REQUIRE(spit(out + "/sah.bin", sah.data(), sah.size() * sizeof(float)));
  {
    std::string s = std::to_string(skipped) + " " + std::to_string(chunkSize * numChunks * iters) + "\n";
    REQUIRE(spit(out + "/skipped.txt", s.data(), s.size()));
  }

  // CUDATracer::allocateMemory / runImpl / freeMemory, the config-1 camera
  Ray *rays = nullptr;
  CUDAPixel *img = nullptr;
  REQUIRE(allocateRays(&rays, w * h));
  REQUIRE(allocateImage(&img, w, h));
  generateRays(rays, w, h, CompatVec3{0.5f, 0.5f, -1.5f}, CompatVec3{0.5f, 0.5f, 0.0f}, CompatVec3{0.0f, 1.0f, 0.0f},
               60.0f);
  std::vector<CUDAPixel> px((size_t)w * h);
  tracerImage(rays, img, gpuBvh.nodes, host.vRootIndex, raw, CompatVec3{2.0f, 2.0f, 2.0f}, w, h, false);
  tracerDoCudaSync();
  copyImageToHost(px.data(), img, w, h);
  REQUIRE(spit(out + "/img.bin", px.data(), px.size() * sizeof(CUDAPixel)));
  tracerImage(rays, img, gpuBvh.nodes, host.vRootIndex, raw, CompatVec3{2.0f, 2.0f, 2.0f}, w, h, true);
  tracerDoCudaSync();
  copyImageToHost(px.data(), img, w, h);
  REQUIRE(spit(out + "/img_bundle.bin", px.data(), px.size() * sizeof(CUDAPixel)));
  freeImage(img);
  freeRays(&rays);
  REQUIRE(rays == nullptr);

  // CopyToHost: the optimised tree and the mesh come back, then the device is reset
  BVH opt;
  REQUIRE(copyBVHToHost(&gpuBvh, &opt));
  REQUIRE(spit(out + "/opt.bin", opt.bvh, opt.vSize * sizeof(BVHNode)));
  Mesh back;
  REQUIRE(copyMeshToHost(&raw, &back));
  REQUIRE(spit(out + "/mesh_vert.bin", back.vert.data(), back.vert.size() * sizeof(CompatVec3)));
  resetCUDA();
  std::free(host.bvh);
  std::free(opt.bvh);
  std::printf("compat_driver: ok\n");
  return 0;
}
