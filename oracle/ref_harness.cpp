// Test infrastructure only: C entry points that drive the reference's own CPU command classes,
// compiled from the reference's sources by oracle/build_ref.py into oracle/_ref/libref.so.
// Tests use them to pin the oracle's restatements to the reference itself:
//   ref_bittner13      -> builder::Bittner13::runImpl + teardown   (lib/builder/Bittner13.cpp:222-392)
//   ref_bittner13par   -> builder::Bittner13Par::setup/runImpl/teardown (Bittner13Par.cpp:370-564)
//   ref_calc_sah       -> base::BVH::calcSAH                         (lib/base/BVH.cpp:23-37)
//   ref_fix_levels     -> base::BVH::fixLevels                       (lib/base/BVH.cpp:39-70)
//   ref_camera_rays    -> misc::Camera::genRays                      (lib/misc/Camera.cpp:67-88)
//   ref_trace          -> tracer::CPUTracer / BruteForceTracer::runImpl (CPUTracer.cpp:56-196,
//                         BruteForceTracer.cpp:56-154)
//   ref_build          -> builder::Median / Wald07::runImpl          (Median.cpp:33-40, Wald07.cpp:35-129)
// The node layout is the reference's 48-byte BVHNode, which is the oracle's orc_node.
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "base/Command.hpp"
#include "builder/Bittner13.hpp"
#include "builder/Bittner13Par.hpp"
#include "builder/Median.hpp"
#include "builder/Wald07.hpp"
#include "misc/Camera.hpp"
#include "tracer/BruteForceTracer.hpp"
#include "tracer/CPUTracer.hpp"

using namespace BVHTest;
using namespace BVHTest::base;

// The reference defines this destructor in lib/base/Command.cpp, whose other members (logging of
// command runs, the progress bar) need generated enum-name tables; the harness calls the command
// phases directly instead of Command::run, so only the destructor is needed.
Command::~Command() {}

namespace {

static_assert(sizeof(BVHNode) == 48, "BVHNode layout");

void set_threads(int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
}

void load_bvh(State &st, const void *nodes, uint32_t n, uint32_t root) {
  st.bvh.resize(n);
  std::memcpy(st.bvh.data(), nodes, sizeof(BVHNode) * (size_t)n);
  st.bvh.setNewRoot(root);
}

void load_mesh(State &st, const float *vert, uint32_t nv, const uint32_t *faces, uint32_t nf) {
  st.mesh.vert.resize(nv);
  for (uint32_t i = 0; i < nv; ++i) st.mesh.vert[i] = glm::vec3(vert[3 * i], vert[3 * i + 1], vert[3 * i + 2]);
  st.mesh.faces.resize(nf);
  for (uint32_t i = 0; i < nf; ++i) st.mesh.faces[i] = {faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]};
}

void store_trace(const State &st, float *sah_trace, uint32_t cap) {
  if (!sah_trace) return;
  const auto &steps = st.optData.optStepps;
  for (uint32_t i = 0; i < cap && i < steps.size(); ++i) sah_trace[i] = steps[i].sah;
}

}  // namespace

extern "C" {

// Sequential optimizer (sort = true, random = false): runs `iters` iterations on the nodes in
// place and writes the SAH before and after every iteration (iters + 1 floats).
int ref_bittner13(void *nodes, uint32_t n_nodes, uint32_t root, uint32_t iters, float batch_percent,
                  int threads, float *sah_trace) {
  set_threads(threads);
  State st;
  load_bvh(st, nodes, n_nodes, root);
  builder::Bittner13 opt;
  opt.fromJSON(json{{"maxNumStepps", iters}, {"batchPercent", batch_percent}, {"base_calcSAH", true},
                    {"sort", true}, {"random", false}});
  ErrorCode e = opt.runImpl(st);
  opt.teardown(st);
  store_trace(st, sah_trace, iters + 1);
  std::memcpy(nodes, st.bvh.data(), sizeof(BVHNode) * (size_t)n_nodes);
  return static_cast<int>(e);
}

// Chunked CPU optimizer (the CPU twin of the GPU algorithm): numChunks chunks per iteration,
// sort = true, random = false, shuffle = false.
int ref_bittner13par(void *nodes, uint32_t n_nodes, uint32_t root, uint32_t iters, float batch_percent,
                     uint32_t num_chunks, int offset_access, int alt_find_node, uint32_t alt_queue, int threads,
                     float *sah_trace, uint32_t *skipped, uint32_t *total) {
  set_threads(threads);
  State st;
  load_bvh(st, nodes, n_nodes, root);
  builder::Bittner13Par opt;
  opt.fromJSON(json{{"maxNumStepps", iters}, {"batchPercent", batch_percent}, {"base_calcSAH", true},
                    {"numChunks", num_chunks}, {"offsetAccess", offset_access != 0},
                    {"altFindNode", alt_find_node != 0}, {"altFindNodeQueueSize", alt_queue}, {"sort", true},
                    {"random", false}, {"shuffle", false}});
  ErrorCode e = opt.setup(st);
  if (e == ErrorCode::OK) e = opt.runImpl(st);
  opt.teardown(st);
  store_trace(st, sah_trace, iters + 1);
  if (skipped) *skipped = st.optData.numSkipped;
  if (total) *total = st.optData.numTotal;
  std::memcpy(nodes, st.bvh.data(), sizeof(BVHNode) * (size_t)n_nodes);
  return static_cast<int>(e);
}

float ref_calc_sah(const void *nodes, uint32_t n_nodes, uint32_t root, int threads) {
  set_threads(threads);
  State st;
  load_bvh(st, nodes, n_nodes, root);
  return st.bvh.calcSAH();
}

uint32_t ref_fix_levels(void *nodes, uint32_t n_nodes, uint32_t root) {
  State st;
  load_bvh(st, nodes, n_nodes, root);
  st.bvh.fixLevels();
  std::memcpy(nodes, st.bvh.data(), sizeof(BVHNode) * (size_t)n_nodes);
  return st.bvh.maxLevel();
}

static std::shared_ptr<misc::Camera> make_camera(const float *pos, const float *lookat, const float *up, float fov,
                                                 uint32_t w, uint32_t h) {
  auto cam = std::make_shared<misc::Camera>();
  cam->setCamera(glm::vec3(pos[0], pos[1], pos[2]), glm::vec3(lookat[0], lookat[1], lookat[2]),
                 glm::vec3(up[0], up[1], up[2]));
  cam->setFOV(fov);
  cam->setResolution(w, h);
  return cam;
}

// Primary rays of a perspective camera: origin, direction, inverse direction and sign per ray.
int ref_camera_rays(const float *pos, const float *lookat, const float *up, float fov, uint32_t w, uint32_t h,
                    int threads, float *org, float *dir) {
  set_threads(threads);
  auto cam = make_camera(pos, lookat, up, fov, w, h);
  std::vector<Ray> rays = cam->genRays();
  for (size_t i = 0; i < rays.size(); ++i) {
    const glm::vec3 &o = rays[i].getOrigin();
    const glm::vec3 &d = rays[i].getDirection();
    org[3 * i] = o.x;
    org[3 * i + 1] = o.y;
    org[3 * i + 2] = o.z;
    dir[3 * i] = d.x;
    dir[3 * i + 1] = d.y;
    dir[3 * i + 2] = d.z;
  }
  return 0;
}

// Traces one camera image with the stackless CPU tracer (brute = 0) or the brute-force tracer
// (brute = 1). Writes per pixel the grey value (r == g == b; 121/167/229 background = miss), the
// inner-node visit count and a hit flag; returns the trace time in nanoseconds.
int64_t ref_trace(int brute, const void *nodes, uint32_t n_nodes, uint32_t root, const float *vert, uint32_t nv,
                  const uint32_t *faces, uint32_t nf, const float *pos, const float *lookat, const float *up, float fov,
                  uint32_t w, uint32_t h, const float *light, int threads, uint8_t *grey, uint32_t *int_count,
                  uint8_t *hit) {
  set_threads(threads);
  State st;
  load_bvh(st, nodes, n_nodes, root);
  load_mesh(st, vert, nv, faces, nf);
  st.cameras.push_back(make_camera(pos, lookat, up, fov, w, h));
  json cfg{{"lightLocation", {{"x", light[0]}, {"y", light[1]}, {"z", light[2]}}}};
  auto run = [&](auto &tr) {
    tr.fromJSON(cfg);
    return tr.runImpl(st);
  };
  ErrorCode e;
  if (brute) {
    tracer::BruteForceTracer tr;
    e = run(tr);
  } else {
    tracer::CPUTracer tr;
    e = run(tr);
  }
  if (e != ErrorCode::OK) return -1;
  const auto &px = st.work.back().img.pixels;
  for (size_t i = 0; i < px.size(); ++i) {
    const bool miss = px[i].r == 121 && px[i].g == 167 && px[i].b == 229;
    if (grey) grey[i] = px[i].r;
    if (int_count) int_count[i] = px[i].intCount;
    if (hit) hit[i] = miss ? 0 : 1;
  }
  return (int64_t)st.work.back().time.count();
}

// CPU top-down builders: which = 0 Median, 1 Wald07 (SAH sweep). Writes up to `cap` nodes and
// returns the node count (or -1 when cap is too small).
int64_t ref_build(int which, const float *vert, uint32_t nv, const uint32_t *faces, uint32_t nf, int threads,
                  void *nodes_out, uint32_t cap, uint32_t *root) {
  set_threads(threads);
  State st;
  load_mesh(st, vert, nv, faces, nf);
  ErrorCode e;
  if (which == 0) {
    builder::Median b;
    e = b.runImpl(st);
  } else {
    builder::Wald07 b;
    e = b.runImpl(st);
  }
  if (e != ErrorCode::OK) return -1;
  if (st.bvh.size() > cap) return -1;
  std::memcpy(nodes_out, st.bvh.data(), sizeof(BVHNode) * st.bvh.size());
  if (root) *root = st.bvh.root();
  return (int64_t)st.bvh.size();
}

}  // extern "C"
