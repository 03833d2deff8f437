/*
 * CPU oracle for the GPU BVH pipeline (LBVH build -> Bittner13 optimizer -> closest-hit tracer).
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: only tests/, __graft_entry__.smoke()
 * and the cpu_baseline / --impl reference legs of bench.py load it. The product (the CUDA
 * library under bvhtest_gb300/) never links or calls it and has no CPU fallback.
 *
 * Parity status: PINNED where the reference has CPU code, through the reference's own sources.
 * oracle/build_ref.py compiles lib/builder/Bittner13.cpp, Bittner13Par.cpp, lib/base/BVH.cpp,
 * lib/misc/Camera.cpp, lib/tracer/CPUTracer.cpp, BruteForceTracer.cpp, Median.cpp and Wald07.cpp
 * (with stand-ins, written here, for its empty math/format/log submodules) into oracle/_ref, and
 * tests/test_ref_pin.py checks: orc_bittner_seq == Bittner13 and orc_bittner_chunked with
 * {heap search, conflict_rule 1, std_select 1} == Bittner13Par, byte for byte on the trees (also on
 * the large scene, whose inefficiencies tie); orc_sah == BVH::calcSAH up to its float summation;
 * orc_camera_rays == Camera::genRays; orc_trace_cpu_reference == CPUTracer (hit mask, visit counts,
 * shading bytes); orc_trace_brute's hit mask == BruteForceTracer's. tests/golden/ref_pin.npz keeps
 * those outputs for machines without the reference. UNPINNED: the LBVH steps (the reference has
 * them only as CUDA kernels, which cannot run here) and the GPU kernels' deterministic conflict
 * rule (conflict_rule 0; the reference's GPU rule is first-come and not deterministic); they rest
 * on hand-derived known answers (tests/golden/) and the reference's runtime invariants
 * (lib/misc/Validate.cpp restated here).
 *
 * Floating point: compiled with -ffp-contract=off so that every a*b+c rounds twice, matching
 * the product kernels, which spell out __fmul_rn/__fadd_rn. The reference's GPU build let nvcc
 * contract surface-area sums into FMAs; the un-contracted form is the documented convention.
 */
#ifndef BVH_ORACLE_H
#define BVH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* lib/base/BVH.hpp:59-60: glm::vec3 minMax[2] (0: min, 1: max). */
typedef struct orc_aabb {
  float mn[3];
  float mx[3];
} orc_aabb;

/* lib/base/BVH.hpp:113-123: 48-byte alignas(16) node. Leaves: left = first face, right = #faces. */
typedef struct orc_node {
  orc_aabb bbox;       /*  0 */
  uint32_t parent;     /* 24 */
  uint32_t left;       /* 28 */
  uint32_t right;      /* 32 */
  uint16_t isLeafFlag; /* 36 */
  uint16_t isLeft;     /* 38 */
  uint16_t level;      /* 40 */
  uint16_t pad;        /* 42: never written by the reference; 0 here */
  float surfaceArea;   /* 44 */
} orc_node;

enum { ORC_TOPO_REFCOMPAT = 0, ORC_TOPO_KARRAS = 1 };

/* ---- LBVH (lib/builder/LBVH_CUDA.cu) ---------------------------------------------------- */

float orc_surface_area(const orc_aabb *b);

/* kInitTriData (LBVH_CUDA.cu:60-96) + ReduceRootAABB with the origin box as initial value
 * (:51-58, :104-106, :112-113). bbox/centroid may be NULL. */
void orc_tri_data(const float *vert, const uint32_t *faces, uint32_t n, orc_aabb *bbox_out,
                  float *centroid_out, orc_aabb *scene_out);

/* Host part of LBVH_calcMortonCodes (:168-180): offset = 0 - min, scale = 1 / (max + offset). */
void orc_morton_params(const orc_aabb *scene, float offset[3], float scale[3]);

/* kCalcMortonCodes (:132-166), 10 bits per axis; and the 21-bit-per-axis extension. */
void orc_morton30(const float *centroid, uint32_t n, const float offset[3], const float scale[3],
                  uint32_t *codes);
void orc_morton63(const float *centroid, uint32_t n, const float offset[3], const float scale[3],
                  uint64_t *codes);

/* cub::DeviceRadixSort::SortPairs (:185-193): stable ascending sort; values = original index. */
void orc_sort_pairs32(const uint32_t *keys, uint32_t n, uint32_t *keys_out, uint32_t *vals_out);
void orc_sort_pairs64(const uint64_t *keys, uint32_t n, uint64_t *keys_out, uint32_t *vals_out);

/* kGenLeafNodes + kBuildTree (determineRange/findSplit/delta, :205-324) and kFixAABBTree
 * (:341-374), top-down Karras construction exactly as the reference evaluates it.
 * keys32 or keys64 (one of them non-NULL) are the sorted Morton codes. */
void orc_build_topology(const uint32_t *keys32, const uint64_t *keys64, uint32_t n, int mode,
                        orc_node *nodes);
void orc_gen_leaves(const float *vert, const uint32_t *faces, const uint32_t *sorted_idx, uint32_t n,
                    orc_node *nodes);
void orc_refit(orc_node *nodes, uint32_t n_nodes, uint32_t root);

/* Whole LBVH::runImpl (LBVH.cpp:41-50). morton_bits: 30 or 63. Writes 2n-1 nodes. */
int orc_lbvh_build(const float *vert, const uint32_t *faces, uint32_t n, int morton_bits, int mode,
                   orc_node *nodes, void *sorted_keys_out, uint32_t *sorted_idx_out);

/* BVH::calcSAH with cInner = cLeaf = 1 (lib/base/BVH.cpp:23-37), summed in double. */
double orc_sah(const orc_node *nodes, uint32_t n_nodes, uint32_t root);
/* BVH::fixLevels (BVH.cpp:39-70); returns max level. */
uint32_t orc_fix_levels(orc_node *nodes, uint32_t n_nodes, uint32_t root);

/* Validate.cpp:42-263. errs[0..4] = tree, bbox, strict bbox, surface area, triangle errors.
 * check_levels = 0 skips the level comparison (levels are only valid after fixLevels). */
int orc_validate(const orc_node *nodes, uint32_t n_nodes, uint32_t root, const float *vert,
                 const uint32_t *faces, uint32_t n_faces, int check_levels, uint32_t errs[5]);

/* ---- Bittner13 ----------------------------------------------------------------------------- */

/* kCalcCost (Bittner13CUDA.cu:480-500) / Bittner13.cpp:271. */
float orc_inefficiency(const orc_node *nodes, uint32_t i);

/* Sequential Bittner13::runMetric (Bittner13.cpp:222-312), sort = true, random = false.
 * Writes the SAH after every iteration to sah_trace[0..iters] (index 0 = before). */
int orc_bittner_seq(orc_node *nodes, uint32_t n_nodes, uint32_t *root, uint32_t iters,
                    float batch_percent, double *sah_trace);

typedef struct orc_bn13_cfg {
  uint32_t num_chunks;   /* numChunks (32) */
  float batch_percent;   /* batchPercent (1.0) */
  uint32_t offset_access;/* offsetAccess */
  uint32_t heap_cap;     /* B&B heap capacity (the reference uses 4096) */
  uint32_t search_mode;  /* 0: batched best-first (32 per round, frontier 128); 1: findNode1 heap;
                          * 2: findNode2, the approximate queue of altFindNode (heap_cap = its
                          *    number of slots: 16 on the GPU, Bittner13CUDA.hpp:30) */
  uint32_t conflict_rule;/* 0: an item is applied iff it holds the lowest batch rank on every node it
                          *    patches, failed items' claims included (the GPU kernels);
                          * 1: items are taken in batch order and an item is applied iff none of its
                          *    nodes was taken by an earlier applied item (Bittner13Par.cpp:470-495,
                          *    where a failed item releases what it claimed) */
  uint32_t std_select;   /* 0: inner nodes by descending inefficiency, ties by node index (GPU
                          *    kernels); 1: the reference CPU optimizers' nth_element + sort order
                          *    (orc_std_select) */
} orc_bn13_cfg;

/* Batch selection of Bittner13.cpp:258-283 / Bittner13Par.cpp:421-437 with the same standard-
 * library calls (ties come out in the reference's order): writes the first k nodes by descending
 * inefficiency to order_out and returns k. */
uint32_t orc_std_select(const orc_node *nodes, uint32_t n_nodes, uint32_t k, int do_sort, uint32_t *order_out);

typedef struct orc_bn13_stats {
  uint64_t items;        /* batch items considered */
  uint64_t applied;      /* items whose patch was applied */
  uint64_t skipped_conflict;
  uint64_t skipped_invalid; /* removeNode refused or best == root */
  uint64_t heap_overflow;
  uint64_t nodes_visited; /* nodes evaluated by the searches of mode 0 */
} orc_bn13_stats;

/* The chunked parallel algorithm of Bittner13CUDA.cu:141-772 + BVHPatch.hpp:87-335, executed
 * in batch order with the deterministic conflict rule of the GPU kernels (an item is applied
 * iff every node it patches is claimed by no lower-ranked item of its chunk). */
int orc_bittner_chunked(orc_node *nodes, uint32_t n_nodes, uint32_t root, uint32_t iters,
                        const orc_bn13_cfg *cfg, double *sah_trace, orc_bn13_stats *stats);

/* The same, stopping after the first iteration whose SAH is <= stop_sah (when stop_sah > 0);
 * iter_ms (optional, iters entries) gets each iteration's wall time without the SAH evaluation,
 * *done the iterations run. */
int orc_bittner_chunked_until(orc_node *nodes, uint32_t n_nodes, uint32_t root, uint32_t iters,
                              const orc_bn13_cfg *cfg, double stop_sah, double *sah_trace, double *iter_ms,
                              orc_bn13_stats *stats, uint32_t *done);

/* One iteration of the chunked algorithm with a given batch order: order[pos] is the node at batch
 * position pos (the role of the sorted todo list). Used to check a GPU iteration whose selection
 * came from the learned scorer. */
int orc_bittner_iteration_ordered(orc_node *nodes, uint32_t n_nodes, uint32_t root, const uint32_t *order,
                                  uint32_t n_order, const orc_bn13_cfg *cfg, orc_bn13_stats *stats);

/* ---- Learned reinsertion scorer (an addition; the reference has no learned part) -------------- */

#define ORC_LR_FEATURES 24

/* 1 / log2(max(#leaves, 2)), the depth feature's scale. */
float orc_lr_inv_log2_leaves(uint32_t n_leaves);

/* Feature rows of every inner node in ascending node order (definition in learned.c); writes the
 * node ids to inner (may be NULL) and returns the number of inner nodes. */
uint32_t orc_lr_features(const orc_node *nodes, uint32_t n_nodes, uint32_t root, float *feat, uint32_t *inner);

/* Realised gain of reinserting each candidate alone: remove the node and its parent, reinsert both
 * children with the batched search (search mode 0), and take the exact SAH reduction (cInner = 1)
 * of the resulting tree against the current one, in units of the root's surface area (summed in
 * double over the changed nodes, then rounded to float). Where the reinsertion is refused
 * (removeNode or best == root) the gain is 0 and ok[i] = 0. */
void orc_bn13_gains(const orc_node *nodes, uint32_t n_nodes, uint32_t root, const uint32_t *cand, uint32_t n,
                    float *gain, uint8_t *ok);

/* ---- Tracer ------------------------------------------------------------------------------ */

typedef struct orc_camera {
  float pos[3], lookat[3], up[3];
  float fov; /* vertical, degrees */
  uint32_t width, height;
} orc_camera;

/* Camera basis (lookAt, right-handed) and per-pixel primary ray (Camera.cpp:67-88,
 * CUDAKernels.cu:43-59): origin and normalised direction for pixel (x, y). */
void orc_camera_ray(const orc_camera *cam, uint32_t x, uint32_t y, float org[3], float dir[3]);
/* All width * height primary rays, row-major. */
void orc_camera_rays(const orc_camera *cam, float *org, float *dir);

/* Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013), FP32 with the paper's
 * double-precision fallback for zero edge functions. Returns 1 and t on a hit in (tmin, tmax]. */
int orc_ray_tri(const float org[3], const float dir[3], const float *v0, const float *v1,
                const float *v2, float tmin, float tmax, int cull, float *t_out);

typedef struct orc_hit {
  uint32_t prim; /* UINT32_MAX = miss */
  float t;
} orc_hit;

/* Closest hit over all triangles (BruteForceTracer.cpp:56-120 with the watertight test).
 * Ties: smallest t, then smallest prim. */
void orc_trace_brute(const float *org, const float *dir, uint32_t n_rays, const float *vert,
                     const uint32_t *faces, uint32_t n_faces, float tmin, float tmax, int cull,
                     orc_hit *hits);
/* Same answers through the BVH (stack traversal, conservative box test). */
void orc_trace_bvh(const float *org, const float *dir, uint32_t n_rays, const orc_node *nodes,
                   uint32_t root, const float *vert, const uint32_t *faces, float tmin, float tmax,
                   int cull, orc_hit *hits);
/* The reference CPU tracer (CPUTracer.cpp:56-162): stackless bit-trail traversal, t0 = 0.01,
 * double-precision Moller-Trumbore (two-sided). Used as the timed CPU baseline. */
void orc_trace_cpu_reference(const float *org, const float *dir, uint32_t n_rays,
                             const orc_node *nodes, uint32_t root, const float *vert,
                             const uint32_t *faces, orc_hit *hits, uint16_t *int_count);

/* Lambert shade of a hit into the CUDAPixel byte (CUDAKernels.cu:208-218). */
uint8_t orc_shade(const float org[3], const float dir[3], float t, const float *v1, const float *v2,
                  const float *v3, const float light[3]);

/* ---- Misc ----------------------------------------------------------------------------------- */
uint32_t orc_adler32(const uint8_t *data, size_t len);
int orc_num_threads(void);
void orc_set_threads(int n); /* OpenMP threads of later calls (n > 0) */

#ifdef __cplusplus
}
#endif
#endif
