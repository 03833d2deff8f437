/*
 * bvhgb — GB300-native (sm_103a) GPU BVH pipeline behind a plain C ABI.
 *
 * Drop-in boundary for BVHTest's GPU path (mensinda/BVHTest): LBVH build (lib/builder/LBVH_CUDA.*),
 * parallel Bittner13 optimizer (lib/builder/Bittner13CUDA.*), closest-hit tracer
 * (lib/tracer/CUDAKernels.*) and the transfer helpers (lib/cuda/cudaFN.*). Every entry point
 * returns a bvhgb_status, takes plain pointers and sizes, and runs stream-ordered on the stream
 * it is given (NULL = legacy default stream). Device pointers are caller-owned unless a function
 * says otherwise; workspaces are opaque and owned by the library.
 *
 * Layouts of the shared data model are byte-identical to the reference (lib/base/BVH.hpp).
 */
#ifndef BVHGB_H
#define BVHGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define BVHGB_API __attribute__((visibility("default")))
#else
#define BVHGB_API
#endif

typedef void *bvhgb_stream; /* a cudaStream_t */

/* ErrorCode (lib/base/Command.hpp:33-42) keeps its values; 8.. are additions. */
typedef enum bvhgb_status {
  BVHGB_OK = 0,
  BVHGB_WARNING = 1,
  BVHGB_IO_ERROR = 2,
  BVHGB_PARSE_ERROR = 3,
  BVHGB_BVH_ERROR = 4,
  BVHGB_GL_ERROR = 5, /* never returned: no graphics path */
  BVHGB_CUDA_ERROR = 6,
  BVHGB_GENERIC_ERROR = 7,
  BVHGB_INVALID_ARGUMENT = 8,
  BVHGB_DEVICE_TIMEOUT = 9, /* a bounded device-side wait gave up; results are not valid */
  BVHGB_OUT_OF_MEMORY = 10,
  BVHGB_TOO_LARGE = 11 /* a size above a documented maximum */
} bvhgb_status;

/* ---- shared data model (lib/base/BVH.hpp) ------------------------------------------------- */

typedef struct bvhgb_vec3 { float x, y, z; } bvhgb_vec3;                  /* glm::vec3 */
typedef struct bvhgb_triangle { uint32_t v1, v2, v3; } bvhgb_triangle;    /* BVH.hpp:38-42 */
typedef struct bvhgb_aabb { bvhgb_vec3 minMax[2]; } bvhgb_aabb;           /* BVH.hpp:59-60 */

/* BVHNode (BVH.hpp:113-123), 48 bytes, 16-byte aligned. Inner nodes of an LBVH are
 * [0, N-1), leaves [N-1, 2N-1); a leaf's left = first face, right = face count. */
typedef struct bvhgb_node {
  bvhgb_aabb bbox;
  uint32_t parent;
  uint32_t left;
  uint32_t right;
  uint16_t isLeafFlag;
  uint16_t isLeft;
  uint16_t level;
  uint16_t pad;
  float surfaceArea;
} bvhgb_node;

/* MeshRaw (BVH.hpp:50-57): device-only arrays. */
typedef struct bvhgb_mesh_raw {
  bvhgb_vec3 *vert;
  bvhgb_vec3 *norm;
  bvhgb_triangle *faces;
  uint32_t numVert;
  uint32_t numNorm;
  uint32_t numFaces;
} bvhgb_mesh_raw;

/* Device-side image of the reference's BVH class (BVH.hpp:138-144). */
typedef struct bvhgb_device_bvh {
  bvhgb_node *bvh;
  size_t vSize;
  size_t vCapacity;
  uint32_t vRootIndex;
  uint16_t vMaxLevel;
  uint16_t pad;
} bvhgb_device_bvh;

/* CUDAMemoryBVHPointer (BVH.hpp:234-238). */
typedef struct bvhgb_bvh_pointer {
  bvhgb_device_bvh *bvh;
  bvhgb_node *nodes;
  uint32_t numNodes;
} bvhgb_bvh_pointer;

/* CUDAPixel (lib/tracer/CUDAKernels.hpp:33-37). */
typedef struct bvhgb_pixel {
  uint8_t hit;
  uint8_t diffuse;
  uint16_t intCount;
} bvhgb_pixel;

/* Closest hit per ray (an addition: the reference keeps only the shaded pixel). */
typedef struct bvhgb_hit {
  uint32_t primId; /* 0xFFFFFFFF = miss */
  float t;
} bvhgb_hit;

/* ---- library -------------------------------------------------------------------------------- */

BVHGB_API const char *bvhgb_version(void);
BVHGB_API const char *bvhgb_status_string(int status);
/* Last CUDA error text seen by this thread (empty if none). */
BVHGB_API const char *bvhgb_last_error(void);
/* Number of kernels this library has launched (process-wide, monotonic; a replayed CUDA graph
 * counts the kernels it holds, a capture counts none). */
BVHGB_API uint64_t bvhgb_launch_count(void);

/* ---- LBVH build (lib/builder/LBVH_CUDA.hpp:49-59, LBVH.cpp:28-55) ------------------------- */

enum { BVHGB_TOPO_REFCOMPAT = 0, BVHGB_TOPO_KARRAS = 1 };

typedef struct bvhgb_lbvh_config {
  uint32_t mortonBits; /* 30 (reference) or 63 */
  uint32_t topology;   /* BVHGB_TOPO_REFCOMPAT: the reference's index-only radix tree (its __clz
                          keeps the low 32 bits of (morton << 32 | index)); BVHGB_TOPO_KARRAS:
                          the radix tree of the full (morton, index) keys */
} bvhgb_lbvh_config;

typedef struct bvhgb_lbvh_workspace bvhgb_lbvh_workspace;

/* LBVH_allocateWorkingMemory (LBVH_CUDA.cu:426-475): device scratch for up to maxFaces. */
BVHGB_API int bvhgb_lbvh_create(uint32_t maxFaces, const bvhgb_lbvh_config *cfg, bvhgb_lbvh_workspace **out);
/* LBVH_freeWorkingMemory (LBVH_CUDA.cu:477-488). */
BVHGB_API int bvhgb_lbvh_destroy(bvhgb_lbvh_workspace *ws);
/* LBVH::runImpl (LBVH.cpp:41-50): tri boxes + scene box, Morton codes, sort, topology and
 * refit into nodes[0 .. 2*numFaces-1). vert: float3[*], faces: uint3[numFaces] (device).
 * Writes nodes[0].parent = 0; inner levels are 0 and leaf levels 255 (fix with
 * bvhgb_fix_levels_host after copying to the host). */
BVHGB_API int bvhgb_lbvh_build(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                               uint32_t numFaces, bvhgb_node *nodes, bvhgb_stream stream);
/* The phases of bvhgb_lbvh_build, for tests and the legacy wrappers:
 * LBVH_initTriData (:98-119) -> scene box kept on the device; LBVH_calcMortonCodes (:168-183);
 * LBVH_sortMortonCodes (:185-193); LBVH_buildBVHTree + LBVH_fixAABB (:326-385, fused). */
BVHGB_API int bvhgb_lbvh_init_tri_data(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                       uint32_t numFaces, bvhgb_stream stream);
BVHGB_API int bvhgb_lbvh_calc_morton(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                     uint32_t numFaces, bvhgb_stream stream);
BVHGB_API int bvhgb_lbvh_sort(bvhgb_lbvh_workspace *ws, uint32_t numFaces, bvhgb_stream stream);
BVHGB_API int bvhgb_lbvh_build_tree(bvhgb_lbvh_workspace *ws, const float *vert, const uint32_t *faces,
                                    uint32_t numFaces, bvhgb_node *nodes, bvhgb_stream stream);
/* Copies of intermediate device results (synchronous on 'stream'). keys: uint32 (30-bit) or
 * uint64 (63-bit) per face; sorted = after bvhgb_lbvh_sort. scene: 6 floats. */
BVHGB_API int bvhgb_lbvh_read_scene_box(bvhgb_lbvh_workspace *ws, bvhgb_aabb *scene, bvhgb_stream stream);
/* The scene box the Morton phase normalises by (LBVH_calcMortonCodes takes it as an argument,
 * LBVH_CUDA.cu:168-183); bvhgb_lbvh_init_tri_data computes it, this call replaces it. */
BVHGB_API int bvhgb_lbvh_set_scene_box(bvhgb_lbvh_workspace *ws, const bvhgb_aabb *scene, bvhgb_stream stream);
BVHGB_API int bvhgb_lbvh_read_keys(bvhgb_lbvh_workspace *ws, int sorted, void *keys_host, uint32_t *idx_host,
                                   uint32_t numFaces, bvhgb_stream stream);
/* Allocation-free LBVH build. No counterpart in the reference (its build allocates in
 * LBVH_allocateWorkingMemory and per call in LBVH_initTriData). For callers that cannot call
 * cudaMalloc while they build — a per-frame rebuild in a render or simulation loop, where an
 * allocation synchronises the device, or a host application that owns all device memory through
 * its own pool. Same node array as bvhgb_lbvh_build, but the working memory is one 12 MiB
 * file-scope device array that every GPU loading the library keeps until exit; nothing is
 * allocated and no allocating library routine is called. The array has no room for the per-face
 * box records the allocating build keeps, so the tree kernel re-reads each leaf's face and three
 * vertices instead of one 32-byte record: the result is the same, the memory traffic and time are
 * not. The caller still passes the mesh and the node array (2 * numFaces - 1 nodes). Limits:
 * numFaces <= BVHGB_STATIC_MAX_FACES, else BVHGB_TOO_LARGE. All calls share the one array: calls
 * that overlap on the GPU (other streams, other host threads) race and must be serialised by the
 * caller. The first call in each context (each device; again after a device reset) looks up the
 * array's device address with that device current; make that first call before any stream
 * capture. */
#define BVHGB_STATIC_MAX_FACES 262144u
BVHGB_API int bvhgb_lbvh_build_static(const float *vert, const uint32_t *faces, uint32_t numFaces,
                                      const bvhgb_lbvh_config *cfg, bvhgb_node *nodes, bvhgb_stream stream);
/* The device error bits of the last bvhgb_lbvh_build_static call (same meaning as
 * bvhgb_lbvh_read_errors; cfg: the configuration that call was given, which fixes where the sort
 * keeps its error word in the shared array). Synchronous on 'stream'; 0 = the tree is valid. */
BVHGB_API int bvhgb_lbvh_static_read_errors(const bvhgb_lbvh_config *cfg, uint32_t *flags, bvhgb_stream stream);
/* Device error bits of the last build (4 = an inconsistent exchange slot was met and the build
 * stopped; 1 = the sort's look-back gave up); synchronous on 'stream'. 0 = the build is valid. */
BVHGB_API int bvhgb_lbvh_read_errors(bvhgb_lbvh_workspace *ws, uint32_t *flags, bvhgb_stream stream);

/* ---- radix sort (used by the build and the optimizer; exposed for tests) --------------------- */

/* Stable ascending LSD sort of (key, uint32 value) pairs on bits [beginBit, endBit) of the key.
 * keyBytes: 4 or 8. temp == NULL: *tempBytes receives the scratch size and nothing runs. */
BVHGB_API int bvhgb_radix_sort_pairs(void *temp, size_t *tempBytes, const void *keysIn, void *keysOut,
                                     const uint32_t *valsIn, uint32_t *valsOut, uint32_t n, uint32_t keyBytes,
                                     uint32_t beginBit, uint32_t endBit, bvhgb_stream stream);

/* The values of the k smallest of n 32-bit keys in stable ascending order (the first k values of
 * bvhgb_radix_sort_pairs over all 32 bits) into valsOut, without sorting all n pairs (k <= n). The
 * optimizer's selection uses it. temp == NULL: *tempBytes receives the scratch size. No counterpart
 * in the reference (its selection sorts every inner node, Bittner13CUDA.cu:659-726). */
BVHGB_API int bvhgb_select_smallest_pairs(void *temp, size_t *tempBytes, const uint32_t *keys, const uint32_t *vals,
                                          uint32_t *valsOut, uint32_t n, uint32_t k, bvhgb_stream stream);

/* Keys per CTA of the onesweep passes (2048, 4096 or 8192) for sorts that are not given one: the
 * LBVH build's and the optimizer's selection sort, launched (or captured into a graph) after the
 * call. tileKeys = 0 only reads the setting. *previous (may be NULL) receives the old value. The
 * results do not depend on it. No counterpart in the reference (cub picks its own tiles). */
BVHGB_API int bvhgb_sort_set_default_tile(uint32_t tileKeys, uint32_t *previous);
/* Diagnostics of the failure paths (no counterpart in the reference). bvhgb_sort_set_spin_limit:
 * how many times a sort tile polls a predecessor that has not published its digit counts before it
 * gives up, sets the timeout bit (1) of the sort's error word (bvhgb_lbvh_read_errors) and scatters
 * with the partial prefix it has (every write stays in bounds; the order is then not valid).
 * 0xFFFFFFFF restores the default (2^24 polls with a short sleep); synchronous, not during stream
 * capture. bvhgb_debug_fail_allocations: after 'after' more successful device allocations inside
 * the library, the next one fails as out of memory (-1: off; *previous, may be NULL, gets the
 * old budget). */
BVHGB_API int bvhgb_sort_set_spin_limit(uint32_t limit, uint32_t *previous);
BVHGB_API int bvhgb_debug_fail_allocations(int64_t after, int64_t *previous);

/* ---- SAH (Bittner13CUDA.cu:776-803, BVH.cpp:23-37) ------------------------------------------- */

/* (sum of all node areas except the root) / root area, cInner = cLeaf = 1; deterministic
 * reduction in double. Synchronous on 'stream'. */
BVHGB_API int bvhgb_calc_sah(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, double *sah,
                             bvhgb_stream stream);

/* ---- Bittner13 optimizer (lib/builder/Bittner13CUDA.hpp:68-83, Bittner13GPU.cpp:78-133) ---- */

typedef struct bvhgb_bn13_config {
  uint32_t numChunks;    /* numChunks = 32 */
  uint32_t blockSize;    /* CUDABlockSize = 128 */
  float batchPercent;    /* batchPercent = 1.0, clamped to [0.01, 75] */
  uint32_t offsetAccess; /* offsetAccess = false */
  uint32_t heapCapacity; /* branch-and-bound queue entries per item (reference: 4096) */
  uint32_t profileKernels; /* 1: bracket every reinsertion-search launch with CUDA events */
  uint32_t searchMode;     /* BVHGB_SEARCH_BATCHED (0, default), BVHGB_SEARCH_HEAP (1) or BVHGB_SEARCH_ALT (2) */
  uint32_t chunkSize;      /* items per chunk; 0: (batchPercent / 100 * numNodes) / numChunks
                            * (Bittner13GPU.cpp:79-80); the reference's allocateMemory passes it */
} bvhgb_bn13_config;

/* Reinsertion search. HEAP: findNode1 (Bittner13CUDA.cu:141-191) one node at a time in the order of
 * the reference's standard-library heap, one thread per item. BATCHED: the same cost model and
 * pruning evaluated 32 lowest-bound frontier nodes per round by a warp per item (frontier of 128
 * kept ordered by (cost, node)); it finds the same positions in practice at a fraction of the
 * latency. Both are deterministic and restated by the oracle. */
enum { BVHGB_SEARCH_BATCHED = 0, BVHGB_SEARCH_HEAP = 1, BVHGB_SEARCH_ALT = 2 };
/* ALT: findNode2 (Bittner13CUDA.cu:194-264), the reference's altFindNode: an approximate search
 * in a fixed queue of 16 slots whose worst entry is overwritten when it is full, one thread per
 * item; cheaper per item, worse positions (the SAH it reaches is reported beside findNode1's). */

typedef struct bvhgb_bn13_stats {
  uint64_t items;            /* batch items processed */
  uint64_t applied;          /* reinsertions applied */
  uint64_t skippedConflict;  /* lost the conflict check (numSkipped in the reference) */
  uint64_t skippedInvalid;   /* removeNode refused or best position == root */
  uint64_t heapOverflow;     /* queue pushes dropped at heapCapacity */
  uint64_t nodesVisited;     /* nodes evaluated by the reinsertion searches */
} bvhgb_bn13_stats;

typedef struct bvhgb_bn13_workspace bvhgb_bn13_workspace;

/* allocateMemory + initData (Bittner13CUDA.cu:836-987) for a tree of numNodes nodes. */
BVHGB_API int bvhgb_bn13_create(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root,
                                const bvhgb_bn13_config *cfg, bvhgb_bn13_workspace **out, bvhgb_stream stream);
BVHGB_API int bvhgb_bn13_destroy(bvhgb_bn13_workspace *ws);
/* bn13_doAlgorithmStep (:768-772): selection + all chunks of one iteration. */
BVHGB_API int bvhgb_bn13_step(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, bvhgb_stream stream);
/* maxNumStepps iterations captured once into a CUDA graph and replayed. */
BVHGB_API int bvhgb_bn13_run(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, uint32_t iterations, bvhgb_stream stream);
/* bn13_selectNodes (:659-726) and bn13_rmAndReinsChunk (:729-766). */
BVHGB_API int bvhgb_bn13_select_nodes(bvhgb_bn13_workspace *ws, const bvhgb_node *nodes, bvhgb_stream stream);
BVHGB_API int bvhgb_bn13_chunk(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, uint32_t chunk, bvhgb_stream stream);
/* fixTree1 (Bittner13CUDA.cu:372-404, 641-648): recomputes every inner node's box and surface area
 * bottom up from the leaves' boxes (all inner nodes, not only the paths a chunk dirtied). */
BVHGB_API int bvhgb_bn13_refit(bvhgb_bn13_workspace *ws, bvhgb_node *nodes, bvhgb_stream stream);
/* calcNumSkipped (:806-821) and friends; synchronous on 'stream'. */
BVHGB_API int bvhgb_bn13_get_stats(bvhgb_bn13_workspace *ws, bvhgb_bn13_stats *stats, bvhgb_stream stream);
/* Number of items per iteration (numChunks * chunkSize, Bittner13GPU.cpp:90-92). */
BVHGB_API uint32_t bvhgb_bn13_batch_size(const bvhgb_bn13_workspace *ws);
/* Kernels one iteration launches (the nodes of the captured graph). */
BVHGB_API uint32_t bvhgb_bn13_launches_per_iteration(const bvhgb_bn13_workspace *ws);
/* With profileKernels = 1: total milliseconds of the reinsertion-search kernel over the chunks of
 * the most recent iteration, and the number of launches that covers (synchronous). */
BVHGB_API int bvhgb_bn13_search_time(bvhgb_bn13_workspace *ws, float *ms, uint32_t *launches);

/* ---- learned reinsertion scorer ------------------------------------------------------------------
 * No counterpart in the reference: its selection is the inefficiency of Bittner13CUDA.cu:480-500.
 * A 24 -> 64 -> 64 -> 1 MLP with GELU (tanh form), BF16 weights, inputs and activations, FP32
 * accumulation, trained by the library's own forward / backward / AdamW kernels on
 * (feature row, realised SAH reduction) pairs logged from plain optimizer runs, and used in place
 * of the inefficiency to pick the batch of each iteration. The plain measure stays the default.
 *
 * Feature row of an inner node x (children l, r, parent p, grand parent g, SA = surface area; p and
 * g are the root where they do not exist; raw values clamped to [-64, 64], NaN -> -64):
 *   0 log2 SA(x)   1 SA(x)/SA(p)   2 SA(x)/SA(g)   3 SA(x)/(SA(l)+SA(r))   4 min(depth,256)/log2(#leaves)
 *   5 log2 leaves(l)   6 log2 leaves(r)   7 log2 SA(x)/SA(root)   8 log2 SA(x)/min(SA(l),SA(r))
 *   9 log2 inefficiency   10..13 ranks (over all inner nodes, 65536-bin histogram) of the
 *   inefficiency, SA(x)/min(SA(l),SA(r)), SA(x)/(SA(l)+SA(r)) and SA(x)   14..23 zero.
 * Parameters, FP32, in this order: W1[64][24] b1[64] W2[64][64] b2[64] W3[64] b3[1]. */
#define BVHGB_LR_FEATURES 24
#define BVHGB_MLP_PARAMS 5825

typedef struct bvhgb_mlp bvhgb_mlp;

/* Parameters initialised from 'seed' (uniform +-sqrt(6/fan_in), last layer scaled by 0.1, zero
 * biases) and zero AdamW state. */
BVHGB_API int bvhgb_mlp_create(uint64_t seed, bvhgb_mlp **out);
BVHGB_API int bvhgb_mlp_destroy(bvhgb_mlp *m);
/* Host FP32 arrays of BVHGB_MLP_PARAMS values; set also resets the AdamW state and step. */
BVHGB_API int bvhgb_mlp_set_params(bvhgb_mlp *m, const float *params);
BVHGB_API int bvhgb_mlp_get_params(const bvhgb_mlp *m, float *params);
/* y[i] = MLP(x[i]) for n device rows of BVHGB_LR_FEATURES BF16 values (raw uint16 bit patterns), on
 * the tcgen05 tensor cores (128-row tiles, FP32 accumulators in tensor memory). */
BVHGB_API int bvhgb_mlp_forward(const bvhgb_mlp *m, const uint16_t *x, uint32_t n, float *y, bvhgb_stream stream);
/* Error bits of the inference kernel (1 = a bounded wait gave up: results not valid); synchronous. */
BVHGB_API int bvhgb_mlp_read_errors(bvhgb_mlp *m, uint32_t *flags, int reset);
/* Gradient of the mean squared error over n device samples (x, target t) without an update:
 * gradHost receives BVHGB_MLP_PARAMS floats, lossHost the loss (either may be NULL). Synchronous.
 * The BF16 rounding of weights and activations is passed through as identity. */
BVHGB_API int bvhgb_mlp_gradient(bvhgb_mlp *m, const uint16_t *x, const float *t, uint32_t n, float *gradHost,
                                 float *lossHost, bvhgb_stream stream);
/* 'steps' AdamW steps (beta 0.9 / 0.999, eps 1e-8, decoupled weight decay on the weights) on
 * batches of 'batch' rows drawn with replacement from numSamples device rows by a counter hash of
 * (seed, step). One step is captured as a CUDA graph and replayed. lossHistory (host, may be NULL)
 * receives each step's batch loss; the call is synchronous when it is given. */
BVHGB_API int bvhgb_mlp_train(bvhgb_mlp *m, const uint16_t *x, const float *t, uint32_t numSamples, uint32_t batch,
                              uint32_t steps, float lr, float weightDecay, uint64_t seed, float *lossHistory,
                              bvhgb_stream stream);

typedef struct bvhgb_lr_features_ctx bvhgb_lr_features_ctx;
/* Device scratch for the features of trees of up to maxNodes nodes. */
BVHGB_API int bvhgb_lr_features_create(uint32_t maxNodes, bvhgb_lr_features_ctx **out);
BVHGB_API int bvhgb_lr_features_destroy(bvhgb_lr_features_ctx *ctx);
/* Feature rows (BF16 bit patterns, numInner x BVHGB_LR_FEATURES, device) of the device inner-node
 * list 'inner' (numInner ids); numLeaves scales the depth feature. */
BVHGB_API int bvhgb_lr_features(bvhgb_lr_features_ctx *ctx, const bvhgb_node *nodes, uint32_t numNodes, uint32_t root,
                                const uint32_t *inner, uint32_t numInner, uint32_t numLeaves, uint16_t *x,
                                bvhgb_stream stream);
/* Realised gain of reinserting each candidate alone with the batched search: the exact SAH
 * reduction (cInner = 1) in units of the root's surface area, 0 where the reinsertion is refused.
 * target (may be NULL) receives the training target sign(g) ln(1 + |g| numLeaves / 0.16): the gain
 * in units of SA(root) / numLeaves, log-compressed so that one scale ranks nodes of every size.
 * Device arrays; the tree is not modified. */
BVHGB_API int bvhgb_bn13_gains(bvhgb_bn13_workspace *ws, const bvhgb_node *nodes, const uint32_t *cand, uint32_t n,
                               float *gain, float *target, bvhgb_stream stream);
/* Number of inner nodes of the workspace's tree; with out != NULL (device, capacity entries) also
 * copies their ids in ascending order (the optimizer's inner-node list) on 'stream'. */
BVHGB_API int bvhgb_bn13_read_inner(const bvhgb_bn13_workspace *ws, uint32_t *out, uint32_t capacity,
                                    uint32_t *numInner, bvhgb_stream stream);
/* Select batches by the scorer's predicted reduction (its output, the target scale above;
 * descending, ties by node id) instead of the inefficiency. With plainEvery = k > 0, every k-th
 * iteration (iteration i with i % k == k - 1, counted from the workspace's creation) still selects
 * by the inefficiency: the plain measure stays in the loop and picks the nodes the scorer misses
 * (k = 2, alternating, is the recommended policy; 0 = scorer only). NULL restores the plain
 * measure. The workspace keeps the pointer: the scorer must outlive its use. */
BVHGB_API int bvhgb_bn13_set_scorer(bvhgb_bn13_workspace *ws, const bvhgb_mlp *scorer, uint32_t plainEvery);
/* Iterations run on this workspace so far (step and run; decides the kind of the next one), and
 * its reset for a new optimisation of a rebuilt tree of the same mesh. */
BVHGB_API uint64_t bvhgb_bn13_iteration(const bvhgb_bn13_workspace *ws);
BVHGB_API int bvhgb_bn13_set_iteration(bvhgb_bn13_workspace *ws, uint64_t iteration);
/* Climbs per warp of the chunk tail's count and refit kernels (1..32; 0 = automatic: the fewest that
 * fit in one wave of resident warps). Results never depend on it; the captured iteration graphs
 * are rebuilt. */
BVHGB_API int bvhgb_bn13_set_tail_packing(bvhgb_bn13_workspace *ws, uint32_t climbsPerWarp);
/* Replaces the selection of the current iteration by a caller order (numInner node ids, device, in
 * batch position order) for the following bvhgb_bn13_chunk calls; a later select overwrites it. */
BVHGB_API int bvhgb_bn13_set_selection(bvhgb_bn13_workspace *ws, const uint32_t *order, uint32_t n,
                                       bvhgb_stream stream);
/* Copies the most recent selection order into out (device, capacity entries) on 'stream': the
 * first min(bvhgb_bn13_batch_size, numInner) node ids in batch position order, which are the ones
 * the chunks process (the reference sorts every inner node; only this prefix is ever read). */
BVHGB_API int bvhgb_bn13_read_selection(const bvhgb_bn13_workspace *ws, uint32_t *out, uint32_t capacity,
                                        bvhgb_stream stream);

/* ---- batched multi-mesh pipeline ------------------------------------------------------------------
 * No counterpart in the reference (its commands take one mesh at a time: LBVH.cpp, Bittner13GPU.cpp,
 * CUDATracer.cpp). Many independent meshes of uneven size are built, optimised and traced together,
 * one launch per phase for the whole batch; bvhgb_batch_run captures build + iterations + trace as one
 * CUDA graph. Each mesh's node array equals what bvhgb_lbvh_build + bvhgb_bn13_run give for that mesh
 * alone (same topology mode, 30-bit Morton codes, same optimizer settings).
 *
 * Inputs: vert = the meshes' float3 vertices concatenated; faces = their uint3 faces concatenated,
 * mesh after mesh (faceCounts[m] faces each), with vertex indices into the concatenated vertices.
 * Output: nodes = mesh m's 2 * faceCounts[m] - 1 nodes at node offset m (bvhgb_batch_offsets), child
 * indices local to the mesh, leaves naming faces by their index within the mesh, root 0. */
typedef struct bvhgb_batch_config {
  uint32_t mortonBits;   /* 30 */
  uint32_t topology;     /* BVHGB_TOPO_REFCOMPAT or BVHGB_TOPO_KARRAS */
  uint32_t numChunks;    /* Bittner13 chunks per iteration (32) */
  float batchPercent;    /* Bittner13 batch, % of each mesh's nodes (1.0) */
  uint32_t sortTileKeys; /* tuning: keys per CTA in the sort passes (2048, 4096, 8192) */
  uint32_t refitBlock;   /* tuning: threads per block of the apply / count / refit kernels (count and refit run one climb per warp) */
  uint32_t traceBlock;   /* tuning: threads per block of the tracer */
} bvhgb_batch_config;

typedef struct bvhgb_batch_workspace bvhgb_batch_workspace;

/* Workspace for numMeshes (<= 4096) meshes of faceCounts[m] (host array) faces; cfg NULL = defaults. */
BVHGB_API int bvhgb_batch_create(uint32_t numMeshes, const uint32_t *faceCounts, const bvhgb_batch_config *cfg,
                                 bvhgb_batch_workspace **out);
BVHGB_API int bvhgb_batch_destroy(bvhgb_batch_workspace *ws);
/* Host copies of the numMeshes + 1 face and node offsets (either may be NULL). */
BVHGB_API int bvhgb_batch_offsets(const bvhgb_batch_workspace *ws, uint32_t *faceOffsets, uint32_t *nodeOffsets);
BVHGB_API int bvhgb_batch_get_config(const bvhgb_batch_workspace *ws, bvhgb_batch_config *cfg);
/* Changes the tuning knobs and the topology (other fields must be unchanged). */
BVHGB_API int bvhgb_batch_set_config(bvhgb_batch_workspace *ws, const bvhgb_batch_config *cfg);
/* LBVH of every mesh (scene boxes, Morton codes, one sort, build + refit). */
BVHGB_API int bvhgb_batch_build(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces, bvhgb_node *nodes,
                                bvhgb_stream stream);
/* Bittner13 iterations of every mesh (selection + chunks, each chunk of all meshes at once). */
BVHGB_API int bvhgb_batch_optimize(bvhgb_batch_workspace *ws, bvhgb_node *nodes, uint32_t iterations,
                                   bvhgb_stream stream);
/* raysPerMesh random rays per mesh (origins uniform in the mesh box grown 1.5x about its centre,
 * directions uniform on the sphere, from a counter hash of seed), closest hit in the mesh's tree:
 * hits[m * raysPerMesh + j] = (face index within the mesh, t). rayOrg / rayDir (float3 per ray, both
 * or neither) receive the rays. */
BVHGB_API int bvhgb_batch_trace_random(bvhgb_batch_workspace *ws, const bvhgb_node *nodes, const float *vert,
                                       const uint32_t *faces, uint32_t raysPerMesh, uint64_t seed, bvhgb_hit *hits,
                                       float *rayOrg, float *rayDir, bvhgb_stream stream);
/* build + iterations + trace captured once as one CUDA graph (again whenever an argument changes)
 * and launched on stream. */
BVHGB_API int bvhgb_batch_run(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces, bvhgb_node *nodes,
                              uint32_t iterations, uint32_t raysPerMesh, uint64_t seed, bvhgb_hit *hits,
                              bvhgb_stream stream);
/* Optimizer statistics summed over the batch, and the device error bits (synchronous). */
BVHGB_API int bvhgb_batch_get_stats(bvhgb_batch_workspace *ws, bvhgb_bn13_stats *stats, uint32_t *errors,
                                    bvhgb_stream stream);

typedef struct bvhgb_batch_tune_report {
  uint32_t sortTileKeys[3];
  float sortTileMs[3];   /* batched build with each sort tile */
  uint32_t refitBlock[3];
  float refitBlockMs[3]; /* one optimizer iteration with each apply / count / refit block */
  uint32_t traceBlock[3];
  float traceBlockMs[3]; /* the random-ray trace with each tracer block */
  bvhgb_batch_config chosen;
} bvhgb_batch_tune_report;

/* Autotuner: times the candidates of each knob on the caller's data (coordinate search, CUDA events,
 * best of two runs each) and keeps the fastest in the workspace. Results do not depend on the knobs.
 * Leaves nodes holding a one-iteration tree; synchronous. */
BVHGB_API int bvhgb_batch_autotune(bvhgb_batch_workspace *ws, const float *vert, const uint32_t *faces,
                                   bvhgb_node *nodes, uint32_t raysPerMesh, uint64_t seed, bvhgb_hit *hits,
                                   bvhgb_batch_tune_report *report, bvhgb_stream stream);

/* ---- tracer (lib/tracer/CUDAKernels.hpp:39-77, CUDATracer.cpp:86-118) ------------------------ */

typedef struct bvhgb_camera {
  float pos[3];
  float lookAt[3];
  float up[3];
  float fov; /* vertical, degrees (Camera.hpp:27-32) */
  uint32_t width;
  uint32_t height;
} bvhgb_camera;

typedef struct bvhgb_trace_config {
  float light[3];       /* lightLocation = (2, 2, 2) (TracerBase.hpp:25) */
  uint32_t faceCulling; /* CUDA_FACE_CULLING: front faces only */
  float tmin;           /* hits need t > tmin (0) */
  float tmax;           /* ... and t <= tmax (+inf) */
  uint32_t rayBundles;  /* rayBundles (CUDATracer.cpp:31-40): image traces run a warp of 32
                         * neighbouring rays as one bundle through the tree (the reference's
                         * kTraceRayBundle, CUDAKernels.cu:240-383); same hits, intCount counts the
                         * bundle's visits. Secondary and arbitrary rays always trace one by one. */
} bvhgb_trace_config;

/* generateRays + tracerImage (CUDAKernels.cu:386-417) fused: one primary ray per pixel,
 * closest hit, Lambert shade into img[y * width + x]; hits (optional) gets (primId, t). */
BVHGB_API int bvhgb_trace_image(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                bvhgb_pixel *img, bvhgb_hit *hits, bvhgb_stream stream);
/* Closest hit for arbitrary rays: org/dir are float3[n] (dir need not be normalised). */
BVHGB_API int bvhgb_trace_rays(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                               const uint32_t *faces, const float *org, const float *dir, uint32_t n,
                               const bvhgb_trace_config *cfg, bvhgb_hit *hits, bvhgb_stream stream);

/* One cosine-weighted diffuse bounce per primary hit (an addition: the reference has no secondary
 * rays). primary: the hits of bvhgb_trace_image for the same camera. The bounce leaves the hit
 * point offset by 'offset' along the normal facing the camera ray; its direction is drawn from a
 * counter-based generator keyed by (seed, pixel). bounce[pixel] gets the closest hit (miss where
 * the primary ray missed). rayOrg/rayDir (float3 per pixel, optional) receive the bounce rays. */
BVHGB_API int bvhgb_trace_bounce(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                 const uint32_t *faces, const bvhgb_camera *cam, const bvhgb_trace_config *cfg,
                                 uint64_t seed, float offset, const bvhgb_hit *primary, bvhgb_hit *bounce,
                                 float *rayOrg, float *rayDir, bvhgb_stream stream);
/* A tracer prepared for one tree (no counterpart in the reference, whose tracer reads the node
 * array): bvhgb_tracer_update builds traversal records (both children's boxes and references per
 * inner node, 64 bytes each, maxNodes of them allocated at create) once, and every trace call on
 * the tracer reuses them, loading one record per visit instead of two 48-byte nodes. The node
 * array must stay as it was at the last update while traces run. Same hits as the calls above. */
typedef struct bvhgb_tracer bvhgb_tracer;
BVHGB_API int bvhgb_tracer_create(uint32_t maxNodes, bvhgb_tracer **out);
BVHGB_API int bvhgb_tracer_destroy(bvhgb_tracer *tr);
BVHGB_API int bvhgb_tracer_update(bvhgb_tracer *tr, const bvhgb_node *nodes, uint32_t numNodes, uint32_t root,
                                  bvhgb_stream stream);
BVHGB_API int bvhgb_tracer_trace_image(const bvhgb_tracer *tr, const float *vert, const uint32_t *faces,
                                       const bvhgb_camera *cam, const bvhgb_trace_config *cfg, bvhgb_pixel *img,
                                       bvhgb_hit *hits, bvhgb_stream stream);
BVHGB_API int bvhgb_tracer_trace_rays(const bvhgb_tracer *tr, const float *vert, const uint32_t *faces,
                                      const float *org, const float *dir, uint32_t n, const bvhgb_trace_config *cfg,
                                      bvhgb_hit *hits, bvhgb_stream stream);
BVHGB_API int bvhgb_tracer_trace_bounce(const bvhgb_tracer *tr, const float *vert, const uint32_t *faces,
                                        const bvhgb_camera *cam, const bvhgb_trace_config *cfg, uint64_t seed,
                                        float offset, const bvhgb_hit *primary, bvhgb_hit *bounce, float *rayOrg,
                                        float *rayDir, bvhgb_stream stream);

/* generateRays (CUDAKernels.cu:43-59, 386-397): one primary ray per pixel written as the
 * reference's 48-byte Ray record (lib/base/Ray.hpp:38-80: origin, direction, 1 / direction, signs,
 * pixel x, y) into rays[y * width + x]; rays must be 16-byte aligned. */
BVHGB_API int bvhgb_generate_rays(void *rays, const bvhgb_camera *cam, bvhgb_stream stream);
/* tracerImage (CUDAKernels.cu:399-417): closest hit of each of the n Ray records, the pixel
 * {hit, diffuse, intCount} into img[i] and (optional) (primId, t) into hits[i]. bundle selects the
 * reference's block-cooperative schedule (rayBundles); the pixels do not depend on it. */
BVHGB_API int bvhgb_trace_ray_image(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const float *vert,
                                    const uint32_t *faces, const void *rays, uint32_t n,
                                    const bvhgb_trace_config *cfg, int bundle, bvhgb_pixel *img, bvhgb_hit *hits,
                                    bvhgb_stream stream);

/* Device-side traversal error bits seen since the last reset (2 = stack overflow, 4 = bad child
 * index); synchronous. */
BVHGB_API int bvhgb_trace_read_errors(uint32_t *flags, int reset);

/* ---- transfer (lib/cuda/cudaFN.hpp:27-33) --------------------------------------------------- */

/* copyMeshToGPU (cudaFN.cu:76-109): allocates and fills out->vert/norm/faces. */
BVHGB_API int bvhgb_copy_mesh_to_gpu(const float *vert, uint32_t numVert, const float *norm, uint32_t numNorm,
                                     const uint32_t *faces, uint32_t numFaces, bvhgb_mesh_raw *out);
/* copyMeshToHost (cudaFN.cu:149-182): copies back and frees the device mesh. */
BVHGB_API int bvhgb_copy_mesh_to_host(bvhgb_mesh_raw *mesh, float *vert, float *norm, uint32_t *faces);
/* copyBVHToGPU (cudaFN.cu:32-74): numNodes == 0 gives null pointers and succeeds. */
BVHGB_API int bvhgb_copy_bvh_to_gpu(const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, uint16_t maxLevel,
                                    bvhgb_bvh_pointer *out);
/* LBVH_allocateBVH (LBVH_CUDA.cu:396-424): fails when out already holds a BVH. */
BVHGB_API int bvhgb_allocate_bvh(bvhgb_bvh_pointer *out, uint32_t numFaces);
/* copyBVHToHost (cudaFN.cu:113-146): copies the nodes (numNodes of them) back, reports root
 * and max level, and frees the device BVH. */
BVHGB_API int bvhgb_copy_bvh_to_host(bvhgb_bvh_pointer *ptr, bvhgb_node *nodes, uint32_t capacity, uint32_t *root,
                                     uint16_t *maxLevel);
BVHGB_API int bvhgb_free_bvh(bvhgb_bvh_pointer *ptr);
BVHGB_API int bvhgb_free_mesh(bvhgb_mesh_raw *mesh);
/* BVH::fixLevels (BVH.cpp:39-70) on a host copy; returns the max level in *maxLevel. */
BVHGB_API int bvhgb_fix_levels_host(bvhgb_node *nodes, uint32_t numNodes, uint32_t root, uint16_t *maxLevel);
/* resetCUDA (cudaFN.cu:184-187): cudaDeviceReset of the current device. Every workspace, tracer
 * and device array made on it before is gone; what the library caches per context (shared-memory
 * opt-ins, the allocation-free build's array address) is looked up again in the new context, also
 * after a cudaDeviceReset the caller makes itself. */
BVHGB_API int bvhgb_reset_device(void);
/* cudaDeviceSynchronize (LBVH_doCUDASyc, doCudaDevSync, tracerDoCudaSync). */
BVHGB_API int bvhgb_device_sync(void);

/* ---- command layer (lib/base/Command.*, Config.*, src/main.cpp) ------------------------------ */

/* `bvhTest run CFG` (src/main.cpp:153-210): parse the JSON config, rewrite it with defaults, run
 * every command for every input. Commands: load, generate, camImport, BVHExport, BVHImport,
 * writeImg, writeData, copyToGPU, copyToHost, LBVH, bittner13GPU, CUDATracer, status, validate,
 * sleep. Returns 0, or the ErrorCode of the command that stopped an input. */
BVHGB_API int bvhgb_run_config(const char *path);
/* The bvhTest command line (list | generate FILE CMDs | run CFG). */
BVHGB_API int bvhgb_cli_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
