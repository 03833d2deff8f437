// Learned reinsertion scorer: internal interface between the feature / MLP kernels and the
// optimizer's node selection.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bvhgb.h"

namespace bvhgb {

constexpr int kMlpIn = BVHGB_LR_FEATURES;  // 24 features (14 used, zero padded)
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = BVHGB_MLP_PARAMS;  // W1[64][24] b1[64] W2[64][64] b2[64] W3[64] b3
constexpr int kMlpRaw = 10;                   // raw (non-rank) features
constexpr uint32_t kRankBins = 65536;         // rank histogram bins (top 16 bits of the ordered image)
constexpr uint32_t kDepthRounds = 8;          // depth features are exact up to 2^8 = 256 levels
constexpr float kTargetEps = 0.16f;           // target = sign(g) ln(1 + |g| numLeaves / kTargetEps)

// Device scratch for the features of one tree (sized for numNodes nodes).
struct LrScratch {
  uint32_t numNodes = 0;
  unsigned long long *ad = nullptr;  // depth pointer jumping: distance << 32 | ancestor
  uint32_t *leafCount = nullptr, *hist = nullptr, *err = nullptr;
  float *sa = nullptr;        // per-node surface area (compact copy)
  uint32_t *par = nullptr;    // per-node parent | leaf bit (compact copy)
  unsigned long long *acc = nullptr;  // leaf-count accumulators: 2^40 per arrival + the arriving count
  uint4 *pend = nullptr;   // per row: the four rank bins (16 bits each) and features 8-9 (BF16)
  uint16_t *x = nullptr;  // BF16 feature rows [numInner][24]
  float *y = nullptr;     // scorer output per inner node
};

int lr_scratch_alloc(LrScratch &s, uint32_t numNodes);
void lr_scratch_free(LrScratch &s);

// Feature rows of the listed inner nodes into s.x (BF16), in list order.
int lr_features(LrScratch &s, const bvhgb_node *nodes, uint32_t numNodes, uint32_t root, const uint32_t *inner,
                uint32_t numInner, float invLog2Leaves, cudaStream_t st);

// Scorer forward over s.x, then the selection keys: key = ~order(y) so that an ascending sort gives
// the descending predicted reduction; vals = node ids.
int lr_score_keys(const bvhgb_mlp *m, LrScratch &s, const bvhgb_node *nodes, uint32_t root, const uint32_t *inner,
                  uint32_t numInner, uint32_t *keys, uint32_t *vals, cudaStream_t st);

float lr_inv_log2_leaves(uint32_t numLeaves);

}  // namespace bvhgb

namespace bvhgb {
// Device word the feature kernels OR error bits into (kErrBadIndex for a broken parent chain).
uint32_t *lr_error_word(LrScratch &s);
}  // namespace bvhgb
