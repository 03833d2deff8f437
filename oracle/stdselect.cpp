// Oracle (test infrastructure only): the batch selection of the reference's CPU optimizers,
// restated with the same standard-library calls so that tied inefficiencies come out in the same
// order as in the reference (std::sort is not stable, so an index tie-break would differ):
//   Bittner13.cpp:258-283 and Bittner13Par.cpp:421-437: every node j gets (j, cost_j), leaves cost
//   0, then nth_element(begin, begin + k, end, cost descending) and sort(begin, begin + k, same).
// The element type is a pair of (node, cost) as in Bittner13Par.hpp:27 (the sequential optimizer's
// tuple has the same two fields); the comparator reads the cost only.
#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

#include "oracle.h"

extern "C" uint32_t orc_std_select(const orc_node *nodes, uint32_t n_nodes, uint32_t k, int do_sort,
                                   uint32_t *order_out) {
  std::vector<std::pair<uint32_t, float>> todo(n_nodes);
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < (int64_t)n_nodes; ++j) todo[j] = {(uint32_t)j, orc_inefficiency(nodes, (uint32_t)j)};
  if (k > n_nodes) k = n_nodes;
  auto comp = [](const std::pair<uint32_t, float> &l, const std::pair<uint32_t, float> &r) {
    return l.second > r.second;
  };
  std::nth_element(todo.begin(), todo.begin() + k, todo.end(), comp);
  if (do_sort) std::sort(todo.begin(), todo.begin() + k, comp);
  for (uint32_t j = 0; j < k; ++j) order_out[j] = todo[j].first;
  return k;
}
