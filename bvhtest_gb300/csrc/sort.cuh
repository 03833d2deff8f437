// Internal interface of the onesweep radix sort (sort.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace bvhgb {
// Sets the kernels' shared-memory attributes; call once before any stream capture.
int sort_prepare();
// Scratch bytes for sorting n pairs on key bits [beginBit, endBit).
size_t sort_temp_bytes(uint32_t n, uint32_t keyBytes, uint32_t beginBit, uint32_t endBit);
// Device word that the look-back sets to a non-zero error bit if a bounded wait gives up.
uint32_t *sort_error_word(void *temp, uint32_t n, uint32_t keyBytes, uint32_t beginBit, uint32_t endBit);
// Stable ascending sort; temp must hold sort_temp_bytes(...) bytes. tileKeys = keys per CTA of the
// onesweep passes (2048, 4096 or 8192; the result does not depend on it); 0 takes the process-wide
// default (kSortTileDefault unless bvhgb_sort_set_default_tile changed it).
constexpr uint32_t kSortTileDefault = 8192;
bool sort_tile_valid(uint32_t tileKeys);
// Polls of an unpublished predecessor before a look-back gives up (0xFFFFFFFF: the default).
int sort_set_spin_limit(uint32_t limit, uint32_t *previous);
int sort_pairs(void *temp, const void *keysIn, void *keysOut, const uint32_t *valsIn, uint32_t *valsOut, uint32_t n,
               uint32_t keyBytes, uint32_t beginBit, uint32_t endBit, cudaStream_t s, uint32_t tileKeys = 0);
// The values of the first k pairs of a stable ascending sort of (keys, vals), 32-bit keys, in that
// order, into valsOut[0, k) (k <= n), without sorting all n pairs; temp must hold
// select_temp_bytes(n, k) bytes.
size_t select_temp_bytes(uint32_t n, uint32_t k);
int select_smallest(void *temp, const uint32_t *keys, const uint32_t *vals, uint32_t n, uint32_t k, uint32_t *valsOut,
                    cudaStream_t s, uint32_t tileKeys = 0);
}  // namespace bvhgb
