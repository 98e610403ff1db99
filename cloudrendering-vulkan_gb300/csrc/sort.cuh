// Scratch layout of the radix sort, shared by the context-owned entry point
// and the fixed-scratch one.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vcr {

constexpr uint32_t kSortTileKeys = 4096;  // keys per tile (256 threads x 16)
constexpr int kSortDigitBits = 8;         // bits a digit pass sorts on
constexpr int kSortRadix = 1 << kSortDigitBits;
constexpr int kSortMaxPasses = 32 / kSortDigitBits;

constexpr size_t sort_round256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t sort_tiles(uint32_t n) { return ((size_t)n + kSortTileKeys - 1) / kSortTileKeys; }
// hist [4][256] + tile counters [4] + look-back words [4][tiles][256]
constexpr size_t sort_scratch_header_bytes(uint32_t n) {
  return ((size_t)kSortMaxPasses * kSortRadix + kSortMaxPasses + (size_t)kSortMaxPasses * sort_tiles(n) * kSortRadix) *
         4;
}
// header + ping-pong copies of keys and values
constexpr size_t sort_scratch_bytes(uint32_t n) {
  return sort_round256(sort_scratch_header_bytes(n)) + 2 * sort_round256((size_t)n * 4);
}

// Queues the whole sort on `st` (no allocation, no synchronisation).
// `scratch` must hold sort_scratch_bytes(n) bytes; `d_err` is set to 2 if a
// look-back wait runs out.
cudaError_t sort_pairs_enqueue(int sm_count, int* d_err, void* scratch, const uint32_t* kin, const uint32_t* vin,
                               uint32_t* kout, uint32_t* vout, uint32_t n, uint32_t begin_bit, uint32_t end_bit,
                               cudaStream_t st);

}  // namespace vcr
