// Exclusive prefix sum of uint32 counts (used to place variable-length
// outputs deterministically, e.g. beam segments per photon).
// Three launches: per-block sums, one-block scan of the sums, per-block scan
// + offset.  n <= 1024 * 2048 = 2^21.
#include "vcr_internal.h"

namespace vcr {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 2;  // items per thread -> 2048 per block

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t& total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (blockDim.x >> 5) ? s_warp[lane] : 0u;
    uint32_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= (uint32_t)o) wi += t;
    }
    if (lane < (blockDim.x >> 5)) s_warp[lane] = wi - w;
    if (lane == 31) s_warp[32] = wi;
  }
  __syncthreads();
  total = s_warp[32];
  uint32_t r = s_warp[warp] + incl - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                                                 uint32_t* __restrict__ sums) {
  __shared__ uint32_t s_warp[33];
  uint32_t base = blockIdx.x * kScanThreads * kScanItems + threadIdx.x * kScanItems;
  uint32_t v = 0;
  for (int j = 0; j < kScanItems; ++j)
    if (base + j < n) v += in[base + j];
  uint32_t total;
  block_exclusive_scan(v, s_warp, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_top_kernel(uint32_t* __restrict__ sums, uint32_t nb,
                                                                uint32_t* __restrict__ grand_total) {
  __shared__ uint32_t s_warp[33];
  uint32_t v = threadIdx.x < nb ? sums[threadIdx.x] : 0u;
  uint32_t total;
  uint32_t ex = block_exclusive_scan(v, s_warp, total);
  if (threadIdx.x < nb) sums[threadIdx.x] = ex;
  if (threadIdx.x == 0 && grand_total) *grand_total = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                                                  const uint32_t* __restrict__ sums,
                                                                  uint32_t* __restrict__ out) {
  __shared__ uint32_t s_warp[33];
  uint32_t base = blockIdx.x * kScanThreads * kScanItems + threadIdx.x * kScanItems;
  uint32_t vals[kScanItems];
  uint32_t v = 0;
  for (int j = 0; j < kScanItems; ++j) {
    vals[j] = base + j < n ? in[base + j] : 0u;
    v += vals[j];
  }
  uint32_t total;
  uint32_t ex = block_exclusive_scan(v, s_warp, total) + sums[blockIdx.x];
  for (int j = 0; j < kScanItems; ++j) {
    if (base + j < n) out[base + j] = ex;
    ex += vals[j];
  }
}

// out[i] = sum of in[0..i); *d_total (optional) = sum of all.  `sums` holds
// at least ceil(n / 2048) words.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums, uint32_t* d_total,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  uint32_t per = kScanThreads * kScanItems;
  uint32_t nb = (n + per - 1) / per;
  if (nb > (uint32_t)kScanThreads) return cudaErrorInvalidValue;
  scan_sums_kernel<<<nb, kScanThreads, 0, st>>>(in, n, sums);
  scan_top_kernel<<<1, kScanThreads, 0, st>>>(sums, nb, d_total);
  scan_apply_kernel<<<nb, kScanThreads, 0, st>>>(in, n, sums, out);
  return cudaGetLastError();
}

}  // namespace vcr
