// Stable LSD radix sort of (uint32 key, uint32 value) pairs, and the Morton
// codes the photon-beam pipeline sorts.
//
// Reference design: PPB_RadixSort_LocalSort.comp (block-local 4-bit sort by
// four 1-bit split passes with a Blelloch scan + 16-bin histogram),
// PPB_RadixSort_PrefixSum.comp and PPB_RadixSort_GlobalSort.comp (scan of
// the histograms, scatter), driven from RenderTechniquePPB.cpp:465-491; keys
// from expandBits/getMortonCode (PPB_PT.comp:317-333).
//
// GB300 design: the same stable order (a stable LSD sort's result does not
// depend on its digit width) from 8-bit digits, so 32-bit keys take 4
// passes instead of the reference's 8.  One histogram kernel computes the
// digit counts of every pass at once and one small kernel turns them into
// offsets; each digit pass is then ONE kernel over 4096-key tiles: stable
// in-tile ranking from eight warp ballots of the digit bits, a decoupled
// look-back across tiles (one thread a digit; tile ids taken in launch
// order from an atomic counter, so every tile waits only on tiles already
// running), shared-memory staging and a coalesced scatter.  Each pass reads
// and writes every pair once (16 B/key per pass).  Spins are bounded: a
// wait that runs out sets the context's error word instead of hanging.
#include "vcr_internal.h"
#include "sort.cuh"

namespace vcr {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys
constexpr int kSortWarps = kSortThreads / 32;
constexpr uint32_t kFlagA = 1u << 30;                 // tile aggregate published
constexpr uint32_t kFlagP = 2u << 30;                 // inclusive prefix published
constexpr uint32_t kCountMask = (1u << 30) - 1u;

struct SortScratch {
  uint32_t* hist;     // [4][256] digit counts per pass, then their exclusive offsets
  uint32_t* tiles;    // [4] tile counters
  uint32_t* desc;     // [4][ntiles][256] look-back words
  uint32_t* keys_tmp; // n
  uint32_t* vals_tmp; // n
};

static_assert(kSortTile == (int)kSortTileKeys, "tile size");
static_assert(kSortThreads == kSortRadix, "one thread a digit in the tile-level steps");

static SortScratch carve(void* base, uint32_t n) {
  uint32_t* p = reinterpret_cast<uint32_t*>(base);
  SortScratch s;
  s.hist = p;
  s.tiles = p + kSortMaxPasses * kSortRadix;
  s.desc = p + kSortMaxPasses * kSortRadix + kSortMaxPasses;
  uint8_t* b = reinterpret_cast<uint8_t*>(base) + sort_round256(sort_scratch_header_bytes(n));
  s.keys_tmp = reinterpret_cast<uint32_t*>(b);
  s.vals_tmp = reinterpret_cast<uint32_t*>(b + sort_round256((size_t)n * 4));
  return s;
}

// Mask of pass p's digit: 8 bits, or the bits left below end_bit in the
// last pass (so bits at or above end_bit never decide the order).
__host__ __device__ __forceinline__ uint32_t digit_mask(uint32_t begin_bit, uint32_t end_bit, uint32_t p) {
  const uint32_t w = end_bit - (begin_bit + kSortDigitBits * p);
  return w >= kSortDigitBits ? (uint32_t)kSortRadix - 1u : (1u << w) - 1u;
}

// Digit counts of all passes in one read of the keys.
__global__ void __launch_bounds__(256) sort_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                        uint32_t begin_bit, uint32_t end_bit, uint32_t passes,
                                                        uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kSortMaxPasses][kSortRadix];
  for (int i = threadIdx.x; i < kSortMaxPasses * kSortRadix; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t k = keys[i];
    for (uint32_t p = 0; p < passes; ++p)
      atomicAdd(&h[p][(k >> (begin_bit + kSortDigitBits * p)) & digit_mask(begin_bit, end_bit, p)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < (int)(passes * kSortRadix); i += blockDim.x) {
    uint32_t v = (&h[0][0])[i];
    if (v) atomicAdd(hist + i, v);
  }
}

// Exclusive block-wide scan of one value a thread (256 threads); `warp_sums`
// holds kSortWarps words of shared memory.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* warp_sums) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  if (lane == 31u) warp_sums[warp] = incl;
  __syncthreads();
  uint32_t before = 0;
  for (uint32_t w = 0; w < warp; ++w) before += warp_sums[w];
  __syncthreads();  // warp_sums may be reused after this
  return before + incl - x;
}

// Each pass's digit counts into exclusive offsets, in place (one CTA of 256
// threads a pass).
__global__ void __launch_bounds__(kSortRadix) sort_offsets_kernel(uint32_t* __restrict__ hist) {
  __shared__ uint32_t ws[kSortWarps];
  uint32_t* h = hist + blockIdx.x * kSortRadix;
  h[threadIdx.x] = block_exclusive_scan(h[threadIdx.x], ws);
}

// One digit pass over 4096-key tiles (tile ids in launch order from an
// atomic counter).  In-warp stable ranking: warp w holds keys
// [w*32*kSortItems, ...) of the tile in kSortItems rounds of 32 (round j,
// lane l = key w*32*I + 32j + l); eight ballots of the digit bits give each
// lane the lanes of its round with the same digit, and the lowest of them
// advances the warp's running count of that digit in shared memory.  Then
// one thread a digit: the exclusive prefix over the warps, the tile's digit
// starts (block scan), the decoupled look-back for the digit's global base.
// The tile's values come to shared memory by asynchronous copies while the
// keys are ranked; the staged keys carry their tile index.
__global__ void __launch_bounds__(kSortThreads, 4) sort_pass_kernel(const uint32_t* __restrict__ kin,
                                                                 const uint32_t* __restrict__ vin,
                                                                 uint32_t* __restrict__ kout,
                                                                 uint32_t* __restrict__ vout, uint32_t n,
                                                                 uint32_t shift, uint32_t dmask, uint32_t pass,
                                                                 SortScratch sc, uint32_t spin_limit,
                                                                 int* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t s_dyn[];
  uint32_t* s_keys = s_dyn;                                   // [kSortTile] sorted keys of the tile
  uint32_t* s_vals = s_keys + kSortTile;                      // [kSortTile] values in tile order
  uint32_t* s_wcnt = s_vals + kSortTile;                      // [kSortWarps][kSortRadix]
  uint16_t* s_src = reinterpret_cast<uint16_t*>(s_wcnt + kSortWarps * kSortRadix);  // [kSortTile]
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_tile_start[kSortRadix];  // digit start inside the tile
  __shared__ uint32_t s_base[kSortRadix];        // global output offset of the digit's run
  __shared__ uint32_t s_ws[kSortWarps];

  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t lt = (1u << lane) - 1u;
  if (threadIdx.x == 0) s_tile = atomicAdd(sc.tiles + pass, 1u);
  uint32_t* wc = s_wcnt + warp * kSortRadix;
  for (uint32_t d = lane; d < (uint32_t)kSortRadix; d += 32u) wc[d] = 0u;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t tile0 = tile * kSortTile;
  const uint32_t count = min((uint32_t)kSortTile, n - tile0);
  if (vin) {
    for (uint32_t i = threadIdx.x; i < count; i += kSortThreads)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(s_vals + i)),
                   "l"(vin + tile0 + i)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  }

  uint32_t key[kSortItems], rank[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t local = warp * (32 * kSortItems) + j * 32 + lane;
    const bool ok = local < count;
    key[j] = ok ? kin[tile0 + local] : 0u;
    const uint32_t d = (key[j] >> shift) & dmask;
    uint32_t peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
    for (int i = 0; i < kSortDigitBits; ++i) {
      const uint32_t b = __ballot_sync(0xffffffffu, ok && ((d >> i) & 1u));
      peers &= ((d >> i) & 1u) ? b : ~b;
    }
    const uint32_t leader = __ffs(peers) - 1u;  // peers includes this lane when ok
    uint32_t base = 0;
    if (ok && lane == leader) {
      base = wc[d];
      wc[d] = base + __popc(peers);
    }
    base = __shfl_sync(0xffffffffu, base, ok ? leader : lane);
    rank[j] = base + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  {
    const uint32_t d = threadIdx.x;  // one thread a digit
    uint32_t total = 0;
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = s_wcnt[w * kSortRadix + d];
      s_wcnt[w * kSortRadix + d] = total;  // exclusive prefix over warps
      total += c;
    }
    s_tile_start[d] = block_exclusive_scan(total, s_ws);
    const uint32_t g = sc.hist[pass * kSortRadix + d];  // exclusive global offset of the digit
    volatile uint32_t* desc = sc.desc + (size_t)pass * ((size_t)gridDim.x * kSortRadix);
    if (tile == 0) {
      desc[d] = kFlagP | total;
      s_base[d] = g;
    } else {
      desc[(size_t)tile * kSortRadix + d] = kFlagA | total;
      uint32_t excl = 0;
      int t = (int)tile - 1;
      uint32_t spins = 0;
      while (t >= 0) {
        uint32_t w = desc[(size_t)t * kSortRadix + d];
        uint32_t flag = w & ~kCountMask;
        if (flag == 0u) {
          if (++spins > spin_limit) {
            atomicExch(err, 2);  // look-back wait ran out
            break;
          }
          continue;
        }
        excl += w & kCountMask;
        if (flag == kFlagP) break;
        --t;
      }
      desc[(size_t)tile * kSortRadix + d] = kFlagP | (excl + total);
      s_base[d] = g + excl;
    }
  }
  __syncthreads();
  // stage the keys in sorted order with the tile-order index they came from
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t local = warp * (32 * kSortItems) + j * 32 + lane;
    if (local < count) {
      const uint32_t d = (key[j] >> shift) & dmask;
      const uint32_t pos = s_tile_start[d] + wc[d] + rank[j];
      s_keys[pos] = key[j];
      s_src[pos] = (uint16_t)local;
    }
  }
  if (vin) asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < count; i += kSortThreads) {
    uint32_t k = s_keys[i];
    uint32_t d = (k >> shift) & dmask;
    uint32_t o = s_base[d] + (i - s_tile_start[d]);
    if (o < n) {  // always true unless a look-back wait ran out (error word set)
      const uint32_t src = s_src[i];
      kout[o] = k;
      vout[o] = vin ? s_vals[src] : tile0 + src;
    }
  }
}

constexpr size_t kSortPassSmem =
    (size_t)(2 * kSortTile + kSortWarps * kSortRadix) * sizeof(uint32_t) + (size_t)kSortTile * sizeof(uint16_t);

// Runs the passes for bits [begin_bit, end_bit) in 8-bit digits (the last
// digit narrower when the range is not a multiple of 8 bits).  The pass
// chain ping-pongs between `out` and the scratch copy so the last pass
// lands in `out`; in-place calls (in == out) with an odd pass count start
// from a copy.
cudaError_t sort_pairs_enqueue(int sm_count, int* d_err, void* scratch, const uint32_t* kin, const uint32_t* vin,
                               uint32_t* kout, uint32_t* vout, uint32_t n, uint32_t begin_bit, uint32_t end_bit,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  uint32_t passes = (end_bit - begin_bit + kSortDigitBits - 1) / kSortDigitBits;
  const uint32_t spins = wait_limits().sort_lookback;
  SortScratch sc = carve(scratch, n);
  uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
  cudaError_t e = cudaMemsetAsync(scratch, 0, sort_scratch_header_bytes(n), st);
  if (e != cudaSuccess) return e;
  int hb = (int)std::min<uint32_t>((n + 255) / 256, (uint32_t)std::max(sm_count, 1) * 4);
  sort_hist_kernel<<<hb, 256, 0, st>>>(kin, n, begin_bit, end_bit, passes, sc.hist);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  sort_offsets_kernel<<<passes, kSortRadix, 0, st>>>(sc.hist);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(sort_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSortPassSmem)) !=
      cudaSuccess)
    return e;
  const uint32_t* ck = kin;
  const uint32_t* cv = vin;
  // Destinations alternate; the first one is `out` when that makes the last
  // pass land in `out` (odd count) unless the input aliases `out`, in which
  // case the chain starts in scratch and ends with one copy.
  bool alias = (kin == kout) || (vin && vin == vout);
  bool first_to_out = (passes % 2u == 1u) && !alias;
  for (uint32_t p = 0; p < passes; ++p) {
    bool to_out = ((p % 2u) == 0u) == first_to_out;
    uint32_t* nk = to_out ? kout : sc.keys_tmp;
    uint32_t* nv = to_out ? vout : sc.vals_tmp;
    sort_pass_kernel<<<ntiles, kSortThreads, kSortPassSmem, st>>>(ck, cv, nk, nv, n, begin_bit + kSortDigitBits * p,
                                                                  digit_mask(begin_bit, end_bit, p), p, sc, spins,
                                                                  d_err);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ck = nk;
    cv = nv;
  }
  if (ck != kout) {
    if ((e = cudaMemcpyAsync(kout, ck, (size_t)n * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(vout, cv, (size_t)n * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Morton codes
// ---------------------------------------------------------------------------
// Spread the low 10 bits of v so two zeros separate each (Karras 2012; the
// reference's 8-bit expandBits is PPB_PT.comp:319-325).
__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__device__ __forceinline__ uint32_t quant(float p, float b0, float ext, float cells) {
  float q = ((p - b0) / ext) * cells;
  q = fminf(fmaxf(q, 0.0f), cells - 1.0f);
  return (uint32_t)q;
}

// bits == 30: 10 bits per axis over the box [b0, b1] (x << 2 | y << 1 | z);
// bits == 24: the reference's getMortonCode (PPB_PT.comp:327-333), relative
// position / 256 clamped to [0, 255] per axis.
__global__ void morton_kernel(const float* __restrict__ pts, uint32_t n, f3 b0, f3 b1, int bits,
                              uint32_t* __restrict__ codes) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  f3 p = mk(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  if (bits == 24) {
    f3 r = p - b0;
    uint32_t x = (uint32_t)fminf(fmaxf(r.x / 256.0f, 0.0f), 255.0f);
    uint32_t y = (uint32_t)fminf(fmaxf(r.y / 256.0f, 0.0f), 255.0f);
    uint32_t z = (uint32_t)fminf(fmaxf(r.z / 256.0f, 0.0f), 255.0f);
    codes[i] = (expand10(x) << 2) + (expand10(y) << 1) + expand10(z);
    return;
  }
  f3 e = b1 - b0;
  uint32_t x = quant(p.x, b0.x, e.x, 1024.0f), y = quant(p.y, b0.y, e.y, 1024.0f), z = quant(p.z, b0.z, e.z, 1024.0f);
  codes[i] = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
}

vcr_status morton_launch(vcr_ctx* ctx, const float* d_pts, uint32_t n, const float b0[3], const float b1[3],
                         int bits, uint32_t* d_codes, cudaStream_t st) {
  if (n == 0) return VCR_OK;
  morton_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_pts, n, mk(b0[0], b0[1], b0[2]), mk(b1[0], b1[1], b1[2]), bits,
                                                 d_codes);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_radix_sort_pairs(vcr_ctx* ctx, const uint32_t* d_keys_in, const uint32_t* d_vals_in,
                                                   uint32_t* d_keys_out, uint32_t* d_vals_out, uint32_t n,
                                                   uint32_t begin_bit, uint32_t end_bit, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (n && (!d_keys_in || !d_keys_out || !d_vals_out)) return fail(ctx, VCR_ERR_INVALID, "null sort buffer");
  if (begin_bit >= end_bit || end_bit > 32) return fail(ctx, VCR_ERR_INVALID, "bit range [%u, %u)", begin_bit, end_bit);
  if (n > (1u << 30) - 1u) return fail(ctx, VCR_ERR_UNSUPPORTED, "sort of %u keys (max 2^30 - 1)", n);
  if (d_vals_in == d_vals_out && d_keys_in != d_keys_out)
    return fail(ctx, VCR_ERR_INVALID, "values may alias only together with keys");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  vcr_status st = ensure_scratch(ctx, sort_scratch_bytes(n));
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  VCR_CUDA(ctx, sort_pairs_enqueue(ctx->sm_count, ctx->d_error, ctx->d_scratch, d_keys_in, d_vals_in, d_keys_out,
                                   d_vals_out, n, begin_bit, end_bit, s));
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_morton_codes(vcr_ctx* ctx, const float* d_points, uint32_t n,
                                               const float bounds_min[3], const float bounds_max[3],
                                               uint32_t bits, uint32_t* d_codes, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (n && (!d_points || !d_codes || !bounds_min || !bounds_max)) return fail(ctx, VCR_ERR_INVALID, "null argument");
  if (bits != 30 && bits != 24) return fail(ctx, VCR_ERR_INVALID, "Morton bits must be 30 or 24");
  return morton_launch(ctx, d_points, n, bounds_min, bounds_max, (int)bits, d_codes, (cudaStream_t)stream);
}
