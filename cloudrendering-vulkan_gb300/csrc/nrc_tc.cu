// Radiance-cache queries on the fifth-generation tensor cores (tcgen05).
// No reference counterpart (the target adds the cache).
//
// A CTA holds kTcGroups warpgroups; each warpgroup of 128 threads runs its
// own 128-record tiles (thread i owns record row i of the tile, which is
// also TMEM lane i of its accumulator), with its own A operand, mbarrier,
// 64 TMEM columns and named barrier, so one group's epilogue overlaps
// another group's MMAs; the groups share the staged weights.  Per tile:
//   1. every thread encodes its record's 64 inputs as BF16 into the A
//      operand in shared memory (rows of 128 bytes in the 128-byte swizzled
//      K-major layout: 16-byte chunk c of row r sits at chunk c ^ (r & 7) of
//      the row, 8-row groups 1024 bytes apart);
//   2. one thread issues the layer as tcgen05.mma M=128, N=64 (N=16 for the
//      output layer), K=64 in four K=16 steps, BF16 operands from shared
//      memory, FP32 accumulators in TMEM, and commits to an mbarrier;
//   3. every thread waits on the mbarrier (bounded), reads its row of the
//      accumulators with tcgen05.ld, applies ReLU, packs BF16 and writes the
//      row back as the next layer's A operand — or, after the output layer,
//      adds throughput x max(y, 0) to its pixel's FP64 sums.
// The weights are staged once per CTA as the B operands: layer l as N rows
// (outputs) of K = 64 inputs, i.e. the transpose of the [in][out] layout,
// in the same swizzled layout.  Every wait is bounded; a wait that runs out
// sets the context's error word.
#include "nrc.cuh"
#include "nrc_mma.cuh"

namespace vcr {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTcRows = 128;                      // records per tile = MMA M = TMEM lanes
constexpr int kTcGroups = 4;                      // warpgroups (independent tiles) per CTA
constexpr int kTcThreads = 128 * kTcGroups;       // one thread per row of each group's tile
constexpr uint32_t kTcGroupCols = 64;             // TMEM columns per group: FP32 accumulators of N = 64
constexpr uint32_t kTcCols = kTcGroupCols * kTcGroups;  // 256 per CTA: two CTAs fill the SM's 512
constexpr int kRowBytes = 128;   // 64 BF16: one 128-byte swizzle span
constexpr int kHiddenB = kNrcWidth * kRowBytes;                    // 8 KB per hidden layer
constexpr int kOutB = kNrcOutPad * kRowBytes;                      // 2 KB output layer
constexpr int kOffA = kNrcHidden * kHiddenB + kOutB;               // 42 KB: 1024-aligned
constexpr int kABytes = kTcRows * kRowBytes;                       // 16 KB per group
constexpr int kOffDirs = kOffA + kTcGroups * kABytes;
constexpr int kTcSmem = kOffDirs + 3 * kNrcPosLevels * 4 + 1024;   // + slack to align the base to 1024
constexpr uint32_t kTcWait = 1u << 22;                             // bounded mbarrier polls
static_assert(kOffA % 1024 == 0, "operands must start on 1024-byte swizzle atoms");

__device__ __forceinline__ uint32_t sw128(uint32_t row, uint32_t chunk) {
  return (row >> 3) * 1024u + (row & 7u) * 128u + ((chunk ^ (row & 7u)) << 4);
}

// Shared-memory matrix descriptor: start address, leading byte offset
// (unused by swizzled K-major operands), 1024-byte stride between 8-row
// groups, the fixed version bits, 128-byte swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)2u << 61;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulators, BF16 A and B,
// both K-major, N and M.
__host__ __device__ constexpr uint32_t mma_idesc(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}

__device__ __forceinline__ uint32_t saddr_of(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0u;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// B operand of layer l from the global [in][out] BF16 weights: row n holds
// W[0..63][n]; gathered 8 inputs (one 16-byte chunk) at a time.
__device__ __forceinline__ void stage_weights(const bf16* __restrict__ w, unsigned char* base) {
  constexpr int kPairs = kNrcHidden * kNrcWidth * 8 + kNrcOutPad * 8;
  for (int p = threadIdx.x; p < kPairs; p += kTcThreads) {
    int l, n, c;
    if (p < kNrcHidden * kNrcWidth * 8) {
      l = p / (kNrcWidth * 8);
      n = (p / 8) % kNrcWidth;
      c = p % 8;
    } else {
      const int q = p - kNrcHidden * kNrcWidth * 8;
      l = kNrcHidden;
      n = q / 8;
      c = q % 8;
    }
    const int cols = nrc_layer_cols(l);
    const bf16* src = w + nrc_layer_offset(l) + (8 * c) * cols + n;
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint16_t lo = __bfloat16_as_ushort(src[(2 * j) * cols]);
      const uint16_t hi = __bfloat16_as_ushort(src[(2 * j + 1) * cols]);
      v[j] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
    *reinterpret_cast<uint4*>(base + l * kHiddenB + sw128((uint32_t)n, (uint32_t)c)) = make_uint4(v[0], v[1], v[2], v[3]);
  }
}

// The 64 inputs of one record (nrc_encode's order) as 8 chunks of 8 BF16.
__device__ __forceinline__ void encode_row(const NrcRecord& r, bool valid, f3 b0, f3 inv_ext, const float* dirs,
                                           unsigned char* a, uint32_t row, int levels, const float* gtab) {
  float ux = 0.f, uy = 0.f, uz = 0.f;
  if (valid) nrc_box_coords(r, b0, inv_ext, ux, uy, uz);
#pragma unroll
  for (int c = 0; c < 4; ++c) {  // position levels 4c .. 4c+3: (sin, cos) pairs
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int l = 4 * c + j;
      float sn = 0.f, cs = 0.f;
      if (valid && l < levels) {
        if (gtab) nrc_grid_level(gtab, l, ux, uy, uz, &sn, &cs);
        else nrc_encode_level_dir(l, dirs[3 * l], dirs[3 * l + 1], dirs[3 * l + 2], ux, uy, uz, &sn, &cs);
      }
      v[j] = pack_bf16(sn, cs);
    }
    *reinterpret_cast<uint4*>(a + sw128(row, (uint32_t)c)) = make_uint4(v[0], v[1], v[2], v[3]);
  }
  float sh[16];
#pragma unroll
  for (int d = 0; d < 2; ++d) {  // view SH (chunks 4, 5), sun SH (chunks 6, 7)
    if (valid) {
      if (d == 0) nrc_sh16(r.vx, r.vy, r.vz, sh);
      else nrc_sh16(r.sx, r.sy, r.sz, sh);
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) sh[i] = 0.f;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int o = 8 * h;
      *reinterpret_cast<uint4*>(a + sw128(row, (uint32_t)(4 + 2 * d + h))) =
          make_uint4(pack_bf16(sh[o], sh[o + 1]), pack_bf16(sh[o + 2], sh[o + 3]), pack_bf16(sh[o + 4], sh[o + 5]),
                     pack_bf16(sh[o + 6], sh[o + 7]));
    }
  }
}

__device__ __forceinline__ void group_sync(uint32_t g) {
  asm volatile("bar.sync %0, %1;" ::"r"(1u + g), "r"(128) : "memory");
}

__global__ void __launch_bounds__(kTcThreads, 2) nrc_infer_tc_kernel(const bf16* __restrict__ wbi, f3 b0, f3 inv_ext,
                                                                     int levels, const float* __restrict__ gtab,
                                                                  const NrcRecord* __restrict__ recs,
                                                                  const uint32_t* __restrict__ count_ptr,
                                                                  uint32_t capacity, double* __restrict__ sum,
                                                                  float* __restrict__ out, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_bar[kTcGroups];
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort[kTcGroups];
  unsigned char* base =
      smem_raw + ((1024u - (saddr_of(smem_raw) & 1023u)) & 1023u);  // 1024-byte aligned operands
  float* dirs = reinterpret_cast<float*>(base + kOffDirs);
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  const uint32_t grp = tid >> 7, row = tid & 127u;  // warpgroup, and this thread's row of its tiles
  unsigned char* A = base + kOffA + grp * kABytes;
  const uint32_t bar = saddr_of(&s_bar[grp]);

  if (warp == 0) {  // TMEM for all groups of the CTA
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr_of(&s_tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (row == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort[grp] = 0;
  }
  stage_weights(wbi, base);
  load_level_dirs(dirs);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = s_tmem + grp * kTcGroupCols;          // this group's accumulator columns
  const uint32_t my_lanes = tmem + ((32u * (warp & 3u)) << 16);  // this warp's 32 TMEM lanes
  const uint32_t count = min(*count_ptr, capacity);
  uint32_t phase = 0;

  for (uint32_t tile = blockIdx.x * kTcGroups + grp; tile * kTcRows < count; tile += gridDim.x * kTcGroups) {
    const uint32_t idx = tile * kTcRows + row;
    const bool valid = idx < count;
    NrcRecord r{};
    if (valid) r = recs[idx];
    encode_row(r, valid, b0, inv_ext, dirs, A, row, levels, gtab);
    float y[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
    for (int l = 0; l < kNrcLayers; ++l) {
      const uint32_t n = (uint32_t)nrc_layer_cols(l);
      fence_async_smem();  // the A rows written by the generic proxy, for the MMA's reads
      fence_before();
      group_sync(grp);
      if (row == 0) {
        fence_after();
        const uint32_t a0 = saddr_of(A), b0s = saddr_of(base + l * kHiddenB);
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k)
          mma_f16(tmem, smem_desc(a0 + 32u * k), smem_desc(b0s + 32u * k), mma_idesc(n), k);
        mma_commit(bar);
      }
      bool ok = false;
      for (uint32_t i = 0; i < kTcWait; ++i)
        if (bar_try_wait(bar, phase)) {
          ok = true;
          break;
        }
      phase ^= 1u;
      if (!ok) {
        atomicExch(err, 4);  // the MMA's completion never arrived: this group stops
        s_abort[grp] = 1;
      }
      fence_after();
      group_sync(grp);
      if (s_abort[grp]) goto done;
      if (l < kNrcHidden) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // 16 columns at a time: ReLU, BF16, two chunks of the next A row
          float v[16];
          tmem_ld16(my_lanes + 16u * q, v);
          tmem_wait_ld();
          uint32_t p[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) p[j] = pack_bf16(fmaxf(v[2 * j], 0.0f), fmaxf(v[2 * j + 1], 0.0f));
          *reinterpret_cast<uint4*>(A + sw128(row, 2u * q)) = make_uint4(p[0], p[1], p[2], p[3]);
          *reinterpret_cast<uint4*>(A + sw128(row, 2u * q + 1u)) = make_uint4(p[4], p[5], p[6], p[7]);
        }
      } else {
        float v[16];
        tmem_ld16(my_lanes, v);
        tmem_wait_ld();
        y[0] = v[0];
        y[1] = v[1];
        y[2] = v[2];
      }
    }
    if (valid) {
      if (out) {
        out[3 * idx] = y[0];
        out[3 * idx + 1] = y[1];
        out[3 * idx + 2] = y[2];
      }
      if (sum) {
        double* o = sum + 3 * (size_t)r.pix;
        atomicAdd(o + 0, (double)(r.w0 * fmaxf(y[0], 0.0f)));
        atomicAdd(o + 1, (double)(r.w1 * fmaxf(y[1], 0.0f)));
        atomicAdd(o + 2, (double)(r.w2 * fmaxf(y[2], 0.0f)));
      }
    }
  }
done:
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s_tmem), "r"(kTcCols) : "memory");
  }
}

}  // namespace

// Queries of one pass on the tensor cores; see nrc.cuh.
vcr_status nrc_infer_tc_launch(vcr_ctx* ctx, const void* wbi, f3 b0, f3 inv_ext, int levels, const float* gtab,
                               const NrcRecord* recs, const uint32_t* d_count, uint32_t capacity, double* sum,
                               float* out, cudaStream_t s) {
  VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
  int per_sm = 0;
  VCR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nrc_infer_tc_kernel, kTcThreads, kTcSmem));
  per_sm = per_sm < 1 ? 1 : (per_sm > (int)(512u / kTcCols) ? (int)(512u / kTcCols) : per_sm);  // TMEM: 512 columns
  const uint32_t tiles = (capacity + kTcRows - 1) / kTcRows;
  uint32_t blocks = (uint32_t)(ctx->sm_count * per_sm);
  const uint32_t need = (tiles + kTcGroups - 1) / kTcGroups;
  if (blocks > need) blocks = need;
  if (blocks == 0) return VCR_OK;
  nrc_infer_tc_kernel<<<blocks, kTcThreads, kTcSmem, s>>>(reinterpret_cast<const bf16*>(wbi), b0, inv_ext, levels,
                                                          gtab, recs, d_count, capacity, sum, out, ctx->d_error);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

}  // namespace vcr
