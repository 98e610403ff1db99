// Density grid: fBm generation, bricking (FP32 / FP16 / BF16 with a per-brick
// FP32 scale), brick majorants, trilinear sampling and the DDA trace.
//
// Replaces the reference's dense R32F 3D image upload (main.cpp:266-335) and
// its single global majorant (Grid3D::GetMajorant, Grid3D.h:180-192;
// main.cpp:152).
#include "vcr_internal.h"
#include "vcr_fbm.cuh"

namespace vcr {

__constant__ FbmConst c_fbm;

__global__ void fbm_kernel(float* __restrict__ out, uint64_t total) {
  uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nx = c_fbm.n[0], ny = c_fbm.n[1];
  for (; idx < total; idx += stride) {
    uint32_t i = (uint32_t)(idx % nx);
    uint64_t r = idx / nx;
    uint32_t j = (uint32_t)(r % ny);
    uint32_t k = (uint32_t)(r / ny);
    out[idx] = fbm_density(c_fbm, i, j, k);
  }
}

// One warp per brick (8 bricks per 256-thread CTA): lane l holds texel rows
// l and l + 32 of the brick (row r = y + 8 z, 8 texels along x, zero
// outside the grid), the warp's maximum is the brick's scale, and each row
// is stored as one 16-byte (FP16 / BF16) or two (FP32) vectors into the
// brick's contiguous 512 texels.
constexpr int kBrickWarps = 8;

template <int P>
__global__ void __launch_bounds__(kBrickWarps * 32) brick_kernel(const float* __restrict__ dense,
                                                                 void* __restrict__ bricks,
                                                                 float* __restrict__ scales, int nx, int ny, int nz,
                                                                 int bx, int by, uint32_t nbricks) {
  const uint32_t b = blockIdx.x * kBrickWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nbricks) return;  // warp-uniform
  const int ib = (int)(b % (uint32_t)bx), jb = (int)((b / (uint32_t)bx) % (uint32_t)by);
  const int kb = (int)(b / ((uint32_t)bx * (uint32_t)by));
  const int i0 = ib * kBrick;
  const bool vec = (nx & 3) == 0 && i0 + kBrick <= nx;  // rows 16-byte aligned and whole
  float v[2][8];
  float m = -INFINITY;  // the max over the brick's 512 values (out-of-grid texels are 0)
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int r = lane + 32 * h;
    const int j = jb * kBrick + (r & 7), k = kb * kBrick + (r >> 3);
    const size_t base = (size_t)i0 + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)k);
    if (j < ny && k < nz && vec) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(dense + base));
      const float4 c = __ldg(reinterpret_cast<const float4*>(dense + base) + 1);
      v[h][0] = a.x; v[h][1] = a.y; v[h][2] = a.z; v[h][3] = a.w;
      v[h][4] = c.x; v[h][5] = c.y; v[h][6] = c.z; v[h][7] = c.w;
    } else {
#pragma unroll
      for (int x = 0; x < 8; ++x) v[h][x] = (j < ny && k < nz && i0 + x < nx) ? __ldg(dense + base + x) : 0.0f;
    }
#pragma unroll
    for (int x = 0; x < 8; ++x) m = fmaxf(m, v[h][x]);
  }
  const size_t brick = (size_t)b << 9;
  if (P == 0) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(bricks) + brick + 8 * (lane + 32 * h));
      dst[0] = make_float4(v[h][0], v[h][1], v[h][2], v[h][3]);
      dst[1] = make_float4(v[h][4], v[h][5], v[h][6], v[h][7]);
    }
    return;
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const float s = m;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    uint32_t w[4];
#pragma unroll
    for (int x = 0; x < 8; x += 2) {
      const float q0 = s > 0.0f ? v[h][x] / s : 0.0f, q1 = s > 0.0f ? v[h][x + 1] / s : 0.0f;
      if (P == 1) {
        const __half2 hv = __halves2half2(__float2half_rn(q0), __float2half_rn(q1));
        w[x / 2] = *reinterpret_cast<const uint32_t*>(&hv);
      } else {
        const __nv_bfloat162 bv = __halves2bfloat162(__float2bfloat16_rn(q0), __float2bfloat16_rn(q1));
        w[x / 2] = *reinterpret_cast<const uint32_t*>(&bv);
      }
    }
    uint16_t* base16 = reinterpret_cast<uint16_t*>(bricks) + brick + 8 * (lane + 32 * h);
    *reinterpret_cast<uint4*>(base16) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  if (lane == 0) scales[b] = s;
}

// The stored grid decoded to dense floats, x fastest (texel() per voxel).
__global__ void decode_kernel(GridView g, float* __restrict__ out, uint64_t total) {
  const uint64_t nx = (uint64_t)g.n[0], ny = (uint64_t)g.n[1];
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = idx / nx;
    out[idx] = texel(g, (int)(idx - r * nx), (int)(r % ny), (int)(r / ny));
  }
}

// Brick majorant: max decoded texel over [8b-1, 8b+8] per axis (clamped),
// which bounds every trilinear sample whose position lies in the brick's
// cell (a sample at texel coordinate u reads floor(u - 1/2) and the next).
__global__ void __launch_bounds__(256) majorant_kernel(GridView g, float* __restrict__ maj,
                                                       unsigned int* __restrict__ gmax) {
  __shared__ float red[8];
  uint32_t b = blockIdx.x;
  int ib = (int)(b % (uint32_t)g.nb[0]), jb = (int)((b / (uint32_t)g.nb[0]) % (uint32_t)g.nb[1]);
  int kb = (int)(b / ((uint32_t)g.nb[0] * (uint32_t)g.nb[1]));
  float m = 0.0f;
  for (int t = threadIdx.x; t < 1000; t += blockDim.x) {
    int di = t % 10, dj = (t / 10) % 10, dk = t / 100;
    int i = min(max(ib * kBrick - 1 + di, 0), g.n[0] - 1);
    int j = min(max(jb * kBrick - 1 + dj, 0), g.n[1] - 1);
    int k = min(max(kb * kBrick - 1 + dk, 0), g.n[2] - 1);
    m = fmaxf(m, texel(g, i, j, k));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
    m = fmaxf(m, red[0]);
    maj[b] = m;
    atomicMax(gmax, __float_as_uint(m));  // non-negative floats order as integers
  }
}

// Level l+1 of the majorant pyramid: max over the (up to) 2x2x2 cells of
// level l it covers.
__global__ void majorant_reduce_kernel(const float* __restrict__ src, int sx, int sy, int sz,
                                       float* __restrict__ dst, int dx, int dy, int dz) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (uint32_t)(dx * dy * dz)) return;
  int i = (int)(c % (uint32_t)dx), j = (int)((c / (uint32_t)dx) % (uint32_t)dy), k = (int)(c / ((uint32_t)dx * dy));
  float m = 0.0f;
  for (int dk = 0; dk < 2; ++dk)
    for (int dj = 0; dj < 2; ++dj)
      for (int di = 0; di < 2; ++di) {
        int a = 2 * i + di, b = 2 * j + dj, e = 2 * k + dk;
        if (a < sx && b < sy && e < sz) m = fmaxf(m, src[(size_t)a + (size_t)sx * ((size_t)b + (size_t)sy * e)]);
      }
  dst[c] = m;
}

__global__ void sample_kernel(GridView g, SceneView s, const float* __restrict__ pos, float* __restrict__ out,
                              uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  f3 p = mk(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  out[i] = density_at(g, s, p);
}

__global__ void dda_trace_kernel(SceneView s, int nc0, int nc1, int nc2, const float* __restrict__ o,
                                 const float* __restrict__ d, uint32_t n, uint32_t max_cells,
                                 uint32_t* __restrict__ cells, float* __restrict__ tt,
                                 uint32_t* __restrict__ count) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nc[3] = {nc0, nc1, nc2};
  f3 org = mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
  f3 dir = mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
  float tmin, tmax;
  uint32_t k = 0;
  if (slab(org, dir, s.b0, s.b1, tmin, tmax) && tmax >= 0.0f) {
    if (tmin > 0.0f) {
      org = along(org, dir, tmin);
      slab(org, dir, s.b0, s.b1, tmin, tmax);
    }
    Dda dd;
    dda_init(dd, org, dir, recip(dir), s.b0, s.cell, s.icell, nc);
    float t = 0.0f;
    while (k < max_cells) {
      float e = dda_cell_exit(dd);
      float se = fminf(e, tmax);
      size_t at = (size_t)i * max_cells + k;
      cells[at] = dda_linear(dd, nc);
      tt[2 * at] = t;
      tt[2 * at + 1] = se;
      ++k;
      if (e >= tmax) break;
      if (!dda_advance(dd, nc)) break;
      t = se;
    }
  }
  count[i] = k;
}

void fbm_permutation(uint64_t seed, uint8_t perm[256]) { fbm_make_perm(seed, perm); }

vcr_status grid_fbm_device(vcr_ctx* ctx, float* d_dense, const vcr_grid_desc* desc, const vcr_fbm_desc* fbm,
                           cudaStream_t s) {
  FbmConst c{};
  fbm_make_perm(fbm->seed, c.perm);
  for (int a = 0; a < 3; ++a) c.n[a] = desc->size[a];
  c.octaves = fbm->octaves;
  c.lacunarity = fbm->lacunarity;
  c.gain = fbm->gain;
  c.f0 = fbm->base_frequency;
  VCR_CUDA(ctx, cudaMemcpyToSymbolAsync(c_fbm, &c, sizeof(c), 0, cudaMemcpyHostToDevice, s));
  uint64_t total = (uint64_t)desc->size[0] * desc->size[1] * desc->size[2];
  int blocks = ctx->sm_count * 8;
  fbm_kernel<<<blocks, 256, 0, s>>>(d_dense, total);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

vcr_status grid_build(vcr_ctx* ctx, const float* d_dense, const vcr_grid_desc* desc, int precision,
                      cudaStream_t s) {
  int n[3] = {(int)desc->size[0], (int)desc->size[1], (int)desc->size[2]};
  int nb[3];
  for (int a = 0; a < 3; ++a) nb[a] = (n[a] + kBrick - 1) / kBrick;
  uint64_t nbricks = (uint64_t)nb[0] * nb[1] * nb[2];
  if (nbricks > (1ull << 22)) return fail(ctx, VCR_ERR_UNSUPPORTED, "grid too large: %llu bricks (max 2^22)",
                                          (unsigned long long)nbricks);
  size_t esz = precision == 0 ? 4 : 2;
  // release the previous grid
  cudaFree(ctx->d_bricks);
  cudaFree(ctx->d_scales);
  cudaFree(ctx->d_majorants);
  ctx->d_bricks = nullptr;
  ctx->d_scales = nullptr;
  ctx->d_majorants = nullptr;
  ctx->has_grid = false;
  VCR_CUDA(ctx, cudaMalloc(&ctx->d_bricks, nbricks * kBrickVoxels * esz));
  VCR_CUDA(ctx, cudaMalloc(&ctx->d_scales, nbricks * sizeof(float)));
  // majorant pyramid: level l has ceil(nb / 2^l) cells per axis; each level
  // starts on a 16-byte boundary (bulk copies into shared memory need it)
  size_t mtotal = 0;
  for (int l = 0; l < 4; ++l) {
    for (int a = 0; a < 3; ++a) ctx->mnb[l][a] = l == 0 ? nb[a] : (ctx->mnb[l - 1][a] + 1) / 2;
    ctx->moff[l] = mtotal;
    size_t cnt = (size_t)ctx->mnb[l][0] * ctx->mnb[l][1] * ctx->mnb[l][2];
    mtotal += (cnt + 3) & ~(size_t)3;
  }
  VCR_CUDA(ctx, cudaMalloc(&ctx->d_majorants, mtotal * sizeof(float)));
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_majorants, 0, mtotal * sizeof(float), s));
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_scales, 0, nbricks * sizeof(float), s));
  if (precision == 0)
    brick_kernel<0><<<(unsigned)((nbricks + kBrickWarps - 1) / kBrickWarps), kBrickWarps * 32, 0, s>>>(
        d_dense, ctx->d_bricks, ctx->d_scales, n[0], n[1], n[2], nb[0], nb[1], (uint32_t)nbricks);
  else if (precision == 1)
    brick_kernel<1><<<(unsigned)((nbricks + kBrickWarps - 1) / kBrickWarps), kBrickWarps * 32, 0, s>>>(
        d_dense, ctx->d_bricks, ctx->d_scales, n[0], n[1], n[2], nb[0], nb[1], (uint32_t)nbricks);
  else
    brick_kernel<2><<<(unsigned)((nbricks + kBrickWarps - 1) / kBrickWarps), kBrickWarps * 32, 0, s>>>(
        d_dense, ctx->d_bricks, ctx->d_scales, n[0], n[1], n[2], nb[0], nb[1], (uint32_t)nbricks);
  VCR_CUDA(ctx, cudaGetLastError());
  ctx->gdesc = *desc;
  ctx->precision = precision;
  for (int a = 0; a < 3; ++a) ctx->nb[a] = nb[a];
  unsigned int* d_gmax = reinterpret_cast<unsigned int*>(ctx->d_counters + 5);
  VCR_CUDA(ctx, cudaMemsetAsync(d_gmax, 0, sizeof(unsigned int), s));
  GridView g = grid_view(ctx);
  majorant_kernel<<<(unsigned)nbricks, 256, 0, s>>>(g, ctx->d_majorants, d_gmax);
  VCR_CUDA(ctx, cudaGetLastError());
  for (int l = 1; l < 4; ++l) {
    const int* sdim = ctx->mnb[l - 1];
    const int* ddim = ctx->mnb[l];
    uint32_t cnt = (uint32_t)(ddim[0] * ddim[1] * ddim[2]);
    majorant_reduce_kernel<<<(cnt + 255) / 256, 256, 0, s>>>(ctx->d_majorants + ctx->moff[l - 1], sdim[0], sdim[1],
                                                              sdim[2], ctx->d_majorants + ctx->moff[l], ddim[0],
                                                              ddim[1], ddim[2]);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  unsigned int gm = 0;
  VCR_CUDA(ctx, cudaMemcpyAsync(&gm, d_gmax, sizeof(gm), cudaMemcpyDeviceToHost, s));
  VCR_CUDA(ctx, cudaStreamSynchronize(s));
  float f;
  memcpy(&f, &gm, sizeof(f));
  if (!(f <= 3.0e38f)) return fail(ctx, VCR_ERR_INVALID, "grid holds non-finite densities");
  ctx->max_density = f;
  ctx->has_grid = true;
  return VCR_OK;
}

vcr_status grid_sample_launch(vcr_ctx* ctx, const float* d_pos, float* d_out, uint32_t n, cudaStream_t s) {
  if (n == 0) return VCR_OK;
  sample_kernel<<<(n + 255) / 256, 256, 0, s>>>(grid_view(ctx), scene_view(ctx), d_pos, d_out, n);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

vcr_status dda_trace_launch(vcr_ctx* ctx, const float* d_o, const float* d_d, uint32_t n, uint32_t max_cells,
                            uint32_t* d_cells, float* d_t, uint32_t* d_count, cudaStream_t s) {
  if (n == 0) return VCR_OK;
  const int* m = ctx->mnb[ctx->tuning.majorant_level];
  dda_trace_kernel<<<(n + 127) / 128, 128, 0, s>>>(scene_view(ctx), m[0], m[1], m[2], d_o, d_d, n, max_cells, d_cells,
                                                   d_t, d_count);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

// The stored grid (its FP32 / FP16 / BF16 bricks) decoded to dense floats,
// x fastest; out is host or device memory.  Synchronous.
extern "C" VCR_API vcr_status vcr_grid_read_dense(vcr_ctx* ctx, float* out, size_t count) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!ctx->has_grid) return fail(ctx, VCR_ERR_STATE, "no grid");
  const uint64_t total = (uint64_t)ctx->gdesc.size[0] * ctx->gdesc.size[1] * ctx->gdesc.size[2];
  if (!out || count != total) return fail(ctx, VCR_ERR_INVALID, "dense grid count %zu != %llu", count,
                                          (unsigned long long)total);
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaPointerAttributes at{};
  VCR_CUDA(ctx, cudaPointerGetAttributes(&at, out));
  const bool on_device = (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == ctx->device;
  float* dst = out;
  if (!on_device) {
    vcr_status vs = ensure_scratch(ctx, total * sizeof(float));
    if (vs) return vs;
    dst = reinterpret_cast<float*>(ctx->d_scratch);
  }
  const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)ctx->sm_count * 64);
  decode_kernel<<<blocks, 256>>>(grid_view(ctx), dst, total);
  VCR_CUDA(ctx, cudaGetLastError());
  if (!on_device) VCR_CUDA(ctx, cudaMemcpy(out, dst, total * sizeof(float), cudaMemcpyDeviceToHost));
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  return VCR_OK;
}
