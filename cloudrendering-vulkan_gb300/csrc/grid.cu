// Density grid: fBm generation, bricking (FP32 / FP16 / BF16 with a per-brick
// FP32 scale), brick majorants, trilinear sampling and the DDA trace.
//
// Replaces the reference's dense R32F 3D image upload (main.cpp:266-335) and
// its single global majorant (Grid3D::GetMajorant, Grid3D.h:180-192;
// main.cpp:152).
#include <algorithm>

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

// `dense` holds z planes [8 kb0, ...) of the grid: the whole grid (kb0 = 0)
// or one slab of brick layers; the launch covers bricks [b0, b0 + count).
template <int P>
__global__ void __launch_bounds__(kBrickWarps * 32) brick_kernel(const float* __restrict__ dense,
                                                                 void* __restrict__ bricks,
                                                                 float* __restrict__ scales, int nx, int ny, int nz,
                                                                 int bx, int by, uint32_t b0, uint32_t count,
                                                                 int kb0) {
  const uint32_t local = blockIdx.x * kBrickWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (local >= count) return;  // warp-uniform
  const uint32_t b = b0 + local;
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
    const size_t base = (size_t)i0 + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)(k - kb0 * kBrick));
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

// Brick summaries for the majorants: per brick, the maximum decoded texel
// over each of the 27 sets "x in X, y in Y, z in Z" with each set one of
// {0} (the low face), {0..7} (the whole brick), {7} (the high face); entry
// sx + 3 sy + 9 sz with 0 = low face, 1 = whole, 2 = high face.  One warp
// per brick, lane l holding texel rows l and l + 32 (row r = y + 8 z).
constexpr int kSumWarps = 8;

__global__ void __launch_bounds__(kSumWarps * 32) brick_summary_kernel(GridView g, float* __restrict__ summary,
                                                                      uint32_t nbricks) {
  const uint32_t b = blockIdx.x * kSumWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nbricks) return;  // warp-uniform
  float m[27];
#pragma unroll
  for (int e = 0; e < 27; ++e) m[e] = 0.0f;
  const float s = g.precision == 0 ? 1.0f : __ldg(g.scales + b);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int r = lane + 32 * h, y = r & 7, z = r >> 3;
    float v[8];
    const size_t off = ((size_t)b << 9) + 8 * (size_t)r;
#pragma unroll
    for (int x = 0; x < 8; ++x) {
      if (g.precision == 0) v[x] = __ldg(reinterpret_cast<const float*>(g.bricks) + off + x);
      else if (g.precision == 1) v[x] = __half2float(__ldg(reinterpret_cast<const __half*>(g.bricks) + off + x)) * s;
      else v[x] = __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(g.bricks) + off + x)) * s;
    }
    float row = v[0];
#pragma unroll
    for (int x = 1; x < 8; ++x) row = fmaxf(row, v[x]);
    const float sel_x[3] = {v[0], row, v[7]};
#pragma unroll
    for (int sz = 0; sz < 3; ++sz) {
      if (!(sz == 1 || (sz == 0 && z == 0) || (sz == 2 && z == 7))) continue;
#pragma unroll
      for (int sy = 0; sy < 3; ++sy) {
        if (!(sy == 1 || (sy == 0 && y == 0) || (sy == 2 && y == 7))) continue;
#pragma unroll
        for (int sx = 0; sx < 3; ++sx) m[sx + 3 * sy + 9 * sz] = fmaxf(m[sx + 3 * sy + 9 * sz], sel_x[sx]);
      }
    }
  }
#pragma unroll
  for (int e = 0; e < 27; ++e)
    for (int o = 16; o > 0; o >>= 1) m[e] = fmaxf(m[e], __shfl_xor_sync(0xffffffffu, m[e], o));
#pragma unroll
  for (int e = 0; e < 27; ++e)
    if (lane == e) summary[(size_t)b * 27 + e] = m[e];
}

// Brick majorant from the summaries: the texels in [8b-1, 8b+8] per axis
// (clamped to the grid) are the brick's own and, from each of the 26
// neighbours inside the grid, its face / edge / corner that touches the
// brick; so the maximum over them is the maximum over 27 summary entries
// (the same texels as a scan of the 10^3 block).
__global__ void majorant_from_summary_kernel(const float* __restrict__ summary, int bx, int by, int bz,
                                             float* __restrict__ maj, unsigned int* __restrict__ gmax) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (uint32_t)(bx * by * bz)) return;
  const int ib = (int)(b % (uint32_t)bx), jb = (int)((b / (uint32_t)bx) % (uint32_t)by);
  const int kb = (int)(b / ((uint32_t)bx * (uint32_t)by));
  float m = 0.0f;
#pragma unroll
  for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int i = ib + dx, j = jb + dy, k = kb + dz;
        if (i < 0 || j < 0 || k < 0 || i >= bx || j >= by || k >= bz) continue;
        // a neighbour below on an axis gives its high face there, above its low face
        const int e = (1 - dx) + 3 * (1 - dy) + 9 * (1 - dz);
        m = fmaxf(m, __ldg(summary + ((size_t)i + (size_t)bx * ((size_t)j + (size_t)by * k)) * 27 + e));
      }
  maj[b] = m;
  atomicMax(gmax, __float_as_uint(m));  // non-negative floats order as integers
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

// Corner blocks: cell (cx, cy, cz) in 0 .. n per axis holds, for the lower
// corner floor(u) = c - 1, the 8 texels a trilinear lookup there reads,
// decoded exactly as the bricks decode them, with the grid-edge clamp
// already applied.  Cells sit in 8^3-cell tiles, x fastest, so the 64
// cells of one z plane of a tile are 2 KB of contiguous output.  One warp
// per such plane (grid-stride over planes, no block barrier): its 9 x 9 x 2
// texels (clamped) are decoded once into the warp's shared memory, then
// each of four stores writes 512 contiguous bytes (lane l the half-cell
// j * 32 + l: the z0 pair block or the z1 pair block of one cell).
constexpr int kCornerWarps = 8;

__global__ void __launch_bounds__(kCornerWarps * 32) corner_kernel(GridView g, float4* __restrict__ out,
                                                                    uint32_t p_begin, uint32_t p_end) {
  __shared__ float tex[kCornerWarps][2 * 81];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  float* tw = tex[w];
  const uint32_t t0 = (uint32_t)g.ctiles[0], t01 = t0 * (uint32_t)g.ctiles[1];
  const uint32_t nwarps = gridDim.x * kCornerWarps;
  for (uint32_t p = p_begin + blockIdx.x * kCornerWarps + w; p < p_end; p += nwarps) {
    const uint32_t t = p >> 3, lz = p & 7u;  // tile, z plane of the tile
    const uint32_t tz = t / t01, ty = (t - tz * t01) / t0, tx = t - tz * t01 - ty * t0;
    const int bx = (int)tx * 8 - 1, by = (int)ty * 8 - 1, bz = (int)(tz * 8u + lz) - 1;
    for (uint32_t k = lane; k < 162u; k += 32u) {
      const int i = (int)(k % 9u), j = (int)((k / 9u) % 9u), l = (int)(k / 81u);
      tw[k] = texel(g, min(max(bx + i, 0), g.n[0] - 1), min(max(by + j, 0), g.n[1] - 1),
                    min(max(bz + l, 0), g.n[2] - 1));
    }
    __syncwarp();
    const bool plane_in = bz + 1 <= g.n[2];  // not padding of the last tile layer
    float4* o = out + 2 * ((size_t)t * 512u + lz * 64u);
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
      const uint32_t h = q * 32u + lane, c = h >> 1;  // half-cell h of cell c = lx + 8 ly
      const int lx = (int)(c & 7u), ly = (int)(c >> 3);
      const float* s = tw + lx + 9 * ly + 81 * (int)(h & 1u);
      if (plane_in && bx + 1 + lx <= g.n[0] && by + 1 + ly <= g.n[1]) o[h] = make_float4(s[0], s[1], s[9], s[10]);
    }
    __syncwarp();
  }
}

// Allocates the corner blocks of the grid description in ctx->gdesc (the
// buffer of the previous grid is kept when its tiles match: freeing and
// mapping 17 GB again costs milliseconds); if the allocation fails there
// are none and lookups gather from the bricks.
static void corner_alloc(vcr_ctx* ctx) {
  ctx->corners_valid = false;
  int tiles3[3];
  for (int a = 0; a < 3; ++a) tiles3[a] = ((int)ctx->gdesc.size[a] + 1 + 7) / 8;
  if (ctx->d_corners && tiles3[0] == ctx->corner_tiles[0] && tiles3[1] == ctx->corner_tiles[1] &&
      tiles3[2] == ctx->corner_tiles[2])
    return;
  cudaFree(ctx->d_corners);
  ctx->d_corners = nullptr;
  for (int a = 0; a < 3; ++a) ctx->corner_tiles[a] = tiles3[a];
  const uint32_t tiles = (uint32_t)tiles3[0] * tiles3[1] * tiles3[2];
  if (cudaMalloc(&ctx->d_corners, (size_t)tiles * 512u * 32u) != cudaSuccess) {
    cudaGetLastError();
    ctx->d_corners = nullptr;
  }
}

// The corner tiles of tile layers [tz0, tz1): tile layer tz reads the
// texels of z planes 8 tz - 1 .. 8 tz + 7 (clamped), i.e. brick layers
// tz - 1 and tz, which must be written.
static vcr_status corner_layers(vcr_ctx* ctx, uint32_t tz0, uint32_t tz1, cudaStream_t s) {
  if (!ctx->d_corners || tz0 >= tz1) return VCR_OK;
  const uint32_t per_layer = (uint32_t)ctx->corner_tiles[0] * ctx->corner_tiles[1] * 8u;  // cell planes
  const uint32_t p0 = tz0 * per_layer, p1 = tz1 * per_layer;
  GridView g = grid_view(ctx);
  g.corners = nullptr;
  const uint32_t blocks =
      std::min<uint32_t>((uint32_t)ctx->sm_count * 8u, (p1 - p0 + kCornerWarps - 1) / kCornerWarps);
  corner_kernel<<<blocks, kCornerWarps * 32, 0, s>>>(g, ctx->d_corners, p0, p1);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

vcr_status corner_build(vcr_ctx* ctx, cudaStream_t s) {
  corner_alloc(ctx);
  vcr_status st = corner_layers(ctx, 0u, (uint32_t)ctx->corner_tiles[2], s);
  if (st) return st;
  ctx->corners_valid = ctx->d_corners != nullptr;
  return VCR_OK;
}

// Makes *p a device buffer of `want` bytes: the current one if it has that
// size, else a new one.
static vcr_status grid_buffer(vcr_ctx* ctx, void** p, size_t& have, size_t want) {
  if (*p && have == want) return VCR_OK;
  cudaFree(*p);
  *p = nullptr;
  have = 0;
  VCR_CUDA(ctx, cudaMalloc(p, want));
  have = want;
  return VCR_OK;
}

// Releases the previous grid and allocates the bricks, scales and majorant
// pyramid of `desc` (levels l = 0..3 with ceil(nb / 2^l) cells per axis,
// each level starting on a 16-byte boundary for the bulk copies into shared
// memory).
static vcr_status grid_alloc(vcr_ctx* ctx, const vcr_grid_desc* desc, int precision, cudaStream_t s) {
  int nb[3];
  for (int a = 0; a < 3; ++a) nb[a] = ((int)desc->size[a] + kBrick - 1) / kBrick;
  uint64_t nbricks = (uint64_t)nb[0] * nb[1] * nb[2];
  if (nbricks > (1ull << 22)) return fail(ctx, VCR_ERR_UNSUPPORTED, "grid too large: %llu bricks (max 2^22)",
                                          (unsigned long long)nbricks);
  size_t esz = precision == 0 ? 4 : 2;
  ctx->has_grid = false;
  ctx->corners_valid = false;
  if (!ctx->tuning.corner_blocks) {  // a same-size buffer is kept only for a grid that builds corners
    cudaFree(ctx->d_corners);
    ctx->d_corners = nullptr;
  }
  ctx->gdesc = *desc;
  ctx->precision = precision;
  for (int a = 0; a < 3; ++a) ctx->nb[a] = nb[a];
  size_t mtotal = 0;
  for (int l = 0; l < 4; ++l) {
    for (int a = 0; a < 3; ++a) ctx->mnb[l][a] = l == 0 ? nb[a] : (ctx->mnb[l - 1][a] + 1) / 2;
    ctx->moff[l] = mtotal;
    size_t cnt = (size_t)ctx->mnb[l][0] * ctx->mnb[l][1] * ctx->mnb[l][2];
    mtotal += (cnt + 3) & ~(size_t)3;
  }
  // the previous grid's buffers are kept where their sizes match
  vcr_status st = grid_buffer(ctx, &ctx->d_bricks, ctx->grid_bytes[0], nbricks * kBrickVoxels * esz);
  if (!st) st = grid_buffer(ctx, reinterpret_cast<void**>(&ctx->d_scales), ctx->grid_bytes[1], nbricks * sizeof(float));
  if (!st) st = grid_buffer(ctx, reinterpret_cast<void**>(&ctx->d_majorants), ctx->grid_bytes[2], mtotal * sizeof(float));
  if (st) return st;
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_majorants, 0, mtotal * sizeof(float), s));
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_scales, 0, nbricks * sizeof(float), s));
  return VCR_OK;
}

// Bricks [b0, b0 + count) from `dense`, which holds z planes [8 kb0, ...).
static vcr_status brick_launch(vcr_ctx* ctx, const float* dense, const vcr_grid_desc* desc, int precision,
                               uint32_t b0, uint32_t count, int kb0, cudaStream_t s) {
  const int n[3] = {(int)desc->size[0], (int)desc->size[1], (int)desc->size[2]};
  const int bx = (n[0] + kBrick - 1) / kBrick, by = (n[1] + kBrick - 1) / kBrick;
  const unsigned blocks = (count + kBrickWarps - 1) / kBrickWarps;
  if (count == 0) return VCR_OK;
  if (precision == 0)
    brick_kernel<0><<<blocks, kBrickWarps * 32, 0, s>>>(dense, ctx->d_bricks, ctx->d_scales, n[0], n[1], n[2], bx,
                                                         by, b0, count, kb0);
  else if (precision == 1)
    brick_kernel<1><<<blocks, kBrickWarps * 32, 0, s>>>(dense, ctx->d_bricks, ctx->d_scales, n[0], n[1], n[2], bx,
                                                         by, b0, count, kb0);
  else
    brick_kernel<2><<<blocks, kBrickWarps * 32, 0, s>>>(dense, ctx->d_bricks, ctx->d_scales, n[0], n[1], n[2], bx,
                                                         by, b0, count, kb0);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

// Once every brick is written: brick summaries, majorant pyramid, global
// maximum, and the corner blocks unless the caller built them already
// (synchronises on s).
static vcr_status grid_finish(vcr_ctx* ctx, const vcr_grid_desc* desc, int precision, cudaStream_t s,
                              bool corners_built = false) {
  int nb[3];
  for (int a = 0; a < 3; ++a) nb[a] = ((int)desc->size[a] + kBrick - 1) / kBrick;
  const uint64_t nbricks = (uint64_t)nb[0] * nb[1] * nb[2];
  ctx->gdesc = *desc;
  ctx->precision = precision;
  for (int a = 0; a < 3; ++a) ctx->nb[a] = nb[a];
  unsigned int* d_gmax = reinterpret_cast<unsigned int*>(ctx->d_counters + 5);
  VCR_CUDA(ctx, cudaMemsetAsync(d_gmax, 0, sizeof(unsigned int), s));
  GridView g = grid_view(ctx);
  vcr_status ss = ensure_scratch(ctx, nbricks * 27 * sizeof(float));
  if (ss) return ss;
  float* summary = reinterpret_cast<float*>(ctx->d_scratch);
  brick_summary_kernel<<<(unsigned)((nbricks + kSumWarps - 1) / kSumWarps), kSumWarps * 32, 0, s>>>(
      g, summary, (uint32_t)nbricks);
  majorant_from_summary_kernel<<<(unsigned)((nbricks + 255) / 256), 256, 0, s>>>(summary, nb[0], nb[1], nb[2],
                                                                                ctx->d_majorants, d_gmax);
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
  if (ctx->tuning.corner_blocks && !corners_built) {
    vcr_status cs = corner_build(ctx, s);
    if (cs) return cs;
  } else if (corners_built) {
    ctx->corners_valid = ctx->d_corners != nullptr;
  }
  VCR_CUDA(ctx, cudaStreamSynchronize(s));
  return VCR_OK;
}

vcr_status grid_build(vcr_ctx* ctx, const float* d_dense, const vcr_grid_desc* desc, int precision,
                      cudaStream_t s) {
  vcr_status st = grid_alloc(ctx, desc, precision, s);
  if (st) return st;
  uint32_t nbricks = 1;
  for (int a = 0; a < 3; ++a) nbricks *= ((uint32_t)desc->size[a] + kBrick - 1) / kBrick;
  st = brick_launch(ctx, d_dense, desc, precision, 0u, nbricks, 0, s);
  if (st) return st;
  return grid_finish(ctx, desc, precision, s);
}

namespace {
// Streams, events and the slab ring of one streamed upload.
struct UploadRing {
  static constexpr int kSlabs = 3;
  float* buf = nullptr;
  cudaStream_t copy = nullptr, brick = nullptr;
  cudaEvent_t copied[kSlabs] = {}, done[kSlabs] = {};
  ~UploadRing() {
    if (copy) cudaStreamSynchronize(copy);
    if (brick) cudaStreamSynchronize(brick);
    for (int r = 0; r < kSlabs; ++r) {
      if (copied[r]) cudaEventDestroy(copied[r]);
      if (done[r]) cudaEventDestroy(done[r]);
    }
    if (copy) cudaStreamDestroy(copy);
    if (brick) cudaStreamDestroy(brick);
    cudaFree(buf);
  }
};
}  // namespace

// A host grid uploaded one brick layer (8 z planes) at a time through a
// ring of three device slabs: the copy of layer k overlaps the bricking of
// layer k - 1 and the corner blocks of tile layer k - 1 (which read brick
// layers k - 2 and k - 1), and no device copy of the whole dense grid is
// made.
vcr_status grid_upload_host(vcr_ctx* ctx, const float* host, const vcr_grid_desc* desc, int precision) {
  vcr_status st = grid_alloc(ctx, desc, precision, 0);
  if (st) return st;
  VCR_CUDA(ctx, cudaDeviceSynchronize());  // the allocations' clears are done
  const size_t nx = desc->size[0], ny = desc->size[1], nz = desc->size[2], plane = nx * ny;
  const uint32_t bx = (uint32_t)((nx + kBrick - 1) / kBrick), by = (uint32_t)((ny + kBrick - 1) / kBrick);
  const int layers = (int)((nz + kBrick - 1) / kBrick);
  const bool corners = ctx->tuning.corner_blocks != 0;
  if (corners) corner_alloc(ctx);
  UploadRing ring;
  VCR_CUDA(ctx, cudaMalloc(&ring.buf, (size_t)UploadRing::kSlabs * kBrick * plane * sizeof(float)));
  VCR_CUDA(ctx, cudaStreamCreateWithFlags(&ring.copy, cudaStreamNonBlocking));
  VCR_CUDA(ctx, cudaStreamCreateWithFlags(&ring.brick, cudaStreamNonBlocking));
  for (int r = 0; r < UploadRing::kSlabs; ++r) {
    VCR_CUDA(ctx, cudaEventCreateWithFlags(&ring.copied[r], cudaEventDisableTiming));
    VCR_CUDA(ctx, cudaEventCreateWithFlags(&ring.done[r], cudaEventDisableTiming));
  }
  for (int kb = 0; kb < layers; ++kb) {
    const int r = kb % UploadRing::kSlabs;
    float* slab = ring.buf + (size_t)r * kBrick * plane;
    if (kb >= UploadRing::kSlabs) VCR_CUDA(ctx, cudaStreamWaitEvent(ring.copy, ring.done[r], 0));
    const size_t z0 = (size_t)kb * kBrick, planes = std::min<size_t>(kBrick, nz - z0);
    VCR_CUDA(ctx, cudaMemcpyAsync(slab, host + z0 * plane, planes * plane * sizeof(float), cudaMemcpyHostToDevice,
                                  ring.copy));
    VCR_CUDA(ctx, cudaEventRecord(ring.copied[r], ring.copy));
    VCR_CUDA(ctx, cudaStreamWaitEvent(ring.brick, ring.copied[r], 0));
    st = brick_launch(ctx, slab, desc, precision, (uint32_t)kb * bx * by, bx * by, kb, ring.brick);
    if (st) return st;
    VCR_CUDA(ctx, cudaEventRecord(ring.done[r], ring.brick));
    if (corners) {
      st = corner_layers(ctx, (uint32_t)kb, (uint32_t)kb + 1u, ring.brick);
      if (st) return st;
    }
  }
  if (corners) {  // the tile layer past the last brick layer (clamped texels)
    st = corner_layers(ctx, (uint32_t)layers, (uint32_t)ctx->corner_tiles[2], ring.brick);
    if (st) return st;
  }
  return grid_finish(ctx, desc, precision, ring.brick, corners);
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
