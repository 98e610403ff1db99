// Device views of the scene and the tracking primitives every tracker uses:
// brick-layout texel fetch, software trilinear filter, majorant-grid DDA,
// delta / ratio tracking steps.
#pragma once

#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "vcr_math.cuh"

namespace vcr {

constexpr int kBrickLog2 = 3;  // 8^3 texels per brick
constexpr int kBrick = 1 << kBrickLog2;
constexpr int kBrickVoxels = kBrick * kBrick * kBrick;

// Density grid in brick layout.  Texel (i,j,k) lives in brick
// b = (i>>3) + B.x*((j>>3) + B.y*(k>>3)) at offset (i&7) + 8(j&7) + 64(k&7);
// reduced-precision bricks store v / scale[b] and decode as float(h) * scale[b].
struct GridView {
  const void* bricks;
  const float* scales;     // per brick (FP16/BF16 only)
  // Optional per-cell corner blocks: cell (cx, cy, cz) for the lower
  // trilinear corner floor(u) = cx - 1 in [-1, n-1] holds the 8 decoded
  // corner texels (clamped to the grid) as two float4, (x, y) pairs of the
  // z0 plane then of the z1 plane; cells in 8^3 tiles, ctiles tiles per axis.
  const float4* corners;
  int ctiles[3];
  const float* majorants;  // the selected pyramid level (max over the cell + halo)
  int n[3];                // voxel counts
  int nb[3];               // brick counts
  int mnb[3];              // cells per axis of the selected majorant level
  int level;               // selected majorant level: cells of 8 << level voxels
  int precision;           // vcr_precision
};

// Scene constants of one pass (CloudProperties + Parameters + light).
struct SceneView {
  f3 b0, b1;        // cloud AABB (CloudProperties.bounds)
  float max_ext;    // global density majorant (CloudProperties.maxExtinction)
  float ds, bs;     // CloudProperties.densityScaling, baseScaling
  float k_sigma;    // ds / bs: sigma_t = k_sigma * density
  f3 cell;          // world size of one majorant cell (8 voxels per axis)
  f3 icell;         // 1 / cell per axis
  f3 iext;          // 1 / (b1 - b0) per axis
  Phase ph;
  float albedo;
  float light;      // sun irradiance
  f3 sun;           // unit direction the sunlight travels
  f3 sky;
  int sky_mode, rng_mode, nee_mode, tracker;
  uint32_t max_events;
  uint32_t nrc_events;  // > 0: paths end in the radiance cache at this event
};

#if defined(__CUDACC__)

__device__ __forceinline__ float texel(const GridView& g, int i, int j, int k) {
  uint32_t b = (uint32_t)(i >> kBrickLog2) +
               (uint32_t)g.nb[0] * ((uint32_t)(j >> kBrickLog2) + (uint32_t)g.nb[1] * (uint32_t)(k >> kBrickLog2));
  uint32_t off = (b << 9) + (uint32_t)(i & 7) + ((uint32_t)(j & 7) << 3) + ((uint32_t)(k & 7) << 6);
  if (g.precision == 0) return __ldg(reinterpret_cast<const float*>(g.bricks) + off);
  float s = __ldg(g.scales + b);
  if (g.precision == 1) {
    __half h = __ldg(reinterpret_cast<const __half*>(g.bricks) + off);
    return __half2float(h) * s;
  }
  __nv_bfloat16 h = __ldg(reinterpret_cast<const __nv_bfloat16*>(g.bricks) + off);
  return __bfloat162float(h) * s;
}

// Software trilinear filter with clamp-to-edge and texel centres at
// (i + 1/2)/N in normalised coordinates (the reference's sampler,
// Initializers.cpp:408-418, sampleCloud PathTracer.comp:115-119).  Lerps are
// fma(t, b - a, a), x then y then z.
// Linear index of corner cell (cx, cy, cz) (each in 0 .. n) in its tiles.
__device__ __forceinline__ uint32_t corner_cell(const GridView& g, uint32_t cx, uint32_t cy, uint32_t cz) {
  const uint32_t t = (cx >> 3) + (uint32_t)g.ctiles[0] * ((cy >> 3) + (uint32_t)g.ctiles[1] * (cz >> 3));
  return (t << 9) + (cx & 7u) + ((cy & 7u) << 3) + ((cz & 7u) << 6);
}

__device__ __forceinline__ float trilinear(const GridView& g, f3 nrm) {
  float ux = nrm.x * (float)g.n[0] - 0.5f;
  float uy = nrm.y * (float)g.n[1] - 0.5f;
  float uz = nrm.z * (float)g.n[2] - 0.5f;
  float fx0 = floorf(ux), fy0 = floorf(uy), fz0 = floorf(uz);
  float tx = ux - fx0, ty = uy - fy0, tz = uz - fz0;
  int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
  if (g.corners) {  // one 32-byte block holds the footprint: the same values, the same lerps
    const uint32_t cx = (uint32_t)(min(max(x0, -1), g.n[0] - 1) + 1);
    const uint32_t cy = (uint32_t)(min(max(y0, -1), g.n[1] - 1) + 1);
    const uint32_t cz = (uint32_t)(min(max(z0, -1), g.n[2] - 1) + 1);
    const float4* c = g.corners + 2 * (size_t)corner_cell(g, cx, cy, cz);
    const float4 a = __ldg(c), b = __ldg(c + 1);
    float c00 = fmaf(tx, a.y - a.x, a.x);
    float c10 = fmaf(tx, a.w - a.z, a.z);
    float c01 = fmaf(tx, b.y - b.x, b.x);
    float c11 = fmaf(tx, b.w - b.z, b.z);
    float c0 = fmaf(ty, c10 - c00, c00);
    float c1 = fmaf(ty, c11 - c01, c01);
    return fmaf(tz, c1 - c0, c0);
  }
  int x1 = min(max(x0 + 1, 0), g.n[0] - 1);
  int y1 = min(max(y0 + 1, 0), g.n[1] - 1);
  int z1 = min(max(z0 + 1, 0), g.n[2] - 1);
  x0 = min(max(x0, 0), g.n[0] - 1);
  y0 = min(max(y0, 0), g.n[1] - 1);
  z0 = min(max(z0, 0), g.n[2] - 1);
  // One brick address for (x0, y0, z0); each +1 neighbour is a step of the
  // element offset (and of the brick index, for the scale) that is 0 where
  // the coordinate is clamped at the grid's edge, 1 / 8 / 64 inside a brick,
  // and the brick stride minus 7 / 56 / 448 where it crosses into the next
  // brick.  The texels read are exactly those of texel(g, x, y, z).
  const uint32_t nb0 = (uint32_t)g.nb[0], nb01 = nb0 * (uint32_t)g.nb[1];
  const uint32_t b = (uint32_t)(x0 >> kBrickLog2) + nb0 * (uint32_t)(y0 >> kBrickLog2) + nb01 * (uint32_t)(z0 >> kBrickLog2);
  const uint32_t o = (b << 9) + (uint32_t)(x0 & 7) + ((uint32_t)(y0 & 7) << 3) + ((uint32_t)(z0 & 7) << 6);
  const bool cx = (x0 & 7) == 7, cy = (y0 & 7) == 7, cz = (z0 & 7) == 7;
  const uint32_t bx = (x1 != x0 && cx) ? 1u : 0u, by = (y1 != y0 && cy) ? nb0 : 0u, bz = (z1 != z0 && cz) ? nb01 : 0u;
  const uint32_t ox = x1 == x0 ? 0u : (cx ? 505u : 1u);
  const uint32_t oy = y1 == y0 ? 0u : (cy ? (nb0 << 9) - 56u : 8u);
  const uint32_t oz = z1 == z0 ? 0u : (cz ? (nb01 << 9) - 448u : 64u);
  float v000, v100, v010, v110, v001, v101, v011, v111;
  if (g.precision == 0) {
    const float* t = reinterpret_cast<const float*>(g.bricks);
    v000 = __ldg(t + o); v100 = __ldg(t + o + ox);
    v010 = __ldg(t + o + oy); v110 = __ldg(t + o + ox + oy);
    v001 = __ldg(t + o + oz); v101 = __ldg(t + o + ox + oz);
    v011 = __ldg(t + o + oy + oz); v111 = __ldg(t + o + ox + oy + oz);
  } else {
    const float* sc = g.scales + b;
    const float s000 = __ldg(sc), s100 = __ldg(sc + bx), s010 = __ldg(sc + by), s110 = __ldg(sc + bx + by);
    const float s001 = __ldg(sc + bz), s101 = __ldg(sc + bx + bz), s011 = __ldg(sc + by + bz);
    const float s111 = __ldg(sc + bx + by + bz);
    if (g.precision == 1) {
      const __half* t = reinterpret_cast<const __half*>(g.bricks);
      v000 = __half2float(__ldg(t + o)) * s000; v100 = __half2float(__ldg(t + o + ox)) * s100;
      v010 = __half2float(__ldg(t + o + oy)) * s010; v110 = __half2float(__ldg(t + o + ox + oy)) * s110;
      v001 = __half2float(__ldg(t + o + oz)) * s001; v101 = __half2float(__ldg(t + o + ox + oz)) * s101;
      v011 = __half2float(__ldg(t + o + oy + oz)) * s011; v111 = __half2float(__ldg(t + o + ox + oy + oz)) * s111;
    } else {
      const __nv_bfloat16* t = reinterpret_cast<const __nv_bfloat16*>(g.bricks);
      v000 = __bfloat162float(__ldg(t + o)) * s000; v100 = __bfloat162float(__ldg(t + o + ox)) * s100;
      v010 = __bfloat162float(__ldg(t + o + oy)) * s010; v110 = __bfloat162float(__ldg(t + o + ox + oy)) * s110;
      v001 = __bfloat162float(__ldg(t + o + oz)) * s001; v101 = __bfloat162float(__ldg(t + o + ox + oz)) * s101;
      v011 = __bfloat162float(__ldg(t + o + oy + oz)) * s011;
      v111 = __bfloat162float(__ldg(t + o + ox + oy + oz)) * s111;
    }
  }
  float c00 = fmaf(tx, v100 - v000, v000);
  float c10 = fmaf(tx, v110 - v010, v010);
  float c01 = fmaf(tx, v101 - v001, v001);
  float c11 = fmaf(tx, v111 - v011, v011);
  float c0 = fmaf(ty, c10 - c00, c00);
  float c1 = fmaf(ty, c11 - c01, c01);
  return fmaf(tz, c1 - c0, c0);
}

// Normalised coordinates (p - b0) / (b1 - b0) as in sampleCloud
// (PathTracer.comp:117), by multiplication with the box's reciprocal extent
// (a GLSL division may be evaluated that way, within 2.5 ulp).
__device__ __forceinline__ float density_at(const GridView& g, const SceneView& s, f3 p) {
  const f3 q = p - s.b0;
  return trilinear(g, mk(q.x * s.iext.x, q.y * s.iext.y, q.z * s.iext.z));
}

#endif  // __CUDACC__

// ---------------------------------------------------------------------------
// Majorant-grid DDA (Amanatides & Woo 1987) over 8^3-voxel cells.
// Ties between axes advance x before y before z.
// ---------------------------------------------------------------------------
struct Dda {
  int c[3];       // current cell
  float tmax[3];  // ray t of the next boundary per axis
  float tdel[3];  // t per cell along the axis, signed like the step (+inf: the axis never advances)
};

// The set-up multiplies by the reciprocal direction `inv` = 1/d (computed
// once per ray and shared with the slab test) and by the reciprocal cell
// size `ics`, so a ray's DDA costs three divisions in all; the sign test is
// on d itself because 1/(+-0) is +-inf.
VCR_HD void dda_axis_init(float o, float d, float inv, float b0, float cs, int c, float& tmax, float& tdel) {
  if (d > 0.0f) {
    tmax = ((b0 + (float)(c + 1) * cs) - o) * inv;
    tdel = cs * inv;
  } else if (d < 0.0f) {
    tmax = ((b0 + (float)c * cs) - o) * inv;
    tdel = cs * inv;  // negative: the axis steps down
  } else {
    tmax = INFINITY;
    tdel = INFINITY;
  }
}

VCR_HD int cell_of(float o, float b0, float ics, int nc) {
  int c = (int)floorf((o - b0) * ics);
  return c < 0 ? 0 : (c > nc - 1 ? nc - 1 : c);
}

VCR_HD void dda_init(Dda& d, f3 o, f3 dir, f3 inv, f3 b0, f3 cs, f3 ics, const int nc[3]) {
  d.c[0] = cell_of(o.x, b0.x, ics.x, nc[0]);
  d.c[1] = cell_of(o.y, b0.y, ics.y, nc[1]);
  d.c[2] = cell_of(o.z, b0.z, ics.z, nc[2]);
  dda_axis_init(o.x, dir.x, inv.x, b0.x, cs.x, d.c[0], d.tmax[0], d.tdel[0]);
  dda_axis_init(o.y, dir.y, inv.y, b0.y, cs.y, d.c[1], d.tmax[1], d.tdel[1]);
  dda_axis_init(o.z, dir.z, inv.z, b0.z, cs.z, d.c[2], d.tmax[2], d.tdel[2]);
}

VCR_HD float dda_cell_exit(const Dda& d) { return fminf(fminf(d.tmax[0], d.tmax[1]), d.tmax[2]); }

// Advance to the next cell; false when it leaves the grid.  The step is the
// sign of tdel and tmax grows by |tdel| (the cell's t extent).
// (Each axis is spelled out so the state stays in registers.)
VCR_HD bool dda_advance(Dda& d, const int nc[3]) {
  if (d.tmax[0] <= d.tmax[1] && d.tmax[0] <= d.tmax[2]) {
    d.c[0] += d.tdel[0] < 0.0f ? -1 : 1;
    d.tmax[0] = d.tmax[0] + fabsf(d.tdel[0]);
    return d.c[0] >= 0 && d.c[0] < nc[0];
  }
  if (d.tmax[1] <= d.tmax[2]) {
    d.c[1] += d.tdel[1] < 0.0f ? -1 : 1;
    d.tmax[1] = d.tmax[1] + fabsf(d.tdel[1]);
    return d.c[1] >= 0 && d.c[1] < nc[1];
  }
  d.c[2] += d.tdel[2] < 0.0f ? -1 : 1;
  d.tmax[2] = d.tmax[2] + fabsf(d.tdel[2]);
  return d.c[2] >= 0 && d.c[2] < nc[2];
}

VCR_HD uint32_t dda_linear(const Dda& d, const int nc[3]) {
  return (uint32_t)d.c[0] + (uint32_t)nc[0] * ((uint32_t)d.c[1] + (uint32_t)nc[1] * (uint32_t)d.c[2]);
}

// One free-flight sample against piecewise-constant majorants: consume the
// optical depth tau = -ln(u) cell by cell.  Returns true with t at a
// tentative collision inside the current cell (majorant *m, density units),
// false when the segment [t, t_end] is used up.
//   per cell: e = min(tmax), s = min(e, t_end), dtau = (m*k)*(s - t);
//   if dtau > tau: t = t + tau/(m*k), stop; else tau -= dtau, t = s, advance.
struct TrackState {
  Dda dda;
  float t, t_end, m;
};

}  // namespace vcr
