// Shared pieces of the path tracers: camera rays, sky, shadow-volume
// lookup, result accumulation, counters and loop guards.
#pragma once

#include "vcr_internal.h"

namespace vcr {

struct CamView {
  f3 pos, fwd, right, up;
  float near_plane, px, py;
  int hw, hh;
};

struct SvView {
  const float* tex;
  int n;
  f3 b0, ext;  // ext = B * (b1 - b0)
  float B[9];
};

struct PassView {
  uint32_t seed, pass, spp, flags;
  uint32_t x0, y0, cw, ch;  // crop
  uint32_t width, height;   // frame
  uint32_t padded_w;        // 32 * (W/32 + 1): the reference's dispatch width
  uint32_t passes;          // consecutive passes in one DDA wavefront launch (0 or 1: one)
};

struct Counters {
  unsigned long long* c;  // [0] paths [1] lookups [2] events [3] cells [4] cursor
};

// ---------------------------------------------------------------------------
// shared helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void camera_ray(const CamView& c, int x, int y, f3& pos, f3& dir) {
  float a = (float)(x - c.hw), b = (float)(y - c.hh);
  f3 d;
  d.x = (c.fwd.x * c.near_plane + (c.right.x * c.px) * a) - (c.up.x * c.py) * b;
  d.y = (c.fwd.y * c.near_plane + (c.right.y * c.px) * a) - (c.up.y * c.py) * b;
  d.z = (c.fwd.z * c.near_plane + (c.right.z * c.px) * a) - (c.up.z * c.py) * b;
  pos = d + c.pos;
  dir = normalize(d);
}

__device__ __forceinline__ f3 sky(const SceneView& s, f3 dir) {
  return s.sky_mode == 0 ? s.sky : sky_gradient(dir);
}

// Dense x-fastest trilinear (shadow volume texture).
__device__ __forceinline__ float trilinear_dense(const float* __restrict__ tex, int n, f3 nrm) {
  float ux = nrm.x * (float)n - 0.5f, uy = nrm.y * (float)n - 0.5f, uz = nrm.z * (float)n - 0.5f;
  float fx0 = floorf(ux), fy0 = floorf(uy), fz0 = floorf(uz);
  float tx = ux - fx0, ty = uy - fy0, tz = uz - fz0;
  int x0 = (int)fx0, y0 = (int)fy0, z0 = (int)fz0;
  int x1 = min(max(x0 + 1, 0), n - 1), y1 = min(max(y0 + 1, 0), n - 1), z1 = min(max(z0 + 1, 0), n - 1);
  x0 = min(max(x0, 0), n - 1);
  y0 = min(max(y0, 0), n - 1);
  z0 = min(max(z0, 0), n - 1);
  size_t sn = (size_t)n, sn2 = sn * sn;
#define T(i, j, k) __ldg(tex + (size_t)(i) + sn * (size_t)(j) + sn2 * (size_t)(k))
  float c00 = fmaf(tx, T(x1, y0, z0) - T(x0, y0, z0), T(x0, y0, z0));
  float c10 = fmaf(tx, T(x1, y1, z0) - T(x0, y1, z0), T(x0, y1, z0));
  float c01 = fmaf(tx, T(x1, y0, z1) - T(x0, y0, z1), T(x0, y0, z1));
  float c11 = fmaf(tx, T(x1, y1, z1) - T(x0, y1, z1), T(x0, y1, z1));
#undef T
  float c0 = fmaf(ty, c10 - c00, c00);
  float c1 = fmaf(ty, c11 - c01, c01);
  return fmaf(tz, c1 - c0, c0);
}

// sampleShadowVolume (PathTracer.comp:121-127).
__device__ __forceinline__ float sv_lookup(const SvView& v, f3 p) {
  f3 d = p - v.b0;
  f3 q;
  q.x = (v.B[0] * d.x + v.B[1] * d.y) + v.B[2] * d.z;
  q.y = (v.B[3] * d.x + v.B[4] * d.y) + v.B[5] * d.z;
  q.z = (v.B[6] * d.x + v.B[7] * d.y) + v.B[8] * d.z;
  return trilinear_dense(v.tex, v.n, div(q, v.ext));
}

__device__ __forceinline__ void flush_counters(Counters c, unsigned long long paths, unsigned long long lookups,
                                               unsigned long long events, unsigned long long cells) {
  for (int o = 16; o > 0; o >>= 1) {
    paths += __shfl_xor_sync(0xffffffffu, paths, o);
    lookups += __shfl_xor_sync(0xffffffffu, lookups, o);
    events += __shfl_xor_sync(0xffffffffu, events, o);
    cells += __shfl_xor_sync(0xffffffffu, cells, o);
  }
  uint32_t lin = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  if ((lin & 31u) == 0) {  // one leader per warp, also for 2D blocks
    if (paths) atomicAdd(c.c + 0, paths);
    if (lookups) atomicAdd(c.c + 1, lookups);
    if (events) atomicAdd(c.c + 2, events);
    if (cells) atomicAdd(c.c + 3, cells);
  }
}

// Adds a sample to the pixel's FP64 sums.  The adds are reductions whose
// result is not read back, so the lane does not wait for the old value; with
// one sample of a pixel per pass they give the same sums as a load-add-store.
__device__ __forceinline__ void write_result(const PassView& pv, double* __restrict__ sum, uint32_t pix, f3 L) {
  double* o = sum + 3 * (size_t)pix;
  if (pv.flags & VCR_PASS_NO_ACCUMULATE) {
    // only valid with spp == 1 (checked on the host)
    o[0] = L.x;
    o[1] = L.y;
    o[2] = L.z;
  } else {
    atomicAdd(o + 0, (double)L.x);
    atomicAdd(o + 1, (double)L.y);
    atomicAdd(o + 2, (double)L.z);
  }
}

// ---------------------------------------------------------------------------
// Per-pixel global-majorant tracker
// ---------------------------------------------------------------------------
constexpr uint32_t kEventCap = 1u << 20;    // safety cap when max_events == 0
constexpr uint32_t kStepCap = 1u << 24;     // tentative collisions per free flight
constexpr uint32_t kPathWorkCap = 1u << 26; // lookups + cell visits per path

// Every loop below ends: a non-finite exit distance (a ray lying in a box
// face with a zero direction component gives NaN) or majorant counts as an
// immediate exit, and the step counts are capped.
__device__ __forceinline__ bool finite_pos(float v) { return v >= 0.0f && v <= 3.0e38f; }

inline CamView cam_view(const vcr_camera& c) {
  CamView v;
  v.pos = mk(c.position[0], c.position[1], c.position[2]);
  v.fwd = mk(c.forward[0], c.forward[1], c.forward[2]);
  v.right = mk(c.right[0], c.right[1], c.right[2]);
  v.up = mk(c.up[0], c.up[1], c.up[2]);
  v.near_plane = c.near_plane;
  v.px = c.pixel_size_x;
  v.py = c.pixel_size_y;
  v.hw = c.half_width;
  v.hh = c.half_height;
  return v;
}

// Pass constants from a vcr_pass_desc (crop defaults to the whole frame).
inline vcr_status make_pass_view(vcr_ctx* ctx, const vcr_pass_desc* pass, PassView& pv) {
  pv.seed = pass->seed;
  pv.pass = pass->pass_index;
  pv.spp = pass->spp ? pass->spp : 1;
  pv.flags = pass->flags;
  pv.width = ctx->width;
  pv.height = ctx->height;
  pv.padded_w = 32u * (ctx->width / 32u + 1u);
  pv.x0 = pass->crop[0];
  pv.y0 = pass->crop[1];
  pv.cw = pass->crop[2] ? pass->crop[2] : ctx->width;
  pv.ch = pass->crop[2] ? pass->crop[3] : ctx->height;
  if ((uint64_t)pv.x0 + pv.cw > ctx->width || (uint64_t)pv.y0 + pv.ch > ctx->height || pv.ch == 0 || pv.cw == 0)
    return fail(ctx, VCR_ERR_INVALID, "crop %u,%u %ux%u outside the %ux%u frame", pv.x0, pv.y0, pv.cw, pv.ch,
                ctx->width, ctx->height);
  if ((pv.flags & VCR_PASS_NO_ACCUMULATE) && pv.spp != 1)
    return fail(ctx, VCR_ERR_INVALID, "VCR_PASS_NO_ACCUMULATE needs spp == 1");
  return VCR_OK;
}

// One view of a batched launch (vcr_batch_*): camera, frame and sun, and
// where the view's work items and pixels start in the batch's ranges.
struct BatchView {
  CamView cam;
  f3 sun;              // direction the sunlight travels
  uint32_t width, height;
  uint32_t path0;      // first work item of the view
  uint32_t pix0;       // first pixel of the view in the batch's sums
};
// View v of a batch draws its paths' streams with seed + v * kViewSeedStep,
// keyed like a single-view pass by its own pixel index and the pass.
constexpr uint32_t kViewSeedStep = 0x9E3779B9u;
static_assert(sizeof(BatchView) % 8 == 0, "BatchView is copied in 8-byte words");
constexpr uint32_t kMaxBatchViews = 256;

struct BatchSink {
  const BatchView* views;    // device table, ascending path0
  uint32_t count;
  const uint32_t* pass_ctr;  // device pass counter added to the pass index
};

// DDA wavefront tracker launch (pt_wavefront.cu).
// `total` camera paths of the pass, preceded by train->paths training paths
// of the radiance cache when `train` is given.  With `batch`, the camera
// paths are those of the batch's views (cam is unused) and sum is the
// batch's sums.
struct NrcTrainSink;
vcr_status wavefront_launch(vcr_ctx* ctx, const GridView& g, const SceneView& s, const CamView& cam,
                            const PassView& pv, uint32_t* stats, Counters cnt, uint32_t total, cudaStream_t st,
                            const NrcTrainSink* train = nullptr, const BatchSink* batch = nullptr,
                            double* sum = nullptr);

}  // namespace vcr
