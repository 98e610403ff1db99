// Path tracing: the per-pixel global-majorant tracker (the reference's
// PathTracer.comp semantics, both RNG modes) and the persistent DDA
// wavefront tracker (per-brick majorants, ratio-tracking NEE).
//
// Reference: PathTracer.comp main (:366-425), findScatterPoint (:318-361),
// samplePhase/scatterRay (:259-311), sampleShadowVolume (:121-127);
// dispatch RenderTechniquePT::RecordDrawCommands (RenderTechniquePT.cpp:129-168).
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

__device__ __forceinline__ void write_result(const PassView& pv, double* __restrict__ sum, uint32_t pix, f3 L,
                                             bool atomic) {
  double* o = sum + 3 * (size_t)pix;
  if (pv.flags & VCR_PASS_NO_ACCUMULATE) {
    // only valid with spp == 1 (checked on the host)
    o[0] = L.x;
    o[1] = L.y;
    o[2] = L.z;
  } else if (atomic) {
    atomicAdd(o + 0, (double)L.x);
    atomicAdd(o + 1, (double)L.y);
    atomicAdd(o + 2, (double)L.z);
  } else {
    o[0] += (double)L.x;
    o[1] += (double)L.y;
    o[2] += (double)L.z;
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

// findScatterPoint (PathTracer.comp:318-361).
__device__ __forceinline__ bool find_scatter_global(const GridView& g, const SceneView& s, float sigma_bar, f3& pos,
                                                    f3 dir, Rng& rng, uint32_t& lookups) {
  float tmin, tmax;
  if (!slab(pos, dir, s.b0, s.b1, tmin, tmax)) return false;
  f3 exitp = along(pos, dir, tmax);
  float dist = length(exitp - pos);
  if (!finite_pos(dist) || !(sigma_bar > 0.0f)) return false;
  float t = 0.0f;
  f3 cp;
  for (uint32_t it = 0;; ++it) {
    if (it >= kStepCap) return false;
    float z = rng_next(rng);
    t = t + (-vlog(z)) / sigma_bar;
    if (t >= dist) return false;
    cp = along(pos, dir, t);
    float ext = density_at(g, s, cp);
    ++lookups;
    float xi = rng_next(rng);
    if (xi < ext / s.max_ext) break;
  }
  pos = cp;
  return true;
}

// Ratio tracking toward the sun with the global majorant.
__device__ __forceinline__ float ratio_global(const GridView& g, const SceneView& s, float sigma_bar, f3 pos, f3 ldir,
                                              Rng& rng, uint32_t& lookups) {
  float tmin, tmax;
  if (!slab(pos, ldir, s.b0, s.b1, tmin, tmax)) return 1.0f;
  float dist = length(along(pos, ldir, tmax) - pos);
  if (!finite_pos(dist) || !(sigma_bar > 0.0f)) return 1.0f;
  float t = 0.0f, T = 1.0f;
  for (uint32_t it = 0; it < kStepCap; ++it) {
    t = t + (-vlog(rng_next(rng))) / sigma_bar;
    if (t >= dist) break;
    float rho = density_at(g, s, along(pos, ldir, t));
    ++lookups;
    T = T * (1.0f - rho / s.max_ext);
    if (T < 0.05f) {
      if (rng_next(rng) >= 0.5f) return 0.0f;
      T = T * 2.0f;
    }
  }
  return T;
}

__global__ void __launch_bounds__(256) pt_global_kernel(GridView g, SceneView s, CamView cam, SvView sv, PassView pv,
                                                        double* __restrict__ sum, uint32_t* __restrict__ stats,
                                                        Counters cnt) {
  uint32_t cx = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cy = blockIdx.y * blockDim.y + threadIdx.y;
  unsigned long long n_paths = 0, n_look = 0, n_ev = 0;
  if (cx < pv.cw && cy < pv.ch) {
    int x = (int)(pv.x0 + cx), y = (int)(pv.y0 + cy);
    uint32_t pix = (uint32_t)y * pv.width + (uint32_t)x;
    float sigma_bar = (s.max_ext * s.ds) / s.bs;  // PathTracer.comp:338
    bool ref = s.rng_mode == 1;
    f3 Lsum = mk(0.f, 0.f, 0.f);
    uint32_t ev_total = 0, look_total = 0;
    for (uint32_t sp = 0; sp < pv.spp; ++sp) {
      Rng rng = ref ? rng_xorshift((uint32_t)pv.seed * ((uint32_t)x + (uint32_t)y * pv.padded_w))
                    : rng_pcg(pv.seed, pix * pv.spp + sp, pv.pass);
      f3 pos, dir;
      camera_ray(cam, x, y, pos, dir);
      f3 L = mk(0.f, 0.f, 0.f);
      uint32_t events = 0, lookups = 0;
      float tmin, tmax;
      if (!slab(pos, dir, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
        L = sky(s, dir);
      } else {
        pos = along(pos, dir, tmax < tmin ? tmax : tmin);
        float beta = 1.0f;
        uint32_t cap = s.max_events ? s.max_events : kEventCap;
        while (true) {
          if (!find_scatter_global(g, s, sigma_bar, pos, dir, rng, lookups)) {
            f3 sk = sky(s, dir);
            L = L + sk * beta;
            break;
          }
          ++events;
          beta = beta * s.albedo;
          float pdf = hg_pdf(s.ph, dot(-dir, s.sun));
          float T = s.nee_mode == 1 ? sv_lookup(sv, pos) : ratio_global(g, s, sigma_bar, pos, -s.sun, rng, lookups);
          float c = ((s.light * pdf) * T) * beta;
          L = L + mk(c, c, c);
          if (events >= cap) break;
          dir = hg_sample(s.ph, dir, rng, !ref);
        }
      }
      Lsum = Lsum + L;
      ev_total += events;
      look_total += lookups;
    }
    write_result(pv, sum, pix, Lsum, false);
    if (stats) {
      uint32_t* st = stats + 4 * (size_t)pix;
      st[0] = ev_total;
      st[1] = look_total;
      st[2] = pv.pass;
      st[3] = 1;
    }
    n_paths = pv.spp;
    n_look = look_total;
    n_ev = ev_total;
  }
  flush_counters(cnt, n_paths, n_look, n_ev, 0);
}

// ---------------------------------------------------------------------------
// Persistent DDA wavefront tracker
// ---------------------------------------------------------------------------
struct Track {
  Dda dda;
  float t, t_end, m;
};

__device__ __forceinline__ void track_init(Track& tr, const GridView& g, const SceneView& s, f3 o, f3 d,
                                           uint32_t& cells) {
  float tmin, tmax;
  if (!slab(o, d, s.b0, s.b1, tmin, tmax) || !finite_pos(tmax)) tmax = 0.0f;
  tr.t = 0.0f;
  tr.t_end = tmax;
  dda_init(tr.dda, o, d, s.b0, s.cell, g.nb);
  tr.m = __ldg(g.majorants + dda_linear(tr.dda, g.nb));
  ++cells;
}

// One free-flight sample (see TrackState in vcr_device.cuh).
__device__ __forceinline__ bool track_step(Track& tr, const GridView& g, float k, float u, uint32_t& cells) {
  float tau = -vlog(u);
  while (true) {
    float e = dda_cell_exit(tr.dda);
    float se = fminf(e, tr.t_end);
    float sig = tr.m * k;
    float dtau = sig * (se - tr.t);
    if (dtau > tau) {
      tr.t = tr.t + tau / sig;
      return true;
    }
    tau = tau - dtau;
    tr.t = se;
    if (e >= tr.t_end) return false;
    if (!dda_advance(tr.dda, g.nb)) return false;
    tr.m = __ldg(g.majorants + dda_linear(tr.dda, g.nb));
    ++cells;
  }
}

enum : uint32_t { kIdle = 0, kScatter = 1, kNee = 2 };

__global__ void __launch_bounds__(256) pt_wavefront_kernel(GridView g, SceneView s, CamView cam, PassView pv,
                                                           double* __restrict__ sum, uint32_t* __restrict__ stats,
                                                           Counters cnt, uint32_t total) {
  const uint32_t lane = threadIdx.x & 31u;
  const float k = s.k_sigma;
  const f3 lsun = -s.sun;
  uint32_t mode = kIdle;
  bool exhausted = false;
  uint32_t pid = 0, pix = 0, events = 0, lookups = 0, cells = 0;
  unsigned long long n_paths = 0, n_look = 0, n_ev = 0, n_cells = 0;
  Rng rng{0u, 0u};
  f3 pos = mk(0.f, 0.f, 0.f), dir = pos, L = pos;
  float beta = 1.0f, T = 1.0f, phase = 0.0f;
  Track tr;
  const bool atomic = pv.spp > 1;

  while (true) {
    // ---- warp-aggregated refill of idle lanes -----------------------------
    bool need = (mode == kIdle) && !exhausted;
    uint32_t mask = __ballot_sync(0xffffffffu, need);
    if (mask) {
      uint32_t leader = __ffs(mask) - 1;
      uint32_t base = 0;
      if (lane == leader) base = (uint32_t)atomicAdd(cnt.c + 4, (unsigned long long)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        uint32_t id = base + __popc(mask & ((1u << lane) - 1u));
        if (id >= total) {
          exhausted = true;
        } else {
          pid = id;
          uint32_t per_row = pv.cw * pv.spp;
          uint32_t cy = id / per_row, rem = id - cy * per_row;
          uint32_t cx = rem / pv.spp, sp = rem - cx * pv.spp;
          int x = (int)(pv.x0 + cx), y = (int)(pv.y0 + cy);
          pix = (uint32_t)y * pv.width + (uint32_t)x;
          rng = rng_pcg(pv.seed, pix * pv.spp + sp, pv.pass);
          camera_ray(cam, x, y, pos, dir);
          L = mk(0.f, 0.f, 0.f);
          beta = 1.0f;
          events = 0;
          lookups = 0;
          cells = 0;
          ++n_paths;
          float tmin, tmax;
          if (!slab(pos, dir, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
            L = sky(s, dir);
            write_result(pv, sum, pix, L, atomic);
            if (stats && sp == 0) {
              uint32_t* st = stats + 4 * (size_t)pix;
              st[0] = 0; st[1] = 0; st[2] = pv.pass; st[3] = 0;
            }
          } else {
            pos = along(pos, dir, tmax < tmin ? tmax : tmin);
            track_init(tr, g, s, pos, dir, cells);
            mode = kScatter;
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, exhausted && mode == kIdle)) break;
    if (mode == kIdle) continue;

    // ---- one tracking step ---------------------------------------------------
    f3 rd = mode == kScatter ? dir : lsun;
    bool nee_done = false, finish = false;
    float u = rng_next(rng);
    if (track_step(tr, g, k, u, cells)) {
      f3 p = along(pos, rd, tr.t);
      float rho = density_at(g, s, p);
      ++lookups;
      if (mode == kScatter) {
        float xi = rng_next(rng);
        if (xi < rho / tr.m) {
          pos = p;
          ++events;
          beta = beta * s.albedo;
          phase = hg_pdf(s.ph, dot(-dir, s.sun));
          T = 1.0f;
          mode = kNee;
          track_init(tr, g, s, pos, lsun, cells);
        }
      } else {
        T = T * (1.0f - rho / tr.m);
        if (T < 0.05f) {
          if (rng_next(rng) >= 0.5f) {
            T = 0.0f;
            nee_done = true;
          } else {
            T = T * 2.0f;
          }
        }
      }
    } else {
      if (mode == kScatter) {
        f3 sk = sky(s, dir);
        L = L + sk * beta;
        finish = true;
      } else {
        nee_done = true;
      }
    }
    if (nee_done) {
      float c = ((s.light * phase) * T) * beta;
      L = L + mk(c, c, c);
      if (s.max_events && events >= s.max_events) {
        finish = true;
      } else {
        dir = hg_sample(s.ph, dir, rng, true);
        mode = kScatter;
        track_init(tr, g, s, pos, dir, cells);
      }
    }
    if (lookups + cells > kPathWorkCap) finish = true;  // runaway guard (non-finite input)
    if (finish) {
      write_result(pv, sum, pix, L, atomic);
      if (stats && (pid % pv.spp) == 0) {
        uint32_t* st = stats + 4 * (size_t)pix;
        st[0] = events; st[1] = lookups; st[2] = pv.pass; st[3] = cells;
      }
      n_look += lookups;
      n_ev += events;
      n_cells += cells;
      mode = kIdle;
    }
  }
  flush_counters(cnt, n_paths, n_look, n_ev, n_cells);
}

// ---------------------------------------------------------------------------
// host launch
// ---------------------------------------------------------------------------
static CamView cam_view(const vcr_camera& c) {
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

vcr_status pt_pass_launch(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t st) {
  if (!ctx->has_grid || !ctx->has_cloud || !ctx->has_cam || !ctx->has_params || !ctx->d_sum)
    return fail(ctx, VCR_ERR_STATE, "vcr_pt_pass needs a grid, cloud, camera, params and frame");
  PassView pv;
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
  if (pv.x0 + pv.cw > ctx->width || pv.y0 + pv.ch > ctx->height || pv.ch == 0)
    return fail(ctx, VCR_ERR_INVALID, "crop %u,%u %ux%u outside the %ux%u frame", pv.x0, pv.y0, pv.cw, pv.ch,
                ctx->width, ctx->height);
  if ((pv.flags & VCR_PASS_NO_ACCUMULATE) && pv.spp != 1)
    return fail(ctx, VCR_ERR_INVALID, "VCR_PASS_NO_ACCUMULATE needs spp == 1");
  const vcr_params& P = ctx->params;
  if (P.rng_mode == VCR_RNG_XORSHIFT && pv.spp != 1)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "the xorshift parity mode renders 1 spp per pass");
  if (P.nee_mode == VCR_NEE_SHADOW_VOLUME && !ctx->has_sv)
    return fail(ctx, VCR_ERR_STATE, "shadow-volume NEE needs vcr_shadow_volume_build first");
  uint64_t total64 = (uint64_t)pv.cw * pv.ch * pv.spp;
  uint64_t pixels = (uint64_t)ctx->width * ctx->height * pv.spp;
  if (total64 > 0xFFFFFFFFull || pixels > 0xFFFFFFFFull)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "more than 2^32 paths in one pass");
  GridView g = grid_view(ctx);
  SceneView s = scene_view(ctx);
  CamView cam = cam_view(ctx->cam);
  uint32_t* stats = (pv.flags & VCR_PASS_RECORD_STATS) ? ctx->d_stats : nullptr;
  Counters cnt{ctx->d_counters};
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 5 * sizeof(unsigned long long), st));
  if (P.tracker == VCR_TRACKER_GLOBAL) {
    SvView sv{};
    if (ctx->has_sv) {
      sv.tex = ctx->d_sv;
      sv.n = (int)ctx->sv.voxel_axis_count;
      sv.b0 = mk(ctx->sv.bounds_min[0], ctx->sv.bounds_min[1], ctx->sv.bounds_min[2]);
      f3 e = mk(ctx->sv.bounds_max[0], ctx->sv.bounds_max[1], ctx->sv.bounds_max[2]) - sv.b0;
      for (int i = 0; i < 9; ++i) sv.B[i] = ctx->sv.basis_change[i];
      sv.ext.x = (sv.B[0] * e.x + sv.B[1] * e.y) + sv.B[2] * e.z;
      sv.ext.y = (sv.B[3] * e.x + sv.B[4] * e.y) + sv.B[5] * e.z;
      sv.ext.z = (sv.B[6] * e.x + sv.B[7] * e.y) + sv.B[8] * e.z;
    }
    dim3 blk(16, 16);
    dim3 grd((pv.cw + 15) / 16, (pv.ch + 15) / 16);
    pt_global_kernel<<<grd, blk, 0, st>>>(g, s, cam, sv, pv, ctx->d_sum, stats, cnt);
  } else {
    if (P.rng_mode != VCR_RNG_PCG || P.nee_mode != VCR_NEE_RATIO)
      return fail(ctx, VCR_ERR_UNSUPPORTED, "the DDA tracker implements PCG streams with ratio-tracking NEE");
    int per_sm = 0;
    VCR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pt_wavefront_kernel, 256, 0));
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)(ctx->sm_count * per_sm);
    uint32_t need = (uint32_t)((total64 + 255) / 256);
    if (blocks > need) blocks = need;
    pt_wavefront_kernel<<<blocks, 256, 0, st>>>(g, s, cam, pv, ctx->d_sum, stats, cnt, (uint32_t)total64);
  }
  VCR_CUDA(ctx, cudaGetLastError());
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, st));
  if (!(pv.flags & VCR_PASS_NO_ACCUMULATE)) {
    ctx->passes += 1;
    ctx->samples += pv.spp;
  }
  return VCR_OK;
}

}  // namespace vcr
