// Path tracing, per-pixel global-majorant tracker (the reference's
// PathTracer.comp semantics, both RNG modes), and the pass dispatch.
//
// Reference: PathTracer.comp main (:366-425), findScatterPoint (:318-361),
// samplePhase/scatterRay (:259-311), sampleShadowVolume (:121-127);
// dispatch RenderTechniquePT::RecordDrawCommands (RenderTechniquePT.cpp:129-168).

#include "pt_common.cuh"

namespace vcr {

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
    write_result(pv, sum, pix, Lsum);
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
// host launch
// ---------------------------------------------------------------------------

vcr_status pt_pass_launch(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t st, const NrcTrainSink* train,
                          uint32_t count) {
  if (!ctx->has_grid || !ctx->has_cloud || !ctx->has_cam || !ctx->has_params || !ctx->d_sum)
    return fail(ctx, VCR_ERR_STATE, "vcr_pt_pass needs a grid, cloud, camera, params and frame");
  PassView pv;
  vcr_status vs = make_pass_view(ctx, pass, pv);
  if (vs) return vs;
  const vcr_params& P = ctx->params;
  if (count == 0) return fail(ctx, VCR_ERR_INVALID, "a launch of zero passes");
  if (count > 1) {
    if (P.tracker != VCR_TRACKER_DDA || train)
      return fail(ctx, VCR_ERR_UNSUPPORTED, "several passes per launch need the DDA tracker and no training paths");
    if (pv.flags & (VCR_PASS_RECORD_STATS | VCR_PASS_NO_ACCUMULATE))
      return fail(ctx, VCR_ERR_INVALID, "several passes per launch accumulate and record no path statistics");
    if ((uint64_t)pass->pass_index + count > 0xFFFFFFFFull)
      return fail(ctx, VCR_ERR_INVALID, "pass indices past 2^32");
  }
  pv.passes = count;
  if (P.rng_mode == VCR_RNG_XORSHIFT && pv.spp != 1)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "the xorshift parity mode renders 1 spp per pass");
  if (P.nee_mode == VCR_NEE_SHADOW_VOLUME && !ctx->has_sv)
    return fail(ctx, VCR_ERR_STATE, "shadow-volume NEE needs vcr_shadow_volume_build first");
  uint64_t total64 = (uint64_t)pv.cw * pv.ch * pv.spp * count;
  uint64_t pixels = (uint64_t)ctx->width * ctx->height * pv.spp;
  if (total64 > 0x7FFFFFFFull || pixels > 0xFFFFFFFFull)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "more than 2^31 paths in one pass");
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
    if (s.nrc_events) {
      if (total64 > nrc_query_capacity(ctx))
        return fail(ctx, VCR_ERR_CAPACITY, "the radiance cache holds %u queries, the pass has %llu paths",
                    nrc_query_capacity(ctx), (unsigned long long)total64);
      vcr_status qs = nrc_reset_queries(ctx, st);
      if (qs) return qs;
    }
    vcr_status ws = wavefront_launch(ctx, g, s, cam, pv, stats, cnt, (uint32_t)total64, st, train);
    if (ws) return ws;
    if (s.nrc_events) {  // add throughput x cache prediction where paths ended
      ws = nrc_infer_queries(ctx, st);
      if (ws) return ws;
    }
  }
  VCR_CUDA(ctx, cudaGetLastError());
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, st));
  if (!(pv.flags & VCR_PASS_NO_ACCUMULATE)) {
    ctx->passes += count;
    ctx->samples += (uint64_t)pv.spp * count;
  }
  return VCR_OK;
}

}  // namespace vcr
