// Volumetric progressive photon mapping: photon emission, photon tree,
// per-pixel gather and the progressive N / R / flux update in FP64, or the
// reference's ray-marched estimate with one global radius per pass.
//
// Reference: PPM_PT.comp (main :452-489, interactWithMedium :393-447,
// depositPhoton :304-321), PPM_PE.comp (samplePhotonMap :304-375, ray march
// :443-546), RenderTechniquePPM.cpp (RecordDrawCommands :229-300,
// UpdateRadius :302-312), KDTree.{h,cpp} (a stub in the reference).
//
// The reference deposits photons into a 100^3 x 32-slot grid hash (extra
// photons dropped) and shrinks one global radius per pass; this build keeps
// every photon, orders them along a 30-bit Morton curve and builds a binary
// radix tree over them (the LBVH of the beam pipeline, with point leaves:
// a spatial median-style subdivision standing in for the kd-tree), and
// keeps per-pixel statistics as stochastic progressive photon mapping
// does: each pass one measurement point per pixel (a delta-tracked
// collision along the camera ray), M photons within the pixel's radius R,
//   N' = N + alpha M,  ratio = (N + alpha M) / (N + M),
//   R' = R ratio^(1/3),  tau' = (tau + Phi) ratio,
// with Phi = sum_p f(w_p . -w_cam) Phi_p / sigma_t(x), and the estimate
//   L = background / k + albedo tau / (4/3 pi R^3 k).
// Photons are stored at every real collision with the power arriving there,
// so direct and multiple scattering both come from the photon map.
#include <cmath>

#include "track.cuh"
#include "sort.cuh"
#include "ppb.cuh"
#include "ppm.cuh"

namespace vcr {

vcr_status lbvh_build_refit(vcr_ctx* ctx, const uint32_t* codes, const uint32_t* order, const float4* seg_a,
                            const float4* seg_b, int n, uint32_t* left, uint32_t* right, uint32_t* parent_int,
                            uint32_t* parent_leaf, uint32_t* flags, float4* leaf_lo, float4* leaf_hi,
                            float4* node_lo, float4* node_hi, cudaStream_t st, float4* node_pk);

// Photon box entry and power: the same sun / constant-sky emission as the
// beams (see ppb.cu).
__device__ __forceinline__ float ppm_box_entry(const SceneView& s, f3 d, Rng& rng, f3& o) {
  f3 e = s.b1 - s.b0;
  float ax = fabsf(d.x) * (e.y * e.z), ay = fabsf(d.y) * (e.x * e.z), az = fabsf(d.z) * (e.x * e.y);
  float at = (ax + ay) + az;
  float sel = rng_next(rng) * at;
  float u = rng_next(rng), v = rng_next(rng);
  if (sel < ax) o = mk(d.x > 0.0f ? s.b0.x : s.b1.x, s.b0.y + u * e.y, s.b0.z + v * e.z);
  else if (sel < ax + ay) o = mk(s.b0.x + u * e.x, d.y > 0.0f ? s.b0.y : s.b1.y, s.b0.z + v * e.z);
  else o = mk(s.b0.x + u * e.x, s.b0.y + v * e.y, d.z > 0.0f ? s.b0.z : s.b1.z);
  return at;
}

// Persistent photon tracing: a lane takes the next photon (one atomic per
// warp on the launch's cursor) whenever its photon has ended, so the lanes
// of a warp whose photons end early keep working while the warp's longest
// path runs.  Deposits at every real collision go to a shared buffer
// through one atomic per warp and round (order fixed later by uid; a
// photon's path, and so every deposit, is the same whichever lane traces
// it).
__device__ __forceinline__ void ppm_start_photon(const SceneView& s, uint32_t p, uint32_t photons, uint32_t seed,
                                                 uint32_t pass, Rng& rng, f3& o, f3& d, f3& power) {
  rng = rng_pcg(seed ^ kPpmEmitSalt, p, pass);
  const float inv = 1.0f / ((float)photons * 0.5f);
  bool sun = rng_next(rng) < 0.5f;
  if (sun) {
    d = s.sun;
  } else {
    float z = 1.0f - 2.0f * rng_next(rng);
    float sn, cs;
    vsincos2pi(rng_next(rng), &sn, &cs);
    float rr = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    d = mk(rr * cs, rr * sn, z);
  }
  float at = ppm_box_entry(s, d, rng, o);
  if (sun) {
    float f = (s.light * at) * inv;
    power = mk(f, f, f);
  } else {
    power = s.sky * (((4.0f * kPI) * at) * inv);
  }
}

__global__ void __launch_bounds__(128) ppm_emit_kernel(GridView g, SceneView s, uint32_t photons, uint32_t seed,
                                                       uint32_t pass, uint32_t cap, float4* __restrict__ pos,
                                                       float4* __restrict__ pw, float4* __restrict__ dir,
                                                       uint32_t* __restrict__ uid, uint32_t* __restrict__ count,
                                                       Counters cnt) {
  const uint32_t lane = threadIdx.x & 31u;
  bool alive = false, exhausted = false;
  uint32_t p = 0, events = 0;
  uint32_t started = 0, lookups = 0, cells = 0, deposits = 0;
  Rng rng{0u, 0u};
  f3 o = mk(0.f, 0.f, 0.f), d = o, power = o;
  while (true) {
    const bool need = !alive && !exhausted;
    const uint32_t want = __ballot_sync(0xffffffffu, need);
    if (want) {
      const uint32_t leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader) base = (uint32_t)atomicAdd(cnt.c + 4, (unsigned long long)__popc(want));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const uint32_t id = base + __popc(want & ((1u << lane) - 1u));
        if (id >= photons) {
          exhausted = true;
        } else {
          p = id;
          events = 0;
          ++started;
          ppm_start_photon(s, p, photons, seed, pass, rng, o, d, power);
          alive = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, !alive && exhausted)) break;
    bool dep = false;
    if (alive) {
      float t;
      if (free_flight(g, s, o, d, rng, t, lookups, cells)) {
        o = along(o, d, t);
        dep = true;
      } else {
        alive = false;
      }
    }
    const uint32_t m = __ballot_sync(0xffffffffu, dep);
    if (m) {
      const uint32_t leader = __ffs(m) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (dep) {
        const uint32_t slot = base + __popc(m & ((1u << lane) - 1u));
        if (slot < cap) {
          pos[slot] = make_float4(o.x, o.y, o.z, 0.0f);
          pw[slot] = make_float4(power.x, power.y, power.z, 0.0f);
          dir[slot] = make_float4(d.x, d.y, d.z, 0.0f);
          uid[slot] = p * kPpmMaxEvents + events;
        }
        ++events;
        ++deposits;
        power = power * s.albedo;
        if ((s.max_events && events >= s.max_events) || events >= kPpmMaxEvents) alive = false;
        else d = hg_sample(s.ph, d, rng, true);
      }
    }
  }
  flush_counters(cnt, started, lookups, deposits, cells);
}

// Morton key of each photon in uid order (order = photons sorted by uid).
__global__ void ppm_keys_kernel(SceneView s, const float4* __restrict__ pos, const uint32_t* __restrict__ by_uid,
                                uint32_t n, uint32_t* __restrict__ codes, uint32_t* __restrict__ idx) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t ph = by_uid[i];
  float4 p = pos[ph];
  f3 e = s.b1 - s.b0;
  float qx = fminf(fmaxf(((p.x - s.b0.x) / e.x) * 1024.0f, 0.0f), 1023.0f);
  float qy = fminf(fmaxf(((p.y - s.b0.y) / e.y) * 1024.0f, 0.0f), 1023.0f);
  float qz = fminf(fmaxf(((p.z - s.b0.z) / e.z) * 1024.0f, 0.0f), 1023.0f);
  codes[i] = (morton_expand10((uint32_t)qx) << 2) | (morton_expand10((uint32_t)qy) << 1) |
             morton_expand10((uint32_t)qz);
  idx[i] = ph;
}

// ratio^(1/3) for ratio in [alpha, 1]: six Newton steps from 1 (converged
// to double precision for ratio >= 0.05), so host and device agree exactly.
__host__ __device__ __forceinline__ double ppm_cbrt_ratio(double r) {
  double y = 1.0;
  for (int i = 0; i < 6; ++i) y = y - (y * y * y - r) / (3.0 * y * y);
  return y;
}

// Photon powers and directions in the tree's leaf order: leaf i holds
// photon order[i].
__global__ void ppm_leaf_order_kernel(const uint32_t* __restrict__ order, const float4* __restrict__ pw,
                                      const float4* __restrict__ dir, uint32_t n, float4* __restrict__ leaf_pw,
                                      float4* __restrict__ leaf_dir) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t ph = order[i];
    leaf_pw[i] = pw[ph];
    leaf_dir[i] = dir[ph];
  }
}

// What the gather and the march read: photon powers and directions in the
// tree's leaf order (leaf i holds photon order[i]), the leaf positions, and
// the internal nodes packed as (low corner, left child bits) (high corner,
// right child bits).
struct PpmGatherView {
  const float4* pw;
  const float4* dir;
  const float4* leaf_lo;
  const float4* node_pk;
  int n;
  double* stats;  // per pixel: N, R, tau rgb, background rgb
  float alpha;
  uint32_t seed, pass;
};

__device__ __forceinline__ float box_dist2(f3 x, float4 lo, float4 hi) {
  float dx = fmaxf(fmaxf(lo.x - x.x, 0.0f), x.x - hi.x);
  float dy = fmaxf(fmaxf(lo.y - x.y, 0.0f), x.y - hi.y);
  float dz = fmaxf(fmaxf(lo.z - x.z, 0.0f), x.z - hi.z);
  return (dx * dx + dy * dy) + dz * dz;
}

__global__ void __launch_bounds__(128, 8) ppm_gather_kernel(GridView g, SceneView s, CamView cam, PassView pv,
                                                         PpmGatherView v, double* __restrict__ sum, Counters cnt,
                                                         unsigned long long* __restrict__ tested) {
  uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t lookups = 0, cells = 0, found = 0, cand = 0;
  if (id < pv.cw * pv.ch) {
    uint32_t cy = id / pv.cw, cx = id - cy * pv.cw;
    int x = (int)(pv.x0 + cx), y = (int)(pv.y0 + cy);
    uint32_t pix = (uint32_t)y * pv.width + (uint32_t)x;
    double* st = v.stats + 8 * (size_t)pix;
    f3 o, rd;
    camera_ray(cam, x, y, o, rd);
    f3 bg = mk(0.f, 0.f, 0.f), phi = bg;
    uint32_t M = 0;
    float tmin, tmax;
    if (!slab(o, rd, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
      bg = sky(s, rd);
    } else {
      f3 entry = along(o, rd, fmaxf(tmin, 0.0f));
      Rng rng = rng_pcg(v.seed ^ kPpmGatherSalt, pix, v.pass);
      float t;
      if (!free_flight(g, s, entry, rd, rng, t, lookups, cells)) {
        bg = sky(s, rd);
      } else if (v.n > 0) {
        f3 xm = along(entry, rd, t);
        float sigma_t = s.k_sigma * density_at(g, s, xm);
        ++lookups;
        float r = (float)st[1];
        float r2 = r * r;
        f3 wo = -rd;
        uint32_t stack[kGatherStack];
        int sp = 0;
        uint32_t node = v.n == 1 ? kLeafBit : 0u;
        while (true) {
          if (node & kLeafBit) {
            uint32_t lf = node & ~kLeafBit;
            ++cand;
            float4 q = v.leaf_lo[lf];
            f3 dq = mk(q.x, q.y, q.z) - xm;
            if (dot(dq, dq) <= r2) {
              float4 w = v.dir[lf], pw = v.pw[lf];
              float f = hg_pdf(s.ph, dot(mk(w.x, w.y, w.z), wo));
              phi = phi + mk(pw.x, pw.y, pw.z) * f;
              ++M;
            }
          } else {
            const float4 lo = v.node_pk[2 * (size_t)node], hi = v.node_pk[2 * (size_t)node + 1];
            if (box_dist2(xm, lo, hi) <= r2) {
              if (sp < kGatherStack) stack[sp++] = __float_as_uint(hi.w);
              node = __float_as_uint(lo.w);
              continue;
            }
          }
          if (sp == 0) break;
          node = stack[--sp];
        }
        if (sigma_t > 0.0f) phi = mk(phi.x / sigma_t, phi.y / sigma_t, phi.z / sigma_t);
        else phi = mk(0.f, 0.f, 0.f);
      }
    }
    // progressive update (FP64)
    double N = st[0], R = st[1];
    double tau[3] = {st[2], st[3], st[4]};
    if (M > 0) {
      double am = (double)v.alpha * (double)M;
      double ratio = (N + am) / (N + (double)M);
      st[0] = N + am;
      st[1] = R * ppm_cbrt_ratio(ratio);
      tau[0] = (tau[0] + (double)phi.x) * ratio;
      tau[1] = (tau[1] + (double)phi.y) * ratio;
      tau[2] = (tau[2] + (double)phi.z) * ratio;
      st[2] = tau[0];
      st[3] = tau[1];
      st[4] = tau[2];
    }
    st[5] += (double)bg.x;
    st[6] += (double)bg.y;
    st[7] += (double)bg.z;
    // current estimate, expressed as a sum over the passes so far
    double Rn = st[1];
    double vol = (4.0 / 3.0) * 3.14159265358979323846 * Rn * Rn * Rn;
    double a = (double)s.albedo / vol;
    double* o3 = sum + 3 * (size_t)pix;
    o3[0] = st[5] + a * tau[0];
    o3[1] = st[6] + a * tau[1];
    o3[2] = st[7] + a * tau[2];
    found = M;
  }
  flush_counters(cnt, id < pv.cw * pv.ch ? 1ull : 0ull, lookups, found, cells);
  warp_count(tested, cand);
}

// ---------------------------------------------------------------------------
// The reference's estimate: a ray march with one global radius
// (PPM_PE.comp main :443-546, samplePhotonMap :304-375)
// ---------------------------------------------------------------------------
constexpr uint32_t kPpmMarchSalt = 0x5F356495u;
constexpr uint32_t kMarchCap = 1u << 20;  // march and ambient steps of one pixel
constexpr float kPI4_3 = kPI * 4.0f / 3.0f;

// samplePhotonMap at x: the photons within the global radius r, phase
// toward wo times power, in the tree's depth-first leaf order, over the
// sphere volume times sigma_s.  Like the reference it draws one random
// number when the sum is positive (its unused six-tap density average).
__device__ f3 march_photon_map(const PpmGatherView& v, const SceneView& s, f3 x, f3 wo, float r, float scatter,
                               Rng& rng, uint32_t& cand) {
  f3 phi = mk(0.f, 0.f, 0.f);
  if (scatter == 0.0f || v.n <= 0) return phi;
  const float r2 = r * r;
  uint32_t stack[kGatherStack];
  int sp = 0;
  uint32_t node = v.n == 1 ? kLeafBit : 0u;
  while (true) {
    if (node & kLeafBit) {
      const uint32_t lf = node & ~kLeafBit;
      ++cand;
      const float4 q = v.leaf_lo[lf];
      const f3 dq = mk(q.x, q.y, q.z) - x;
      if (dot(dq, dq) <= r2) {
        const float4 w = v.dir[lf], pw = v.pw[lf];
        const float f = hg_pdf(s.ph, dot(wo, mk(w.x, w.y, w.z)));
        phi = phi + mk(f * pw.x, f * pw.y, f * pw.z);
      }
    } else {
      const float4 lo = v.node_pk[2 * (size_t)node], hi = v.node_pk[2 * (size_t)node + 1];
      if (box_dist2(x, lo, hi) <= r2) {
        if (sp < kGatherStack) stack[sp++] = __float_as_uint(hi.w);
        node = __float_as_uint(lo.w);
        continue;
      }
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
  if ((phi.x + phi.y) + phi.z <= 0.0f) return mk(0.f, 0.f, 0.f);
  rng_next(rng);
  const float den = ((kPI4_3 * r) * r2) * scatter;
  return mk(phi.x / den, phi.y / den, phi.z / den);
}

__global__ void __launch_bounds__(128) ppm_march_kernel(GridView g, SceneView s, CamView cam, SvView sv, PassView pv,
                                                        PpmGatherView v, float radius, float step, float amb_step,
                                                        double* __restrict__ sum, Counters cnt,
                                                        unsigned long long* __restrict__ tested) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t lookups = 0, cand = 0;
  if (id < pv.cw * pv.ch) {
    const uint32_t cy = id / pv.cw, cx = id - cy * pv.cw;
    const int x = (int)(pv.x0 + cx), y = (int)(pv.y0 + cy);
    const uint32_t pix = (uint32_t)y * pv.width + (uint32_t)x;
    Rng rng = s.rng_mode == 1 ? rng_xorshift(pv.seed * ((uint32_t)x + (uint32_t)y * pv.padded_w))
                              : rng_pcg(pv.seed ^ kPpmMarchSalt, pix, pv.pass);
    f3 pos, rd;
    camera_ray(cam, x, y, pos, rd);
    f3 L = sky(s, rd);
    float tmin, tmax;
    if (slab(pos, rd, s.b0, s.b1, tmin, tmax) && s.ds > 0.0f) {
      const f3 closest = along(pos, rd, tmin);
      pos = along(pos, rd, tmax - step * rng_next(rng));
      const float max_d = length(pos - closest);
      const f3 wo = -rd;
      float cur = 0.0f;
      for (uint32_t it = 0; cur < max_d && it < kMarchCap; ++it) {
        pos = pos - rd * step;
        cur = cur + step;
        const float ext = (density_at(g, s, pos) * s.ds) / s.bs;
        ++lookups;
        const float scatter = s.albedo * ext;
        const float pdf = hg_pdf(s.ph, dot(wo, s.sun));
        const float dl = (s.light * pdf) * sv_lookup(sv, pos);
        f3 direct = mk(dl, dl, dl);
        // ambient: the sky along a phase-sampled direction, attenuated by
        // the mean extinction of a coarse march to the box
        const f3 adir = hg_sample(s.ph, rd, rng, false);
        f3 ap = pos;
        float acc = 0.0f, adist = 0.0f;
        uint32_t n = 0;
        f3 amb = sky(s, adir);
        while (in_box(ap, s.b0, s.b1) && n < kMarchCap) {
          ap = ap + adir * amb_step;
          acc = acc + density_at(g, s, ap);
          adist = adist + amb_step;
          ++n;
        }
        lookups += n;
        if (n > 0) {
          acc = acc * (s.ds / s.bs);
          const float att = vexp(((-adist) * acc) / (float)n);
          amb = amb * att;
          if (amb.x > 0.0f) direct = direct + amb;
        }
        const f3 ind = march_photon_map(v, s, pos, wo, radius, scatter, rng, cand) * s.albedo;
        const float a = vexp((-step) * ext);
        const f3 src = direct + ind;
        L = L * a + mk((scatter * src.x) * step, (scatter * src.y) * step, (scatter * src.z) * step);
      }
    }
    write_result(pv, sum, pix, L);
  }
  flush_counters(cnt, id < pv.cw * pv.ch ? 1ull : 0ull, lookups, 0, 0);
  warp_count(tested, cand);
}

__global__ void ppm_init_stats_kernel(double* __restrict__ stats, size_t pixels, double r0) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pixels) return;
  double* st = stats + 8 * i;
  st[0] = 0.0;
  st[1] = r0;
  for (int k = 2; k < 8; ++k) st[k] = 0.0;
}

void ppm_free(vcr_ctx* ctx) {
  PpmState* st = ctx->ppm;
  if (!st) return;
  void* ptrs[] = {st->pos, st->pw, st->dir, st->uid, st->count, st->by_uid, st->uid_sorted, st->codes, st->idx,
                  st->codes_sorted, st->order, st->left, st->right, st->parent_int, st->parent_leaf, st->flags,
                  st->leaf_lo, st->leaf_hi, st->node_lo, st->node_hi, st->node_pk, st->leaf_pw, st->leaf_dir,
                  st->stats, st->iota};
  for (void* p : ptrs) cudaFree(p);
  probe_free(st->gather);
  delete st;
  ctx->ppm = nullptr;
}

__global__ void iota_kernel(uint32_t* __restrict__ v, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

vcr_status ppm_setup(vcr_ctx* ctx, const vcr_ppm_params* p) {
  if (!p || p->photons == 0 || p->photons > (1u << 26) || p->capacity < 2 || p->capacity > (1u << 28) ||
      !(p->radius > 0.0f) || !(p->alpha > 0.0f && p->alpha <= 1.0f) || p->estimator > VCR_PPM_MARCH ||
      (p->estimator == VCR_PPM_MARCH && !(p->march_step > 0.0f && p->ambient_step > 0.0f)))
    return fail(ctx, VCR_ERR_INVALID,
                "ppm params: photons 1..2^26, capacity 2..2^28, radius > 0, alpha in (0,1], estimator "
                "VCR_PPM_GATHER or VCR_PPM_MARCH (with march_step > 0, ambient_step > 0)");
  if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "vcr_ppm_setup needs a frame (vcr_set_frame)");
  ppm_free(ctx);
  PpmState* st = new PpmState();
  ctx->ppm = st;
  st->prm = *p;
  size_t C = p->capacity;
#define VCR_ALLOC(ptr, bytes) VCR_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(&(ptr)), (bytes)))
  VCR_ALLOC(st->pos, C * 16);
  VCR_ALLOC(st->pw, C * 16);
  VCR_ALLOC(st->dir, C * 16);
  VCR_ALLOC(st->uid, C * 4);
  VCR_ALLOC(st->count, 4);
  VCR_ALLOC(st->by_uid, C * 4);
  VCR_ALLOC(st->uid_sorted, C * 4);
  VCR_ALLOC(st->codes, C * 4);
  VCR_ALLOC(st->idx, C * 4);
  VCR_ALLOC(st->codes_sorted, C * 4);
  VCR_ALLOC(st->order, C * 4);
  VCR_ALLOC(st->left, C * 4);
  VCR_ALLOC(st->right, C * 4);
  VCR_ALLOC(st->parent_int, C * 4);
  VCR_ALLOC(st->parent_leaf, C * 4);
  VCR_ALLOC(st->flags, C * 4);
  VCR_ALLOC(st->leaf_lo, C * 16);
  VCR_ALLOC(st->leaf_hi, C * 16);
  VCR_ALLOC(st->node_lo, C * 16);
  VCR_ALLOC(st->node_hi, C * 16);
  VCR_ALLOC(st->node_pk, 2 * C * 16);
  VCR_ALLOC(st->leaf_pw, C * 16);
  VCR_ALLOC(st->leaf_dir, C * 16);
  VCR_ALLOC(st->iota, C * 4);
  size_t px = (size_t)ctx->width * ctx->height;
  VCR_ALLOC(st->stats, px * 8 * sizeof(double));
#undef VCR_ALLOC
  iota_kernel<<<(unsigned)((C + 255) / 256), 256>>>(st->iota, (uint32_t)C);
  ppm_init_stats_kernel<<<(unsigned)((px + 255) / 256), 256>>>(st->stats, px, (double)p->radius);
  VCR_CUDA(ctx, cudaGetLastError());
  st->pixels = px;
  return ensure_scratch(ctx, sort_scratch_bytes(p->capacity));
}

// RenderTechniquePPM::UpdateRadius (:302-312) for frame k + 1 (pass k):
// r_1 = R0, r_n = r_(n-1) ((n - 1 + alpha) / n)^0.33333, in float.
float ppm_global_radius(float r0, float alpha, uint32_t pass) {
  float r = r0;
  for (uint32_t n = 2; n <= pass + 1; ++n) r = r * std::pow(((float)(n - 1) + alpha) / (float)n, 0.33333f);
  return r;
}

static SvView sv_view(const vcr_ctx* ctx) {
  SvView sv{};
  sv.tex = ctx->d_sv;
  sv.n = (int)ctx->sv.voxel_axis_count;
  sv.b0 = mk(ctx->sv.bounds_min[0], ctx->sv.bounds_min[1], ctx->sv.bounds_min[2]);
  const f3 e = mk(ctx->sv.bounds_max[0], ctx->sv.bounds_max[1], ctx->sv.bounds_max[2]) - sv.b0;
  for (int i = 0; i < 9; ++i) sv.B[i] = ctx->sv.basis_change[i];
  sv.ext.x = (sv.B[0] * e.x + sv.B[1] * e.y) + sv.B[2] * e.z;
  sv.ext.y = (sv.B[3] * e.x + sv.B[4] * e.y) + sv.B[5] * e.z;
  sv.ext.z = (sv.B[6] * e.x + sv.B[7] * e.y) + sv.B[8] * e.z;
  return sv;
}

vcr_status ppm_pass_launch(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t cs) {
  PpmState* st = ctx->ppm;
  if (!st) return fail(ctx, VCR_ERR_STATE, "vcr_ppm_pass needs vcr_ppm_setup");
  if (!ctx->has_grid || !ctx->has_cloud || !ctx->has_cam || !ctx->has_params || !ctx->d_sum)
    return fail(ctx, VCR_ERR_STATE, "vcr_ppm_pass needs a grid, cloud, camera, params and frame");
  if ((size_t)ctx->width * ctx->height != st->pixels)
    return fail(ctx, VCR_ERR_STATE, "the frame changed since vcr_ppm_setup");
  const bool march = st->prm.estimator == VCR_PPM_MARCH;
  if (ctx->params.rng_mode != VCR_RNG_PCG && !march)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "the gather estimate uses PCG streams");
  if (march && !ctx->has_sv)
    return fail(ctx, VCR_ERR_STATE, "the march estimate needs vcr_shadow_volume_build first");
  PassView pv;
  vcr_status vs = make_pass_view(ctx, pass, pv);
  if (vs) return vs;
  if (pv.spp != 1 || (pv.flags & VCR_PASS_NO_ACCUMULATE))
    return fail(ctx, VCR_ERR_UNSUPPORTED, "photon mapping keeps its own statistics: spp 1, accumulating passes");
  GridView g = grid_view(ctx);
  SceneView s = scene_view(ctx);
  const uint32_t P = st->prm.photons, C = st->prm.capacity;
  Counters cnt{ctx->d_counters};
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 5 * sizeof(unsigned long long), cs));
  VCR_CUDA(ctx, cudaMemsetAsync(st->count, 0, 4, cs));
  {  // persistent: as many CTAs as fit, up to one lane a photon
    int per_sm = 0;
    VCR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppm_emit_kernel, 128, 0));
    const uint32_t blocks = std::min<uint32_t>((uint32_t)(ctx->sm_count * std::max(per_sm, 1)), (P + 127) / 128);
    ppm_emit_kernel<<<blocks, 128, 0, cs>>>(g, s, P, pass->seed, pass->pass_index, C, st->pos, st->pw, st->dir,
                                            st->uid, st->count, cnt);
  }
  VCR_CUDA(ctx, cudaGetLastError());
  uint32_t total = 0;
  VCR_CUDA(ctx, cudaMemcpyAsync(&total, st->count, 4, cudaMemcpyDeviceToHost, cs));
  VCR_CUDA(ctx, cudaStreamSynchronize(cs));
  uint32_t n = std::min(total, C);
  st->photons_stored = n;
  st->dropped = total - n;
  // deterministic order: by (photon, event) uid, then stable along the Morton
  // curve; the uid sort covers only the bits a uid of this photon count uses
  uint32_t uid_bits = 1;
  while (uid_bits < 32 && (1ull << uid_bits) <= (uint64_t)P * kPpmMaxEvents + kPpmMaxEvents) ++uid_bits;
  VCR_CUDA(ctx, sort_pairs_enqueue(ctx->sm_count, ctx->d_error, ctx->d_scratch, st->uid, st->iota, st->uid_sorted,
                                   st->by_uid, n, 0, uid_bits, cs));
  if (n) {
    ppm_keys_kernel<<<(n + 255) / 256, 256, 0, cs>>>(s, st->pos, st->by_uid, n, st->codes, st->idx);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  VCR_CUDA(ctx, sort_pairs_enqueue(ctx->sm_count, ctx->d_error, ctx->d_scratch, st->codes, st->idx,
                                   st->codes_sorted, st->order, n, 0, 30, cs));
  vs = lbvh_build_refit(ctx, st->codes_sorted, st->order, st->pos, st->pos, (int)n, st->left, st->right,
                        st->parent_int, st->parent_leaf, st->flags, st->leaf_lo, st->leaf_hi, st->node_lo,
                        st->node_hi, cs, st->node_pk);
  if (vs) return vs;
  if (n) {  // powers and directions in leaf order, read with the leaf's position
    ppm_leaf_order_kernel<<<ctx->sm_count * 8, 256, 0, cs>>>(st->order, st->pw, st->dir, n, st->leaf_pw,
                                                             st->leaf_dir);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  PpmGatherView gv{st->leaf_pw, st->leaf_dir, st->leaf_lo, st->node_pk, (int)n, st->stats, st->prm.alpha, pass->seed,
                   pass->pass_index};
  uint32_t pixels = pv.cw * pv.ch;
  vcr_status ps = probe_begin(ctx, st->gather, cs);
  if (ps) return ps;
  if (march) {
    ppm_march_kernel<<<(pixels + 127) / 128, 128, 0, cs>>>(
        g, s, cam_view(ctx->cam), sv_view(ctx), pv, gv, ppm_global_radius(st->prm.radius, st->prm.alpha, pv.pass),
        st->prm.march_step, st->prm.ambient_step, ctx->d_sum, cnt, st->gather.d_count);
  } else {
    ppm_gather_kernel<<<(pixels + 127) / 128, 128, 0, cs>>>(g, s, cam_view(ctx->cam), pv, gv, ctx->d_sum, cnt,
                                                            st->gather.d_count);
  }
  VCR_CUDA(ctx, cudaGetLastError());
  ps = probe_end(ctx, st->gather, cs);
  if (ps) return ps;
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, cs));
  // the sums hold the running estimate times the pass count
  ctx->passes += 1;
  ctx->samples += 1;
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_ppm_setup(vcr_ctx* ctx, const vcr_ppm_params* p) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  vcr_status st = ppm_setup(ctx, p);
  if (st) return st;
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  return vcr_reset_accumulation(ctx);
}

extern "C" VCR_API vcr_status vcr_ppm_free(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaDeviceSynchronize();
  ppm_free(ctx);
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_ppm_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  return ppm_pass_launch(ctx, pass, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_ppm_info(vcr_ctx* ctx, vcr_ppm_info_t* out) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  if (!ctx->ppm) return fail(ctx, VCR_ERR_STATE, "no photon-map state");
  out->photons_stored = ctx->ppm->photons_stored;
  out->dropped = ctx->ppm->dropped;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_ppm_gather_stats(vcr_ctx* ctx, uint64_t* count, float* ms) {
  if (!ctx || !count || !ms) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->ppm) return fail(ctx, VCR_ERR_STATE, "no photon-map state");
  return probe_read(ctx, ctx->ppm->gather, *count, *ms);
}

extern "C" VCR_API vcr_status vcr_ppm_read(vcr_ctx* ctx, vcr_ppm_buffer which, void* host, size_t bytes) {
  if (!ctx || !host) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  PpmState* st = ctx->ppm;
  if (!st) return fail(ctx, VCR_ERR_STATE, "no photon-map state");
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  size_t n = st->photons_stored;
  const void* src = nullptr;
  size_t want = 0;
  switch (which) {
    case VCR_PPM_STATS: src = st->stats; want = st->pixels * 8 * sizeof(double); break;
    case VCR_PPM_POS: src = st->pos; want = n * 16; break;
    case VCR_PPM_POWER: src = st->pw; want = n * 16; break;
    case VCR_PPM_DIR: src = st->dir; want = n * 16; break;
    case VCR_PPM_UID: src = st->uid; want = n * 4; break;
    case VCR_PPM_ORDER: src = st->order; want = n * 4; break;
    case VCR_PPM_LEFT: src = st->left; want = n > 1 ? (n - 1) * 4 : 0; break;
    case VCR_PPM_RIGHT: src = st->right; want = n > 1 ? (n - 1) * 4 : 0; break;
    default: return fail(ctx, VCR_ERR_INVALID, "unknown photon buffer %d", (int)which);
  }
  if (bytes != want) return fail(ctx, VCR_ERR_INVALID, "photon buffer %d is %zu bytes, not %zu", (int)which, want, bytes);
  if (want) VCR_CUDA(ctx, cudaMemcpy(host, src, want, cudaMemcpyDeviceToHost));
  return VCR_OK;
}
