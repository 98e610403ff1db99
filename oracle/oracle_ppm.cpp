// ORACLE — test infrastructure only (see oracle_math.h).  CPU restatement of
// volumetric progressive photon mapping:
//   emission : PPM_PT.comp main (:452-489) / interactWithMedium (:393-447) /
//              depositPhoton (:304-321), with a deposit at every real
//              collision carrying the power arriving there
//   tree     : photons in (photon, event) order, stable Morton order, binary
//              radix tree with point leaves (see oracle_ppb.cpp)
//   gather   : samplePhotonMap (PPM_PE.comp:304-375) at one delta-tracked
//              measurement point per pixel, with the pixel's radius
//   update   : stochastic progressive photon mapping per pixel in FP64
//              (instead of the global UpdateRadius, RenderTechniquePPM.cpp
//              :302-312)
//   march    : the reference's estimate instead of the gather (PPM_PE.comp
//              main :443-546, samplePhotonMap :304-375) with the global
//              radius of UpdateRadius (RenderTechniquePPM.cpp:302-312)
// The algorithm is the reference's (the lines cited above; where it departs,
// the departure is named).  Its evaluation order is written out explicitly
// (every fused multiply-add as fma, sums in a stated order), and the CUDA
// kernels keep that same order, so the two compare bit for bit.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "oracle_lbvh.h"
#include "oracle_scene.h"

namespace oracle {

const uint32_t kPpmMaxEvents = 64;
const uint32_t kPpmEmitSalt = 0x27D4EB2Fu;
const uint32_t kPpmGatherSalt = 0x165667B1u;
const uint32_t kPpmMarchSalt = 0x5F356495u;
const uint32_t kMarchCap = 1u << 20;

struct Photon {
  F4 pos, pw, dir;
  uint32_t uid;
};

static float box_entry(const Scene& s, V3 d, Rng& rng, V3& o) {
  V3 e = sub(s.b1, s.b0);
  float ax = std::fabs(d.x) * (e.y * e.z), ay = std::fabs(d.y) * (e.x * e.z), az = std::fabs(d.z) * (e.x * e.y);
  float at = (ax + ay) + az;
  float sel = rng.next() * at;
  float u = rng.next(), v = rng.next();
  if (sel < ax) o = v3(d.x > 0.0f ? s.b0.x : s.b1.x, s.b0.y + u * e.y, s.b0.z + v * e.z);
  else if (sel < ax + ay) o = v3(s.b0.x + u * e.x, d.y > 0.0f ? s.b0.y : s.b1.y, s.b0.z + v * e.z);
  else o = v3(s.b0.x + u * e.x, s.b0.y + v * e.y, d.z > 0.0f ? s.b0.z : s.b1.z);
  return at;
}

static double cbrt_ratio(double r) {
  double y = 1.0;
  for (int i = 0; i < 6; ++i) y = y - (y * y * y - r) / (3.0 * y * y);
  return y;
}

static float box_dist2(V3 x, F4 lo, F4 hi) {
  float dx = std::fmax(std::fmax(lo.x - x.x, 0.0f), x.x - hi.x);
  float dy = std::fmax(std::fmax(lo.y - x.y, 0.0f), x.y - hi.y);
  float dz = std::fmax(std::fmax(lo.z - x.z, 0.0f), x.z - hi.z);
  return (dx * dx + dy * dy) + dz * dz;
}

struct PhotonTree {
  std::vector<Photon> ph;  // (photon, event) order
  uint32_t dropped = 0;
  std::vector<uint32_t> order, left, right;
  std::vector<F4> leaf_lo, leaf_hi, node_lo, node_hi;
};

// The radius query of samplePhotonMap (PPM_PE.comp:304-375) over the tree:
// depth first, left child before right, a subtree entered when its box
// comes within r of x (box_dist2 <= r2), a photon taken when its own
// squared distance is <= r2; `take` receives each taken leaf (tree order)
// in walk order, which fixes the order of the caller's sums.
template <class Take>
static void tree_query(const PhotonTree& T, V3 x, float r2, Take&& take) {
  const int n = (int)T.ph.size();
  if (n <= 0) return;
  uint32_t stack[64];
  int sp = 0;
  uint32_t node = n == 1 ? kLeafBit : 0u;
  while (true) {
    if (node & kLeafBit) {
      uint32_t lf = node & ~kLeafBit;
      F4 q = T.leaf_lo[lf];
      V3 dq = sub(v3(q.x, q.y, q.z), x);
      if (dot(dq, dq) <= r2) take(lf);
    } else if (box_dist2(x, T.node_lo[node], T.node_hi[node]) <= r2) {
      if (sp < 64) stack[sp++] = T.right[node];
      node = T.left[node];
      continue;
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
}

static void emit(const Scene& s, uint32_t P, uint32_t cap, uint32_t seed, uint32_t pass, PhotonTree& T,
                 int threads) {
  std::vector<std::vector<Photon>> per(P);
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : 1)
  for (int64_t pi = 0; pi < (int64_t)P; ++pi) {
    uint32_t p = (uint32_t)pi;
    Counts c;
    Rng rng = rng_pcg(seed ^ kPpmEmitSalt, p, pass);
    const float inv = 1.0f / ((float)P * 0.5f);
    V3 d, o, power;
    bool sun = rng.next() < 0.5f;
    if (sun) {
      d = s.sun;
    } else {
      float z = 1.0f - 2.0f * rng.next();
      float sn, cs;
      osincos2pi(rng.next(), &sn, &cs);
      float rr = std::sqrt(std::fmax(0.0f, 1.0f - z * z));
      d = v3(rr * cs, rr * sn, z);
    }
    float at = box_entry(s, d, rng, o);
    if (sun) {
      float f = (s.light * at) * inv;
      power = v3(f, f, f);
    } else {
      power = scale(s.sky, ((4.0f * kPI) * at) * inv);
    }
    uint32_t events = 0;
    while (true) {
      float t;
      if (!free_flight(s, o, d, rng, t, c)) break;
      o = along(o, d, t);
      per[p].push_back(Photon{F4{o.x, o.y, o.z, 0.f}, F4{power.x, power.y, power.z, 0.f}, F4{d.x, d.y, d.z, 0.f},
                              p * kPpmMaxEvents + events});
      ++events;
      power = scale(power, s.albedo);
      if ((s.max_events && events >= s.max_events) || events >= kPpmMaxEvents) break;
      d = hg_sample(s, d, rng, true);
    }
  }
  size_t total = 0;
  for (auto& v : per) total += v.size();
  T.ph.clear();
  T.ph.reserve(std::min<size_t>(total, cap));
  for (auto& v : per)
    for (auto& x : v)
      if (T.ph.size() < cap) T.ph.push_back(x);
  T.dropped = (uint32_t)(total - T.ph.size());
}

static void build(const Scene& s, PhotonTree& T) {
  uint32_t n = (uint32_t)T.ph.size();
  std::vector<uint32_t> codes(n);
  V3 e = sub(s.b1, s.b0);
  for (uint32_t i = 0; i < n; ++i) {
    F4 p = T.ph[i].pos;
    float qx = std::fmin(std::fmax(((p.x - s.b0.x) / e.x) * 1024.0f, 0.0f), 1023.0f);
    float qy = std::fmin(std::fmax(((p.y - s.b0.y) / e.y) * 1024.0f, 0.0f), 1023.0f);
    float qz = std::fmin(std::fmax(((p.z - s.b0.z) / e.z) * 1024.0f, 0.0f), 1023.0f);
    codes[i] = (expand10((uint32_t)qx) << 2) | (expand10((uint32_t)qy) << 1) | expand10((uint32_t)qz);
  }
  T.order.resize(n);
  std::iota(T.order.begin(), T.order.end(), 0u);
  std::stable_sort(T.order.begin(), T.order.end(), [&](uint32_t a, uint32_t b) { return codes[a] < codes[b]; });
  std::vector<uint32_t> sorted(n);
  for (uint32_t i = 0; i < n; ++i) sorted[i] = codes[T.order[i]];
  T.left.assign(n > 1 ? n - 1 : 0, 0);
  T.right.assign(n > 1 ? n - 1 : 0, 0);
  T.leaf_lo.assign(n, F4{});
  T.leaf_hi.assign(n, F4{});
  T.node_lo.assign(n > 1 ? n - 1 : 0, F4{});
  T.node_hi.assign(n > 1 ? n - 1 : 0, F4{});
  if (n > 1) lbvh_build(sorted.data(), (int)n, T.left.data(), T.right.data());
  for (uint32_t i = 0; i < n; ++i) segment_box(T.ph[T.order[i]].pos, T.ph[T.order[i]].pos, T.leaf_lo[i], T.leaf_hi[i]);
  if (n > 1) refit(0, T.left.data(), T.right.data(), T.leaf_lo, T.leaf_hi, T.node_lo, T.node_hi);
}

static void gather(const Scene& s, const PhotonTree& T, const vcr_camera& cam, uint32_t W, uint32_t H,
                   const vcr_pass_desc* pass, float alpha, double* stats, double* sum, int threads) {
  uint32_t x0 = pass->crop[0], y0 = pass->crop[1];
  uint32_t cw = pass->crop[2] ? pass->crop[2] : W, ch = pass->crop[2] ? pass->crop[3] : H;
  int n = (int)T.ph.size();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
  for (int64_t row = 0; row < (int64_t)ch; ++row) {
    for (uint32_t cx = 0; cx < cw; ++cx) {
      int x = (int)(x0 + cx), y = (int)(y0 + (uint32_t)row);
      uint32_t pix = (uint32_t)y * W + (uint32_t)x;
      double* st = stats + 8 * (size_t)pix;
      Counts c;
      V3 o, rd;
      camera_ray(cam, x, y, o, rd);
      V3 bg = v3(0, 0, 0), phi = bg;
      uint32_t M = 0;
      float tmin, tmax;
      if (!slab(o, rd, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
        bg = sky(s, rd);
      } else {
        V3 entry = along(o, rd, std::fmax(tmin, 0.0f));
        Rng rng = rng_pcg(pass->seed ^ kPpmGatherSalt, pix, pass->pass_index);
        float t;
        if (!free_flight(s, entry, rd, rng, t, c)) {
          bg = sky(s, rd);
        } else if (n > 0) {
          V3 xm = along(entry, rd, t);
          float sigma_t = s.k * density(s, xm);
          float r = (float)st[1];
          float r2 = r * r;
          V3 wo = neg(rd);
          tree_query(T, xm, r2, [&](uint32_t lf) {
            const Photon& ph = T.ph[T.order[lf]];
            float f = hg_pdf(s, dot(v3(ph.dir.x, ph.dir.y, ph.dir.z), wo));
            phi = add(phi, scale(v3(ph.pw.x, ph.pw.y, ph.pw.z), f));
            ++M;
          });
          if (sigma_t > 0.0f) phi = v3(phi.x / sigma_t, phi.y / sigma_t, phi.z / sigma_t);
          else phi = v3(0, 0, 0);
        }
      }
      double N = st[0], R = st[1];
      double tau[3] = {st[2], st[3], st[4]};
      if (M > 0) {
        double am = (double)alpha * (double)M;
        double ratio = (N + am) / (N + (double)M);
        st[0] = N + am;
        st[1] = R * cbrt_ratio(ratio);
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
      double Rn = st[1];
      double vol = (4.0 / 3.0) * 3.14159265358979323846 * Rn * Rn * Rn;
      double a = (double)s.albedo / vol;
      double* o3 = sum + 3 * (size_t)pix;
      o3[0] = st[5] + a * tau[0];
      o3[1] = st[6] + a * tau[1];
      o3[2] = st[7] + a * tau[2];
    }
  }
}

// RenderTechniquePPM::UpdateRadius (:302-312) for frame k + 1 (pass k).
static float global_radius(float r0, float alpha, uint32_t pass) {
  float r = r0;
  for (uint32_t n = 2; n <= pass + 1; ++n) r = r * std::pow(((float)(n - 1) + alpha) / (float)n, 0.33333f);
  return r;
}

static bool inside(V3 p, V3 b0, V3 b1) {
  return !(p.x < b0.x || p.y < b0.y || p.z < b0.z || p.x > b1.x || p.y > b1.y || p.z > b1.z);
}

// samplePhotonMap (PPM_PE.comp:304-375) with the global radius r.
static V3 photon_map(const Scene& s, const PhotonTree& T, V3 x, V3 wo, float r, float scatter, Rng& rng) {
  V3 phi = v3(0, 0, 0);
  int n = (int)T.ph.size();
  if (scatter == 0.0f || n <= 0) return phi;
  const float r2 = r * r;
  tree_query(T, x, r2, [&](uint32_t lf) {
    const Photon& ph = T.ph[T.order[lf]];
    float f = hg_pdf(s, dot(wo, v3(ph.dir.x, ph.dir.y, ph.dir.z)));
    phi = add(phi, v3(f * ph.pw.x, f * ph.pw.y, f * ph.pw.z));
  });
  if ((phi.x + phi.y) + phi.z <= 0.0f) return v3(0, 0, 0);
  rng.next();  // the reference's unused six-tap density average draws one number
  const float kPI4_3 = kPI * 4.0f / 3.0f;
  float den = ((kPI4_3 * r) * r2) * scatter;
  return v3(phi.x / den, phi.y / den, phi.z / den);
}

// PPM_PE.comp main (:443-546): back-to-front march, direct light from the
// shadow volume, an ambient sky term, the photon map; sums += L.
static void march(const Scene& s, const PhotonTree& T, const vcr_camera& cam, uint32_t W, uint32_t H,
                  const vcr_pass_desc* pass, float radius, float step, float amb_step, double* sum, int threads) {
  uint32_t x0 = pass->crop[0], y0 = pass->crop[1];
  uint32_t cw = pass->crop[2] ? pass->crop[2] : W, ch = pass->crop[2] ? pass->crop[3] : H;
  const uint32_t padded_w = 32u * (W / 32u + 1u);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
  for (int64_t row = 0; row < (int64_t)ch; ++row) {
    for (uint32_t cx = 0; cx < cw; ++cx) {
      int x = (int)(x0 + cx), y = (int)(y0 + (uint32_t)row);
      uint32_t pix = (uint32_t)y * W + (uint32_t)x;
      Rng rng = s.rng_mode == 1 ? rng_xorshift(pass->seed * ((uint32_t)x + (uint32_t)y * padded_w))
                                : rng_pcg(pass->seed ^ kPpmMarchSalt, pix, pass->pass_index);
      V3 pos, rd;
      camera_ray(cam, x, y, pos, rd);
      V3 L = sky(s, rd);
      float tmin, tmax;
      if (slab(pos, rd, s.b0, s.b1, tmin, tmax) && s.ds > 0.0f) {
        V3 closest = along(pos, rd, tmin);
        pos = along(pos, rd, tmax - step * rng.next());
        float max_d = length(sub(pos, closest));
        V3 wo = neg(rd);
        float cur = 0.0f;
        for (uint32_t it = 0; cur < max_d && it < kMarchCap; ++it) {
          pos = sub(pos, scale(rd, step));
          cur = cur + step;
          float ext = (density(s, pos) * s.ds) / s.bs;
          float scatter = s.albedo * ext;
          float pdf = hg_pdf(s, dot(wo, s.sun));
          float dl = (s.light * pdf) * sv_lookup(s, pos);
          V3 direct = v3(dl, dl, dl);
          V3 adir = hg_sample(s, rd, rng, false);
          V3 ap = pos;
          float acc = 0.0f, adist = 0.0f;
          uint32_t n = 0;
          V3 amb = sky(s, adir);
          while (inside(ap, s.b0, s.b1) && n < kMarchCap) {
            ap = add(ap, scale(adir, amb_step));
            acc = acc + density(s, ap);
            adist = adist + amb_step;
            ++n;
          }
          if (n > 0) {
            acc = acc * (s.ds / s.bs);
            float att = oexp(((-adist) * acc) / (float)n);
            amb = scale(amb, att);
            if (amb.x > 0.0f) direct = add(direct, amb);
          }
          V3 ind = scale(photon_map(s, T, pos, wo, radius, scatter, rng), s.albedo);
          float a = oexp((-step) * ext);
          V3 src = add(direct, ind);
          L = add(scale(L, a), v3((scatter * src.x) * step, (scatter * src.y) * step, (scatter * src.z) * step));
        }
      }
      double* o3 = sum + 3 * (size_t)pix;
      o3[0] += (double)L.x;
      o3[1] += (double)L.y;
      o3[2] += (double)L.z;
    }
  }
}

}  // namespace oracle

using namespace oracle;

extern "C" {

// stats: float64 x8 per pixel (N, R, tau rgb, background rgb), initialised
// by the caller to (0, R0, 0...).  out_n[2] = stored photons, dropped.
// If `photons_out` is non-null it receives pos/pw/dir (12 floats) + uid per
// stored photon in (photon, event) order, and `order_out` the leaf order.
int oracle_ppm_pass(void* h, int level, const vcr_cloud* cl, const vcr_camera* cam, const vcr_params* prm,
                    uint32_t photons, uint32_t cap, float alpha, uint32_t W, uint32_t H, const vcr_pass_desc* pass,
                    double* stats, double* sum, uint32_t* out_n, float* photons_out, uint32_t* uid_out,
                    uint32_t* order_out, uint32_t* left_out, uint32_t* right_out, int threads) {
  Scene s = make_scene(static_cast<Grid*>(h), *cl, *prm, nullptr, level, nullptr);
  PhotonTree T;
  emit(s, photons, cap, pass->seed, pass->pass_index, T, threads);
  build(s, T);
  gather(s, T, *cam, W, H, pass, alpha, stats, sum, threads);
  uint32_t n = (uint32_t)T.ph.size();
  if (out_n) {
    out_n[0] = n;
    out_n[1] = T.dropped;
  }
  if (photons_out)
    for (uint32_t i = 0; i < n; ++i) {
      const Photon& p = T.ph[i];
      float* q = photons_out + 12 * (size_t)i;
      q[0] = p.pos.x; q[1] = p.pos.y; q[2] = p.pos.z; q[3] = p.pos.w;
      q[4] = p.pw.x; q[5] = p.pw.y; q[6] = p.pw.z; q[7] = p.pw.w;
      q[8] = p.dir.x; q[9] = p.dir.y; q[10] = p.dir.z; q[11] = p.dir.w;
    }
  if (uid_out)
    for (uint32_t i = 0; i < n; ++i) uid_out[i] = T.ph[i].uid;
  if (order_out) std::copy(T.order.begin(), T.order.end(), order_out);
  if (left_out) std::copy(T.left.begin(), T.left.end(), left_out);
  if (right_out) std::copy(T.right.begin(), T.right.end(), right_out);
  return 0;
}

// One pass of the march estimate (VCR_PPM_MARCH): the same photons and tree
// as oracle_ppm_pass, then the ray march per pixel of the crop; sums +=
// the pass's estimate.  The shadow volume `sv_tex` is oracle_sv_build's.
int oracle_ppm_march_pass(void* h, int level, const vcr_cloud* cl, const vcr_camera* cam, const vcr_params* prm,
                          const vcr_shadow_volume* sv, const float* sv_tex, uint32_t photons, uint32_t cap, float r0,
                          float alpha, float step, float amb_step, uint32_t W, uint32_t H, const vcr_pass_desc* pass,
                          double* sum, uint32_t* out_n, float* radius_out, int threads) {
  Scene s = make_scene(static_cast<Grid*>(h), *cl, *prm, sv, level, sv_tex);
  PhotonTree T;
  emit(s, photons, cap, pass->seed, pass->pass_index, T, threads);
  build(s, T);
  float r = global_radius(r0, alpha, pass->pass_index);
  march(s, T, *cam, W, H, pass, r, step, amb_step, sum, threads);
  if (out_n) {
    out_n[0] = (uint32_t)T.ph.size();
    out_n[1] = T.dropped;
  }
  if (radius_out) *radius_out = r;
  return 0;
}

// The photon tree alone: built over n photon positions (xyz floats) in the
// box [b0, b1] as a pass builds it (30-bit Morton order, radix tree, refit),
// then, for each of m query points q with radius r, the photons the
// gather's walk takes: counts[i] and their input indices in hits (walk
// order, queries one after another, at most cap entries).  Returns the
// total number taken.
uint64_t oracle_ppm_tree_query(const float* pos, uint32_t n, const float b0[3], const float b1[3], const float* q,
                               const float* r, uint32_t m, uint32_t* counts, uint32_t* hits, uint64_t cap) {
  Scene s{};
  s.b0 = v3(b0[0], b0[1], b0[2]);
  s.b1 = v3(b1[0], b1[1], b1[2]);
  PhotonTree T;
  T.ph.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    T.ph[i] = Photon{};
    T.ph[i].pos = F4{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.0f};
    T.ph[i].uid = i;
  }
  build(s, T);
  uint64_t total = 0;
  for (uint32_t i = 0; i < m; ++i) {
    uint32_t c = 0;
    tree_query(T, v3(q[3 * i], q[3 * i + 1], q[3 * i + 2]), r[i] * r[i], [&](uint32_t lf) {
      if (total < cap) hits[total] = T.order[lf];
      ++total;
      ++c;
    });
    counts[i] = c;
  }
  return total;
}

}  // extern "C"
