// ORACLE — test infrastructure only (see oracle_math.h).  CPU restatement of
// progressive photon beams:
//   emission  : PPB_PT.comp main (:506-539), generateSunRay (:396-430, with
//               the missing else restored), interactWithMedium (:453-501),
//               depositPhotonBeam (:334-393: beam to the box exit, 16
//               free-flight distances, segments of about the radius)
//   keys      : 30-bit Morton of segment midpoints over the cloud box
//   sort      : stable sort by key (what the LocalSort/PrefixSum/GlobalSort
//               pipeline is meant to produce; see oracle_sort.cpp)
//   LBVH      : PPB_GenerateHierarchy.comp (:62-168) with index-augmented
//               common prefixes for equal keys
//   refit     : PPB_CalculateAABB.comp (:64-120), upper bounds fixed
//   gather    : PPB_PE.comp traverseTree (:408-466) / accumulateRadiance
//               (:362-404) as the beam x beam 1D estimator
// The algorithm is the reference's (the lines cited above; departures are
// named).  Per photon, beam and pixel its evaluation order is written out
// explicitly and the CUDA kernels keep the same order, so results agree bit
// for bit.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "oracle_lbvh.h"
#include "oracle_scene.h"

namespace oracle {

const int kBeamDists = 16;
// A transmittance distance whose free flight left the box: beyond every
// point of the beam or camera ray, whatever the rounding of the box exit.
const float kEscaped = 3.0e38f;
const int kSlotFloats = 28;
const uint32_t kMaxBeamsPerPhoton = 65;
const uint32_t kMaxSegPerBeam = 4096;
const uint32_t kEmitSalt = 0x85EBCA6Bu;
const uint32_t kGatherSalt = 0xC2B2AE35u;

static uint32_t segments_of(float len, float r) {
  float q = len / r;
  return q < (float)(kMaxSegPerBeam - 1) ? (uint32_t)q + 1u : kMaxSegPerBeam;
}

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

uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

static int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }

static int lbvh_delta(const uint32_t* keys, int n, int i, int j) {
  if (j < 0 || j > n - 1) return -1;
  uint32_t a = keys[i], b = keys[j];
  if (a == b) return 32 + clz32((uint32_t)i ^ (uint32_t)j);
  return clz32(a ^ b);
}

void lbvh_build(const uint32_t* keys, int n, uint32_t* left, uint32_t* right) {
  for (int i = 0; i < n - 1; ++i) {
    int d = lbvh_delta(keys, n, i, i + 1) - lbvh_delta(keys, n, i, i - 1) > 0 ? 1 : -1;
    int dmin = lbvh_delta(keys, n, i, i - d);
    int lmax = 2;
    while (lbvh_delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
      if (lbvh_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = lbvh_delta(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
      int t = (l + div - 1) / div;
      if (lbvh_delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
      if (t == 1) break;
    }
    int gamma = i + s * d + (d < 0 ? -1 : 0);
    left[i] = (std::min(i, j) == gamma) ? ((uint32_t)gamma | kLeafBit) : (uint32_t)gamma;
    right[i] = (std::max(i, j) == gamma + 1) ? ((uint32_t)(gamma + 1) | kLeafBit) : (uint32_t)(gamma + 1);
  }
}

void segment_box(F4 A, F4 B, F4& lo, F4& hi) {
  V3 pa = v3(A.x, A.y, A.z), pb = v3(B.x, B.y, B.z);
  float r = A.w;
  V3 a = sub(pb, pa);
  float dd = dot(a, a);
  V3 e;
  if (dd > 0.0f) {
    e.x = r * std::sqrt(std::fmax(0.0f, 1.0f - (a.x * a.x) / dd));
    e.y = r * std::sqrt(std::fmax(0.0f, 1.0f - (a.y * a.y) / dd));
    e.z = r * std::sqrt(std::fmax(0.0f, 1.0f - (a.z * a.z) / dd));
  } else {
    e = v3(r, r, r);
  }
  lo = F4{std::fmin(pa.x - e.x, pb.x - e.x), std::fmin(pa.y - e.y, pb.y - e.y), std::fmin(pa.z - e.z, pb.z - e.z), 0.f};
  hi = F4{std::fmax(pa.x + e.x, pb.x + e.x), std::fmax(pa.y + e.y, pb.y + e.y), std::fmax(pa.z + e.z, pb.z + e.z), 0.f};
}

// Boxes of the whole tree, recursively (same min/max as the GPU refit).
void refit(uint32_t node, const uint32_t* left, const uint32_t* right, const std::vector<F4>& llo,
           const std::vector<F4>& lhi, std::vector<F4>& nlo, std::vector<F4>& nhi) {
  uint32_t c[2] = {left[node], right[node]};
  F4 lo[2], hi[2];
  for (int k = 0; k < 2; ++k) {
    if (c[k] & kLeafBit) {
      lo[k] = llo[c[k] & ~kLeafBit];
      hi[k] = lhi[c[k] & ~kLeafBit];
    } else {
      refit(c[k], left, right, llo, lhi, nlo, nhi);
      lo[k] = nlo[c[k]];
      hi[k] = nhi[c[k]];
    }
  }
  nlo[node] = F4{std::fmin(lo[0].x, lo[1].x), std::fmin(lo[0].y, lo[1].y), std::fmin(lo[0].z, lo[1].z), 0.f};
  nhi[node] = F4{std::fmax(hi[0].x, hi[1].x), std::fmax(hi[0].y, hi[1].y), std::fmax(hi[0].z, hi[1].z), 0.f};
}

static bool ray_box(V3 o, V3 inv, float t0, float t1, F4 lo, F4 hi) {
  float ax = (lo.x - o.x) * inv.x, bx = (hi.x - o.x) * inv.x;
  float ay = (lo.y - o.y) * inv.y, by = (hi.y - o.y) * inv.y;
  float az = (lo.z - o.z) * inv.z, bz = (hi.z - o.z) * inv.z;
  float tn = std::fmax(std::fmax(std::fmin(ax, bx), std::fmin(ay, by)), std::fmax(std::fmin(az, bz), t0));
  float tf = std::fmin(std::fmin(std::fmax(ax, bx), std::fmax(ay, by)), std::fmin(std::fmax(az, bz), t1));
  return tn <= tf;
}

struct Beams {
  uint32_t P = 0, K = 0;
  std::vector<float> slots;
  std::vector<uint32_t> nbeams, slot_segs, slot_off, photon_off;
  uint32_t n = 0, dropped = 0;
  std::vector<F4> seg_a, seg_b;
  std::vector<uint32_t> seg_beam, codes, order, sorted;
  std::vector<uint32_t> left, right;
  std::vector<F4> leaf_lo, leaf_hi, node_lo, node_hi;
};

// The gather's walk over the beam tree (PPB_PE.comp:408-466 visits every
// beam whose box the camera ray crosses): depth first, left child before
// right, a subtree entered when the ray's [t_in, t_out] crosses its box
// (ray_box), `visit` called with each leaf (tree order) whose own box the
// ray crosses, in walk order, which fixes the order of the caller's sums.
template <class Visit>
static void beam_walk(const Beams& B, V3 o, V3 inv, float t_in, float t_out, Visit&& visit) {
  const int n = (int)B.n;
  if (n <= 0) return;
  uint32_t stack[64];
  int sp = 0;
  uint32_t node = n == 1 ? (0u | kLeafBit) : 0u;
  while (true) {
    if (node & kLeafBit) {
      uint32_t lf = node & ~kLeafBit;
      if (ray_box(o, inv, t_in, t_out, B.leaf_lo[lf], B.leaf_hi[lf])) visit(lf);
    } else if (ray_box(o, inv, t_in, t_out, B.node_lo[node], B.node_hi[node])) {
      if (sp < 64) stack[sp++] = B.right[node];
      node = B.left[node];
      continue;
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
}

static V3 beam_contribution(const Scene& s, const Beams& B, uint32_t sid, V3 o, V3 rd, float t_in, float t_out,
                            const float* cam_d, Counts& c) {
  F4 A = B.seg_a[sid], Bq = B.seg_b[sid];
  V3 pa = v3(A.x, A.y, A.z), pb = v3(Bq.x, Bq.y, Bq.z);
  float r = A.w;
  V3 ax = sub(pb, pa);
  float segl = length(ax);
  V3 zero = v3(0, 0, 0);
  if (!(segl > 0.0f)) return zero;
  V3 bd = v3(ax.x / segl, ax.y / segl, ax.z / segl);
  float b = dot(rd, bd);
  float den = 1.0f - b * b;
  if (!(den > 1e-6f)) return zero;
  V3 w0 = sub(o, pa);
  float dw = dot(rd, w0), ew = dot(bd, w0);
  float t = (b * ew - dw) / den;
  float sb = ew + t * b;
  if (t < t_in || t > t_out || sb < 0.0f || sb > segl) return zero;
  V3 xc = along(o, rd, t);
  V3 xb = along(pa, bd, sb);
  float dist = length(sub(xc, xb));
  if (!(dist < r)) return zero;
  float u = dist / r;
  float q = 1.0f - u * u;
  float kern = ((0.9375f * q) * q) / r;
  float rho = density(s, xc);
  ++c.lookups;
  float sigma_s = (s.albedo * s.k) * rho;
  const float* sl = &B.slots[(size_t)B.seg_beam[sid] * kSlotFloats];
  float sbeam = sb + Bq.w;
  uint32_t cb = 0, cc = 0;
  float tc = t - t_in;
  for (int i = 0; i < kBeamDists; ++i) {
    cb += sl[10 + i] >= sbeam ? 1u : 0u;
    cc += cam_d[i] >= tc ? 1u : 0u;
  }
  float tb = (float)cb * (1.0f / kBeamDists), tcam = (float)cc * (1.0f / kBeamDists);
  float ph = hg_pdf(s, dot(bd, neg(rd)));
  float w = ((((kern * sigma_s) * tcam) * tb) * ph) / std::sqrt(den);
  return v3(sl[7] * w, sl[8] * w, sl[9] * w);
}

static void run_ppb(const Scene& s, uint32_t P, uint32_t cap, float radius, uint32_t seed, uint32_t pass, Beams& B,
                    int threads) {
  uint32_t K = s.max_events ? std::min<uint32_t>(s.max_events + 1u, kMaxBeamsPerPhoton) : kMaxBeamsPerPhoton;
  B.P = P;
  B.K = K;
  B.slots.assign((size_t)P * K * kSlotFloats, 0.0f);
  B.nbeams.assign(P, 0);
  B.slot_segs.assign((size_t)P * K, 0);
  B.slot_off.assign((size_t)P * K, 0);
  std::vector<uint32_t> photon_segs(P, 0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
  for (int64_t pi = 0; pi < (int64_t)P; ++pi) {
    uint32_t p = (uint32_t)pi;
    Counts c;
    Rng rng = rng_pcg(seed ^ kEmitSalt, p, pass);
    V3 d, power;
    const float inv = 1.0f / ((float)P * 0.5f);
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
    V3 o;
    float at = box_entry(s, d, rng, o);
    if (sun) {
      float f = (s.light * at) * inv;
      power = v3(f, f, f);
    } else {
      float f = ((4.0f * kPI) * at) * inv;
      power = scale(s.sky, f);
    }
    uint32_t beams = 0, events = 0, seg_total = 0;
    while (beams < K) {
      float tmin, tmax;
      if (!slab(o, d, s.b0, s.b1, tmin, tmax) || !finite_pos(tmax)) break;
      float* sl = &B.slots[((size_t)p * K + beams) * kSlotFloats];
      sl[0] = o.x; sl[1] = o.y; sl[2] = o.z;
      sl[3] = d.x; sl[4] = d.y; sl[5] = d.z;
      sl[6] = tmax;
      sl[7] = power.x; sl[8] = power.y; sl[9] = power.z;
      for (int i = 0; i < kBeamDists; ++i) {
        float t;
        sl[10 + i] = free_flight(s, o, d, rng, t, c) ? t : kEscaped;
      }
      uint32_t ns = segments_of(tmax, radius);
      B.slot_segs[(size_t)p * K + beams] = ns;
      B.slot_off[(size_t)p * K + beams] = seg_total;
      seg_total += ns;
      ++beams;
      float t;
      if (!free_flight(s, o, d, rng, t, c)) break;
      o = along(o, d, t);
      ++events;
      power = scale(power, s.albedo);
      if (s.max_events && events >= s.max_events) break;
      d = hg_sample(s, d, rng, true);
    }
    B.nbeams[p] = beams;
    photon_segs[p] = seg_total;
  }
  B.photon_off.assign(P, 0);
  uint64_t total = 0;
  for (uint32_t p = 0; p < P; ++p) {
    B.photon_off[p] = (uint32_t)total;
    total += photon_segs[p];
  }
  uint32_t n = (uint32_t)std::min<uint64_t>(total, cap);
  B.n = n;
  B.dropped = (uint32_t)(total - n);
  B.seg_a.assign(n, F4{});
  B.seg_b.assign(n, F4{});
  B.seg_beam.assign(n, 0);
  B.codes.assign(n, 0);
  V3 e = sub(s.b1, s.b0);
  for (uint32_t p = 0; p < P; ++p)
    for (uint32_t k = 0; k < B.nbeams[p]; ++k) {
      size_t slot = (size_t)p * K + k;
      const float* sl = &B.slots[slot * kSlotFloats];
      V3 o = v3(sl[0], sl[1], sl[2]), d = v3(sl[3], sl[4], sl[5]);
      float len = sl[6];
      uint32_t ns = B.slot_segs[slot];
      uint32_t base = B.photon_off[p] + B.slot_off[slot];
      float segl = len / (float)ns;
      for (uint32_t j = 0; j < ns; ++j) {
        uint32_t gi = base + j;
        if (gi >= cap) break;
        float off = (float)j * segl;
        V3 a = along(o, d, off);
        V3 b = along(a, d, segl);
        B.seg_a[gi] = F4{a.x, a.y, a.z, radius};
        B.seg_b[gi] = F4{b.x, b.y, b.z, off};
        B.seg_beam[gi] = (uint32_t)slot;
        V3 m = scale(add(a, b), 0.5f);
        float qx = std::fmin(std::fmax(((m.x - s.b0.x) / e.x) * 1024.0f, 0.0f), 1023.0f);
        float qy = std::fmin(std::fmax(((m.y - s.b0.y) / e.y) * 1024.0f, 0.0f), 1023.0f);
        float qz = std::fmin(std::fmax(((m.z - s.b0.z) / e.z) * 1024.0f, 0.0f), 1023.0f);
        B.codes[gi] = (expand10((uint32_t)qx) << 2) | (expand10((uint32_t)qy) << 1) | expand10((uint32_t)qz);
      }
    }
  // stable sort by key
  B.order.resize(n);
  std::iota(B.order.begin(), B.order.end(), 0u);
  std::stable_sort(B.order.begin(), B.order.end(), [&](uint32_t a, uint32_t b) { return B.codes[a] < B.codes[b]; });
  B.sorted.resize(n);
  for (uint32_t i = 0; i < n; ++i) B.sorted[i] = B.codes[B.order[i]];
  B.left.assign(n > 1 ? n - 1 : 0, 0);
  B.right.assign(n > 1 ? n - 1 : 0, 0);
  B.leaf_lo.assign(n, F4{});
  B.leaf_hi.assign(n, F4{});
  B.node_lo.assign(n > 1 ? n - 1 : 0, F4{});
  B.node_hi.assign(n > 1 ? n - 1 : 0, F4{});
  if (n > 1) lbvh_build(B.sorted.data(), (int)n, B.left.data(), B.right.data());
  for (uint32_t i = 0; i < n; ++i) segment_box(B.seg_a[B.order[i]], B.seg_b[B.order[i]], B.leaf_lo[i], B.leaf_hi[i]);
  if (n > 1) refit(0, B.left.data(), B.right.data(), B.leaf_lo, B.leaf_hi, B.node_lo, B.node_hi);
}

static void gather(const Scene& s, const Beams& B, const vcr_camera& cam, uint32_t W, uint32_t H,
                   const vcr_pass_desc* pass, double* sum, int threads) {
  uint32_t x0 = pass->crop[0], y0 = pass->crop[1];
  uint32_t cw = pass->crop[2] ? pass->crop[2] : W, ch = pass->crop[2] ? pass->crop[3] : H;
  int n = (int)B.n;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
  for (int64_t row = 0; row < (int64_t)ch; ++row) {
    for (uint32_t cx = 0; cx < cw; ++cx) {
      int x = (int)(x0 + cx), y = (int)(y0 + (uint32_t)row);
      uint32_t pix = (uint32_t)y * W + (uint32_t)x;
      Counts c;
      V3 o, rd;
      camera_ray(cam, x, y, o, rd);
      V3 L = v3(0, 0, 0);
      float tmin, tmax;
      if (!slab(o, rd, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
        L = sky(s, rd);
      } else {
        float t_in = std::fmax(tmin, 0.0f), t_out = tmax;
        V3 entry = along(o, rd, t_in);
        Rng rng = rng_pcg(pass->seed ^ kGatherSalt, pix, pass->pass_index);
        float cam_d[kBeamDists];
        for (int i = 0; i < kBeamDists; ++i) {
          float t;
          cam_d[i] = free_flight(s, entry, rd, rng, t, c) ? t : kEscaped;
        }
        uint32_t cexit = 0;
        for (int i = 0; i < kBeamDists; ++i) cexit += cam_d[i] >= (t_out - t_in) ? 1u : 0u;
        L = scale(sky(s, rd), (float)cexit * (1.0f / kBeamDists));
        if (n > 0) {
          V3 inv = v3(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
          beam_walk(B, o, inv, t_in, t_out, [&](uint32_t lf) {
            L = add(L, beam_contribution(s, B, B.order[lf], o, rd, t_in, t_out, cam_d, c));
          });
        }
      }
      double* out = sum + 3 * (size_t)pix;
      if (pass->flags & VCR_PASS_NO_ACCUMULATE) {
        out[0] = L.x; out[1] = L.y; out[2] = L.z;
      } else {
        out[0] += L.x; out[1] += L.y; out[2] += L.z;
      }
    }
  }
}

}  // namespace oracle

using namespace oracle;

extern "C" {

// Outputs of one oracle beam pass (each pointer may be NULL).
struct OraclePpbOut {
  uint32_t* n;          // [2]: segments, dropped
  float* slots;         // P*K*28
  uint32_t* nbeams;     // P
  float* seg_a;         // n*4
  float* seg_b;         // n*4
  uint32_t* seg_beam;   // n
  uint32_t* codes;      // n
  uint32_t* order;      // n
  uint32_t* left;       // n-1
  uint32_t* right;      // n-1
  float* node_lo;       // (n-1)*4
  float* node_hi;
  float* leaf_lo;       // n*4
  float* leaf_hi;
  uint32_t capacity_out;  // capacity of the per-segment arrays
};

float oracle_ppb_radius(float r0, float alpha, uint32_t pass) {
  double r = r0;
  for (uint32_t i = 1; i <= pass; ++i) r *= ((double)i + (double)alpha) / ((double)i + 1.0);
  return (float)r;
}

int oracle_ppb_pass(void* h, int level, const vcr_cloud* cl, const vcr_camera* cam, const vcr_params* prm,
                    uint32_t photons, uint32_t cap, float r0, float alpha, uint32_t W, uint32_t H,
                    const vcr_pass_desc* pass, double* sum, OraclePpbOut* out, int threads) {
  Scene s = make_scene(static_cast<Grid*>(h), *cl, *prm, nullptr, level, nullptr);
  Beams B;
  float radius = oracle_ppb_radius(r0, alpha, pass->pass_index);
  run_ppb(s, photons, cap, radius, pass->seed, pass->pass_index, B, threads);
  if (sum) gather(s, B, *cam, W, H, pass, sum, threads);
  if (out) {
    uint32_t n = B.n;
    if (out->n) { out->n[0] = n; out->n[1] = B.dropped; }
    if (out->slots) std::copy(B.slots.begin(), B.slots.end(), out->slots);
    if (out->nbeams) std::copy(B.nbeams.begin(), B.nbeams.end(), out->nbeams);
    if (n <= out->capacity_out) {
      if (out->seg_a) std::memcpy(out->seg_a, B.seg_a.data(), n * 16);
      if (out->seg_b) std::memcpy(out->seg_b, B.seg_b.data(), n * 16);
      if (out->seg_beam) std::copy(B.seg_beam.begin(), B.seg_beam.end(), out->seg_beam);
      if (out->codes) std::copy(B.codes.begin(), B.codes.end(), out->codes);
      if (out->order) std::copy(B.order.begin(), B.order.end(), out->order);
      if (out->left) std::copy(B.left.begin(), B.left.end(), out->left);
      if (out->right) std::copy(B.right.begin(), B.right.end(), out->right);
      if (out->node_lo && n > 1) std::memcpy(out->node_lo, B.node_lo.data(), (n - 1) * 16);
      if (out->node_hi && n > 1) std::memcpy(out->node_hi, B.node_hi.data(), (n - 1) * 16);
      if (out->leaf_lo) std::memcpy(out->leaf_lo, B.leaf_lo.data(), n * 16);
      if (out->leaf_hi) std::memcpy(out->leaf_hi, B.leaf_hi.data(), n * 16);
    }
  }
  return 0;
}

// The gather's walk alone over a given tree (left / right children, node
// and leaf boxes as float4, n leaves): for each of m rays (origin,
// direction, [t0, t1]) the leaves it visits, counts[i] and the leaf indices
// in hits (walk order, rays one after another, at most cap entries).
// Returns the total.
uint64_t oracle_ppb_walk(const uint32_t* left, const uint32_t* right, const float* node_lo, const float* node_hi,
                         const float* leaf_lo, const float* leaf_hi, uint32_t n, const float* ro, const float* rdir,
                         const float* t01, uint32_t m, uint32_t* counts, uint32_t* hits, uint64_t cap) {
  Beams B;
  B.n = n;
  const size_t ni = n > 1 ? n - 1 : 0;
  B.left.assign(left, left + ni);
  B.right.assign(right, right + ni);
  B.node_lo.assign(reinterpret_cast<const F4*>(node_lo), reinterpret_cast<const F4*>(node_lo) + ni);
  B.node_hi.assign(reinterpret_cast<const F4*>(node_hi), reinterpret_cast<const F4*>(node_hi) + ni);
  B.leaf_lo.assign(reinterpret_cast<const F4*>(leaf_lo), reinterpret_cast<const F4*>(leaf_lo) + n);
  B.leaf_hi.assign(reinterpret_cast<const F4*>(leaf_hi), reinterpret_cast<const F4*>(leaf_hi) + n);
  uint64_t total = 0;
  for (uint32_t i = 0; i < m; ++i) {
    const V3 o = v3(ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]), d = v3(rdir[3 * i], rdir[3 * i + 1], rdir[3 * i + 2]);
    const V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t c = 0;
    beam_walk(B, o, inv, t01[2 * i], t01[2 * i + 1], [&](uint32_t lf) {
      if (total < cap) hits[total] = lf;
      ++total;
      ++c;
    });
    counts[i] = c;
  }
  return total;
}

// LBVH + refit over given sorted keys / segments (for the primitive test).
void oracle_lbvh(const uint32_t* sorted, const uint32_t* order, const float* seg_a, const float* seg_b, uint32_t n,
                 uint32_t* left, uint32_t* right, float* node_lo, float* node_hi, float* leaf_lo, float* leaf_hi) {
  std::vector<F4> llo(n), lhi(n), nlo(n > 1 ? n - 1 : 0), nhi(n > 1 ? n - 1 : 0);
  const F4* A = reinterpret_cast<const F4*>(seg_a);
  const F4* Bq = reinterpret_cast<const F4*>(seg_b);
  if (n > 1) lbvh_build(sorted, (int)n, left, right);
  for (uint32_t i = 0; i < n; ++i) segment_box(A[order[i]], Bq[order[i]], llo[i], lhi[i]);
  if (n > 1) refit(0, left, right, llo, lhi, nlo, nhi);
  std::memcpy(leaf_lo, llo.data(), n * 16);
  std::memcpy(leaf_hi, lhi.data(), n * 16);
  if (n > 1) {
    std::memcpy(node_lo, nlo.data(), (n - 1) * 16);
    std::memcpy(node_hi, nhi.data(), (n - 1) * 16);
  }
}

}  // extern "C"
