// ORACLE — test infrastructure only (see oracle_math.h).  CPU restatement of
// the reference's volumetric path tracer and its supporting pieces:
//   grid     : Grid3D (Grid3D.h:5-192) + the brick encoding the GPU stores
//   sampler  : sampleCloud (PathTracer.comp:115-119), trilinear, clamp-to-edge
//   tracker  : findScatterPoint (PathTracer.comp:318-361) and the DDA
//              majorant-grid variant; ratio tracking toward the sun
//   phase    : calculatePDF / invertCDF / scatterRay (PathTracer.comp:247-311)
//   camera   : getCameraRay (PathTracer.comp:144-151)
//   main     : PathTracer.comp:366-425
//   shadow   : ShadowVolume.comp:77-93, sampleShadowVolume (:121-127)
//   fBm      : the synthetic cloud generator (Perlin 2002 improved noise)
#include <algorithm>
#include <vector>

#include "oracle_scene.h"

namespace oracle {

// ---------------------------------------------------------------------------
// grid: decoded texels (what the GPU reads back from its bricks) + majorants
// ---------------------------------------------------------------------------
Grid* grid_new(const uint32_t size[3], const float* dense, int precision) {
  Grid* g = new Grid();
  for (int a = 0; a < 3; ++a) {
    g->n[a] = (int)size[a];
    g->nb[a] = (g->n[a] + 7) / 8;
  }
  size_t total = (size_t)g->n[0] * g->n[1] * g->n[2];
  g->tex.assign(dense, dense + total);
  if (precision != 0) {
    // per-brick scale = brick maximum; texel stored as RNE(v / scale)
#pragma omp parallel for schedule(dynamic, 1)
    for (int kb = 0; kb < g->nb[2]; ++kb)
      for (int jb = 0; jb < g->nb[1]; ++jb)
        for (int ib = 0; ib < g->nb[0]; ++ib) {
          float s = 0.0f;
          for (int k = kb * 8; k < std::min(kb * 8 + 8, g->n[2]); ++k)
            for (int j = jb * 8; j < std::min(jb * 8 + 8, g->n[1]); ++j)
              for (int i = ib * 8; i < std::min(ib * 8 + 8, g->n[0]); ++i) s = std::fmax(s, g->at(i, j, k));
          for (int k = kb * 8; k < std::min(kb * 8 + 8, g->n[2]); ++k)
            for (int j = jb * 8; j < std::min(jb * 8 + 8, g->n[1]); ++j)
              for (int i = ib * 8; i < std::min(ib * 8 + 8, g->n[0]); ++i) {
                float& v = g->tex[(size_t)i + (size_t)g->n[0] * ((size_t)j + (size_t)g->n[1] * k)];
                float q = s > 0.0f ? v / s : 0.0f;
                float d = precision == 1 ? f16_to_f32(f32_to_f16(q)) : bf16_to_f32(f32_to_bf16(q));
                v = d * s;
              }
        }
  }
  // majorant over [8b-1, 8b+8] per axis, clamped
  g->maj.assign((size_t)g->nb[0] * g->nb[1] * g->nb[2], 0.0f);
#pragma omp parallel for schedule(dynamic, 1)
  for (int kb = 0; kb < g->nb[2]; ++kb)
    for (int jb = 0; jb < g->nb[1]; ++jb)
      for (int ib = 0; ib < g->nb[0]; ++ib) {
        float m = 0.0f;
        for (int dk = 0; dk < 10; ++dk)
          for (int dj = 0; dj < 10; ++dj)
            for (int di = 0; di < 10; ++di) {
              int i = std::min(std::max(ib * 8 - 1 + di, 0), g->n[0] - 1);
              int j = std::min(std::max(jb * 8 - 1 + dj, 0), g->n[1] - 1);
              int k = std::min(std::max(kb * 8 - 1 + dk, 0), g->n[2] - 1);
              m = std::fmax(m, g->at(i, j, k));
            }
        g->maj[(size_t)ib + (size_t)g->nb[0] * ((size_t)jb + (size_t)g->nb[1] * kb)] = m;
      }
  for (float m : g->maj) g->max_density = std::fmax(g->max_density, m);
  g->lv[0] = g->maj;
  for (int a = 0; a < 3; ++a) g->lnb[0][a] = g->nb[a];
  for (int l = 1; l < 4; ++l) {
    const int* sd = g->lnb[l - 1];
    int* dd = g->lnb[l];
    for (int a = 0; a < 3; ++a) dd[a] = (sd[a] + 1) / 2;
    g->lv[l].assign((size_t)dd[0] * dd[1] * dd[2], 0.0f);
    for (int k = 0; k < dd[2]; ++k)
      for (int j = 0; j < dd[1]; ++j)
        for (int i = 0; i < dd[0]; ++i) {
          float m = 0.0f;
          for (int c = 0; c < 8; ++c) {
            int a = 2 * i + (c & 1), b = 2 * j + ((c >> 1) & 1), e = 2 * k + (c >> 2);
            if (a < sd[0] && b < sd[1] && e < sd[2])
              m = std::fmax(m, g->lv[l - 1][(size_t)a + (size_t)sd[0] * ((size_t)b + (size_t)sd[1] * e)]);
          }
          g->lv[l][(size_t)i + (size_t)dd[0] * ((size_t)j + (size_t)dd[1] * k)] = m;
        }
  }
  return g;
}

// texel centres at (i + 1/2)/N; lerp = fma(t, b - a, a), x then y then z
float trilinear(const float* tex, const int n[3], V3 nrm) {
  float ux = nrm.x * (float)n[0] - 0.5f, uy = nrm.y * (float)n[1] - 0.5f, uz = nrm.z * (float)n[2] - 0.5f;
  float fx = std::floor(ux), fy = std::floor(uy), fz = std::floor(uz);
  float tx = ux - fx, ty = uy - fy, tz = uz - fz;
  int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
  int x1 = std::min(std::max(x0 + 1, 0), n[0] - 1), y1 = std::min(std::max(y0 + 1, 0), n[1] - 1),
      z1 = std::min(std::max(z0 + 1, 0), n[2] - 1);
  x0 = std::min(std::max(x0, 0), n[0] - 1);
  y0 = std::min(std::max(y0, 0), n[1] - 1);
  z0 = std::min(std::max(z0, 0), n[2] - 1);
  auto T = [&](int i, int j, int k) { return tex[(size_t)i + (size_t)n[0] * ((size_t)j + (size_t)n[1] * k)]; };
  float c00 = std::fma(tx, T(x1, y0, z0) - T(x0, y0, z0), T(x0, y0, z0));
  float c10 = std::fma(tx, T(x1, y1, z0) - T(x0, y1, z0), T(x0, y1, z0));
  float c01 = std::fma(tx, T(x1, y0, z1) - T(x0, y0, z1), T(x0, y0, z1));
  float c11 = std::fma(tx, T(x1, y1, z1) - T(x0, y1, z1), T(x0, y1, z1));
  float c0 = std::fma(ty, c10 - c00, c00);
  float c1 = std::fma(ty, c11 - c01, c01);
  return std::fma(tz, c1 - c0, c0);
}

// sampleCloud (PathTracer.comp:115-119)
// normalised coordinates (p - b0) / (b1 - b0), by the reciprocal extent
float density(const Scene& s, V3 p) {
  V3 q = sub(p, s.b0);
  return trilinear(s.g->tex.data(), s.g->n, v3(q.x * s.iext.x, q.y * s.iext.y, q.z * s.iext.z));
}

// slab test, intersectCloud (PathTracer.comp:154-184)
bool slab(V3 pos, V3 dir, V3 b0, V3 b1, float& tmin, float& tmax) {
  V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  bool sx = inv.x < 0.0f, sy = inv.y < 0.0f, sz = inv.z < 0.0f;
  tmin = ((sx ? b1.x : b0.x) - pos.x) * inv.x;
  tmax = ((sx ? b0.x : b1.x) - pos.x) * inv.x;
  float tymin = ((sy ? b1.y : b0.y) - pos.y) * inv.y;
  float tymax = ((sy ? b0.y : b1.y) - pos.y) * inv.y;
  if ((tmin > tymax) || (tymin > tmax)) return false;
  if (tymin > tmin) tmin = tymin;
  if (tymax < tmax) tmax = tymax;
  float tzmin = ((sz ? b1.z : b0.z) - pos.z) * inv.z;
  float tzmax = ((sz ? b0.z : b1.z) - pos.z) * inv.z;
  if ((tmin > tzmax) || (tzmin > tmax)) return false;
  if (tzmin > tmin) tmin = tzmin;
  if (tzmax < tmax) tmax = tzmax;
  return true;
}

bool in_box(V3 p, V3 b0, V3 b1) {
  return !(p.x < b0.x || p.y < b0.y || p.z < b0.z || p.x > b1.x || p.y > b1.y || p.z > b1.z);
}

// sampleBackground (PathTracer.comp:104-113); smoothstep / mix per GLSL
V3 sky_gradient(V3 dir) {
  const float C[5][3] = {{0.00f, 0.0f, 0.02f}, {0.01f, 0.05f, 0.2f}, {0.7f, 0.9f, 1.0f},
                         {0.1f, 0.3f, 1.0f}, {0.01f, 0.1f, 0.7f}};
  const float D[5] = {-1.0f, -0.04f, 0.0f, 0.5f, 1.0f};
  float col[3] = {C[0][0], C[0][1], C[0][2]};
  for (int i = 1; i < 5; ++i) {
    float t = clampf((dir.y - D[i - 1]) / (D[i] - D[i - 1]), 0.0f, 1.0f);
    float sm = t * t * (3.0f - 2.0f * t);
    for (int c = 0; c < 3; ++c) col[c] = col[c] * (1.0f - sm) + C[i][c] * sm;
  }
  return v3(col[0], col[1], col[2]);
}

V3 sky(const Scene& s, V3 dir) { return s.sky_mode == 0 ? s.sky : sky_gradient(dir); }

// calculatePDF / samplePhase (PathTracer.comp:247-274); pow(x, 1.5) = x sqrt(x)
float hg_pdf(const Scene& s, float c) {
  if (s.iso) return kINV_4PI;
  float d = s.opg2 - (2.0f * s.g_) * c;
  return (kINV_4PI * s.omg2) / (d * std::sqrt(d));
}

// createOrthonormalBasis (PathTracer.comp:197-206)
void onb(V3 n, V3& xp, V3& yp) {
  float sz = n.z >= 0.0f ? 1.0f : -1.0f;
  float a = n.y / (1.0f + std::fabs(n.z));
  float b = n.y * a;
  float c = -n.x * a;
  xp = v3(n.z + sz * b, sz * c, -n.x);
  yp = v3(c, 1.0f - b, -sz * n.y);
}

// scatterRay (PathTracer.comp:277-311); `renorm` as PPM_PT/PPB_PT do
V3 hg_sample(const Scene& s, V3 in, Rng& rng, bool renorm) {
  V3 out;
  if (s.iso) {
    float xi = rng.next();
    out.z = xi * 2.0f - 1.0f;
    float s2 = 1.0f - out.z * out.z;
    if (s2 > 0.0f) {
      float st = std::sqrt(std::fmax(0.0f, s2));
      float sn, cs;
      osincos2pi(rng.next(), &sn, &cs);
      out.x = st * cs;
      out.y = st * sn;
    } else {
      out.x = out.y = 0.0f;
    }
  } else {
    float u_phi = rng.next();
    float xi = rng.next();
    float sq = s.omg2 / ((1.0f - s.g_) + (2.0f * s.g_) * xi);  // invertCDF
    float ct = s.o2g * (s.opg2 - sq * sq);
    float st = std::sqrt(std::fmax(0.0f, 1.0f - ct * ct));
    float sn, cs;
    osincos2pi(u_phi, &sn, &cs);
    V3 t0, t1;
    onb(in, t0, t1);
    float a = st * cs, b = st * sn;
    out = v3((a * t0.x + b * t1.x) + ct * in.x, (a * t0.y + b * t1.y) + ct * in.y, (a * t0.z + b * t1.z) + ct * in.z);
  }
  return renorm ? normalize(out) : out;
}

// getCameraRay (PathTracer.comp:144-151)
void camera_ray(const vcr_camera& c, int x, int y, V3& pos, V3& dir) {
  float a = (float)(x - c.half_width), b = (float)(y - c.half_height);
  V3 d;
  d.x = (c.forward[0] * c.near_plane + (c.right[0] * c.pixel_size_x) * a) - (c.up[0] * c.pixel_size_y) * b;
  d.y = (c.forward[1] * c.near_plane + (c.right[1] * c.pixel_size_x) * a) - (c.up[1] * c.pixel_size_y) * b;
  d.z = (c.forward[2] * c.near_plane + (c.right[2] * c.pixel_size_x) * a) - (c.up[2] * c.pixel_size_y) * b;
  pos = add(d, v3(c.position[0], c.position[1], c.position[2]));
  dir = normalize(d);
}

float dense_trilinear(const float* tex, int n, V3 nrm) {
  int nn[3] = {n, n, n};
  return trilinear(tex, nn, nrm);
}

// sampleShadowVolume (PathTracer.comp:121-127)
float sv_lookup(const Scene& s, V3 p) {
  V3 d = sub(p, s.sv_b0);
  V3 q = v3((s.B[0] * d.x + s.B[1] * d.y) + s.B[2] * d.z, (s.B[3] * d.x + s.B[4] * d.y) + s.B[5] * d.z,
            (s.B[6] * d.x + s.B[7] * d.y) + s.B[8] * d.z);
  return dense_trilinear(s.sv_tex, s.sv_n, vdiv(q, s.sv_ext));
}

// ---------------------------------------------------------------------------
// global-majorant tracking (reference semantics)
// ---------------------------------------------------------------------------

// findScatterPoint (PathTracer.comp:318-361)
bool find_scatter_global(const Scene& s, float sigma_bar, V3& pos, V3 dir, Rng& rng, Counts& c) {
  float tmin, tmax;
  if (!slab(pos, dir, s.b0, s.b1, tmin, tmax)) return false;
  V3 exitp = along(pos, dir, tmax);
  float dist = length(sub(exitp, pos));
  if (!finite_pos(dist) || !(sigma_bar > 0.0f)) return false;
  float t = 0.0f;
  V3 cp;
  for (uint32_t it = 0;; ++it) {
    if (it >= kStepCap) return false;
    float z = rng.next();
    t = t + (-olog(z)) / sigma_bar;
    if (t >= dist) return false;
    cp = along(pos, dir, t);
    float ext = density(s, cp);
    ++c.lookups;
    float xi = rng.next();
    if (xi < ext / s.max_ext) break;
  }
  pos = cp;
  return true;
}

float ratio_global(const Scene& s, float sigma_bar, V3 pos, V3 ldir, Rng& rng, Counts& c) {
  float tmin, tmax;
  if (!slab(pos, ldir, s.b0, s.b1, tmin, tmax)) return 1.0f;
  float dist = length(sub(along(pos, ldir, tmax), pos));
  if (!finite_pos(dist) || !(sigma_bar > 0.0f)) return 1.0f;
  float t = 0.0f, T = 1.0f;
  for (uint32_t it = 0; it < kStepCap; ++it) {
    t = t + (-olog(rng.next())) / sigma_bar;
    if (t >= dist) break;
    float rho = density(s, along(pos, ldir, t));
    ++c.lookups;
    T = T * (1.0f - rho / s.max_ext);
    if (T < 0.05f) {
      if (rng.next() >= 0.5f) return 0.0f;
      T = T * 2.0f;
    }
  }
  return T;
}

// ---------------------------------------------------------------------------
// DDA over 8^3-voxel majorant cells (Amanatides & Woo); ties x < y < z
// ---------------------------------------------------------------------------

// Set-up by multiplication with the reciprocal direction inv = 1/d and the
// reciprocal cell size ics; the sign test is on d (1/(+-0) is +-inf).
static void dda_axis(float o, float d, float inv, float b0, float cs, int c, int& step, float& tmax, float& tdel) {
  if (d > 0.0f) {
    step = 1;
    tmax = ((b0 + (float)(c + 1) * cs) - o) * inv;
    tdel = cs * inv;
  } else if (d < 0.0f) {
    step = -1;
    tmax = ((b0 + (float)c * cs) - o) * inv;
    tdel = -(cs * inv);
  } else {
    step = 0;
    tmax = INFINITY;
    tdel = INFINITY;
  }
}

static int cell_of(float o, float b0, float ics, int nc) {
  int c = (int)std::floor((o - b0) * ics);
  return c < 0 ? 0 : (c > nc - 1 ? nc - 1 : c);
}

void dda_init(Dda& d, V3 o, V3 dir, V3 b0, V3 cs, V3 ics, const int nc[3]) {
  V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  d.c[0] = cell_of(o.x, b0.x, ics.x, nc[0]);
  d.c[1] = cell_of(o.y, b0.y, ics.y, nc[1]);
  d.c[2] = cell_of(o.z, b0.z, ics.z, nc[2]);
  dda_axis(o.x, dir.x, inv.x, b0.x, cs.x, d.c[0], d.step[0], d.tmax[0], d.tdel[0]);
  dda_axis(o.y, dir.y, inv.y, b0.y, cs.y, d.c[1], d.step[1], d.tmax[1], d.tdel[1]);
  dda_axis(o.z, dir.z, inv.z, b0.z, cs.z, d.c[2], d.step[2], d.tmax[2], d.tdel[2]);
}

float dda_exit(const Dda& d) { return std::fmin(std::fmin(d.tmax[0], d.tmax[1]), d.tmax[2]); }

bool dda_advance(Dda& d, const int nc[3]) {
  int a = (d.tmax[0] <= d.tmax[1] && d.tmax[0] <= d.tmax[2]) ? 0 : (d.tmax[1] <= d.tmax[2] ? 1 : 2);
  d.c[a] += d.step[a];
  d.tmax[a] = d.tmax[a] + d.tdel[a];
  return d.c[a] >= 0 && d.c[a] < nc[a];
}

uint32_t dda_linear(const Dda& d, const int nc[3]) {
  return (uint32_t)d.c[0] + (uint32_t)nc[0] * ((uint32_t)d.c[1] + (uint32_t)nc[1] * (uint32_t)d.c[2]);
}


void track_init(const Scene& s, Track& tr, V3 o, V3 d, Counts& c) {
  float tmin, tmax;
  if (!slab(o, d, s.b0, s.b1, tmin, tmax) || !finite_pos(tmax)) tmax = 0.0f;
  tr.t = 0.0f;
  tr.t_end = tmax;
  dda_init(tr.dda, o, d, s.b0, s.cell, s.icell, s.mnb);
  tr.m = s.maj[dda_linear(tr.dda, s.mnb)];
  ++c.cells;
}

// free flight against piecewise-constant majorants: consume tau = -ln u
bool track_step(const Scene& s, Track& tr, float u, Counts& c) {
  float tau = -olog(u);
  while (true) {
    float e = dda_exit(tr.dda);
    float se = std::fmin(e, tr.t_end);
    float sig = tr.m * s.k;
    float dtau = sig * (se - tr.t);
    if (dtau > tau) {
      tr.t = tr.t + tau / sig;
      return true;
    }
    tau = tau - dtau;
    tr.t = se;
    if (e >= tr.t_end) return false;
    if (!dda_advance(tr.dda, s.mnb)) return false;
    tr.m = s.maj[dda_linear(tr.dda, s.mnb)];
    ++c.cells;
  }
}

const uint32_t kEventCap = 1u << 20;

// One camera path.  Global tracker: PathTracer.comp main (:366-417); DDA
// tracker: the same loop with DDA free flights and ratio-tracking NEE.
V3 trace_path(const Scene& s, const vcr_camera& cam, int x, int y, Rng& rng, Counts& c) {
  V3 pos, dir;
  camera_ray(cam, x, y, pos, dir);
  float tmin, tmax;
  if (!slab(pos, dir, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) return sky(s, dir);
  pos = along(pos, dir, tmax < tmin ? tmax : tmin);
  V3 L = v3(0, 0, 0);
  float beta = 1.0f;
  bool ref = s.rng_mode == 1;
  if (s.tracker == 0) {
    float sigma_bar = (s.max_ext * s.ds) / s.bs;
    uint32_t cap = s.max_events ? s.max_events : kEventCap;
    while (true) {
      if (!find_scatter_global(s, sigma_bar, pos, dir, rng, c)) {
        V3 sk = sky(s, dir);
        L = add(L, scale(sk, beta));
        break;
      }
      ++c.events;
      beta = beta * s.albedo;
      float pdf = hg_pdf(s, dot(neg(dir), s.sun));
      float T = s.nee_mode == 1 ? sv_lookup(s, pos) : ratio_global(s, sigma_bar, pos, neg(s.sun), rng, c);
      float contrib = ((s.light * pdf) * T) * beta;
      L = add(L, v3(contrib, contrib, contrib));
      if (c.events >= cap) break;
      dir = hg_sample(s, dir, rng, !ref);
    }
    return L;
  }
  V3 lsun = neg(s.sun);
  Track tr;
  while (true) {
    track_init(s, tr, pos, dir, c);
    bool hit = false;
    V3 p;
    while (track_step(s, tr, rng.next(), c)) {
      p = along(pos, dir, tr.t);
      float rho = density(s, p);
      ++c.lookups;
      float xi = rng.next();
      if (xi * tr.m < rho) {
        hit = true;
        break;
      }
    }
    if (!hit) {
      V3 sk = sky(s, dir);
      L = add(L, scale(sk, beta));
      break;
    }
    if (c.lookups + c.cells > kPathWorkCap) break;
    pos = p;
    ++c.events;
    if (s.nrc_events && c.events == s.nrc_events) break;  // ends in the radiance cache (added separately)
    beta = beta * s.albedo;
    float phase = hg_pdf(s, dot(neg(dir), s.sun));
    float T = 1.0f;
    track_init(s, tr, pos, lsun, c);
    while (track_step(s, tr, rng.next(), c)) {
      float rho = density(s, along(pos, lsun, tr.t));
      ++c.lookups;
      T = T * (1.0f - rho / tr.m);
      if (T < 0.05f) {
        if (rng.next() >= 0.5f) {
          T = 0.0f;
          break;
        }
        T = T * 2.0f;
      }
    }
    float contrib = ((s.light * phase) * T) * beta;
    L = add(L, v3(contrib, contrib, contrib));
    if (s.max_events && c.events >= s.max_events) break;
    dir = hg_sample(s, dir, rng, true);
  }
  return L;
}

Scene make_scene(const Grid* g, const vcr_cloud& cl, const vcr_params& p, const vcr_shadow_volume* sv, int level,
                 const float* sv_tex) {
  Scene s{};
  s.g = g;
  s.b0 = v3(cl.bounds_min[0], cl.bounds_min[1], cl.bounds_min[2]);
  s.b1 = v3(cl.bounds_max[0], cl.bounds_max[1], cl.bounds_max[2]);
  s.max_ext = cl.max_extinction > 0.0f ? cl.max_extinction : std::fmax(g->max_density, 0.01f);
  s.ds = cl.density_scaling;
  s.bs = cl.base_scaling;
  s.k = cl.density_scaling / cl.base_scaling;
  V3 ext = sub(s.b1, s.b0);
  const float cv = (float)(8 << level);  // voxels per majorant cell
  s.cell = v3((ext.x / (float)g->n[0]) * cv, (ext.y / (float)g->n[1]) * cv, (ext.z / (float)g->n[2]) * cv);
  s.icell = v3(1.0f / s.cell.x, 1.0f / s.cell.y, 1.0f / s.cell.z);
  s.iext = v3(1.0f / ext.x, 1.0f / ext.y, 1.0f / ext.z);
  s.maj = g->lv[level].data();
  for (int a = 0; a < 3; ++a) s.mnb[a] = g->lnb[level][a];
  s.g_ = p.phase_g;
  s.opg2 = p.phase_one_plus_g2;
  s.omg2 = p.phase_one_minus_g2;
  s.o2g = p.phase_one_over_2g;
  s.iso = p.isotropic != 0;
  s.albedo = p.albedo;
  s.light = p.light_intensity;
  s.sun = v3(p.sun_dir[0], p.sun_dir[1], p.sun_dir[2]);
  s.sky = v3(p.sky[0], p.sky[1], p.sky[2]);
  s.sky_mode = p.sky_mode;
  s.rng_mode = p.rng_mode;
  s.nee_mode = p.nee_mode;
  s.tracker = p.tracker;
  s.max_events = p.max_events;
  s.nrc_events = p.nrc_events;
  if (sv && sv_tex) {
    s.sv_tex = sv_tex;
    s.sv_n = (int)sv->voxel_axis_count;
    s.sv_b0 = v3(sv->bounds_min[0], sv->bounds_min[1], sv->bounds_min[2]);
    for (int i = 0; i < 9; ++i) s.B[i] = sv->basis_change[i];
    V3 e = sub(v3(sv->bounds_max[0], sv->bounds_max[1], sv->bounds_max[2]), s.sv_b0);
    s.sv_ext = v3((s.B[0] * e.x + s.B[1] * e.y) + s.B[2] * e.z, (s.B[3] * e.x + s.B[4] * e.y) + s.B[5] * e.z,
                  (s.B[6] * e.x + s.B[7] * e.y) + s.B[8] * e.z);
  }
  return s;
}

// ---------------------------------------------------------------------------
// fBm (same formulas as the product generator, restated)
// ---------------------------------------------------------------------------
static float fade(float t) { return ((t * t) * t) * ((t * ((t * 6.0f) - 15.0f)) + 10.0f); }
static float grad(uint32_t h, float x, float y, float z) {
  h &= 15u;
  float u = h < 8u ? x : y;
  float v = h < 4u ? y : ((h == 12u || h == 14u) ? x : z);
  return ((h & 1u) == 0u ? u : -u) + ((h & 2u) == 0u ? v : -v);
}
static float lerp(float t, float a, float b) { return std::fma(t, b - a, a); }

static float perlin(const uint8_t* P, float x, float y, float z) {
  float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  uint32_t X = (uint32_t)(int)fx & 255u, Y = (uint32_t)(int)fy & 255u, Z = (uint32_t)(int)fz & 255u;
  x -= fx;
  y -= fy;
  z -= fz;
  float u = fade(x), v = fade(y), w = fade(z);
  auto p = [&](uint32_t i) { return (uint32_t)P[i & 255u]; };
  uint32_t A = p(X) + Y, AA = p(A) + Z, AB = p(A + 1) + Z, B = p(X + 1) + Y, BA = p(B) + Z, BB = p(B + 1) + Z;
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float r0 = lerp(v, lerp(u, grad(p(AA), x, y, z), grad(p(BA), x1, y, z)),
                  lerp(u, grad(p(AB), x, y1, z), grad(p(BB), x1, y1, z)));
  float r1 = lerp(v, lerp(u, grad(p(AA + 1), x, y, z1), grad(p(BA + 1), x1, y, z1)),
                  lerp(u, grad(p(AB + 1), x, y1, z1), grad(p(BB + 1), x1, y1, z1)));
  return lerp(w, r0, r1);
}

void fbm_perm(uint64_t seed, uint8_t perm[256]) {
  for (int i = 0; i < 256; ++i) perm[i] = (uint8_t)i;
  uint64_t s = seed;
  for (int i = 255; i > 0; --i) {
    s += 0x9E3779B97F4A7C15ull;  // splitmix64
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    uint64_t j = z % (uint64_t)(i + 1);
    std::swap(perm[i], perm[j]);
  }
}

float fbm_voxel(const uint8_t* perm, const uint32_t n[3], uint32_t oct, float lac, float gain, float f0, uint32_t i,
                uint32_t j, uint32_t k) {
  uint32_t nmax = std::max(std::max(n[0], n[1]), n[2]);
  float fn = (float)nmax;
  float qx = ((float)i + 0.5f) / fn, qy = ((float)j + 0.5f) / fn, qz = ((float)k + 0.5f) / fn;
  float sum = 0.0f, norm = 0.0f, amp = 1.0f, freq = f0;
  for (uint32_t o = 0; o < oct; ++o) {
    sum = std::fma(amp, perlin(perm, qx * freq, qy * freq, qz * freq), sum);
    norm = norm + amp;
    amp = amp * gain;
    freq = freq * lac;
  }
  float nz = sum / norm;
  float hx = ((float)n[0] * 0.5f) / fn, hy = ((float)n[1] * 0.5f) / fn, hz = ((float)n[2] * 0.5f) / fn;
  float dx = (qx - hx) / hx, dy = (qy - hy) / hy, dz = (qz - hz) / hz;
  float r = std::sqrt((dx * dx + dy * dy) + dz * dz);
  float fall = clampf(1.0f - r, 0.0f, 1.0f);
  return clampf((3.0f * fall) * (1.0f + 4.0f * nz), 0.0f, 1.0f);
}

}  // namespace oracle

// ===========================================================================
// C entry points (loaded by the tests through ctypes)
// ===========================================================================
using namespace oracle;

extern "C" {

void* oracle_grid_new(const uint32_t size[3], const float* dense, int precision) {
  return grid_new(size, dense, precision);
}
void oracle_grid_free(void* h) { delete static_cast<Grid*>(h); }
float oracle_grid_max(void* h) { return static_cast<Grid*>(h)->max_density; }
void oracle_grid_majorants(void* h, int level, float* out) {
  Grid* g = static_cast<Grid*>(h);
  std::copy(g->lv[level].begin(), g->lv[level].end(), out);
}
void oracle_grid_decoded(void* h, float* out) {
  Grid* g = static_cast<Grid*>(h);
  std::copy(g->tex.begin(), g->tex.end(), out);
}

// ---- single functions, for checks against the reference's shader code run
// on the CPU (oracle/ref_shaders.cpp) ----------------------------------------
void oracle_sky_gradient(const float dir[3], float out[3]) {
  V3 c = sky_gradient(v3(dir[0], dir[1], dir[2]));
  out[0] = c.x; out[1] = c.y; out[2] = c.z;
}

int oracle_slab(const float b0[3], const float b1[3], const float pos[3], const float dir[3], float* tmin,
                float* tmax) {
  return slab(v3(pos[0], pos[1], pos[2]), v3(dir[0], dir[1], dir[2]), v3(b0[0], b0[1], b0[2]), v3(b1[0], b1[1], b1[2]),
              *tmin, *tmax) ? 1 : 0;
}

void oracle_onb(const float n[3], float xp[3], float yp[3]) {
  V3 a, b;
  onb(v3(n[0], n[1], n[2]), a, b);
  xp[0] = a.x; xp[1] = a.y; xp[2] = a.z;
  yp[0] = b.x; yp[1] = b.y; yp[2] = b.z;
}

void oracle_camera_ray(const vcr_camera* cam, int x, int y, float pos[3], float dir[3]) {
  V3 p, d;
  camera_ray(*cam, x, y, p, d);
  pos[0] = p.x; pos[1] = p.y; pos[2] = p.z;
  dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
}

// The reference-parity RNG: the state after initializeRandom(seed), and n
// numbers from a state (returning the state after them).
uint32_t oracle_xorshift_init(uint32_t seed) { return rng_xorshift(seed).s; }
uint32_t oracle_xorshift_numbers(uint32_t state, uint32_t n, float* out) {
  Rng r{state, true};
  for (uint32_t i = 0; i < n; ++i) out[i] = r.next();
  return r.s;
}

// One scattering direction as the reference-parity path draws it (no
// renormalisation) from the xorshift state *state.
void oracle_hg_sample_xorshift(const vcr_params* p, const float in[3], uint32_t* state, float out[3]) {
  Scene s{};
  s.g_ = p->phase_g;
  s.opg2 = p->phase_one_plus_g2;
  s.omg2 = p->phase_one_minus_g2;
  s.o2g = p->phase_one_over_2g;
  s.iso = p->isotropic != 0;
  Rng rng{*state, true};
  V3 o = hg_sample(s, v3(in[0], in[1], in[2]), rng, false);
  out[0] = o.x; out[1] = o.y; out[2] = o.z;
  *state = rng.s;
}

// find_scatter_global from (pos, dir) with the xorshift state *state.
int oracle_find_scatter_global(void* h, const vcr_cloud* cl, float pos[3], const float dir[3], uint32_t* state) {
  vcr_params p{};
  Scene s = make_scene(static_cast<Grid*>(h), *cl, p, nullptr, 0, nullptr);
  const float sigma_bar = (s.max_ext * s.ds) / s.bs;
  Rng rng{*state, true};
  Counts c;
  V3 q = v3(pos[0], pos[1], pos[2]);
  const bool hit = find_scatter_global(s, sigma_bar, q, v3(dir[0], dir[1], dir[2]), rng, c);
  pos[0] = q.x; pos[1] = q.y; pos[2] = q.z;
  *state = rng.s;
  return hit ? 1 : 0;
}

float oracle_sv_lookup(void* h, const vcr_cloud* cl, const vcr_shadow_volume* sv, const float* sv_tex,
                       const float pos[3]) {
  vcr_params p{};
  Scene s = make_scene(static_cast<Grid*>(h), *cl, p, sv, 0, sv_tex);
  return sv_lookup(s, v3(pos[0], pos[1], pos[2]));
}

// The phase function alone (hg_pdf / hg_sample above, as the tracker calls
// them): its density at n cosines, and m directions scattered from `in`,
// sample i drawn from the stream rng_pcg(seed, i, 0).
void oracle_hg(const vcr_params* p, const float* cosines, uint32_t n, float* pdf, const float in[3], uint32_t seed,
               uint32_t m, float* dirs) {
  Scene s{};
  s.g_ = p->phase_g;
  s.opg2 = p->phase_one_plus_g2;
  s.omg2 = p->phase_one_minus_g2;
  s.o2g = p->phase_one_over_2g;
  s.iso = p->isotropic != 0;
  for (uint32_t i = 0; i < n; ++i) pdf[i] = hg_pdf(s, cosines[i]);
  const V3 d = v3(in[0], in[1], in[2]);
  for (uint32_t i = 0; i < m; ++i) {
    Rng rng = rng_pcg(seed, i, 0u);
    V3 o = hg_sample(s, d, rng, true);
    dirs[3 * i] = o.x;
    dirs[3 * i + 1] = o.y;
    dirs[3 * i + 2] = o.z;
  }
}

void oracle_grid_sample(void* h, const vcr_cloud* cl, const float* pos, uint32_t n, float* out) {
  vcr_params p{};
  Scene s = make_scene(static_cast<Grid*>(h), *cl, p, nullptr, 0, nullptr);
  for (uint32_t i = 0; i < n; ++i) out[i] = density(s, v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
}

void oracle_dda_trace(void* h, const vcr_cloud* cl, int level, const float* o, const float* d, uint32_t n, uint32_t max_cells,
                      uint32_t* cells, float* tt, uint32_t* count) {
  vcr_params p{};
  Scene s = make_scene(static_cast<Grid*>(h), *cl, p, nullptr, level, nullptr);
  const int* nc = s.mnb;
  for (uint32_t i = 0; i < n; ++i) {
    V3 org = v3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    V3 dir = v3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    float tmin, tmax;
    uint32_t k = 0;
    if (slab(org, dir, s.b0, s.b1, tmin, tmax) && tmax >= 0.0f) {
      if (tmin > 0.0f) {
        org = along(org, dir, tmin);
        slab(org, dir, s.b0, s.b1, tmin, tmax);
      }
      Dda dd;
      dda_init(dd, org, dir, s.b0, s.cell, s.icell, nc);
      float t = 0.0f;
      while (k < max_cells) {
        float e = dda_exit(dd);
        float se = std::fmin(e, tmax);
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
}

// One progressive pass over the crop: adds spp paths per pixel into sum
// (float64 RGB, W*H*3) and writes stats (uint32 x4: events, lookups, pass, cells).
int oracle_pt_pass(void* h, int level, const vcr_cloud* cl, const vcr_camera* cam, const vcr_params* prm,
                   const vcr_shadow_volume* sv, const float* sv_tex, uint32_t width, uint32_t height,
                   const vcr_pass_desc* pass, double* sum, uint32_t* stats, int threads) {
  Scene s = make_scene(static_cast<Grid*>(h), *cl, *prm, sv, level, sv_tex);
  uint32_t x0 = pass->crop[0], y0 = pass->crop[1];
  uint32_t cw = pass->crop[2] ? pass->crop[2] : width, ch = pass->crop[2] ? pass->crop[3] : height;
  uint32_t spp = pass->spp ? pass->spp : 1;
  uint32_t padded_w = 32u * (width / 32u + 1u);
  bool ref = prm->rng_mode == 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
  for (int64_t row = 0; row < (int64_t)ch; ++row) {
    for (uint32_t cx = 0; cx < cw; ++cx) {
      int x = (int)(x0 + cx), y = (int)(y0 + (uint32_t)row);
      uint32_t pix = (uint32_t)y * width + (uint32_t)x;
      double Ls[3] = {0.0, 0.0, 0.0};  // every sample is added in FP64, as the GPU does
      Counts c;
      for (uint32_t sp = 0; sp < spp; ++sp) {
        Rng rng = ref ? rng_xorshift(pass->seed * ((uint32_t)x + (uint32_t)y * padded_w))
                      : rng_pcg(pass->seed, pix * spp + sp, pass->pass_index);
        Counts cs;
        V3 L = trace_path(s, *cam, x, y, rng, cs);
        Ls[0] += (double)L.x;
        Ls[1] += (double)L.y;
        Ls[2] += (double)L.z;
        if (sp == 0 || s.tracker == 0) {
          c.events += cs.events;
          c.lookups += cs.lookups;
          c.cells += cs.cells;
        }
      }
      double* o = sum + 3 * (size_t)pix;
      if (pass->flags & VCR_PASS_NO_ACCUMULATE) {
        o[0] = Ls[0]; o[1] = Ls[1]; o[2] = Ls[2];
      } else {
        o[0] += Ls[0]; o[1] += Ls[1]; o[2] += Ls[2];
      }
      if (stats) {
        uint32_t* st = stats + 4 * (size_t)pix;
        st[0] = c.events;
        st[1] = c.lookups;
        st[2] = pass->pass_index;
        st[3] = s.tracker == 0 ? 1u : c.cells;
      }
    }
  }
  return 0;
}

// ShadowVolume.comp:77-93: one column per (x, y), z marching along the light.
void oracle_sv_build(void* h, const vcr_cloud* cl, const vcr_shadow_volume* sv, float* out) {
  vcr_params p{};
  Scene s = make_scene(static_cast<Grid*>(h), *cl, p, nullptr, 0, nullptr);
  uint32_t n = sv->voxel_axis_count;
  V3 b0 = v3(sv->bounds_min[0], sv->bounds_min[1], sv->bounds_min[2]);
  V3 R = v3(sv->right[0], sv->right[1], sv->right[2]), U = v3(sv->up[0], sv->up[1], sv->up[2]),
     Ld = v3(sv->light_dir[0], sv->light_dir[1], sv->light_dir[2]);
  float vs = sv->voxel_size;
  size_t plane = (size_t)n * n;
  for (uint32_t y = 0; y < n; ++y)
    for (uint32_t x = 0; x < n; ++x) {
      float acc = 0.0f, dist = 0.0f;
      for (uint32_t z = 0; z < n; ++z) {
        float fx = (float)x * vs, fy = (float)y * vs, fz = (float)z * vs;
        V3 pp = v3(((b0.x + fx * R.x) + fy * U.x) + fz * Ld.x, ((b0.y + fx * R.y) + fy * U.y) + fz * Ld.y,
                   ((b0.z + fx * R.z) + fy * U.z) + fz * Ld.z);
        if (in_box(pp, s.b0, s.b1)) acc = acc + (density(s, pp) * s.ds) / s.bs;
        dist = dist + vs;
        out[(size_t)x + (size_t)n * y + plane * z] = oexp(((-dist) * acc) / (float)(z + 1));
      }
    }
}

void oracle_fbm_fill(const uint32_t n[3], uint64_t seed, uint32_t octaves, float lac, float gain, float f0, float* out,
                     int threads) {
  uint8_t perm[256];
  fbm_perm(seed, perm);
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1)
  for (int64_t k = 0; k < (int64_t)n[2]; ++k)
    for (uint32_t j = 0; j < n[1]; ++j)
      for (uint32_t i = 0; i < n[0]; ++i)
        out[(size_t)i + (size_t)n[0] * ((size_t)j + (size_t)n[1] * (size_t)k)] =
            fbm_voxel(perm, n, octaves, lac, gain, f0, i, j, (uint32_t)k);
}

// Display image (the blit of RenderTechniquePT.cpp:143-167 into an sRGB
// swapchain, VulkanSwapchain.cpp:72): mean = float(sum * inv), times
// exposure, clamped to [0, 1], sRGB-encoded, rounded to 8 bits; alpha 255;
// order 0 writes R G B A bytes, 1 writes B G R A.
void oracle_display(const double* sum, size_t npx, double inv, float exposure, uint32_t order, uint32_t* out) {
  for (size_t p = 0; p < npx; ++p) {
    uint32_t q[3];
    for (int c = 0; c < 3; ++c) {
      float v = (float)(sum[3 * p + c] * inv) * exposure;
      v = std::fmin(std::fmax(v, 0.0f), 1.0f);
      q[c] = (uint32_t)(osrgb_encode(v) * 255.0f + 0.5f);
    }
    const uint32_t r = order ? q[2] : q[0], b = order ? q[0] : q[2];
    out[p] = r | (q[1] << 8) | (b << 16) | (255u << 24);
  }
}
float oracle_srgb_encode(float v) { return osrgb_encode(v); }

float oracle_log(float x) { return olog(x); }
float oracle_exp(float x) { return oexp(x); }
void oracle_sincos2pi(float u, float* s, float* c) { osincos2pi(u, s, c); }
uint32_t oracle_pcg_hash(uint32_t v) { return pcg_hash(v); }
uint16_t oracle_f32_to_f16(float f) { return f32_to_f16(f); }
uint16_t oracle_f32_to_bf16(float f) { return f32_to_bf16(f); }

}  // extern "C"
