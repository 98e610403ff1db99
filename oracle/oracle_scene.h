// ORACLE — test infrastructure only (see oracle_math.h).  Scene, grid and
// tracking pieces of the CPU restatement shared by its translation units
// (path tracing in oracle_pt.cpp, photon beams in oracle_ppb.cpp, photon
// mapping in oracle_ppm.cpp).
#pragma once

#include <cstdint>
#include <vector>

#include "../include/vcr/abi.h"
#include "oracle_math.h"

namespace oracle {

// Decoded texels (what the GPU reads back from its bricks) + the majorant
// pyramid.
struct Grid {
  int n[3];
  int nb[3];
  std::vector<float> tex;    // decoded, x fastest
  std::vector<float> maj;    // per 8^3 brick, halo included (pyramid level 0)
  std::vector<float> lv[4];  // pyramid: level l+1 = max over 2x2x2 cells of level l
  int lnb[4][3];
  float max_density = 0.0f;

  float at(int i, int j, int k) const { return tex[(size_t)i + (size_t)n[0] * ((size_t)j + (size_t)n[1] * k)]; }
};

struct Scene {
  const Grid* g;
  const float* maj;  // majorants of the selected pyramid level
  int mnb[3];
  V3 b0, b1;
  float max_ext, ds, bs, k;
  V3 cell;
  V3 icell;  // 1 / cell
  V3 iext;   // 1 / (b1 - b0)
  float g_, opg2, omg2, o2g;  // Parameters (UniformBuffers.h:80-112)
  bool iso;
  float albedo, light;
  V3 sun, sky;
  uint32_t sky_mode, rng_mode, nee_mode, tracker, max_events;
  uint32_t nrc_events = 0;  // > 0: paths end at this event (radiance cache)
  const float* sv_tex = nullptr;  // shadow volume (reference-parity NEE)
  int sv_n = 0;
  V3 sv_b0, sv_ext;
  float B[9];
};

struct Counts {
  uint32_t events = 0, lookups = 0, cells = 0;
};

// Loop guards, identical to the kernels': a non-finite exit distance counts
// as an immediate exit and step counts are capped.
const uint32_t kStepCap = 1u << 24;
const uint32_t kPathWorkCap = 1u << 26;
inline bool finite_pos(float v) { return v >= 0.0f && v <= 3.0e38f; }

struct Dda {
  int c[3], step[3];
  float tmax[3], tdel[3];
};

struct Track {
  Dda dda;
  float t, t_end, m;
};

Grid* grid_new(const uint32_t size[3], const float* dense, int precision);
Scene make_scene(const Grid* g, const vcr_cloud& cl, const vcr_params& p, const vcr_shadow_volume* sv, int level,
                 const float* sv_tex);
float density(const Scene& s, V3 p);
bool slab(V3 pos, V3 dir, V3 b0, V3 b1, float& tmin, float& tmax);
V3 sky(const Scene& s, V3 dir);
float hg_pdf(const Scene& s, float c);
float sv_lookup(const Scene& s, V3 p);  // sampleShadowVolume (PathTracer.comp:121-127)
V3 hg_sample(const Scene& s, V3 in, Rng& rng, bool renorm);
void camera_ray(const vcr_camera& c, int x, int y, V3& pos, V3& dir);
void track_init(const Scene& s, Track& tr, V3 o, V3 d, Counts& c);
bool track_step(const Scene& s, Track& tr, float u, Counts& c);

// One delta-tracking free flight from o along unit d (DDA majorants): true
// with the distance of the first real collision, false on escape (t =
// distance to the box exit).
inline bool free_flight(const Scene& s, V3 o, V3 d, Rng& rng, float& t, Counts& c) {
  Track tr;
  track_init(s, tr, o, d, c);
  while (true) {
    if (!track_step(s, tr, rng.next(), c)) {
      t = tr.t_end;
      return false;
    }
    float rho = density(s, along(o, d, tr.t));
    ++c.lookups;
    if (rng.next() * tr.m < rho) {
      t = tr.t;
      return true;
    }
    if (c.lookups + c.cells > kPathWorkCap) {
      t = tr.t_end;
      return false;
    }
  }
}

}  // namespace oracle
