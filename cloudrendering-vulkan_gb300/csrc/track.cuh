// DDA free-flight tracking over a majorant pyramid level, shared by the
// path tracer, the photon-beam emitter and the photon emitter.
#pragma once

#include "pt_common.cuh"

namespace vcr {

struct Track {
  Dda dda;
  float t, t_end, m;
};

__device__ __forceinline__ void track_init(Track& tr, const GridView& g, const SceneView& s, const float* maj, f3 o,
                                           f3 d, uint32_t& cells) {
  float tmin, tmax;
  const f3 inv = recip(d);
  if (!slab_inv(o, inv, s.b0, s.b1, tmin, tmax) || !finite_pos(tmax)) tmax = 0.0f;
  tr.t = 0.0f;
  tr.t_end = tmax;
  dda_init(tr.dda, o, d, inv, s.b0, s.cell, s.icell, g.mnb);
  tr.m = maj[dda_linear(tr.dda, g.mnb)];
  ++cells;
}

enum : int { kPending = 0, kCandidate = 1, kExit = 2 };

// Up to `steps` cells of one free flight: consume the optical depth `tau`
// cell by cell (dtau = (m k)(min(exit, t_end) - t)); a tentative collision
// lands at t + tau/(m k) inside the cell where tau runs out.
__device__ __forceinline__ int track_walk(Track& tr, const GridView& g, const float* maj, float k, float& tau,
                                          uint32_t& cells, uint32_t steps) {
  for (uint32_t i = 0; i < steps; ++i) {
    float e = dda_cell_exit(tr.dda);
    float se = fminf(e, tr.t_end);
    float sig = tr.m * k;
    float dtau = sig * (se - tr.t);
    if (dtau > tau) {
      tr.t = tr.t + tau / sig;
      return kCandidate;
    }
    tau = tau - dtau;
    tr.t = se;
    if (e >= tr.t_end) return kExit;
    if (!dda_advance(tr.dda, g.mnb)) return kExit;
    tr.m = maj[dda_linear(tr.dda, g.mnb)];
    ++cells;
  }
  return kPending;
}

// One delta-tracking free flight from o along unit d (DDA majorants):
// true with the distance t of the first real collision, false on escape
// (t = distance to the box exit).  Draw order: per tentative collision one
// uniform for the optical depth, then one for the acceptance test.
__device__ __forceinline__ bool free_flight(const GridView& g, const SceneView& s, f3 o, f3 d, Rng& rng, float& t,
                                            uint32_t& lookups, uint32_t& cells) {
  Track tr;
  track_init(tr, g, s, g.majorants, o, d, cells);
  while (true) {
    float tau = -vlog(rng_next(rng));
    if (track_walk(tr, g, g.majorants, s.k_sigma, tau, cells, 0xFFFFFFFFu) != kCandidate) {
      t = tr.t_end;
      return false;
    }
    float rho = density_at(g, s, along(o, d, tr.t));
    ++lookups;
    if (rng_next(rng) * tr.m < rho) {  // xi < rho / m without the division
      t = tr.t;
      return true;
    }
    if (lookups + cells > kPathWorkCap) {  // runaway guard (non-finite input)
      t = tr.t_end;
      return false;
    }
  }
}

}  // namespace vcr
