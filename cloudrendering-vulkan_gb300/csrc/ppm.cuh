// Photon-map state owned by a context (RenderTechniquePPM's photon map and
// collision map, RenderTechniquePPM.cpp:115-156, plus per-pixel statistics).
#pragma once

#include "vcr_internal.h"

namespace vcr {

constexpr uint32_t kPpmMaxEvents = 64;  // deposits per photon path (uid = photon * 64 + event)
constexpr uint32_t kPpmEmitSalt = 0x27D4EB2Fu;
constexpr uint32_t kPpmGatherSalt = 0x165667B1u;

struct PpmState {
  vcr_ppm_params prm{};
  size_t pixels = 0;
  uint32_t photons_stored = 0, dropped = 0;
  float4 *pos = nullptr, *pw = nullptr, *dir = nullptr;
  uint32_t *uid = nullptr, *count = nullptr, *by_uid = nullptr, *uid_sorted = nullptr, *codes = nullptr,
           *idx = nullptr, *codes_sorted = nullptr, *order = nullptr, *iota = nullptr;
  uint32_t *left = nullptr, *right = nullptr, *parent_int = nullptr, *parent_leaf = nullptr, *flags = nullptr;
  float4 *leaf_lo = nullptr, *leaf_hi = nullptr, *node_lo = nullptr, *node_hi = nullptr;
  float4* node_pk = nullptr;   // internal nodes packed for the gather: (lo, left), (hi, right)
  float4* leaf_pw = nullptr;   // photon powers in leaf order
  float4* leaf_dir = nullptr;  // photon directions in leaf order
  double* stats = nullptr;  // per pixel: N, R, tau rgb, background rgb
  GatherProbe gather;       // photons the last gather tested, its device time
};

}  // namespace vcr
