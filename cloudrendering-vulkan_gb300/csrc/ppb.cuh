// Photon-beam state owned by a context (RenderTechniquePPB's buffers:
// photon beams, beam data, LBVH, histograms — RenderTechniquePPB.h:100-104).
#pragma once

#include "vcr_internal.h"

namespace vcr {

constexpr int kBeamDists = 16;             // BEAM_TRANSMITTANCE_SAMPLES (PPB_PT.comp, PPB_PE.comp:31)
// A transmittance distance whose free flight left the box: beyond every point
// of the beam or camera ray, whatever the rounding of the box exit.
constexpr float kEscaped = 3.0e38f;
constexpr int kSlotFloats = 28;            // start 3, dir 3, length, power 3, 16 distances, 2 pad
constexpr uint32_t kMaxBeamsPerPhoton = 65;  // 64 scatter events + the entering beam
constexpr uint32_t kMaxSegPerBeam = 4096;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kGatherStack = 64;
constexpr uint32_t kEmitSalt = 0x85EBCA6Bu;
constexpr uint32_t kGatherSalt = 0xC2B2AE35u;

struct PpbState {
  vcr_ppb_params prm{};
  uint32_t K = 0;  // beam slots per photon
  float radius = 0.0f;
  uint32_t segments = 0, dropped = 0;
  float* slots = nullptr;
  uint32_t *nbeams = nullptr, *slot_segs = nullptr, *slot_off = nullptr, *photon_segs = nullptr,
           *photon_off = nullptr, *scan_sums = nullptr, *total = nullptr;
  float4 *seg_a = nullptr, *seg_b = nullptr;
  // the segments again in the LBVH's leaf (Morton) order, for the gather:
  // leaf i's segment is at i, loaded together with the leaf's box
  float4 *leaf_a = nullptr, *leaf_b = nullptr;
  uint32_t* leaf_beam = nullptr;
  uint32_t *seg_beam = nullptr, *codes = nullptr, *idx = nullptr, *codes_sorted = nullptr, *idx_sorted = nullptr;
  uint32_t *left = nullptr, *right = nullptr, *parent_int = nullptr, *parent_leaf = nullptr, *flags = nullptr;
  float4 *leaf_lo = nullptr, *leaf_hi = nullptr, *node_lo = nullptr, *node_hi = nullptr;
  float4* node_pk = nullptr;  // internal nodes packed for the gather: (lo, left), (hi, right)
  float4* node2 = nullptr;    // per internal node: its packed node and its two children's (6 float4)
  GatherProbe gather;  // segments the last gather evaluated, its device time
};

// Spread the low 10 bits of v so two zeros separate each bit (Karras 2012;
// the reference's 8-bit expandBits is PPB_PT.comp:319-325).
__device__ __forceinline__ uint32_t morton_expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

}  // namespace vcr
