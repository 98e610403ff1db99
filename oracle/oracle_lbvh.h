// ORACLE — test infrastructure only (see oracle_math.h).  Binary radix tree
// pieces shared by the photon-beam and photon-map restatements.
#pragma once

#include <cstdint>
#include <vector>

namespace oracle {

struct F4 {
  float x, y, z, w;
};

const uint32_t kLeafBit = 0x80000000u;

uint32_t expand10(uint32_t v);
void lbvh_build(const uint32_t* keys, int n, uint32_t* left, uint32_t* right);
void segment_box(F4 A, F4 B, F4& lo, F4& hi);
void refit(uint32_t node, const uint32_t* left, const uint32_t* right, const std::vector<F4>& llo,
           const std::vector<F4>& lhi, std::vector<F4>& nlo, std::vector<F4>& nhi);

}  // namespace oracle
