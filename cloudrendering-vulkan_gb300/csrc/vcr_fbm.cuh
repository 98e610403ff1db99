// Seeded Perlin-fBm cloud density, the synthetic stand-in for the
// reference's .xyz cloud files (main.cpp:100, models/ is empty).
//
// noise  : Perlin's improved gradient noise (Perlin, "Improving Noise",
//          SIGGRAPH 2002): 256-entry permutation, fade 6t^5-15t^4+10t^3,
//          12 cube-edge gradients.
// fbm    : sum_o gain^o * noise(f0 * lacunarity^o * q) / sum_o gain^o.
// density: clamp(3 falloff (1 + 4 fbm), 0, 1), falloff = clamp(1 - |d|, 0, 1)
//          with d the voxel centre relative to the grid centre, divided by
//          the half extent per axis (an ellipsoid filling the box).
// q is the voxel centre ((i + 1/2)/N_max, ...), N_max the longest axis.
#pragma once

#include "vcr_math.cuh"

namespace vcr {

struct FbmConst {
  uint8_t perm[256];
  uint32_t n[3];
  uint32_t octaves;
  float lacunarity, gain, f0;
};

VCR_HD float fbm_fade(float t) { return ((t * t) * t) * ((t * ((t * 6.0f) - 15.0f)) + 10.0f); }

VCR_HD float fbm_grad(uint32_t h, float x, float y, float z) {
  h &= 15u;
  float u = h < 8u ? x : y;
  float v = h < 4u ? y : ((h == 12u || h == 14u) ? x : z);
  return ((h & 1u) == 0u ? u : -u) + ((h & 2u) == 0u ? v : -v);
}

VCR_HD float fbm_lerp(float t, float a, float b) { return fmaf(t, b - a, a); }

VCR_HD float perlin(const uint8_t* P, float x, float y, float z) {
  float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  uint32_t X = (uint32_t)(int)fx & 255u, Y = (uint32_t)(int)fy & 255u, Z = (uint32_t)(int)fz & 255u;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  float u = fbm_fade(x), v = fbm_fade(y), w = fbm_fade(z);
#define VCR_P(i) ((uint32_t)P[(i) & 255u])
  uint32_t A = VCR_P(X) + Y, AA = VCR_P(A) + Z, AB = VCR_P(A + 1u) + Z;
  uint32_t B = VCR_P(X + 1u) + Y, BA = VCR_P(B) + Z, BB = VCR_P(B + 1u) + Z;
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float r0 = fbm_lerp(v, fbm_lerp(u, fbm_grad(VCR_P(AA), x, y, z), fbm_grad(VCR_P(BA), x1, y, z)),
                      fbm_lerp(u, fbm_grad(VCR_P(AB), x, y1, z), fbm_grad(VCR_P(BB), x1, y1, z)));
  float r1 = fbm_lerp(v, fbm_lerp(u, fbm_grad(VCR_P(AA + 1u), x, y, z1), fbm_grad(VCR_P(BA + 1u), x1, y, z1)),
                      fbm_lerp(u, fbm_grad(VCR_P(AB + 1u), x, y1, z1), fbm_grad(VCR_P(BB + 1u), x1, y1, z1)));
#undef VCR_P
  return fbm_lerp(w, r0, r1);
}

VCR_HD float fbm_density(const FbmConst& c, uint32_t i, uint32_t j, uint32_t k) {
  uint32_t nmax = c.n[0] > c.n[1] ? c.n[0] : c.n[1];
  nmax = nmax > c.n[2] ? nmax : c.n[2];
  float fn = (float)nmax;
  float qx = ((float)i + 0.5f) / fn, qy = ((float)j + 0.5f) / fn, qz = ((float)k + 0.5f) / fn;
  float sum = 0.0f, norm = 0.0f, amp = 1.0f, freq = c.f0;
  for (uint32_t o = 0; o < c.octaves; ++o) {
    sum = fmaf(amp, perlin(c.perm, qx * freq, qy * freq, qz * freq), sum);
    norm = norm + amp;
    amp = amp * c.gain;
    freq = freq * c.lacunarity;
  }
  float n = sum / norm;
  float hx = ((float)c.n[0] * 0.5f) / fn, hy = ((float)c.n[1] * 0.5f) / fn, hz = ((float)c.n[2] * 0.5f) / fn;
  float dx = (qx - hx) / hx, dy = (qy - hy) / hy, dz = (qz - hz) / hz;
  float r = sqrtf((dx * dx + dy * dy) + dz * dz);
  float fall = clampf(1.0f - r, 0.0f, 1.0f);
  return clampf((3.0f * fall) * (1.0f + 4.0f * n), 0.0f, 1.0f);
}

// splitmix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) driving a Fisher-Yates shuffle of 0..255.
inline uint64_t splitmix64(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline void fbm_make_perm(uint64_t seed, uint8_t perm[256]) {
  for (int i = 0; i < 256; ++i) perm[i] = (uint8_t)i;
  uint64_t s = seed;
  for (int i = 255; i > 0; --i) {
    uint64_t j = splitmix64(s) % (uint64_t)(i + 1);
    uint8_t t = perm[i];
    perm[i] = perm[j];
    perm[j] = t;
  }
}

}  // namespace vcr
