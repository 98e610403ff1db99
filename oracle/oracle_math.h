// ORACLE — test infrastructure only.  A CPU restatement of the reference's
// shader arithmetic, used as the checker by tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg.  Nothing in the shipped library includes,
// links or calls this code.
//
// Parity status: the reference's render path is GLSL run through Vulkan,
// which cannot run here (no graphics stack), so no reference output pins
// these formulas ("parity unpinned" for the shader math).  What is pinned:
// the radix-sort fixture of Tests.cpp:113-131 and the closed-form checks in
// tests/test_oracle.py.
//
// Float semantics (shared with the CUDA kernels by specification, not by
// code): compiled with -ffp-contract=off; every FMA is an explicit std::fma;
// log / exp / sin / cos are the series below, not libm.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 scale(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 vdiv(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) {
  float l = std::sqrt(dot(a, a));
  return V3{a.x / l, a.y / l, a.z / l};
}
// p + t*d, per component, two roundings (GLSL `ray.pos + t * ray.dir`)
inline V3 along(V3 p, V3 d, float t) { return V3{p.x + t * d.x, p.y + t * d.y, p.z + t * d.z}; }
inline float clampf(float v, float lo, float hi) { return std::fmin(std::fmax(v, lo), hi); }

inline uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline float from_bits(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

const float kPI = 3.14159265359f;  // PathTracer.comp:18
const float kINV_4PI = 0.0795774715f;

// ln x: x = 2^e m, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1))
// summed to the s^9 term.
inline float olog(float x) {
  if (!(x > 0.0f)) return -INFINITY;
  uint32_t b = bits(x);
  int e = (int)(b >> 23) - 127;
  float m = from_bits((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e = e + 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = 0.222222222f;
  p = std::fma(p, s2, 0.285714286f);
  p = std::fma(p, s2, 0.4f);
  p = std::fma(p, s2, 0.666666667f);
  p = std::fma(p, s2, 2.0f);
  float fe = (float)e;
  return std::fma(fe, 0.693145751953125f, std::fma(fe, 1.428606765330187e-06f, s * p));
}

// e^x = 2^k e^r, r = x - k ln2 (two-constant split), Taylor to r^8.
inline float oexp(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return INFINITY;
  float k = std::floor(std::fma(x, 1.44269504088896341f, 0.5f));
  float r = std::fma(-k, 0.693145751953125f, x);
  r = std::fma(-k, 1.428606765330187e-06f, r);
  const float c[9] = {2.48015873e-05f, 1.98412698e-04f, 1.38888889e-03f, 8.33333333e-03f,
                      4.16666667e-02f, 1.66666667e-01f, 0.5f, 1.0f, 1.0f};
  float p = c[0];
  for (int i = 1; i < 9; ++i) p = std::fma(p, r, c[i]);
  int ki = (int)k;
  int k1 = ki / 2, k2 = ki - k1;
  return (p * from_bits((uint32_t)(k1 + 127) << 23)) * from_bits((uint32_t)(k2 + 127) << 23);
}

// sin / cos of 2 pi u: quadrant from round(4u), Taylor on [-pi/4, pi/4].
// sRGB transfer function (IEC 61966-2-1), the power as exp(log(v) / 2.4)
// with olog / oexp (the device's srgb_encode, bit for bit).
inline float osrgb_encode(float v) {
  if (v <= 0.0031308f) return 12.92f * v;
  return 1.055f * oexp(olog(v) * (1.0f / 2.4f)) - 0.055f;
}

inline void osincos2pi(float u, float* s, float* c) {
  float q = std::floor(std::fma(u, 4.0f, 0.5f));
  float r = std::fma(q, -0.25f, u);
  float x = r * 6.28318530717958648f;
  float x2 = x * x;
  float sp = -2.50521084e-08f;
  sp = std::fma(sp, x2, 2.75573192e-06f);
  sp = std::fma(sp, x2, -1.98412698e-04f);
  sp = std::fma(sp, x2, 8.33333333e-03f);
  sp = std::fma(sp, x2, -1.66666667e-01f);
  sp = std::fma(sp * x2, x, x);
  float cp = -2.75573192e-07f;
  cp = std::fma(cp, x2, 2.48015873e-05f);
  cp = std::fma(cp, x2, -1.38888889e-03f);
  cp = std::fma(cp, x2, 4.16666667e-02f);
  cp = std::fma(cp, x2, -0.5f);
  cp = std::fma(cp, x2, 1.0f);
  switch (((int)q) & 3) {
    case 0: *s = sp; *c = cp; break;
    case 1: *s = cp; *c = -sp; break;
    case 2: *s = -sp; *c = -cp; break;
    default: *s = -cp; *c = sp; break;
  }
}

// ---- random numbers ------------------------------------------------------
// "pcg hash" (Jarzynski & Olano, JCGT 2020): one PCG LCG step + RXS-M-XS.
inline uint32_t pcg_hash(uint32_t v) {
  uint32_t st = v * 747796405u + 2891336453u;
  uint32_t w = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
  return (w >> 22u) ^ w;
}

struct Rng {
  uint32_t s;
  bool xorshift;
  float next() {
    if (!xorshift) {
      s = s * 747796405u + 2891336453u;
      uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
      uint32_t o = (w >> 22u) ^ w;
      return (float)((o >> 8) + 1u) * 5.96046448e-08f;
    }
    // rand_xorshift + generateRandomNumber (PathTracer.comp:221-233)
    s ^= (s << 13);
    s ^= (s >> 17);
    s ^= (s << 5);
    return (float)s / 4294967296.0f;
  }
};

inline Rng rng_pcg(uint32_t seed, uint32_t path, uint32_t pass) {
  uint32_t k0 = pcg_hash(pass + 0x68E31DA4u);
  uint32_t k1 = pcg_hash(path ^ k0);
  return Rng{pcg_hash(seed + k1), false};
}

// initializeRandom (PathTracer.comp:235-241)
inline Rng rng_xorshift(uint32_t seed) {
  Rng r{seed, true};
  for (uint32_t i = 0; i < seed % 7u + 2u; ++i) r.next();
  return r;
}

// ---- half / bfloat16 round-to-nearest-even -------------------------------
inline uint16_t f32_to_f16(float f) {
  uint32_t u = bits(f);
  uint32_t sign = (u >> 16) & 0x8000u;
  int exp = (int)((u >> 23) & 0xFFu);
  uint32_t mant = u & 0x7FFFFFu;
  if (exp == 0xFF) return (uint16_t)(sign | 0x7C00u | (mant ? 0x200u : 0u));
  int e = exp - 127 + 15;
  if (e >= 31) return (uint16_t)(sign | 0x7C00u);
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;
    uint32_t full = mant | 0x800000u;
    int shift = 14 - e;
    uint32_t hm = full >> shift;
    uint32_t rem = full & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1);
    if (rem > half || (rem == half && (hm & 1u))) ++hm;
    return (uint16_t)(sign | hm);
  }
  uint32_t hm = mant >> 13;
  uint32_t rem = mant & 0x1FFFu;
  uint32_t r = sign | ((uint32_t)e << 10) | hm;
  if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) ++r;
  return (uint16_t)r;
}

inline float f16_to_f32(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
  if (e == 0) {
    float v = (float)m * 5.9604644775390625e-08f;  // m * 2^-24, exact
    return sign ? -v : v;
  }
  if (e == 31) return from_bits(sign | 0x7F800000u | (m << 13));
  return from_bits(sign | ((e - 15 + 127) << 23) | (m << 13));
}

inline uint16_t f32_to_bf16(float f) {
  uint32_t u = bits(f);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
inline float bf16_to_f32(uint16_t h) { return from_bits((uint32_t)h << 16); }

}  // namespace oracle
