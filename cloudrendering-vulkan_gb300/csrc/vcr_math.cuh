// Scalar math and sampling primitives shared by every vcr kernel.
//
// Float semantics are pinned so that a CPU restatement can reproduce the
// kernels bit for bit: the library is compiled with -fmad=false (no implicit
// FMA contraction) and every fused multiply-add is written out with fmaf();
// +, -, *, / and sqrtf are IEEE round-to-nearest on both sides.  The
// transcendental functions below are the project's own, written from the
// classical series named at each one, so they give the same bits on the CPU
// and the GPU (CUDA's logf/expf/sinf would not match a host libm).  A
// translation unit built with VCR_FAST_MATH (the fast-math tracker) swaps
// them, in device code only, for CUDA's __logf / __expf / __sincosf.
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define VCR_HD __host__ __device__ __forceinline__
#else
#define VCR_HD inline
#endif

namespace vcr {

// ---------------------------------------------------------------------------
// float3
// ---------------------------------------------------------------------------
struct f3 {
  float x, y, z;
};

VCR_HD f3 mk(float x, float y, float z) { return f3{x, y, z}; }
VCR_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
VCR_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
VCR_HD f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
VCR_HD f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
VCR_HD f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
VCR_HD f3 mul(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
VCR_HD f3 div(f3 a, f3 b) { return f3{a.x / b.x, a.y / b.y, a.z / b.z}; }
// dot = (x*x' + y*y') + z*z', evaluated left to right, no fusion.
VCR_HD float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
VCR_HD float length(f3 a) { return sqrtf(dot(a, a)); }
VCR_HD f3 normalize(f3 a) {
  float l = sqrtf(dot(a, a));
  return f3{a.x / l, a.y / l, a.z / l};
}
VCR_HD f3 cross(f3 a, f3 b) {
  return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// p + t*d per component (two roundings).
VCR_HD f3 along(f3 p, f3 d, float t) { return f3{p.x + t * d.x, p.y + t * d.y, p.z + t * d.z}; }

VCR_HD float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

VCR_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  union { float f; uint32_t u; } c; c.f = f; return c.u;
#endif
}
VCR_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  union { float f; uint32_t u; } c; c.u = u; return c.f;
#endif
}

// ---------------------------------------------------------------------------
// Transcendentals (own implementations, see file header)
// ---------------------------------------------------------------------------
constexpr float kPI = 3.14159265359f;
constexpr float kINV_4PI = 0.0795774715f;  // 1 / (4 pi)
constexpr float kLN2_HI = 0.693145751953125f;
constexpr float kLN2_LO = 1.428606765330187e-06f;
constexpr float kLOG2E = 1.44269504088896341f;
constexpr float kTWO_PI = 6.28318530717958648f;

// Natural log of a positive normal float.  x = 2^e * m, m folded into
// [sqrt(1/2), sqrt(2)); log m = 2 atanh(s), s = (m-1)/(m+1), summed as the
// odd series 2(s + s^3/3 + ... + s^9/9) (|s| <= 0.1716, truncation < 1e-9).
// log(0) = -inf, matching the shaders' log(0) in the xorshift parity mode.
VCR_HD float vlog(float x) {
  if (!(x > 0.0f)) return -INFINITY;
#if defined(VCR_FAST_MATH) && defined(__CUDA_ARCH__)
  return __logf(x);
#endif
  uint32_t b = f2u(x);
  int e = (int)(b >> 23) - 127;
  float m = u2f((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e = e + 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = 0.222222222f;           // 2/9
  p = fmaf(p, s2, 0.285714286f);    // 2/7
  p = fmaf(p, s2, 0.4f);            // 2/5
  p = fmaf(p, s2, 0.666666667f);    // 2/3
  p = fmaf(p, s2, 2.0f);
  float lm = s * p;
  float fe = (float)e;
  return fmaf(fe, kLN2_HI, fmaf(fe, kLN2_LO, lm));
}

// e^x: x = k ln2 + r (Cody-Waite split of ln2), e^r by its Taylor series to
// r^8/8! (|r| <= ln2/2, truncation < 5e-9), scaled by 2^k through the
// exponent bits.  Underflows to 0 below -87.
VCR_HD float vexp(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return INFINITY;
#if defined(VCR_FAST_MATH) && defined(__CUDA_ARCH__)
  return __expf(x);
#endif
  float k = floorf(fmaf(x, kLOG2E, 0.5f));
  float r = fmaf(-k, kLN2_HI, x);
  r = fmaf(-k, kLN2_LO, r);
  float p = 2.48015873e-05f;        // 1/8!
  p = fmaf(p, r, 1.98412698e-04f);  // 1/7!
  p = fmaf(p, r, 1.38888889e-03f);  // 1/6!
  p = fmaf(p, r, 8.33333333e-03f);  // 1/5!
  p = fmaf(p, r, 4.16666667e-02f);  // 1/4!
  p = fmaf(p, r, 1.66666667e-01f);  // 1/3!
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int ki = (int)k;
  // two-step scale keeps 2^k representable near the ends of the range
  int k1 = ki / 2, k2 = ki - k1;
  return (p * u2f((uint32_t)(k1 + 127) << 23)) * u2f((uint32_t)(k2 + 127) << 23);
}

// sRGB transfer function (IEC 61966-2-1) of a linear value in [0, 1]:
// 12.92 v up to 0.0031308, else 1.055 v^(1/2.4) - 0.055, the power taken as
// exp(log(v) / 2.4) with the functions above (so CPU and GPU agree).
VCR_HD float srgb_encode(float v) {
  if (v <= 0.0031308f) return 12.92f * v;
  return 1.055f * vexp(vlog(v) * (1.0f / 2.4f)) - 0.055f;
}

// sin(2 pi u) and cos(2 pi u): u = q/4 + r with q = round(4u), x = 2 pi r in
// [-pi/4, pi/4]; Taylor series of sin to x^11 and cos to x^10, then the
// quadrant rotation.
VCR_HD void vsincos2pi(float u, float* s, float* c) {
#if defined(VCR_FAST_MATH) && defined(__CUDA_ARCH__)
  __sincosf(kTWO_PI * (u - floorf(u + 0.5f)), s, c);  // argument reduced to [-pi, pi]
  return;
#endif
  float q = floorf(fmaf(u, 4.0f, 0.5f));
  float r = fmaf(q, -0.25f, u);
  float x = r * kTWO_PI;
  float x2 = x * x;
  float sp = -2.50521084e-08f;          // -1/11!
  sp = fmaf(sp, x2, 2.75573192e-06f);   // 1/9!
  sp = fmaf(sp, x2, -1.98412698e-04f);  // -1/7!
  sp = fmaf(sp, x2, 8.33333333e-03f);   // 1/5!
  sp = fmaf(sp, x2, -1.66666667e-01f);  // -1/3!
  sp = fmaf(sp * x2, x, x);
  float cp = -2.75573192e-07f;          // -1/10!
  cp = fmaf(cp, x2, 2.48015873e-05f);   // 1/8!
  cp = fmaf(cp, x2, -1.38888889e-03f);  // -1/6!
  cp = fmaf(cp, x2, 4.16666667e-02f);   // 1/4!
  cp = fmaf(cp, x2, -0.5f);
  cp = fmaf(cp, x2, 1.0f);
  int qi = ((int)q) & 3;
  if (qi == 0) { *s = sp; *c = cp; }
  else if (qi == 1) { *s = cp; *c = -sp; }
  else if (qi == 2) { *s = -sp; *c = -cp; }
  else { *s = -cp; *c = sp; }
}

// ---------------------------------------------------------------------------
// Random numbers
// ---------------------------------------------------------------------------
// PCG-RXS-M-XS 32-bit output permutation of one LCG step (the "pcg hash" of
// Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020).
VCR_HD uint32_t pcg_hash(uint32_t v) {
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

// Per-path generator keyed on (seed, path, pass): resuming at pass k gives
// the same streams as an uninterrupted run.  Draws are in (0, 1].
struct Rng {
  uint32_t state;
  uint32_t mode;  // vcr_rng_mode
};

VCR_HD uint32_t path_key(uint32_t seed, uint32_t path, uint32_t pass) {
  uint32_t k0 = pcg_hash(pass + 0x68E31DA4u);
  uint32_t k1 = pcg_hash(path ^ k0);
  return pcg_hash(seed + k1);
}

VCR_HD Rng rng_pcg(uint32_t seed, uint32_t path, uint32_t pass) {
  return Rng{path_key(seed, path, pass), 0u};
}

VCR_HD float rng_next(Rng& r) {
  if (r.mode == 0u) {
    r.state = r.state * 747796405u + 2891336453u;
    uint32_t word = ((r.state >> ((r.state >> 28u) + 4u)) ^ r.state) * 277803737u;
    uint32_t out = (word >> 22u) ^ word;
    return (float)((out >> 8) + 1u) * 5.96046448e-08f;  // 2^-24
  }
  // xorshift32 (13, 17, 5), u = float(state) / 2^32 (PathTracer.comp:221-233)
  r.state ^= (r.state << 13);
  r.state ^= (r.state >> 17);
  r.state ^= (r.state << 5);
  return (float)r.state / 4294967296.0f;
}

// initializeRandom (PathTracer.comp:235-241): state = seed, seed%7+2 draws.
VCR_HD Rng rng_xorshift(uint32_t seed) {
  Rng r{seed, 1u};
  for (uint32_t i = 0; i < seed % 7u + 2u; ++i) rng_next(r);
  return r;
}

// ---------------------------------------------------------------------------
// Henyey-Greenstein (PathTracer.comp:247-311)
// ---------------------------------------------------------------------------
struct Phase {
  float g, opg2, omg2, o2g;
  int iso;
};

VCR_HD float hg_pdf(const Phase& ph, float cos_theta) {
  if (ph.iso) return kINV_4PI;
  float d = ph.opg2 - (2.0f * ph.g) * cos_theta;
  return (kINV_4PI * ph.omg2) / (d * sqrtf(d));
}

VCR_HD float hg_invert_cdf(const Phase& ph, float xi) {
  float sq = ph.omg2 / ((1.0f - ph.g) + (2.0f * ph.g) * xi);
  return ph.o2g * (ph.opg2 - sq * sq);
}

// Branchless orthonormal basis (createOrthonormalBasis, PathTracer.comp:197-206;
// utilities::GetOrthonormalBasis, Utilities.cpp:7-16).
VCR_HD void onb(f3 n, f3& xp, f3& yp) {
  float sz = n.z >= 0.0f ? 1.0f : -1.0f;
  float a = n.y / (1.0f + fabsf(n.z));
  float b = n.y * a;
  float c = -n.x * a;
  xp = f3{n.z + sz * b, sz * c, -n.x};
  yp = f3{c, 1.0f - b, -sz * n.y};
}

// scatterRay (PathTracer.comp:277-311): phi first, then cos theta.
// `renorm` applies the normalisation the PPM/PPB shaders do.
VCR_HD f3 hg_sample(const Phase& ph, f3 in, Rng& rng, bool renorm) {
  f3 out;
  if (ph.iso) {
    float xi = rng_next(rng);
    out.z = xi * 2.0f - 1.0f;
    float s2 = 1.0f - out.z * out.z;
    if (s2 > 0.0f) {
      float st = sqrtf(fmaxf(0.0f, s2));
      float sn, cs;
      vsincos2pi(rng_next(rng), &sn, &cs);
      out.x = st * cs;
      out.y = st * sn;
    } else {
      out.x = out.y = 0.0f;
    }
  } else {
    float u_phi = rng_next(rng);
    float ct = hg_invert_cdf(ph, rng_next(rng));
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float sn, cs;
    vsincos2pi(u_phi, &sn, &cs);
    f3 t0, t1;
    onb(in, t0, t1);
    float a = st * cs, b = st * sn;
    out = f3{(a * t0.x + b * t1.x) + ct * in.x, (a * t0.y + b * t1.y) + ct * in.y,
             (a * t0.z + b * t1.z) + ct * in.z};
  }
  return renorm ? normalize(out) : out;
}

// ---------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------
// Slab test (intersectCloud, PathTracer.comp:154-184), same comparisons.
VCR_HD f3 recip(f3 d) { return f3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z}; }

// Slab test with the ray's reciprocal direction already computed.
VCR_HD bool slab_inv(f3 pos, f3 inv, f3 b0, f3 b1, float& tmin, float& tmax) {
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

VCR_HD bool slab(f3 pos, f3 dir, f3 b0, f3 b1, float& tmin, float& tmax) {
  return slab_inv(pos, recip(dir), b0, b1, tmin, tmax);
}

VCR_HD bool in_box(f3 p, f3 b0, f3 b1) {
  return !(p.x < b0.x || p.y < b0.y || p.z < b0.z || p.x > b1.x || p.y > b1.y || p.z > b1.z);
}

// Five-stop sky gradient on dir.y (sampleBackground, PathTracer.comp:104-113),
// smoothstep/mix as GLSL defines them.
VCR_HD f3 sky_gradient(f3 dir) {
  const float C[5][3] = {{0.00f, 0.0f, 0.02f}, {0.01f, 0.05f, 0.2f}, {0.7f, 0.9f, 1.0f},
                         {0.1f, 0.3f, 1.0f}, {0.01f, 0.1f, 0.7f}};
  const float D[5] = {-1.0f, -0.04f, 0.0f, 0.5f, 1.0f};
  float col[3] = {C[0][0], C[0][1], C[0][2]};
  float y = dir.y;
  for (int i = 1; i < 5; ++i) {
    float t = clampf((y - D[i - 1]) / (D[i] - D[i - 1]), 0.0f, 1.0f);
    float s = t * t * (3.0f - 2.0f * t);
    for (int c = 0; c < 3; ++c) col[c] = col[c] * (1.0f - s) + C[i][c] * s;
  }
  return f3{col[0], col[1], col[2]};
}

}  // namespace vcr
