// ORACLE — test infrastructure only (see oracle_math.h).  FP64 restatement
// of the radiance-cache network for the gradient check: the same encoding
// (frequency encoding of the box position, 4-band real SH of the view and
// sun directions), the same 64 -> 5x64 ReLU -> 3 layers without biases,
// the relative L2 loss, and analytic backpropagation.  Where the GPU rounds
// to BF16 (weights, encoded inputs, hidden activations, output and hidden
// gradients) this code rounds too; sums run in double.
#include <cmath>
#include <cstdint>
#include <vector>

#include "oracle_math.h"

namespace oracle {

const int kIn = 64, kW = 64, kHidden = 5, kLayers = 6, kOut = 3, kOutPad = 16;
const int kWeights = kHidden * kW * kW + kW * kOutPad;

struct Rec {
  float px, py, pz, vx, vy, vz, sx, sy, sz, w0, w1, w2;
  uint32_t pix, pad[3];
};

static bool g_exact = false;  // true: no BF16 rounding (finite-difference checks of the analytic gradient)
static int g_levels = 16;     // position levels encoded; the inputs of the others are 0
static const float* g_grid = nullptr;  // grid encoding's tables [16][2^17][2], or null: frequency encoding

// Grid encoding: level l has kGridRes[l] cells per box axis and a table of
// 2^17 two-feature entries, dense while the (n+1)^3 vertices fit, else
// indexed by the spatial hash x ^ 2654435761 y ^ 805459861 z; the level's
// two inputs interpolate its cell's 8 vertices trilinearly.
const uint32_t kGridTable = 1u << 17;
const int kGridRes[16] = {16, 21, 27, 36, 48, 64, 84, 111, 147, 194, 256, 337, 445, 588, 776, 1024};

static uint32_t grid_index(int n, uint32_t x, uint32_t y, uint32_t z) {
  const uint64_t v = (uint64_t)n + 1u;
  if (v * v * v <= kGridTable) return (uint32_t)(x + v * (y + v * z));
  return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (kGridTable - 1u);
}

struct GridCell {
  uint32_t c[3];
  float f[3];
};

static GridCell grid_cell(int n, const float u[3]) {
  GridCell g;
  for (int a = 0; a < 3; ++a) {
    const float p = std::fmin(std::fmax(u[a], 0.0f), 1.0f) * (float)n;
    const int i = (int)p < n - 1 ? (int)p : n - 1;
    g.c[a] = (uint32_t)i;
    g.f[a] = p - (float)i;
  }
  return g;
}

// Corner k (bit 0: +x, 1: +y, 2: +z): its table entry and trilinear weight.
static void grid_corner(int n, const GridCell& g, int k, uint32_t& idx, float& w) {
  idx = grid_index(n, g.c[0] + (k & 1), g.c[1] + ((k >> 1) & 1), g.c[2] + (k >> 2));
  const float wx = (k & 1) ? g.f[0] : 1.0f - g.f[0];
  const float wy = (k & 2) ? g.f[1] : 1.0f - g.f[1];
  const float wz = (k & 4) ? g.f[2] : 1.0f - g.f[2];
  w = (wx * wy) * wz;
}
static double bf(double x) { return g_exact ? x : (double)bf16_to_f32(f32_to_bf16((float)x)); }
static int layer_off(int l) { return l * kW * kW; }
static int layer_cols(int l) { return l < kHidden ? kW : kOutPad; }

static void level_dir(int l, float& dx, float& dy, float& dz) {
  const float z = 1.0f - (2.0f * (float)l + 1.0f) / 16.0f;
  const float r = std::sqrt(std::fmax(0.0f, 1.0f - z * z));
  float t = 0.61803398875f * (float)l;
  t = t - std::floor(t);
  float sn, cs;
  osincos2pi(t, &sn, &cs);
  dx = r * cs;
  dy = r * sn;
  dz = z;
}

static void sh16(float x, float y, float z, float* o) {
  const float xx = x * x, yy = y * y, zz = z * z;
  o[0] = 0.28209479177f;
  o[1] = -0.48860251190f * y;
  o[2] = 0.48860251190f * z;
  o[3] = -0.48860251190f * x;
  o[4] = 1.09254843059f * (x * y);
  o[5] = -1.09254843059f * (y * z);
  o[6] = 0.31539156525f * (3.0f * zz - 1.0f);
  o[7] = -1.09254843059f * (x * z);
  o[8] = 0.54627421529f * (xx - yy);
  o[9] = -0.59004358993f * y * (3.0f * xx - yy);
  o[10] = 2.89061144264f * (x * y) * z;
  o[11] = -0.45704579946f * y * (5.0f * zz - 1.0f);
  o[12] = 0.37317633259f * z * (5.0f * zz - 3.0f);
  o[13] = -0.45704579946f * x * (5.0f * zz - 1.0f);
  o[14] = 1.44530572132f * z * (xx - yy);
  o[15] = -0.59004358993f * x * (xx - 3.0f * yy);
}

static void encode(const Rec& r, const float* b0, const float* inv_ext, float* o) {
  float ux = (r.px - b0[0]) * inv_ext[0], uy = (r.py - b0[1]) * inv_ext[1], uz = (r.pz - b0[2]) * inv_ext[2];
  for (int l = 0; l < 16; ++l) {
    if (l >= g_levels) {
      o[2 * l] = o[2 * l + 1] = 0.0f;
      continue;
    }
    if (g_grid) {
      const float u[3] = {ux, uy, uz};
      const GridCell g = grid_cell(kGridRes[l], u);
      const float* t = g_grid + (size_t)l * kGridTable * 2;
      float a0 = 0.0f, a1 = 0.0f;
      for (int k = 0; k < 8; ++k) {
        uint32_t idx;
        float w;
        grid_corner(kGridRes[l], g, k, idx, w);
        a0 = std::fma(w, t[2 * idx], a0);
        a1 = std::fma(w, t[2 * idx + 1], a1);
      }
      o[2 * l] = a0;
      o[2 * l + 1] = a1;
      continue;
    }
    float dx, dy, dz;
    level_dir(l, dx, dy, dz);
    float f = (float)(1u << (l >> 1)) * ((l & 1) ? 1.41421356f : 1.0f);
    float ph = f * ((dx * ux + dy * uy) + dz * uz);
    ph = ph - std::floor(ph);
    float sn, cs;
    osincos2pi(ph, &sn, &cs);
    o[2 * l] = sn;
    o[2 * l + 1] = cs;
  }
  sh16(r.vx, r.vy, r.vz, o + 32);
  sh16(r.sx, r.sy, r.sz, o + 48);
}

// h[l] (l = 0..5) activations and the output of one record.
static void forward(const std::vector<double>& wb, const Rec& r, const float* b0, const float* inv_ext,
                    std::vector<std::vector<double>>& h, double* y) {
  float enc[kIn];
  encode(r, b0, inv_ext, enc);
  h.assign(kLayers, std::vector<double>(kW, 0.0));
  for (int i = 0; i < kIn; ++i) h[0][i] = bf(enc[i]);
  for (int l = 0; l < kLayers; ++l) {
    int cols = layer_cols(l);
    std::vector<double> z(cols, 0.0);
    for (int i = 0; i < kW; ++i)
      for (int o = 0; o < cols; ++o) z[o] += h[l][i] * wb[layer_off(l) + i * cols + o];
    if (l < kHidden) {
      for (int o = 0; o < kW; ++o) h[l + 1][o] = bf(std::fmax(z[o], 0.0));
    } else {
      for (int c = 0; c < kOut; ++c) y[c] = z[c];
    }
  }
}

static std::vector<double> round_weights(const float* w) {
  std::vector<double> wb(kWeights);
  for (int i = 0; i < kWeights; ++i) wb[i] = bf(w[i]);
  return wb;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int oracle_nrc_weight_count() { return kWeights; }

void oracle_nrc_set_exact(int exact) { g_exact = exact != 0; }

void oracle_nrc_set_levels(int levels) { g_levels = levels < 0 ? 0 : levels > 16 ? 16 : levels; }

void oracle_nrc_set_grid(const float* tables) { g_grid = tables; }

void oracle_nrc_encode(const void* recs, uint32_t n, const float* b0, const float* inv_ext, float* out) {
  const Rec* r = static_cast<const Rec*>(recs);
  for (uint32_t i = 0; i < n; ++i) encode(r[i], b0, inv_ext, out + (size_t)i * kIn);
}

void oracle_nrc_forward(const float* w, const void* recs, uint32_t n, const float* b0, const float* inv_ext,
                        double* out) {
  std::vector<double> wb = round_weights(w);
  const Rec* r = static_cast<const Rec*>(recs);
  std::vector<std::vector<double>> h;
  for (uint32_t i = 0; i < n; ++i) forward(wb, r[i], b0, inv_ext, h, out + 3 * (size_t)i);
}

// Gradient of (1/3n) sum_s sum_c (y - t)^2 / (y^2 + 0.01), with y held
// constant in the denominator (stop-gradient), over n records; with the
// grid encoding and gtab given, also the gradient of the tables
// (dX_0 = dY_0 W_0^T of the 32 position inputs, spread over each level's 8
// vertices by their trilinear weights).
double oracle_nrc_gradient_tables(const float* w, const void* recs, uint32_t n, const float* b0, const float* inv_ext,
                                  double* grad, double* gtab) {
  std::vector<double> wb = round_weights(w);
  const Rec* r = static_cast<const Rec*>(recs);
  for (int i = 0; i < kWeights; ++i) grad[i] = 0.0;
  const double inv_n = 1.0 / (3.0 * (double)n);
  double loss = 0.0;
  std::vector<std::vector<double>> h;
  for (uint32_t s = 0; s < n; ++s) {
    double y[3];
    forward(wb, r[s], b0, inv_ext, h, y);
    std::vector<double> dy(kOutPad, 0.0);
    const float t[3] = {r[s].w0, r[s].w1, r[s].w2};
    for (int c = 0; c < kOut; ++c) {
      double den = y[c] * y[c] + 0.01;
      double diff = y[c] - (double)t[c];
      loss += diff * diff / den * inv_n;
      dy[c] = bf(2.0 * diff / den * inv_n);
    }
    for (int l = kLayers - 1; l >= 0; --l) {
      int cols = layer_cols(l);
      for (int i = 0; i < kW; ++i)
        for (int o = 0; o < cols; ++o) grad[layer_off(l) + i * cols + o] += h[l][i] * dy[o];
      if (l > 0) {
        std::vector<double> dn(kW, 0.0);
        for (int i = 0; i < kW; ++i) {
          double acc = 0.0;
          for (int o = 0; o < cols; ++o) acc += dy[o] * wb[layer_off(l) + i * cols + o];
          dn[i] = bf(h[l][i] > 0.0 ? acc : 0.0);
        }
        dy = dn;
      } else if (g_grid && gtab) {
        const float u[3] = {(r[s].px - b0[0]) * inv_ext[0], (r[s].py - b0[1]) * inv_ext[1],
                            (r[s].pz - b0[2]) * inv_ext[2]};
        for (int lv = 0; lv < g_levels; ++lv) {
          double d[2];
          for (int e = 0; e < 2; ++e) {
            const int i = 2 * lv + e;
            double acc = 0.0;
            for (int o = 0; o < cols; ++o) acc += dy[o] * wb[layer_off(0) + i * cols + o];
            d[e] = acc;
          }
          const GridCell g = grid_cell(kGridRes[lv], u);
          double* gl = gtab + (size_t)lv * kGridTable * 2;
          for (int k = 0; k < 8; ++k) {
            uint32_t idx;
            float wk;
            grid_corner(kGridRes[lv], g, k, idx, wk);
            gl[2 * idx] += (double)wk * d[0];
            gl[2 * idx + 1] += (double)wk * d[1];
          }
        }
      }
    }
  }
  return loss;
}

double oracle_nrc_gradient(const float* w, const void* recs, uint32_t n, const float* b0, const float* inv_ext,
                           double* grad) {
  return oracle_nrc_gradient_tables(w, recs, n, b0, inv_ext, grad, nullptr);
}

}  // extern "C"
