// Radiance-cache network: encoding, sizes and state (no counterpart in the
// reference; the target adds it on top of the path tracer).
#pragma once

#include "vcr_internal.h"

namespace vcr {

constexpr int kNrcIn = 64;       // 32 position + 16 view SH + 16 sun SH
constexpr int kNrcWidth = 64;
constexpr int kNrcHidden = 5;    // hidden layers (ReLU)
constexpr int kNrcLayers = 6;    // weight matrices: 5 x (64x64) + output (64x16, 3 used)
constexpr int kNrcOut = 3;
constexpr int kNrcOutPad = 16;
constexpr int kNrcPosLevels = 16;
constexpr int kNrcWeightCount = kNrcHidden * kNrcWidth * kNrcWidth + kNrcWidth * kNrcOutPad;  // 21504
constexpr int kNrcTile = 64;     // samples per CTA tile (4 warps x 16 rows)

// One query / training record: the position of a real collision, the
// direction radiance leaves toward the previous vertex, the sun direction.
struct NrcRecord {
  float px, py, pz;  // world position
  float vx, vy, vz;  // unit direction toward the viewer (-travel direction)
  float sx, sy, sz;  // unit direction the sunlight travels
  float w0, w1, w2;  // query: path throughput (rgb); training: target radiance
  uint32_t pix;      // query: pixel index; training: unused
  uint32_t pad[3];   // training, while its path runs: beta before the vertex
                     // (float bits), slot of the path's previous record
};
static_assert(sizeof(NrcRecord) == 64, "record size");

// Training paths: extended (unbiased, full length) paths from uniformly
// drawn pixels of the crop that record their first kNrcRecordEvents
// scattering vertices.  They run as the first work items of a wavefront
// launch, ahead of the pass's camera paths.
constexpr int kNrcRecordEvents = 4;
// training sets one vcr_nrc_train_step may trace in its launch (pass.spp)
constexpr uint32_t kNrcMaxSets = 64;
constexpr uint32_t kNrcTrainSalt = 0x3C6EF372u;  // RNG stream salt of training paths
constexpr uint32_t kNrcNoSlot = 0xFFFFFFFFu;

struct NrcTrainSink {
  NrcRecord* rec;
  uint32_t* count;
  uint32_t capacity;
  uint32_t paths;   // training paths of the launch (0: none)
  float survival;   // Russian-roulette survival past the last recorded vertex (0: off)
};

struct NrcState {
  vcr_nrc_params prm{};
  float* w = nullptr;        // FP32 master weights [kNrcWeightCount]
  void* wb = nullptr;        // BF16 copy used by the kernels
  float* m = nullptr;        // Adam first moment
  float* v = nullptr;        // Adam second moment
  float* grad = nullptr;     // gradient accumulator [kNrcWeightCount]
  float* gpart = nullptr;    // per-CTA gradients of one training launch [gpart_blocks][kNrcWeightCount]
  int gpart_blocks = 0;
  float* ema = nullptr;      // exponential moving average of w (ema_decay > 0)
  void* wbi = nullptr;       // BF16 copy of ema used for inference (ema_decay > 0)
  float* loss = nullptr;     // [2]: the running step's loss sum (zeroed by the reduction), the last step's loss
  // grid encoding (prm.encoding == VCR_NRC_ENCODING_GRID): the tables
  // [kNrcGridParams], their Adam moments, gradient accumulator and moving
  // average (ema_decay > 0)
  float* gw = nullptr;
  float* gm = nullptr;
  float* gv = nullptr;
  float* ggrad = nullptr;
  float* gema = nullptr;
  NrcRecord* train = nullptr;  // training records [train_cap]
  uint32_t* train_count = nullptr;
  uint32_t train_cap = 0;      // 2 x train_samples x sets: room for the yield's spread
  uint32_t sets = 1;           // training sets (of ~train_samples records) in the buffer
  uint32_t cursor = 0;         // first record of the next vcr_nrc_train_more batch
  bool records = false;        // the buffer holds a training step's or frame's records
  NrcRecord* query = nullptr;  // cache queries of one pass [query_capacity]
  uint32_t* query_count = nullptr;
  uint32_t query_capacity = 0;
  uint32_t step = 0;
  float last_loss = 0.0f;
  uint32_t last_train = 0, last_queries = 0;
  // training paths per step, calibrated so that a step yields about
  // train_samples records for the bound camera and cloud (0 = recalibrate)
  uint32_t npaths = 0;
  vcr_camera calib_cam{};
  vcr_cloud calib_cloud{};
  uint32_t calib_w = 0, calib_h = 0;
};

// Position encoding: level l uses frequency 2^(l/2) cycles per unit box
// along a fixed unit direction d_l (a spherical Fibonacci set), giving
// (sin, cos)(2 pi 2^(l/2) d_l . p) with p in [0,1]^3 box coordinates.
// Directions: real spherical harmonics of degree 3 (16 coefficients, bands
// 0..3) with the usual normalisation constants.
__host__ __device__ __forceinline__ void nrc_level_dir(int l, float& dx, float& dy, float& dz) {
  // spherical Fibonacci point l of 16 (fixed constants, same on host and device)
  const float z = 1.0f - (2.0f * (float)l + 1.0f) / 16.0f;
  const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
  float t = 0.61803398875f * (float)l;  // golden-ratio turns
  t = t - floorf(t);
  float sn, cs;
  vsincos2pi(t, &sn, &cs);
  dx = r * cs;
  dy = r * sn;
  dz = z;
}

__host__ __device__ __forceinline__ void nrc_sh16(float x, float y, float z, float* o) {
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

// 64 encoded inputs of one record.  `b0`, `inv_ext` map world positions to
// [0,1]^3 box coordinates.
// (sin, cos) of position level l along its direction (dx, dy, dz) for box
// coordinates (ux, uy, uz).
__host__ __device__ __forceinline__ void nrc_encode_level_dir(int l, float dx, float dy, float dz, float ux, float uy,
                                                              float uz, float* sn, float* cs) {
  float f = (float)(1u << (l >> 1)) * ((l & 1) ? 1.41421356f : 1.0f);
  float ph = f * ((dx * ux + dy * uy) + dz * uz);
  ph = ph - floorf(ph);
  vsincos2pi(ph, sn, cs);
}

// (sin, cos) of position level l for box coordinates (ux, uy, uz).
__host__ __device__ __forceinline__ void nrc_encode_level(int l, float ux, float uy, float uz, float* sn, float* cs) {
  float dx, dy, dz;
  nrc_level_dir(l, dx, dy, dz);
  nrc_encode_level_dir(l, dx, dy, dz, ux, uy, uz, sn, cs);
}


__host__ __device__ __forceinline__ void nrc_box_coords(const NrcRecord& r, f3 b0, f3 inv_ext, float& ux, float& uy,
                                                        float& uz) {
  ux = (r.px - b0.x) * inv_ext.x;
  uy = (r.py - b0.y) * inv_ext.y;
  uz = (r.pz - b0.z) * inv_ext.z;
}

__host__ __device__ __forceinline__ void nrc_encode_position(const NrcRecord& r, f3 b0, f3 inv_ext, float* o) {
  float ux, uy, uz;
  nrc_box_coords(r, b0, inv_ext, ux, uy, uz);
#pragma unroll
  for (int l = 0; l < kNrcPosLevels; ++l) nrc_encode_level(l, ux, uy, uz, &o[2 * l], &o[2 * l + 1]);
}

// The 32 direction inputs: SH of the view direction, then of the sun.
__host__ __device__ __forceinline__ void nrc_encode_directions(const NrcRecord& r, float* o) {
  nrc_sh16(r.vx, r.vy, r.vz, o);
  nrc_sh16(r.sx, r.sy, r.sz, o + 16);
}

__host__ __device__ __forceinline__ void nrc_encode(const NrcRecord& r, f3 b0, f3 inv_ext, float* o) {
  nrc_encode_position(r, b0, inv_ext, o);
  nrc_encode_directions(r, o + 32);
}

// Multiresolution grid encoding, the alternative to the frequency encoding
// (vcr_nrc_params.encoding = VCR_NRC_ENCODING_GRID): level l has N_l =
// floor(16 * 64^(l/15)) cells per box axis (16 .. 1024) and a table of
// kNrcGridTable entries of 2 FP32 features, dense when the level's
// (N_l + 1)^3 vertices fit (levels 0..4) and indexed by the spatial hash
// x ^ 2654435761 y ^ 805459861 z of the vertex otherwise; the level's two
// network inputs (where the frequency encoding has its sin and cos) are the
// trilinear interpolation of its 8 vertices' features at the box position.
// The tables are parameters trained with the network.
constexpr int kNrcGridLog2 = 17;
constexpr uint32_t kNrcGridTable = 1u << kNrcGridLog2;  // entries per level
constexpr size_t kNrcGridParams = (size_t)kNrcPosLevels * kNrcGridTable * 2;  // 4,194,304 floats
constexpr float kNrcGridLrScale = 10.0f;  // the tables' Adam step size relative to the network's

__host__ __device__ __forceinline__ int nrc_grid_res(int l) {
  switch (l) {
    case 0: return 16;   case 1: return 21;   case 2: return 27;   case 3: return 36;
    case 4: return 48;   case 5: return 64;   case 6: return 84;   case 7: return 111;
    case 8: return 147;  case 9: return 194;  case 10: return 256; case 11: return 337;
    case 12: return 445; case 13: return 588; case 14: return 776; default: return 1024;
  }
}

// Table entry of vertex (x, y, z) of a level with n cells per axis.
__host__ __device__ __forceinline__ uint32_t nrc_grid_index(int n, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t v = (uint32_t)n + 1u;
  if ((uint64_t)v * v * v <= kNrcGridTable) return x + v * (y + v * z);
  return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (kNrcGridTable - 1u);
}

// The level's cell and trilinear fractions at box coordinates (ux, uy, uz)
// (clamped to the box).
struct NrcGridCell {
  uint32_t x, y, z;
  float fx, fy, fz;
};
__host__ __device__ __forceinline__ NrcGridCell nrc_grid_cell(int n, float ux, float uy, float uz) {
  NrcGridCell c;
  const float px = fminf(fmaxf(ux, 0.0f), 1.0f) * (float)n;
  const float py = fminf(fmaxf(uy, 0.0f), 1.0f) * (float)n;
  const float pz = fminf(fmaxf(uz, 0.0f), 1.0f) * (float)n;
  c.x = (uint32_t)((int)px < n - 1 ? (int)px : n - 1);
  c.y = (uint32_t)((int)py < n - 1 ? (int)py : n - 1);
  c.z = (uint32_t)((int)pz < n - 1 ? (int)pz : n - 1);
  c.fx = px - (float)c.x;
  c.fy = py - (float)c.y;
  c.fz = pz - (float)c.z;
  return c;
}

// Weight of corner k (bit 0: +x, bit 1: +y, bit 2: +z) of the cell.
__host__ __device__ __forceinline__ float nrc_grid_weight(const NrcGridCell& c, int k) {
  const float wx = (k & 1) ? c.fx : 1.0f - c.fx;
  const float wy = (k & 2) ? c.fy : 1.0f - c.fy;
  const float wz = (k & 4) ? c.fz : 1.0f - c.fz;
  return (wx * wy) * wz;
}

// The two features of level l at box coordinates (ux, uy, uz) from the
// tables `tab` (kNrcPosLevels x kNrcGridTable x 2 floats).
__host__ __device__ __forceinline__ void nrc_grid_level(const float* tab, int l, float ux, float uy, float uz,
                                                        float* f0, float* f1) {
  const int n = nrc_grid_res(l);
  const NrcGridCell c = nrc_grid_cell(n, ux, uy, uz);
  const float* t = tab + (size_t)l * kNrcGridTable * 2;
  float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint32_t idx = nrc_grid_index(n, c.x + (k & 1), c.y + ((k >> 1) & 1), c.z + (k >> 2));
    const float w = nrc_grid_weight(c, k);
#if defined(__CUDA_ARCH__)
    const float2 v = __ldg(reinterpret_cast<const float2*>(t) + idx);
#else
    const float2 v = reinterpret_cast<const float2*>(t)[idx];
#endif
    a0 = fmaf(w, v.x, a0);
    a1 = fmaf(w, v.y, a1);
  }
  *f0 = a0;
  *f1 = a1;
}

// Layer l weights start at this offset; hidden layers are [in][out] = 64x64
// row-major, the output layer 64 x 16 (columns 3..15 stay zero).
__host__ __device__ constexpr int nrc_layer_offset(int l) { return l * kNrcWidth * kNrcWidth; }
__host__ __device__ constexpr int nrc_layer_cols(int l) { return l < kNrcHidden ? kNrcWidth : kNrcOutPad; }

// nrc_tc.cu: the queries' forward on tcgen05 (128-record tiles, TMEM
// accumulators): reads the *d_count (<= capacity) records, adds
// throughput x max(y, 0) to sum[pix] and/or writes y to out.
// Network weights plus, with the grid encoding, the tables.
size_t nrc_param_count(const NrcState* st);

// `gtab`: the grid encoding's tables (nullptr: the frequency encoding).
vcr_status nrc_infer_tc_launch(vcr_ctx* ctx, const void* wbi, f3 b0, f3 inv_ext, int levels, const float* gtab,
                               const NrcRecord* recs, const uint32_t* d_count, uint32_t capacity, double* sum,
                               float* out, cudaStream_t s);

}  // namespace vcr
