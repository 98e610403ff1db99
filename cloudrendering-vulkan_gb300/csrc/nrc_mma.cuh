// Register-resident forward pass of the radiance-cache MLP on the tensor
// cores: mma.sync m16n8k16 with BF16 operands and FP32 accumulation.  A warp
// owns 16 samples; their activations never leave registers, because the
// accumulator fragment of one layer (rows g and g+8, columns 2t and 2t+1 of
// each 8-column tile, g = lane/4, t = lane%4) is, after ReLU and BF16
// packing, exactly the A fragment of the next layer (rows g and g+8,
// columns 2t, 2t+1 and 2t+8, 2t+9 of each 16-column tile).  Only the
// weights live in shared memory, in their [in][out] layout with padded
// rows (144 bytes for the hidden layers), copied 16 bytes at a time; the B
// fragments come from ldmatrix.trans, two 8-column tiles per load, on 32
// distinct banks.
#pragma once

#include "nrc.cuh"

namespace vcr {

// Shared-memory row strides are padded off powers of two, so the 16 rows of
// a matrix fragment load or store fall on different banks.
constexpr int kLdX = kNrcWidth + 8;  // BF16 activation / gradient tiles: 144-byte rows
__host__ __device__ constexpr int ldw(int l) { return nrc_layer_cols(l) + 8; }  // BF16 weights of layer l
__host__ __device__ constexpr int woff(int l) { return l * kNrcWidth * (kNrcWidth + 8); }
constexpr int kWs = woff(kNrcLayers - 1) + kNrcWidth * (kNrcOutPad + 8);  // BF16 weights in shared memory

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ldmatrix: four 8x8 BF16 matrices from shared memory; lane j gives the
// address of row j%8 of matrix j/8 (16-byte aligned).  Without .trans lane
// (g, t) = (lane/4, lane%4) receives row g, columns 2t, 2t+1 of each
// matrix; with .trans column g, rows 2t, 2t+1.
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a)
               : "memory");
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a)
               : "memory");
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(a)
               : "memory");
}

// Global [in][out] BF16 weights (ld = cols) into the padded shared layout,
// 16 bytes at a time by a CTA of kThreads threads: all of a thread's loads
// are issued before its stores, so the copy costs one L2 round trip, not
// eleven.
template <int kThreads>
__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ g, __nv_bfloat16* s) {
  constexpr int kPieces = kNrcWeightCount / 8;
  constexpr int kIters = (kPieces + kThreads - 1) / kThreads;
  const uint4* src = reinterpret_cast<const uint4*>(g);
  uint4 v[kIters];
#pragma unroll
  for (int k = 0; k < kIters; ++k) {
    const int c = (int)threadIdx.x + k * kThreads;
    if (c < kPieces) v[k] = src[c];
  }
#pragma unroll
  for (int k = 0; k < kIters; ++k) {
    const int c = (int)threadIdx.x + k * kThreads;
    if (c >= kPieces) break;
    const int e = c * 8;
    const int l = e < kNrcHidden * kNrcWidth * kNrcWidth ? e / (kNrcWidth * kNrcWidth) : kNrcHidden;
    const int cols = nrc_layer_cols(l);
    const int rel = e - nrc_layer_offset(l);
    const int row = rel / cols, col = rel - row * cols;
    *reinterpret_cast<uint4*>(s + woff(l) + row * ldw(l) + col) = v[k];
  }
}

// acc = X W_l for the NT 8-column output tiles of layer l: X the A
// fragments a[kt] (4 input tiles), W_l the [in][out] rows of ldw(l); the B
// fragments come from ldmatrix.trans, two output tiles per load.
template <int NT>
__device__ __forceinline__ void mma_layer_in_out(const __nv_bfloat16* Wl, int ld, const uint32_t (&a)[4][4],
                                                 float (&acc)[NT][4], int lane) {
  const int rr = lane & 7, q = lane >> 3;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
#pragma unroll
    for (int np = 0; np < NT / 2; ++np) {
      uint32_t b[4];  // (in 16kt.., out 16np..), (in +8, out), (in, out +8), (in +8, out +8)
      ldsm_x4_t(b, Wl + (kt * 16 + rr + 8 * (q & 1)) * ld + np * 16 + 8 * (q >> 1));
      mma_bf16(acc[2 * np], a[kt], b[0], b[1]);
      mma_bf16(acc[2 * np + 1], a[kt], b[2], b[3]);
    }
  }
}

// The 16 position-level directions into shared memory (x, y, z each): the
// same function as the per-sample encoder, so the values are identical.
__device__ __forceinline__ void load_level_dirs(float* dirs) {
  if (threadIdx.x < kNrcPosLevels)
    nrc_level_dir((int)threadIdx.x, dirs[3 * threadIdx.x], dirs[3 * threadIdx.x + 1], dirs[3 * threadIdx.x + 2]);
}

// ReLU, BF16, and the accumulator layout of 8 tiles turned into the A
// fragments of 4 input tiles.
__device__ __forceinline__ void relu_to_a(const float (&acc)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    a[kt][0] = pack_bf16(fmaxf(acc[2 * kt][0], 0.0f), fmaxf(acc[2 * kt][1], 0.0f));
    a[kt][1] = pack_bf16(fmaxf(acc[2 * kt][2], 0.0f), fmaxf(acc[2 * kt][3], 0.0f));
    a[kt][2] = pack_bf16(fmaxf(acc[2 * kt + 1][0], 0.0f), fmaxf(acc[2 * kt + 1][1], 0.0f));
    a[kt][3] = pack_bf16(fmaxf(acc[2 * kt + 1][2], 0.0f), fmaxf(acc[2 * kt + 1][3], 0.0f));
  }
}

// Coefficients 2t, 2t+1, 8+2t, 9+2t of a 16-vector (constant indices only).
__device__ __forceinline__ void pick4(const float (&v)[16], int t, float& x0, float& x1, float& x2, float& x3) {
  x0 = t == 0 ? v[0] : t == 1 ? v[2] : t == 2 ? v[4] : v[6];
  x1 = t == 0 ? v[1] : t == 1 ? v[3] : t == 2 ? v[5] : v[7];
  x2 = t == 0 ? v[8] : t == 1 ? v[10] : t == 2 ? v[12] : v[14];
  x3 = t == 0 ? v[9] : t == 1 ? v[11] : t == 2 ? v[13] : v[15];
}

// The A fragments of the 64 encoded inputs of one sample row (h = 0: the
// row g half of each register pair, h = 1: row g + 8).  Column 2l / 2l+1
// are sin / cos of position level l (k-tiles 0, 1), columns 32.. the view
// SH, 48.. the sun SH (k-tiles 2, 3), as nrc_encode lays them out.
// `dirs` holds the 16 level directions (nrc_level_dir) as x, y, z triples.
// `gtab`: the grid encoding's tables (nullptr: the frequency encoding).
__device__ __forceinline__ void encode_a(const NrcRecord& r, bool valid, f3 b0, f3 inv_ext, const float* dirs, int t,
                                         int h, uint32_t (&a)[4][4], int levels = kNrcPosLevels,
                                         const float* gtab = nullptr) {
  float s[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
  float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f, w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f;
  if (valid) {
    float ux, uy, uz;
    nrc_box_coords(r, b0, inv_ext, ux, uy, uz);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int l = 4 * j + t;
      if (l >= levels) continue;
      if (gtab) nrc_grid_level(gtab, l, ux, uy, uz, &s[j], &c[j]);
      else nrc_encode_level_dir(l, dirs[3 * l], dirs[3 * l + 1], dirs[3 * l + 2], ux, uy, uz, &s[j], &c[j]);
    }
    float sh[16];
    nrc_sh16(r.vx, r.vy, r.vz, sh);
    pick4(sh, t, v0, v1, v2, v3);
    nrc_sh16(r.sx, r.sy, r.sz, sh);
    pick4(sh, t, w0, w1, w2, w3);
  }
  a[0][h] = pack_bf16(s[0], c[0]);      // cols 2t, 2t+1: level t
  a[0][h + 2] = pack_bf16(s[1], c[1]);  // cols 8+2t: level 4+t
  a[1][h] = pack_bf16(s[2], c[2]);      // level 8+t
  a[1][h + 2] = pack_bf16(s[3], c[3]);  // level 12+t
  a[2][h] = pack_bf16(v0, v1);
  a[2][h + 2] = pack_bf16(v2, v3);
  a[3][h] = pack_bf16(w0, w1);
  a[3][h + 2] = pack_bf16(w2, w3);
}

// Forward of rows g and g+8 of one 16-sample tile: outputs y (cols 0..2)
// land in lanes with t == 0 (row g in yg, row g + 8 in yh).
// W holds the weights in the shared [in][out] layout (load_weights).
__device__ __forceinline__ void mlp_forward_mma(const __nv_bfloat16* W, uint32_t (&a)[4][4], int lane,
                                                float (&yg)[3], float (&yh)[3]) {
#pragma unroll 1
  for (int l = 0; l < kNrcHidden; ++l) {
    float acc[8][4];
    mma_layer_in_out<8>(W + woff(l), ldw(l), a, acc, lane);
    relu_to_a(acc, a);
  }
  float out[2][4];
  mma_layer_in_out<2>(W + woff(kNrcHidden), ldw(kNrcHidden), a, out, lane);
  // tile 0 holds cols 2t, 2t+1: lane t = 0 has cols 0, 1 and lane t = 1 col 2
  const float c2g = __shfl_down_sync(0xffffffffu, out[0][0], 1);
  const float c2h = __shfl_down_sync(0xffffffffu, out[0][2], 1);
  yg[0] = out[0][0];
  yg[1] = out[0][1];
  yg[2] = c2g;
  yh[0] = out[0][2];
  yh[1] = out[0][3];
  yh[2] = c2h;
}

}  // namespace vcr
