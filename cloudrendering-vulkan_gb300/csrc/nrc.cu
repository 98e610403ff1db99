// Neural radiance cache: a 64 -> 5x64 (ReLU) -> 3 MLP that predicts the
// radiance leaving a scattering vertex toward the previous vertex, trained
// online on paths the tracer itself produces and queried where paths
// terminate into it.  No reference counterpart.
//
// Tensor cores, BF16 operands, FP32 accumulation.  Queries: a
// register-resident forward (mma.sync m16n8k16, nrc_mma.cuh) — each warp
// runs 16-sample tiles whose activations stay in the MMA fragments, the CTA
// shares only the BF16 weights.  Training: one 8-warp CTA per
// SM holds the BF16 weights and, for a 128-sample tile, the six activation
// tiles and the gradient ping-pong in padded shared memory (197 KB); the
// forward and the backward's dY_l W_l^T run register-resident on the same
// mma.sync fragments, and ldmatrix.trans feeds X_l^T dY_l over the tile.
// The weight gradient stays in the warps' accumulator fragments (each warp
// owns a 16x32 block of every hidden layer) across all the CTA's tiles; at
// the end each CTA stores it into its own slot and one kernel sums the
// slots in a fixed order and takes the Adam step (one atomic add per
// weight per CTA cost as much as the tiles themselves).  Adam runs on FP32
// master weights and refreshes the BF16 copies (training weights, and the
// moving average the queries use).
#include <cmath>
#include <cstring>

#include "nrc.cuh"
#include "nrc_mma.cuh"
#include "track.cuh"

namespace vcr {

using bf16 = __nv_bfloat16;

// Training CTA: 8 warps, 16 records each, one 128-record tile at a time.
constexpr int kTrainWarps = 8;
constexpr int kTrainThreads = kTrainWarps * 32;
constexpr int kTrainTile = kTrainWarps * 16;

constexpr int kTileX = kTrainTile * kLdX;                                  // one activation tile

struct NrcView {
  const bf16* wb;   // training weights
  const bf16* wbi;  // inference weights (the moving average, or wb)
  f3 b0, inv_ext;
  int levels;       // position-encoding levels the network sees (the rest are 0)
  // grid encoding (nullptr: the frequency encoding): the tables training
  // reads, the tables queries read (their moving average, or gtab), and the
  // tables' gradient accumulator
  const float* gtab;
  const float* gtab_i;
  float* ggrad;
};

// ---------------------------------------------------------------------------
// inference: sum[pix] += throughput * max(cache(x, view, sun), 0); out (if
// given) receives the 3 outputs.  Register-resident forward (nrc_mma.cuh):
// every warp runs whole 16-sample tiles, the CTA shares only the weights.
// ---------------------------------------------------------------------------
constexpr int kInferThreads = 256;

__global__ void __launch_bounds__(kInferThreads, 3) nrc_infer_kernel(NrcView v, const NrcRecord* __restrict__ recs,
                                                                     const uint32_t* __restrict__ count_ptr,
                                                                     uint32_t capacity, double* __restrict__ sum,
                                                                     float* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char smem[];
  bf16* W = reinterpret_cast<bf16*>(smem);
  float* dirs = reinterpret_cast<float*>(W + kWs);  // 16 level directions
  load_weights<kInferThreads>(v.wbi, W);
  load_level_dirs(dirs);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t count = min(*count_ptr, capacity);
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16u < count; tile += warps) {
    const uint32_t i0 = tile * 16u + (uint32_t)g, i1 = i0 + 8u;
    NrcRecord r0{}, r1{};
    if (i0 < count) r0 = recs[i0];
    if (i1 < count) r1 = recs[i1];
    uint32_t a[4][4];
    encode_a(r0, i0 < count, v.b0, v.inv_ext, dirs, t, 0, a, v.levels, v.gtab_i);
    encode_a(r1, i1 < count, v.b0, v.inv_ext, dirs, t, 1, a, v.levels, v.gtab_i);
    float yg[3], yh[3];
    mlp_forward_mma(W, a, lane, yg, yh);
    if (t == 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint32_t idx = h ? i1 : i0;
        if (idx >= count) continue;
        const NrcRecord& r = h ? r1 : r0;
        const float* y = h ? yh : yg;
        if (out) {
          out[3 * idx] = y[0];
          out[3 * idx + 1] = y[1];
          out[3 * idx + 2] = y[2];
        }
        if (sum) {
          double* o = sum + 3 * (size_t)r.pix;
          atomicAdd(o + 0, (double)(r.w0 * fmaxf(y[0], 0.0f)));
          atomicAdd(o + 1, (double)(r.w1 * fmaxf(y[1], 0.0f)));
          atomicAdd(o + 2, (double)(r.w2 * fmaxf(y[2], 0.0f)));
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// training: relative L2 loss sum_c (y - t)^2 / (sg(y)^2 + 0.01) / (3 B)
// ---------------------------------------------------------------------------

// The lane's four BF16 pairs of an A fragment (rows g, g+8; columns 2t and
// 8+2t of each 16-column tile kt) to / from a [record][feature] tile with
// kLdX rows: 4-byte accesses on 32 distinct banks.
__device__ __forceinline__ void store_a(bf16* T, int row, int t, const uint32_t (&a)[4][4], int tiles) {
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    if (kt >= tiles) break;
    uint32_t* p0 = reinterpret_cast<uint32_t*>(T + row * kLdX + kt * 16 + 2 * t);
    uint32_t* p1 = reinterpret_cast<uint32_t*>(T + (row + 8) * kLdX + kt * 16 + 2 * t);
    p0[0] = a[kt][0];
    p1[0] = a[kt][1];
    p0[4] = a[kt][2];
    p1[4] = a[kt][3];
  }
}

// One 8-warp CTA per SM; a 128-record tile at a time, 16 records per warp.
// The forward keeps a warp's activations in its MMA fragments (as the
// queries do) and stores each layer's input X_l once, as BF16, into the
// tile's shared [record][feature] buffers; the backward runs dY_l W_l^T in
// registers as well (the dY A fragments of one layer are the masked
// accumulators of the last), so only X_l and dY_l go through shared memory,
// for the weight gradient dW_l = X_l^T dY_l over all 128 records.  Warp w
// owns the 16 x 32 block (rows 16(w/2).., columns 32(w%2)..) of every 64x64
// hidden-layer gradient and the 16 x 8 block (rows 16(w/2).., columns
// 8(w%2)..) of the 64x16 output layer's, in registers across the CTA's
// tiles; X_l^T and dY_l fragments come from ldmatrix.trans.  At the end each
// CTA stores its gradient into its own slot of gpart.
//
// kGrid (the grid encoding): the backward also forms dX_0 = dY_0 W_0^T for
// the 32 position inputs in registers and adds, for every record, level and
// feature, the 8 trilinear shares of it into the tables' gradient (float
// atomics, so their order, and the last bits of the sums, vary).
template <bool kGrid>
__global__ void __launch_bounds__(kTrainThreads, 1) nrc_train_kernel(NrcView v, const NrcRecord* __restrict__ recs,
                                                                     const uint32_t* __restrict__ count_ptr,
                                                                     uint32_t capacity, uint32_t first_rec,
                                                                     float* __restrict__ gpart, float* __restrict__ loss) {
  extern __shared__ __align__(128) unsigned char smem[];
  bf16* W = reinterpret_cast<bf16*>(smem);              // [in][out], rows of ldw(l)
  bf16* X = W + kWs;                                     // X_0 .. X_5 of the tile
  bf16* D = X + kNrcLayers * kTileX;                     // dY ping-pong: 2 tiles
  float* dirs = reinterpret_cast<float*>(D + 2 * kTileX);  // 16 position-level directions
  // records [first_rec, first_rec + capacity) of the *count_ptr written; a
  // CTA without a tile leaves its slot alone (the reduction reads the slots
  // of the first ceil(count / kTrainTile) CTAs only)
  const uint32_t total = *count_ptr;
  const uint32_t count = total > first_rec ? min(total - first_rec, capacity) : 0u;
  if (blockIdx.x * kTrainTile >= count) return;
  load_weights<kTrainThreads>(v.wb, W);
  load_level_dirs(dirs);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int rr = lane & 7, q = lane >> 3;
  const int mt = warp >> 1, half = warp & 1;  // the warp's gradient blocks
  float dwh[kNrcHidden][4][4], dwo[4];
#pragma unroll
  for (int l = 0; l < kNrcHidden; ++l)
#pragma unroll
    for (int j = 0; j < 4; ++j) dwh[l][j][0] = dwh[l][j][1] = dwh[l][j][2] = dwh[l][j][3] = 0.0f;
  dwo[0] = dwo[1] = dwo[2] = dwo[3] = 0.0f;
  __syncthreads();
  recs += first_rec;
  const float inv_n = 1.0f / (3.0f * (float)max(count, 1u));
  float loss_local = 0.0f;
  const int row = warp * 16 + g;  // the lane's tile rows: row and row + 8
  for (uint32_t first = blockIdx.x * kTrainTile; first < count; first += gridDim.x * kTrainTile) {
    const uint32_t i0 = first + (uint32_t)row, i1 = i0 + 8u;
    uint32_t a[4][4];
    {
      NrcRecord r0{}, r1{};
      if (i0 < count) r0 = recs[i0];
      if (i1 < count) r1 = recs[i1];
      encode_a(r0, i0 < count, v.b0, v.inv_ext, dirs, t, 0, a, v.levels, kGrid ? v.gtab : nullptr);
      encode_a(r1, i1 < count, v.b0, v.inv_ext, dirs, t, 1, a, v.levels, kGrid ? v.gtab : nullptr);
    }
    store_a(X, row, t, a, 4);
#pragma unroll 1
    for (int l = 0; l < kNrcHidden; ++l) {
      float acc[8][4];
      mma_layer_in_out<8>(W + woff(l), ldw(l), a, acc, lane);
      relu_to_a(acc, a);
      store_a(X + (l + 1) * kTileX, row, t, a, 4);
    }
    // output layer and the loss gradient dY_5 (columns 0..2 of 16)
    uint32_t da[4][4];
    {
      float out[2][4];
      mma_layer_in_out<2>(W + woff(kNrcHidden), ldw(kNrcHidden), a, out, lane);
      float d5[4];  // (row, 2t), (row, 2t+1), (row+8, 2t), (row+8, 2t+1)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint32_t idx = h ? i1 : i0;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int c = 2 * t + e;
          float gval = 0.0f;
          if (c < kNrcOut && idx < count) {
            const NrcRecord& rec = recs[idx];
            const float tv = c == 0 ? rec.w0 : (c == 1 ? rec.w1 : rec.w2);
            const float y = out[0][2 * h + e];
            const float den = y * y + 0.01f;
            const float diff = y - tv;
            loss_local += (diff * diff / den) * inv_n;
            gval = (2.0f * diff / den) * inv_n;
          }
          d5[2 * h + e] = gval;
        }
      }
      da[0][0] = pack_bf16(d5[0], d5[1]);
      da[0][1] = pack_bf16(d5[2], d5[3]);
      da[0][2] = 0u;  // columns 8..15: padding
      da[0][3] = 0u;
      store_a(D, row, t, da, 1);  // dY_5 in buffer 0
    }
    // backward through layers 5..0 (unrolled: the gradient blocks are indexed by layer)
#pragma unroll
    for (int l = kNrcLayers - 1; l >= 0; --l) {
      const bf16* Xl = X + l * kTileX;
      const bf16* Dl = D + ((kNrcLayers - 1 - l) & 1) * kTileX;  // dY_5 in buffer 0, dY_4 in 1, ...
      __syncthreads();                                           // X_l and dY_l complete for every row
      // dW_l += X_l^T dY_l over the tile's 128 records (k)
#pragma unroll 2
      for (int kt = 0; kt < kTrainTile / 16; ++kt) {
        uint32_t xa[4];  // X_l^T rows 16mt.. (features), columns 16kt.. (records)
        ldsm_x4_t(xa, Xl + (kt * 16 + rr + 8 * (q >> 1)) * kLdX + mt * 16 + 8 * (q & 1));
        if (l == kNrcLayers - 1) {
          uint32_t b[2];  // dY_5 records 16kt.., columns 8 half..
          ldsm_x2_t(b, Dl + (kt * 16 + rr + 8 * (q & 1)) * kLdX + half * 8);
          mma_bf16(dwo, xa, b[0], b[1]);
        } else {
#pragma unroll
          for (int np = 0; np < 2; ++np) {
            uint32_t b[4];  // dY_l records 16kt.., columns 32 half + 16 np ..
            ldsm_x4_t(b, Dl + (kt * 16 + rr + 8 * (q & 1)) * kLdX + half * 32 + np * 16 + 8 * (q >> 1));
            mma_bf16(dwh[l < kNrcHidden ? l : 0][2 * np], xa, b[0], b[1]);
            mma_bf16(dwh[l < kNrcHidden ? l : 0][2 * np + 1], xa, b[2], b[3]);
          }
        }
      }
      if (l > 0) {
        // dY_{l-1} = (dY_l W_l^T) * (X_l > 0) for the warp's rows, in registers
        const bf16* Wl = W + woff(l);
        const int ld = ldw(l), ktiles = nrc_layer_cols(l) / 16;
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
          if (kt >= ktiles) break;
#pragma unroll
          for (int np = 0; np < 4; ++np) {
            uint32_t b[4];  // W_l rows (in) 16np.., columns (out) 16kt..: (in, out), (in, out+8), (in+8, out), (in+8, out+8)
            ldsm_x4(b, Wl + (np * 16 + rr + 8 * (q >> 1)) * ld + kt * 16 + 8 * (q & 1));
            mma_bf16(acc[2 * np], da[kt], b[0], b[1]);
            mma_bf16(acc[2 * np + 1], da[kt], b[2], b[3]);
          }
        }
        bf16* Dn = D + ((kNrcLayers - l) & 1) * kTileX;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
          const uint32_t* h0 = reinterpret_cast<const uint32_t*>(Xl + row * kLdX + kt * 16 + 2 * t);
          const uint32_t* h1 = reinterpret_cast<const uint32_t*>(Xl + (row + 8) * kLdX + kt * 16 + 2 * t);
          const uint32_t hv[4] = {h0[0], h1[0], h0[4], h1[4]};
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const __nv_bfloat162 hq = *reinterpret_cast<const __nv_bfloat162*>(&hv[p]);
            const float* y = &acc[2 * kt + (p >> 1)][2 * (p & 1)];
            const float m0 = __low2float(hq) > 0.0f ? 1.0f : 0.0f, m1 = __high2float(hq) > 0.0f ? 1.0f : 0.0f;
            da[kt][p] = pack_bf16(y[0] * m0, y[1] * m1);
          }
        }
        store_a(Dn, row, t, da, 4);
      } else if (kGrid) {
        // dX_0 for inputs 0..31 (n-tiles 0..3): acc[nt] holds (row, 8nt+2t+e)
        // and (row+8, 8nt+2t+e), i.e. level 4nt+t, feature e
        const bf16* W0 = W + woff(0);
        float acc[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
          for (int np = 0; np < 2; ++np) {
            uint32_t b[4];
            ldsm_x4(b, W0 + (np * 16 + rr + 8 * (q >> 1)) * ldw(0) + kt * 16 + 8 * (q & 1));
            mma_bf16(acc[2 * np], da[kt], b[0], b[1]);
            mma_bf16(acc[2 * np + 1], da[kt], b[2], b[3]);
          }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t idx = h ? i1 : i0;
          if (idx >= count) continue;
          const NrcRecord& rec = recs[idx];
          float ux, uy, uz;
          nrc_box_coords(rec, v.b0, v.inv_ext, ux, uy, uz);
#pragma unroll
          for (int nt = 0; nt < 4; ++nt) {
            const int lv = 4 * nt + t;
            if (lv >= v.levels) continue;
            const float d0 = acc[nt][2 * h], d1 = acc[nt][2 * h + 1];
            const int n = nrc_grid_res(lv);
            const NrcGridCell c = nrc_grid_cell(n, ux, uy, uz);
            float* gl = v.ggrad + (size_t)lv * kNrcGridTable * 2;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const uint32_t e = nrc_grid_index(n, c.x + (k & 1), c.y + ((k >> 1) & 1), c.z + (k >> 2));
              const float w = nrc_grid_weight(c, k);
              atomicAdd(gl + 2 * e, w * d0);
              atomicAdd(gl + 2 * e + 1, w * d1);
            }
          }
        }
      }
    }
    __syncthreads();  // every warp is done with X_0 and dY_0 before the next tile's
  }
  // the CTA's gradient ([in][out] layout per layer) into its own slot of
  // gpart, every weight written (the warps' blocks cover each layer once);
  // nrc_grad_reduce_kernel sums the slots in a fixed order
  float* slot = gpart + (size_t)blockIdx.x * kNrcWeightCount;
#pragma unroll
  for (int l = 0; l < kNrcHidden; ++l)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float* base = slot + nrc_layer_offset(l) + (mt * 16 + g) * kNrcWidth + half * 32 + j * 8 + 2 * t;
      *reinterpret_cast<float2*>(base) = make_float2(dwh[l][j][0], dwh[l][j][1]);
      *reinterpret_cast<float2*>(base + 8 * kNrcWidth) = make_float2(dwh[l][j][2], dwh[l][j][3]);
    }
  {
    float* base = slot + nrc_layer_offset(kNrcHidden) + (mt * 16 + g) * kNrcOutPad + half * 8 + 2 * t;
    *reinterpret_cast<float2*>(base) = make_float2(dwo[0], dwo[1]);
    *reinterpret_cast<float2*>(base + 8 * kNrcOutPad) = make_float2(dwo[2], dwo[3]);
  }
  for (int o = 16; o > 0; o >>= 1) loss_local += __shfl_xor_sync(0xffffffffu, loss_local, o);
  if (lane == 0) atomicAdd(loss, loss_local);
}

// The optimiser state Adam updates, and the hyper-parameters of one step
// (bias corrections c1 = 1 - b1^t, c2 = 1 - b2^t; moving-average decay).
struct AdamView {
  float* w;
  bf16* wb;
  float* m;
  float* v;
  float* ema;
  bf16* wbi;
};
struct AdamStep {
  float lr, b1, b2, eps, c1, c2, decay;
};

constexpr int kReduceCols = 64;    // weights per reduction CTA
constexpr int kReduceGroups = 4;   // slot groups per weight (b mod 4)
constexpr int kReduceUnroll = 8;   // independent loads in flight per thread
static_assert(kNrcWeightCount % kReduceCols == 0, "reduction tiling");

// Sums the slots of the CTAs that had records (the first
// ceil(count / kTrainTile)) in a fixed order: thread group g adds slots
// g, g+4, g+8, ... into eight partial sums (slot g + 4u + 32k into sum u),
// combined pairwise, then the four groups in order.  Without kAdam the sum
// is added to grad; with kAdam the Adam step follows on grad + sum and grad
// is cleared.  One launch of kNrcWeightCount / 64 CTAs: every weight's 152
// loads are spread over four threads with eight in flight each.  Its first
// thread also moves the step's loss sum to loss[1] and clears loss[0] for
// the next step's training kernel.
template <bool kAdam>
__global__ void __launch_bounds__(kReduceCols * kReduceGroups)
    nrc_grad_reduce_kernel(const float* __restrict__ gpart, int blocks, const uint32_t* __restrict__ count_ptr,
                           uint32_t capacity, uint32_t first_rec, float* __restrict__ grad, AdamView a, AdamStep h,
                           float* __restrict__ loss) {
  __shared__ float part[kReduceGroups][kReduceCols];
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // the step's loss, and a zero sum for the next step
    loss[1] = loss[0];
    loss[0] = 0.0f;
  }
  const int col = threadIdx.x % kReduceCols, grp = threadIdx.x / kReduceCols;
  const int i = blockIdx.x * kReduceCols + col;
  const uint32_t total = *count_ptr;
  const uint32_t count = total > first_rec ? min(total - first_rec, capacity) : 0u;
  const int active = (int)min((uint32_t)blocks, (count + kTrainTile - 1) / kTrainTile);
  float s[kReduceUnroll];
#pragma unroll
  for (int u = 0; u < kReduceUnroll; ++u) s[u] = 0.0f;
  constexpr int kStride = kReduceGroups * kReduceUnroll;
  int b = grp;
  for (; b + kStride - kReduceGroups < active; b += kStride) {
    float x[kReduceUnroll];
#pragma unroll
    for (int u = 0; u < kReduceUnroll; ++u) x[u] = gpart[(size_t)(b + kReduceGroups * u) * kNrcWeightCount + i];
#pragma unroll
    for (int u = 0; u < kReduceUnroll; ++u) s[u] += x[u];
  }
#pragma unroll
  for (int u = 0; u < kReduceUnroll; ++u)  // the last slots of the group: < 8 of them
    if (b + kReduceGroups * u < active) s[u] += gpart[(size_t)(b + kReduceGroups * u) * kNrcWeightCount + i];
  part[grp][col] = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
  __syncthreads();
  if (grp != 0) return;
  const float sum = (part[0][col] + part[1][col]) + (part[2][col] + part[3][col]);
  if (!kAdam) {
    grad[i] += sum;
    return;
  }
  const float gi = grad[i] + sum;
  const float mi = h.b1 * a.m[i] + (1.0f - h.b1) * gi;
  const float vi = h.b2 * a.v[i] + (1.0f - h.b2) * gi * gi;
  a.m[i] = mi;
  a.v[i] = vi;
  const float wi = a.w[i] - h.lr * (mi / h.c1) / (sqrtf(vi / h.c2) + h.eps);
  a.w[i] = wi;
  a.wb[i] = __float2bfloat16_rn(wi);
  grad[i] = 0.0f;
  if (a.ema) {
    const float e = h.decay * a.ema[i] + (1.0f - h.decay) * wi;
    a.ema[i] = e;
    a.wbi[i] = __float2bfloat16_rn(e);
  }
}

__global__ void nrc_copy_weights_kernel(const float* __restrict__ w, float* __restrict__ ema, bf16* __restrict__ wbi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kNrcWeightCount) {
    ema[i] = w[i];
    wbi[i] = __float2bfloat16_rn(w[i]);
  }
}

__global__ void nrc_to_bf16_kernel(const float* __restrict__ w, bf16* __restrict__ wb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kNrcWeightCount) wb[i] = __float2bfloat16_rn(w[i]);
}

// Adam step on the grid encoding's tables (step size h.lr x
// kNrcGridLrScale), clearing their gradient; the moving average as for the
// weights.
__global__ void nrc_grid_adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                                     float* __restrict__ grad, float* __restrict__ ema, AdamStep h) {
  const float lr = h.lr * kNrcGridLrScale;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < kNrcGridParams;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = grad[i];
    const float mi = h.b1 * m[i] + (1.0f - h.b1) * gi;
    const float vi = h.b2 * v[i] + (1.0f - h.b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / h.c1) / (sqrtf(vi / h.c2) + h.eps);
    w[i] = wi;
    grad[i] = 0.0f;
    if (ema) ema[i] = h.decay * ema[i] + (1.0f - h.decay) * wi;
  }
}

// The tables' initial values: uniform in [-1e-4, 1e-4] from a seeded hash
// (the moving average starts equal).
__global__ void nrc_grid_init_kernel(float* __restrict__ w, float* __restrict__ ema, uint32_t seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < kNrcGridParams;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t hsh = pcg_hash(seed ^ 0x9E3779B9u ^ pcg_hash((uint32_t)i));
    const float u = (float)(hsh >> 8) * 5.96046448e-08f;  // [0,1)
    const float x = (2.0f * u - 1.0f) * 1e-4f;
    w[i] = x;
    if (ema) ema[i] = x;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t infer_smem() { return (size_t)kWs * 2 + kNrcPosLevels * 3 * sizeof(float); }
static size_t train_smem() {
  return (size_t)kWs * 2 + (size_t)(kNrcLayers + 2) * kTileX * 2 + kNrcPosLevels * 3 * sizeof(float);
}

size_t nrc_param_count(const NrcState* st) {
  return (size_t)kNrcWeightCount + (st && st->gw ? kNrcGridParams : 0);
}

NrcView nrc_view(const vcr_ctx* ctx) {
  NrcView v;
  v.wb = reinterpret_cast<const bf16*>(ctx->nrc->wb);
  v.wbi = reinterpret_cast<const bf16*>(ctx->nrc->wbi ? ctx->nrc->wbi : ctx->nrc->wb);
  const vcr_cloud& c = ctx->cloud;
  v.b0 = mk(c.bounds_min[0], c.bounds_min[1], c.bounds_min[2]);
  v.inv_ext = mk(1.0f / (c.bounds_max[0] - c.bounds_min[0]), 1.0f / (c.bounds_max[1] - c.bounds_min[1]),
                 1.0f / (c.bounds_max[2] - c.bounds_min[2]));
  v.levels = kNrcPosLevels - (int)ctx->nrc->prm.position_drop;
  const NrcState* st = ctx->nrc;
  v.gtab = st->gw;
  v.gtab_i = st->gema ? st->gema : st->gw;
  v.ggrad = st->ggrad;
  return v;
}

void nrc_free(vcr_ctx* ctx) {
  NrcState* st = ctx->nrc;
  if (!st) return;
  void* ptrs[] = {st->w,      st->wb,          st->m,     st->v,           st->grad, st->gpart, st->ema,
                  st->wbi,    st->loss,        st->train, st->train_count, st->query, st->query_count,
                  st->gw,     st->gm,          st->gv,    st->ggrad,       st->gema};
  for (void* p : ptrs) cudaFree(p);
  delete st;
  ctx->nrc = nullptr;
}

// Kaiming-uniform initial weights from a seeded hash (host).
static void nrc_init_weights(std::vector<float>& w, uint32_t seed) {
  w.assign(kNrcWeightCount, 0.0f);
  uint32_t c = 0;
  for (int l = 0; l < kNrcLayers; ++l) {
    int cols = nrc_layer_cols(l);
    float bound = l < kNrcHidden ? sqrtf(6.0f / (float)kNrcWidth) : sqrtf(1.0f / (float)kNrcWidth);
    for (int i = 0; i < kNrcWidth; ++i)
      for (int o = 0; o < cols; ++o) {
        uint32_t hsh = pcg_hash(seed ^ pcg_hash(c++));
        float u = (float)(hsh >> 8) * 5.96046448e-08f;  // [0,1)
        w[(size_t)nrc_layer_offset(l) + (size_t)i * cols + o] =
            (l == kNrcLayers - 1 && o >= kNrcOut) ? 0.0f : (2.0f * u - 1.0f) * bound;
      }
  }
}

vcr_status nrc_setup(vcr_ctx* ctx, const vcr_nrc_params* p) {
  if (!p || p->train_samples == 0 || p->train_samples > (1u << 22) || !(p->learning_rate > 0.0f) ||
      p->query_capacity == 0 || !(p->ema_decay >= 0.0f && p->ema_decay < 1.0f) ||
      !(p->tail_survival >= 0.0f && p->tail_survival < 1.0f) || p->query_kernel > VCR_NRC_QUERY_TCGEN05 ||
      p->position_drop > (uint32_t)kNrcPosLevels || p->encoding > VCR_NRC_ENCODING_GRID)
    return fail(ctx, VCR_ERR_INVALID,
                "nrc params: train_samples 1..2^22, learning_rate > 0, query_capacity > 0, ema_decay and "
                "tail_survival in [0,1), query_kernel a VCR_NRC_QUERY_* value, position_drop 0..16, encoding a "
                "VCR_NRC_ENCODING_* value");
  nrc_free(ctx);
  NrcState* st = new NrcState();
  ctx->nrc = st;
  st->prm = *p;
  st->query_capacity = p->query_capacity;
  st->train_cap = 2 * p->train_samples;
#define VCR_ALLOC(ptr, bytes) VCR_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(&(ptr)), (bytes)))
  VCR_ALLOC(st->w, kNrcWeightCount * 4);
  VCR_ALLOC(st->wb, kNrcWeightCount * 2);
  VCR_ALLOC(st->m, kNrcWeightCount * 4);
  VCR_ALLOC(st->v, kNrcWeightCount * 4);
  VCR_ALLOC(st->grad, kNrcWeightCount * 4);
  st->gpart_blocks = ctx->sm_count;
  VCR_ALLOC(st->gpart, (size_t)st->gpart_blocks * kNrcWeightCount * 4);
  VCR_ALLOC(st->loss, 8);
  VCR_ALLOC(st->train, (size_t)st->train_cap * sizeof(NrcRecord));
  if (p->ema_decay > 0.0f) {
    VCR_ALLOC(st->ema, kNrcWeightCount * 4);
    VCR_ALLOC(st->wbi, kNrcWeightCount * 2);
  }
  VCR_ALLOC(st->train_count, 4);
  VCR_ALLOC(st->query, (size_t)p->query_capacity * sizeof(NrcRecord));
  VCR_ALLOC(st->query_count, 4);
  if (p->encoding == VCR_NRC_ENCODING_GRID) {
    VCR_ALLOC(st->gw, kNrcGridParams * 4);
    VCR_ALLOC(st->gm, kNrcGridParams * 4);
    VCR_ALLOC(st->gv, kNrcGridParams * 4);
    VCR_ALLOC(st->ggrad, kNrcGridParams * 4);
    if (p->ema_decay > 0.0f) VCR_ALLOC(st->gema, kNrcGridParams * 4);
  }
#undef VCR_ALLOC
  VCR_CUDA(ctx, cudaMemset(st->train_count, 0, 4));
  VCR_CUDA(ctx, cudaMemset(st->loss, 0, 8));
  std::vector<float> w;
  nrc_init_weights(w, p->seed);
  VCR_CUDA(ctx, cudaMemcpy(st->w, w.data(), kNrcWeightCount * 4, cudaMemcpyHostToDevice));
  VCR_CUDA(ctx, cudaMemset(st->m, 0, kNrcWeightCount * 4));
  VCR_CUDA(ctx, cudaMemset(st->v, 0, kNrcWeightCount * 4));
  VCR_CUDA(ctx, cudaMemset(st->grad, 0, kNrcWeightCount * 4));
  VCR_CUDA(ctx, cudaMemset(st->query_count, 0, 4));
  nrc_to_bf16_kernel<<<(kNrcWeightCount + 255) / 256, 256>>>(st->w, reinterpret_cast<bf16*>(st->wb));
  VCR_CUDA(ctx, cudaGetLastError());
  if (st->ema) {
    nrc_copy_weights_kernel<<<(kNrcWeightCount + 255) / 256, 256>>>(st->w, st->ema, reinterpret_cast<bf16*>(st->wbi));
    VCR_CUDA(ctx, cudaGetLastError());
  }
  if (st->gw) {
    VCR_CUDA(ctx, cudaMemset(st->gm, 0, kNrcGridParams * 4));
    VCR_CUDA(ctx, cudaMemset(st->gv, 0, kNrcGridParams * 4));
    VCR_CUDA(ctx, cudaMemset(st->ggrad, 0, kNrcGridParams * 4));
    nrc_grid_init_kernel<<<ctx->sm_count * 8, 256>>>(st->gw, st->gema, p->seed);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_smem()));
  VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_train_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)train_smem()));
  VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_train_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)train_smem()));
  return VCR_OK;
}

// Gradient of the loss over records [first, first + capacity) of the
// *d_count written (device): added to grad, or (adam) followed by one Adam
// step in the same reduction launch.
static vcr_status nrc_grad(vcr_ctx* ctx, const NrcRecord* recs, const uint32_t* d_count, uint32_t capacity,
                           cudaStream_t s, uint32_t first, bool adam) {
  NrcState* st = ctx->nrc;
  const int blocks = st->gpart_blocks;
  if (st->gw) {
    VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_train_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)train_smem()));
    nrc_train_kernel<true><<<blocks, kTrainThreads, train_smem(), s>>>(nrc_view(ctx), recs, d_count, capacity, first,
                                                                       st->gpart, st->loss);
  } else {
    VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_train_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)train_smem()));
    nrc_train_kernel<false><<<blocks, kTrainThreads, train_smem(), s>>>(nrc_view(ctx), recs, d_count, capacity,
                                                                        first, st->gpart, st->loss);
  }
  VCR_CUDA(ctx, cudaGetLastError());
  AdamView a{st->w, reinterpret_cast<bf16*>(st->wb), st->m, st->v, st->ema, reinterpret_cast<bf16*>(st->wbi)};
  AdamStep h{};
  if (adam) {
    st->step += 1;
    h.lr = st->prm.learning_rate;
    h.b1 = 0.9f;
    h.b2 = 0.99f;
    h.eps = 1e-8f;
    h.c1 = 1.0f - (float)std::pow(0.9, (double)st->step);
    h.c2 = 1.0f - (float)std::pow(0.99, (double)st->step);
    // moving-average decay ramps up over the first steps: min(d, (1+k)/(10+k))
    h.decay = std::min(st->prm.ema_decay, (1.0f + (float)st->step) / (10.0f + (float)st->step));
  }
  const dim3 grid(kNrcWeightCount / kReduceCols), block(kReduceCols * kReduceGroups);
  if (adam)
    nrc_grad_reduce_kernel<true><<<grid, block, 0, s>>>(st->gpart, blocks, d_count, capacity, first, st->grad, a, h,
                                                        st->loss);
  else
    nrc_grad_reduce_kernel<false><<<grid, block, 0, s>>>(st->gpart, blocks, d_count, capacity, first, st->grad, a, h,
                                                         st->loss);
  VCR_CUDA(ctx, cudaGetLastError());
  if (adam && st->gw) {
    nrc_grid_adam_kernel<<<ctx->sm_count * 8, 256, 0, s>>>(st->gw, st->gm, st->gv, st->ggrad, st->gema, h);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  return VCR_OK;
}

// BF16 copies from the FP32 master weights and their moving average (after
// the FP32 state was written from outside, e.g. a checkpoint).
vcr_status nrc_refresh_copies(vcr_ctx* ctx) {
  NrcState* st = ctx->nrc;
  nrc_to_bf16_kernel<<<(kNrcWeightCount + 255) / 256, 256>>>(st->w, reinterpret_cast<bf16*>(st->wb));
  VCR_CUDA(ctx, cudaGetLastError());
  if (st->ema) {
    nrc_to_bf16_kernel<<<(kNrcWeightCount + 255) / 256, 256>>>(st->ema, reinterpret_cast<bf16*>(st->wbi));
    VCR_CUDA(ctx, cudaGetLastError());
  }
  return VCR_OK;
}

uint32_t nrc_query_capacity(const vcr_ctx* ctx) { return ctx->nrc ? ctx->nrc->query_capacity : 0u; }

vcr_status nrc_reset_queries(vcr_ctx* ctx, cudaStream_t s) {
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->nrc->query_count, 0, 4, s));
  return VCR_OK;
}

// Which kernel serves the queries (vcr_nrc_params.query_kernel).
static bool use_tc(const NrcState* st) { return st->prm.query_kernel == VCR_NRC_QUERY_TCGEN05; }

vcr_status nrc_infer_queries(vcr_ctx* ctx, cudaStream_t s) {
  NrcState* st = ctx->nrc;
  if (use_tc(st)) {
    const NrcView v = nrc_view(ctx);
    return nrc_infer_tc_launch(ctx, v.wbi, v.b0, v.inv_ext, v.levels, v.gtab_i, st->query, st->query_count,
                               st->query_capacity, ctx->d_sum, nullptr, s);
  }
  VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_smem()));
  int per_sm = 0;
  VCR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nrc_infer_kernel, kInferThreads, infer_smem()));
  int blocks = ctx->sm_count * std::max(per_sm, 1);
  nrc_infer_kernel<<<blocks, kInferThreads, infer_smem(), s>>>(nrc_view(ctx), st->query, st->query_count,
                                                               st->query_capacity, ctx->d_sum, nullptr);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

static vcr_status nrc_check_scene(vcr_ctx* ctx, const char* who) {
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "%s needs vcr_nrc_setup", who);
  if (!ctx->has_grid || !ctx->has_cloud || !ctx->has_cam || !ctx->has_params || !ctx->d_sum)
    return fail(ctx, VCR_ERR_STATE, "%s needs a grid, cloud, camera, params and frame", who);
  return VCR_OK;
}

static bool nrc_calibrated(const vcr_ctx* ctx) {
  const NrcState* st = ctx->nrc;
  return st->npaths && !memcmp(&st->calib_cam, &ctx->cam, sizeof(vcr_camera)) &&
         !memcmp(&st->calib_cloud, &ctx->cloud, sizeof(vcr_cloud)) && st->calib_w == ctx->width &&
         st->calib_h == ctx->height;
}

// Training paths: extended paths from uniformly drawn pixels that record
// the radiance leaving each of their first kNrcRecordEvents scattering
// vertices toward the previous vertex, target_i = (L_total - L_before_i) /
// beta_i.  They run in the persistent wavefront kernel, alone
// (vcr_nrc_train_step) or as the first work items of a pass (vcr_nrc_frame),
// where their long paths overlap the pass's short ones.  The first step for
// a camera/cloud/frame calibrates the path count so that a step yields
// about train_samples records (synchronises once; deterministic, as the
// yield of a seeded launch is).  A step with pass.spp = S > 1 traces S
// sets of paths in its one launch: a training-only launch is as long as
// its longest path, so S sets take far less than S launches (0.95 ms for
// four sets against 0.65 ms for one on the 1920x1080 cloud scene).
static NrcTrainSink nrc_sink(vcr_ctx* ctx) {
  NrcState* st = ctx->nrc;
  return NrcTrainSink{st->train, st->train_count, st->train_cap, st->npaths, st->prm.tail_survival};
}

static vcr_status nrc_launch_training(vcr_ctx* ctx, const PassView& pv, uint32_t paths, cudaStream_t s) {
  NrcTrainSink ts = nrc_sink(ctx);
  ts.paths = paths;
  VCR_CUDA(ctx, cudaMemsetAsync(ts.count, 0, 4, s));
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 5 * sizeof(unsigned long long), s));
  return wavefront_launch(ctx, grid_view(ctx), scene_view(ctx), cam_view(ctx->cam), pv, nullptr,
                          Counters{ctx->d_counters}, 0u, s, &ts);
}

static vcr_status nrc_calibrate(vcr_ctx* ctx, const PassView& pv, cudaStream_t s) {
  NrcState* st = ctx->nrc;
  const uint32_t want = st->prm.train_samples, paths = std::max(1u, want / 2);
  vcr_status vs = nrc_launch_training(ctx, pv, paths, s);
  if (vs) return vs;
  uint32_t got = 0;
  VCR_CUDA(ctx, cudaMemcpyAsync(&got, st->train_count, 4, cudaMemcpyDeviceToHost, s));
  VCR_CUDA(ctx, cudaStreamSynchronize(s));
  double n = std::ceil((double)paths * (double)want / (double)std::max(got, 1u));
  st->npaths = (uint32_t)std::min(std::max(n, (double)std::max(1u, want / 4)), 16.0 * (double)want);
  st->calib_cam = ctx->cam;
  st->calib_cloud = ctx->cloud;
  st->calib_w = ctx->width;
  st->calib_h = ctx->height;
  return VCR_OK;
}

// Loss gradient over the step's records, then Adam.
static vcr_status nrc_update(vcr_ctx* ctx, cudaStream_t s, uint32_t first = 0, uint32_t limit = 0) {
  NrcState* st = ctx->nrc;
  return nrc_grad(ctx, st->train, st->train_count, limit ? limit : st->train_cap, s, first, true);
}

// Record room for `sets` training sets; growing the buffer synchronises.
static vcr_status nrc_reserve_sets(vcr_ctx* ctx, uint32_t sets) {
  NrcState* st = ctx->nrc;
  const uint64_t cap = 2ull * st->prm.train_samples * sets;
  if (sets > kNrcMaxSets || cap > (1ull << 25))
    return fail(ctx, VCR_ERR_INVALID, "training sets (pass.spp) 1..%u with sets x train_samples <= 2^24", kNrcMaxSets);
  if (cap <= st->train_cap) return VCR_OK;
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  VCR_CUDA(ctx, cudaFree(st->train));
  st->train = nullptr;
  st->train_cap = 0;
  VCR_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(&st->train), (size_t)cap * sizeof(NrcRecord)));
  st->train_cap = (uint32_t)cap;
  return VCR_OK;
}

vcr_status nrc_train_step(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t s) {
  vcr_status vs = nrc_check_scene(ctx, "vcr_nrc_train_step");
  if (vs) return vs;
  PassView pv;
  vs = make_pass_view(ctx, pass, pv);
  if (vs) return vs;
  const uint32_t sets = pv.spp;
  vs = nrc_reserve_sets(ctx, sets);
  if (vs) return vs;
  NrcState* st = ctx->nrc;
  if (!nrc_calibrated(ctx)) {
    vs = nrc_calibrate(ctx, pv, s);  // its records serve a one-set step
    if (!vs && sets > 1) vs = nrc_launch_training(ctx, pv, st->npaths * sets, s);
  } else {
    vs = nrc_launch_training(ctx, pv, st->npaths * sets, s);
  }
  if (vs) return vs;
  st->records = true;
  st->sets = sets;
  // one set: a step over all its records; several: over the first
  // train_samples, and vcr_nrc_train_more continues after them
  vs = sets == 1 ? nrc_update(ctx, s) : nrc_update(ctx, s, 0, st->prm.train_samples);
  if (vs) return vs;
  st->cursor = sets == 1 ? 0u : st->prm.train_samples;
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  return VCR_OK;
}

// One frame of the cached tracker: one wavefront launch runs this frame's
// training paths first and the pass's camera paths after them (the latter
// end in the cache at nrc_events, queried with the weights before this
// frame's update), then the loss gradient and Adam.  Same result as
// vcr_pt_pass followed by vcr_nrc_train_step with the same pass.
vcr_status nrc_frame(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t s) {
  vcr_status vs = nrc_check_scene(ctx, "vcr_nrc_frame");
  if (vs) return vs;
  if (ctx->params.nrc_events == 0 || ctx->params.tracker != VCR_TRACKER_DDA)
    return fail(ctx, VCR_ERR_STATE, "vcr_nrc_frame needs the DDA tracker and params.nrc_events > 0");
  PassView pv;
  vs = make_pass_view(ctx, pass, pv);
  if (vs) return vs;
  if (!nrc_calibrated(ctx)) {  // the calibration synchronises: training launch first, then the pass
    vs = nrc_calibrate(ctx, pv, s);
    if (vs) return vs;
    vs = pt_pass_launch(ctx, pass, s);
  } else {
    NrcTrainSink ts = nrc_sink(ctx);
    VCR_CUDA(ctx, cudaMemsetAsync(ts.count, 0, 4, s));
    vs = pt_pass_launch(ctx, pass, s, &ts);
  }
  if (vs) return vs;
  ctx->nrc->records = true;
  ctx->nrc->sets = 1;
  ctx->nrc->cursor = 0;
  vs = nrc_update(ctx, s);
  if (vs) return vs;
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_nrc_setup(vcr_ctx* ctx, const vcr_nrc_params* p) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  vcr_status st = nrc_setup(ctx, p);
  if (st) return st;
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_nrc_free(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaDeviceSynchronize();
  nrc_free(ctx);
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_nrc_train_step(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  return nrc_train_step(ctx, pass, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_nrc_train_more(vcr_ctx* ctx, uint32_t steps, uint32_t max_records,
                                                 void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  if (!ctx->nrc->records)
    return fail(ctx, VCR_ERR_STATE, "no training records (vcr_nrc_train_step or vcr_nrc_frame first)");
  cudaStream_t s = (cudaStream_t)stream;
  NrcState* st = ctx->nrc;
  const uint32_t want = st->prm.train_samples * st->sets;
  const uint32_t batch = (max_records && max_records < want) ? max_records : 0u;
  for (uint32_t k = 0; k < steps; ++k) {
    // consecutive steps, and consecutive calls, walk through the records
    // batch by batch, from the start again after the last whole batch
    if (batch && st->cursor + batch > want) st->cursor = 0;
    vcr_status vs = batch ? nrc_update(ctx, s, st->cursor, batch) : nrc_update(ctx, s);
    if (vs) return vs;
    if (batch) st->cursor += batch;
  }
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_nrc_set_learning_rate(vcr_ctx* ctx, float learning_rate) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  if (!(learning_rate > 0.0f) || !std::isfinite(learning_rate))
    return fail(ctx, VCR_ERR_INVALID, "learning rate must be finite and > 0");
  ctx->nrc->prm.learning_rate = learning_rate;  // read on the host when the next step is enqueued
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_nrc_frame(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  return nrc_frame(ctx, pass, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_nrc_info(vcr_ctx* ctx, vcr_nrc_info_t* out) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  NrcState* st = ctx->nrc;
  if (!st) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  float loss = 0.0f;
  uint32_t ntrain = 0, nq = 0;
  VCR_CUDA(ctx, cudaMemcpy(&loss, st->loss + 1, 4, cudaMemcpyDeviceToHost));
  VCR_CUDA(ctx, cudaMemcpy(&ntrain, st->train_count, 4, cudaMemcpyDeviceToHost));
  VCR_CUDA(ctx, cudaMemcpy(&nq, st->query_count, 4, cudaMemcpyDeviceToHost));
  out->steps = st->step;
  out->last_loss = loss;
  out->train_records = std::min(ntrain, st->train_cap);
  out->queries = std::min(nq, st->query_capacity);
  out->weights = (uint32_t)nrc_param_count(st);
  return VCR_OK;
}

// `count` is the network's weight count, or (grid encoding) the full
// parameter count with the tables after the weights.
static vcr_status nrc_check_count(vcr_ctx* ctx, size_t count) {
  const size_t all = nrc_param_count(ctx->nrc);
  if (count != (size_t)kNrcWeightCount && count != all)
    return fail(ctx, VCR_ERR_INVALID, "the cache has %d weights (%zu parameters with the grid tables)",
                kNrcWeightCount, all);
  return VCR_OK;
}

// Weights: FP32 master copy in the layer layout of vcr_nrc_params.
extern "C" VCR_API vcr_status vcr_nrc_get_weights(vcr_ctx* ctx, float* host, size_t count) {
  if (!ctx || !host) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  vcr_status cs = nrc_check_count(ctx, count);
  if (cs) return cs;
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  VCR_CUDA(ctx, cudaMemcpy(host, ctx->nrc->w, kNrcWeightCount * 4, cudaMemcpyDeviceToHost));
  if (count > (size_t)kNrcWeightCount)
    VCR_CUDA(ctx, cudaMemcpy(host + kNrcWeightCount, ctx->nrc->gw, kNrcGridParams * 4, cudaMemcpyDeviceToHost));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_nrc_set_weights(vcr_ctx* ctx, const float* host, size_t count) {
  if (!ctx || !host) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  vcr_status cs = nrc_check_count(ctx, count);
  if (cs) return cs;
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  VCR_CUDA(ctx, cudaMemcpy(ctx->nrc->w, host, kNrcWeightCount * 4, cudaMemcpyHostToDevice));
  if (count > (size_t)kNrcWeightCount) {
    VCR_CUDA(ctx, cudaMemcpy(ctx->nrc->gw, host + kNrcWeightCount, kNrcGridParams * 4, cudaMemcpyHostToDevice));
    if (ctx->nrc->gema)
      VCR_CUDA(ctx, cudaMemcpy(ctx->nrc->gema, ctx->nrc->gw, kNrcGridParams * 4, cudaMemcpyDeviceToDevice));
  }
  nrc_to_bf16_kernel<<<(kNrcWeightCount + 255) / 256, 256>>>(ctx->nrc->w, reinterpret_cast<bf16*>(ctx->nrc->wb));
  VCR_CUDA(ctx, cudaGetLastError());
  if (ctx->nrc->ema) {
    nrc_copy_weights_kernel<<<(kNrcWeightCount + 255) / 256, 256>>>(ctx->nrc->w, ctx->nrc->ema,
                                                                     reinterpret_cast<bf16*>(ctx->nrc->wbi));
    VCR_CUDA(ctx, cudaGetLastError());
  }
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  return VCR_OK;
}

// Evaluate the cache on n records (device NrcRecord array, 64 B each);
// writes 3 floats per record to d_out.  For tests and tools.
extern "C" VCR_API vcr_status vcr_nrc_forward(vcr_ctx* ctx, const void* d_records, uint32_t n, float* d_out,
                                              void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  if (n == 0) return VCR_OK;
  if (!d_records || !d_out) return fail(ctx, VCR_ERR_INVALID, "null buffer");
  if (!ctx->has_cloud) return fail(ctx, VCR_ERR_STATE, "the encoding needs the cloud box (vcr_set_cloud)");
  cudaStream_t s = (cudaStream_t)stream;
  vcr_status vs = ensure_scratch(ctx, 4);
  if (vs) return vs;
  uint32_t* d_n = reinterpret_cast<uint32_t*>(ctx->d_scratch);
  VCR_CUDA(ctx, cudaMemcpyAsync(d_n, &n, 4, cudaMemcpyHostToDevice, s));
  if (use_tc(ctx->nrc)) {
    const NrcView v = nrc_view(ctx);
    vs = nrc_infer_tc_launch(ctx, v.wbi, v.b0, v.inv_ext, v.levels, v.gtab_i,
                             reinterpret_cast<const NrcRecord*>(d_records), d_n, n, nullptr, d_out, s);
    if (vs) return vs;
  } else {
    VCR_CUDA(ctx, cudaFuncSetAttribute(nrc_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)infer_smem()));
    nrc_infer_kernel<<<ctx->sm_count * 3, kInferThreads, infer_smem(), s>>>(
        nrc_view(ctx), reinterpret_cast<const NrcRecord*>(d_records), d_n, n, nullptr, d_out);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  VCR_CUDA(ctx, cudaStreamSynchronize(s));
  return VCR_OK;
}

// `steps` Adam steps on n caller records (targets in w0..w2).
extern "C" VCR_API vcr_status vcr_nrc_fit(vcr_ctx* ctx, const void* d_records, uint32_t n, uint32_t steps,
                                          void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  if (!d_records || n == 0) return fail(ctx, VCR_ERR_INVALID, "bad fit arguments");
  if (!ctx->has_cloud) return fail(ctx, VCR_ERR_STATE, "the encoding needs the cloud box (vcr_set_cloud)");
  cudaStream_t s = (cudaStream_t)stream;
  vcr_status vs = ensure_scratch(ctx, 4);
  if (vs) return vs;
  uint32_t* d_n = reinterpret_cast<uint32_t*>(ctx->d_scratch);
  VCR_CUDA(ctx, cudaMemcpyAsync(d_n, &n, 4, cudaMemcpyHostToDevice, s));
  for (uint32_t k = 0; k < steps; ++k) {
    vs = nrc_grad(ctx, reinterpret_cast<const NrcRecord*>(d_records), d_n, n, s, 0, true);
    if (vs) return vs;
  }
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  return VCR_OK;
}

// Loss gradient over n records (targets in w0..w2), without an update:
// copies the gradient to host (count = weight count) and returns the loss.
extern "C" VCR_API vcr_status vcr_nrc_gradient(vcr_ctx* ctx, const void* d_records, uint32_t n, float* host_grad,
                                               size_t count, float* out_loss) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->nrc) return fail(ctx, VCR_ERR_STATE, "no radiance cache");
  if (!d_records || !host_grad || n == 0) return fail(ctx, VCR_ERR_INVALID, "bad gradient arguments");
  vcr_status cs = nrc_check_count(ctx, count);
  if (cs) return cs;
  if (!ctx->has_cloud) return fail(ctx, VCR_ERR_STATE, "the encoding needs the cloud box (vcr_set_cloud)");
  vcr_status vs = ensure_scratch(ctx, 4);
  if (vs) return vs;
  uint32_t* d_n = reinterpret_cast<uint32_t*>(ctx->d_scratch);
  VCR_CUDA(ctx, cudaMemcpy(d_n, &n, 4, cudaMemcpyHostToDevice));
  NrcState* st = ctx->nrc;
  VCR_CUDA(ctx, cudaMemset(st->grad, 0, kNrcWeightCount * 4));
  if (st->ggrad) VCR_CUDA(ctx, cudaMemset(st->ggrad, 0, kNrcGridParams * 4));
  vs = nrc_grad(ctx, reinterpret_cast<const NrcRecord*>(d_records), d_n, n, 0, 0, false);
  if (vs) return vs;
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  VCR_CUDA(ctx, cudaMemcpy(host_grad, st->grad, kNrcWeightCount * 4, cudaMemcpyDeviceToHost));
  if (count > (size_t)kNrcWeightCount)
    VCR_CUDA(ctx, cudaMemcpy(host_grad + kNrcWeightCount, st->ggrad, kNrcGridParams * 4, cudaMemcpyDeviceToHost));
  if (out_loss) VCR_CUDA(ctx, cudaMemcpy(out_loss, st->loss + 1, 4, cudaMemcpyDeviceToHost));
  VCR_CUDA(ctx, cudaMemset(st->grad, 0, kNrcWeightCount * 4));
  if (st->ggrad) VCR_CUDA(ctx, cudaMemset(st->ggrad, 0, kNrcGridParams * 4));
  return VCR_OK;
}
