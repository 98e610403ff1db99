// Progressive photon beams: emission, beam segments, LBVH build and refit,
// camera-ray beam gather.
//
// Reference: PPB_PT.comp (main :506-539, generateSunRay :396-430,
// generateAmbientRay :432-445, interactWithMedium :453-501,
// depositPhotonBeam :334-393), PPB_GenerateHierarchy.comp (:62-168),
// PPB_CalculateAABB.comp (:64-120), PPB_PE.comp (traverseTree :408-466,
// accumulateRadiance :362-404), RenderTechniquePPB.cpp (RecordDrawCommands
// :436-519, UpdateRadius :530-546).
//
// Differences from the shipped shaders, all deliberate (the reference's PPB
// never ran end to end): the sun-face choice has its missing `else`
// (PPB_PT.comp:413); beam capacity is enforced; the radius schedule is the
// intended product r_{k+1} = r_k (k + alpha) / (k + 1) (the shader host sums,
// RenderTechniquePPB.cpp:538-544); LBVH leaves keep their primitive and the
// split uses index-augmented prefixes for equal Morton codes; the refit max
// uses the upper bounds (PPB_CalculateAABB.comp:90 used bounds[0]); the
// estimator is the beam x beam 1D one (normalised biweight, 1/sin theta)
// with camera transmittance from 16 free-flight samples along the camera ray,
// the way each beam carries 16 along itself.
//
// Determinism: every photon writes its beams into its own slots; a prefix
// sum over photons places the segments, so the segment order, the sort and
// the BVH are identical from run to run.
#include "track.cuh"
#include "sort.cuh"
#include "ppb.cuh"

namespace vcr {

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums, uint32_t* d_total,
                               cudaStream_t st);

// ---------------------------------------------------------------------------
// emission
// ---------------------------------------------------------------------------
struct PpbEmitView {
  float* slots;         // [P * K * kSlotFloats]
  uint32_t* nbeams;     // [P]
  uint32_t* slot_segs;  // [P * K] segments of each beam
  uint32_t* slot_off;   // [P * K] exclusive prefix inside the photon
  uint32_t* photon_segs;// [P]
  uint32_t photons, K;
  float radius;
  uint32_t seed, pass;
};

__device__ __forceinline__ uint32_t segments_of(float len, float r) {
  float q = len / r;
  uint32_t n = q < (float)(kMaxSegPerBeam - 1) ? (uint32_t)q + 1u : kMaxSegPerBeam;
  return n;
}

// Origin on the box face the direction enters through, uniform over the
// projected area; returns the projected area.  Face weights are |d_a| times
// the face area (generateSunRay, PPB_PT.comp:396-430, with the else-if).
__device__ __forceinline__ float box_entry(const SceneView& s, f3 d, Rng& rng, f3& o) {
  f3 e = s.b1 - s.b0;
  float ax = fabsf(d.x) * (e.y * e.z), ay = fabsf(d.y) * (e.x * e.z), az = fabsf(d.z) * (e.x * e.y);
  float at = (ax + ay) + az;
  float sel = rng_next(rng) * at;
  float u = rng_next(rng), v = rng_next(rng);
  if (sel < ax) {
    o = mk(d.x > 0.0f ? s.b0.x : s.b1.x, s.b0.y + u * e.y, s.b0.z + v * e.z);
  } else if (sel < ax + ay) {
    o = mk(s.b0.x + u * e.x, d.y > 0.0f ? s.b0.y : s.b1.y, s.b0.z + v * e.z);
  } else {
    o = mk(s.b0.x + u * e.x, s.b0.y + v * e.y, d.z > 0.0f ? s.b0.z : s.b1.z);
  }
  return at;
}

__global__ void __launch_bounds__(128) ppb_emit_kernel(GridView g, SceneView s, PpbEmitView v, Counters cnt) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t lookups = 0, cells = 0, events = 0, beams = 0;
  if (p < v.photons) {
    Rng rng = rng_pcg(v.seed ^ kEmitSalt, p, v.pass);
    f3 d, power;
    const float inv = 1.0f / ((float)v.photons * 0.5f);
    bool sun = rng_next(rng) < 0.5f;
    if (sun) {
      d = s.sun;
    } else {  // uniform direction for the constant sky
      float z = 1.0f - 2.0f * rng_next(rng);
      float sn, cs;
      vsincos2pi(rng_next(rng), &sn, &cs);
      float rr = sqrtf(fmaxf(0.0f, 1.0f - z * z));
      d = mk(rr * cs, rr * sn, z);
    }
    f3 o;
    float at = box_entry(s, d, rng, o);
    if (sun) {
      float f = (s.light * at) * inv;
      power = mk(f, f, f);
    } else {
      float f = ((4.0f * kPI) * at) * inv;
      power = s.sky * f;
    }
    uint32_t seg_total = 0;
    while (beams < v.K) {
      float tmin, tmax;
      if (!slab(o, d, s.b0, s.b1, tmin, tmax) || !finite_pos(tmax)) break;
      // deposit a beam from o to the box exit (depositPhotonBeam, PPB_PT.comp:334-393)
      float* sl = v.slots + ((size_t)p * v.K + beams) * kSlotFloats;
      sl[0] = o.x; sl[1] = o.y; sl[2] = o.z;
      sl[3] = d.x; sl[4] = d.y; sl[5] = d.z;
      sl[6] = tmax;
      sl[7] = power.x; sl[8] = power.y; sl[9] = power.z;
      for (int i = 0; i < kBeamDists; ++i) {
        float t;
        sl[10 + i] = free_flight(g, s, o, d, rng, t, lookups, cells) ? t : kEscaped;
      }
      uint32_t ns = segments_of(tmax, v.radius);
      v.slot_segs[(size_t)p * v.K + beams] = ns;
      v.slot_off[(size_t)p * v.K + beams] = seg_total;
      seg_total += ns;
      ++beams;
      // next interaction (interactWithMedium, PPB_PT.comp:453-501)
      float t;
      if (!free_flight(g, s, o, d, rng, t, lookups, cells)) break;
      o = along(o, d, t);
      ++events;
      power = power * s.albedo;
      if (s.max_events && events >= s.max_events) break;
      d = hg_sample(s.ph, d, rng, true);
    }
    v.nbeams[p] = beams;
    v.photon_segs[p] = seg_total;
  }
  flush_counters(cnt, p < v.photons ? 1ull : 0ull, lookups, events, cells);
}

// One thread per (photon, beam): split into equal segments of about the
// radius, 30-bit Morton code of each midpoint.
__global__ void ppb_segment_kernel(SceneView s, const float* __restrict__ slots, const uint32_t* __restrict__ nbeams,
                                   const uint32_t* __restrict__ slot_segs, const uint32_t* __restrict__ slot_off,
                                   const uint32_t* __restrict__ photon_off, uint32_t photons, uint32_t K, float radius,
                                   uint32_t cap, float4* __restrict__ seg_a, float4* __restrict__ seg_b,
                                   uint32_t* __restrict__ seg_beam, uint32_t* __restrict__ codes,
                                   uint32_t* __restrict__ idx) {
  uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t p = gid / K, k = gid - p * K;
  if (p >= photons || k >= nbeams[p]) return;
  size_t slot = (size_t)p * K + k;
  const float* sl = slots + slot * kSlotFloats;
  f3 o = mk(sl[0], sl[1], sl[2]), d = mk(sl[3], sl[4], sl[5]);
  float len = sl[6];
  uint32_t ns = slot_segs[slot];
  uint32_t base = photon_off[p] + slot_off[slot];
  float segl = len / (float)ns;
  f3 e = s.b1 - s.b0;
  for (uint32_t j = 0; j < ns; ++j) {
    uint32_t gi = base + j;
    if (gi >= cap) return;
    float off = (float)j * segl;
    f3 a = along(o, d, off);
    f3 b = along(a, d, segl);
    seg_a[gi] = make_float4(a.x, a.y, a.z, radius);
    seg_b[gi] = make_float4(b.x, b.y, b.z, off);
    seg_beam[gi] = (uint32_t)slot;
    f3 m = (a + b) * 0.5f;
    float qx = fminf(fmaxf(((m.x - s.b0.x) / e.x) * 1024.0f, 0.0f), 1023.0f);
    float qy = fminf(fmaxf(((m.y - s.b0.y) / e.y) * 1024.0f, 0.0f), 1023.0f);
    float qz = fminf(fmaxf(((m.z - s.b0.z) / e.z) * 1024.0f, 0.0f), 1023.0f);
    codes[gi] = (morton_expand10((uint32_t)qx) << 2) | (morton_expand10((uint32_t)qy) << 1) |
                morton_expand10((uint32_t)qz);
    idx[gi] = gi;
  }
}

// ---------------------------------------------------------------------------
// LBVH (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012) over sorted 30-bit keys
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lbvh_delta(const uint32_t* __restrict__ keys, int n, int i, int j) {
  if (j < 0 || j > n - 1) return -1;
  uint32_t a = keys[i], b = keys[j];
  if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
  return __clz(a ^ b);
}

__global__ void lbvh_build_kernel(const uint32_t* __restrict__ keys, int n, uint32_t* __restrict__ left,
                                  uint32_t* __restrict__ right, uint32_t* __restrict__ parent_int,
                                  uint32_t* __restrict__ parent_leaf) {
  int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= n - 1) return;
  int d = lbvh_delta(keys, n, i, i + 1) - lbvh_delta(keys, n, i, i - 1) > 0 ? 1 : -1;
  int dmin = lbvh_delta(keys, n, i, i - d);
  int lmax = 2;
  while (lbvh_delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (lbvh_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = lbvh_delta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div <<= 1) {
    int t = (l + div - 1) / div;
    if (lbvh_delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  int gamma = i + s * d + (d < 0 ? -1 : 0);
  uint32_t lc = (min(i, j) == gamma) ? ((uint32_t)gamma | kLeafBit) : (uint32_t)gamma;
  uint32_t rc = (max(i, j) == gamma + 1) ? ((uint32_t)(gamma + 1) | kLeafBit) : (uint32_t)(gamma + 1);
  left[i] = lc;
  right[i] = rc;
  if (lc & kLeafBit) parent_leaf[lc & ~kLeafBit] = (uint32_t)i;
  else parent_int[lc] = (uint32_t)i;
  if (rc & kLeafBit) parent_leaf[rc & ~kLeafBit] = (uint32_t)i;
  else parent_int[rc] = (uint32_t)i;
  if (i == 0) parent_int[0] = 0xFFFFFFFFu;
}

// Capped-cylinder AABB of a segment (calculateBeamBounds,
// PPB_CalculateAABB.comp:64-80): e = r sqrt(1 - a^2/|a|^2) per axis.
__device__ __forceinline__ void segment_box(float4 A, float4 B, float4& lo, float4& hi) {
  f3 pa = mk(A.x, A.y, A.z), pb = mk(B.x, B.y, B.z);
  float r = A.w;
  f3 a = pb - pa;
  float dd = dot(a, a);
  f3 e;
  if (dd > 0.0f) {
    e.x = r * sqrtf(fmaxf(0.0f, 1.0f - (a.x * a.x) / dd));
    e.y = r * sqrtf(fmaxf(0.0f, 1.0f - (a.y * a.y) / dd));
    e.z = r * sqrtf(fmaxf(0.0f, 1.0f - (a.z * a.z) / dd));
  } else {
    e = mk(r, r, r);
  }
  lo = make_float4(fminf(pa.x - e.x, pb.x - e.x), fminf(pa.y - e.y, pb.y - e.y), fminf(pa.z - e.z, pb.z - e.z), 0.f);
  hi = make_float4(fmaxf(pa.x + e.x, pb.x + e.x), fmaxf(pa.y + e.y, pb.y + e.y), fmaxf(pa.z + e.z, pb.z + e.z), 0.f);
}

// The segments in leaf order: leaf i holds segment order[i].
__global__ void ppb_leaf_order_kernel(const uint32_t* __restrict__ order, const float4* __restrict__ seg_a,
                                      const float4* __restrict__ seg_b, const uint32_t* __restrict__ seg_beam,
                                      uint32_t n, float4* __restrict__ leaf_a, float4* __restrict__ leaf_b,
                                      uint32_t* __restrict__ leaf_beam) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t sid = order[i];
    leaf_a[i] = seg_a[sid];
    leaf_b[i] = seg_b[sid];
    leaf_beam[i] = seg_beam[sid];
  }
}

// Arrival counter of the refit: an atomic add with acquire-release
// semantics at GPU scope, so the box a thread stored before its arrival is
// visible to the sibling that arrives second, without separate fences.
__device__ __forceinline__ uint32_t arrive_acq_rel(uint32_t* p) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// Leaf boxes, then a bottom-up walk: the second child to arrive at a node
// (atomic counter) computes its box from both children and moves up; it
// holds its own child's box and loads only the sibling's.
__global__ void lbvh_refit_kernel(const float4* __restrict__ seg_a, const float4* __restrict__ seg_b,
                                  const uint32_t* __restrict__ order, int n, const uint32_t* __restrict__ left,
                                  const uint32_t* __restrict__ right, const uint32_t* __restrict__ parent_int,
                                  const uint32_t* __restrict__ parent_leaf, uint32_t* __restrict__ flags,
                                  float4* __restrict__ leaf_lo, float4* __restrict__ leaf_hi,
                                  float4* __restrict__ node_lo, float4* __restrict__ node_hi,
                                  float4* __restrict__ node_pk) {
  int g = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (g >= n) return;
  uint32_t sid = order[g];
  float4 lo, hi;
  segment_box(seg_a[sid], seg_b[sid], lo, hi);
  leaf_lo[g] = lo;
  leaf_hi[g] = hi;
  if (n == 1) return;
  uint32_t me = (uint32_t)g | kLeafBit;  // the child this thread climbs from, and its box (lo, hi)
  uint32_t node = parent_leaf[g];
  for (int guard = 0; node != 0xFFFFFFFFu && guard < 64; ++guard) {
    if (arrive_acq_rel(flags + node) == 0u) return;  // first arrival: the sibling finishes this node
    const uint32_t l = left[node], r = right[node];
    const bool mine_left = l == me;
    const uint32_t sib = mine_left ? r : l;
    const float4 slo = (sib & kLeafBit) ? __ldcg(leaf_lo + (sib & ~kLeafBit)) : __ldcg(node_lo + sib);
    const float4 shi = (sib & kLeafBit) ? __ldcg(leaf_hi + (sib & ~kLeafBit)) : __ldcg(node_hi + sib);
    const float4 al = mine_left ? lo : slo, ah = mine_left ? hi : shi;  // left child's box
    const float4 bl = mine_left ? slo : lo, bh = mine_left ? shi : hi;  // right child's box
    lo = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.f);
    hi = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.f);
    node_lo[node] = lo;
    node_hi[node] = hi;
    if (node_pk) {  // box and children together: one 32-byte sector per node for the gathers
      node_pk[2 * (size_t)node] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(l));
      node_pk[2 * (size_t)node + 1] = make_float4(hi.x, hi.y, hi.z, __uint_as_float(r));
    }
    me = node;
    node = parent_int[node];
  }
}

// ---------------------------------------------------------------------------
// gather
// ---------------------------------------------------------------------------
// What the gather reads: the segments in the LBVH's leaf order (leaf i
// holds segment order[i]), the leaf boxes, and per internal node its own
// packed node (low corner, left child bits) (high corner, right child bits)
// followed by its two children's (a child leaf: its box), so that one round
// of loads covers two levels of the tree.
struct PpbGatherView {
  const float4* seg_a;
  const float4* seg_b;
  const uint32_t* seg_beam;
  const float* slots;
  const float4* leaf_lo;
  const float4* leaf_hi;
  const float4* node2;
  int n;
  uint32_t seed, pass;
};

// Two levels of the LBVH per internal node b: node2[6b..6b+1] = b's packed
// node, [6b+2..6b+3] and [6b+4..6b+5] = its left and right child's packed
// node, or the child leaf's box (its leaf id stays in b's child bits).
__global__ void lbvh_node2_kernel(const float4* __restrict__ node_pk, const float4* __restrict__ leaf_lo,
                                  const float4* __restrict__ leaf_hi, uint32_t internal,
                                  float4* __restrict__ node2) {
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < internal; b += gridDim.x * blockDim.x) {
    const float4 q0 = node_pk[2 * (size_t)b], q1 = node_pk[2 * (size_t)b + 1];
    float4* o = node2 + 6 * (size_t)b;
    o[0] = q0;
    o[1] = q1;
    const uint32_t ch[2] = {__float_as_uint(q0.w), __float_as_uint(q1.w)};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const uint32_t c = ch[k];
      if (c & kLeafBit) {
        o[2 + 2 * k] = leaf_lo[c & ~kLeafBit];
        o[3 + 2 * k] = leaf_hi[c & ~kLeafBit];
      } else {
        o[2 + 2 * k] = node_pk[2 * (size_t)c];
        o[3 + 2 * k] = node_pk[2 * (size_t)c + 1];
      }
    }
  }
}

// Ray-box overlap of [t0, t1] with the slab interval.
__device__ __forceinline__ bool ray_box(f3 o, f3 inv, float t0, float t1, float4 lo, float4 hi) {
  float ax = (lo.x - o.x) * inv.x, bx = (hi.x - o.x) * inv.x;
  float ay = (lo.y - o.y) * inv.y, by = (hi.y - o.y) * inv.y;
  float az = (lo.z - o.z) * inv.z, bz = (hi.z - o.z) * inv.z;
  float tn = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), t0));
  float tf = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fminf(fmaxf(az, bz), t1));
  return tn <= tf;
}

// Beam x beam (1D) estimate of one segment (accumulateRadiance,
// PPB_PE.comp:362-404, with the fixes named at the top of the file); A, B:
// its endpoints (with the radius and the offset from the beam origin).
__device__ __forceinline__ f3 beam_contribution(const GridView& g, const SceneView& s, const PpbGatherView& v,
                                                float4 A, float4 B, uint32_t beam, f3 o, f3 rd, float t_in,
                                                float t_out, const float* cam_d, uint32_t& lookups) {
  f3 pa = mk(A.x, A.y, A.z), pb = mk(B.x, B.y, B.z);
  float r = A.w;
  f3 ax = pb - pa;
  float segl = length(ax);
  f3 zero = mk(0.f, 0.f, 0.f);
  if (!(segl > 0.0f)) return zero;
  f3 bd = mk(ax.x / segl, ax.y / segl, ax.z / segl);
  float b = dot(rd, bd);
  float den = 1.0f - b * b;
  if (!(den > 1e-6f)) return zero;  // (nearly) parallel
  f3 w0 = o - pa;
  float dw = dot(rd, w0), ew = dot(bd, w0);
  float t = (b * ew - dw) / den;
  float sb = ew + t * b;
  if (t < t_in || t > t_out || sb < 0.0f || sb > segl) return zero;
  f3 xc = along(o, rd, t);
  f3 xb = along(pa, bd, sb);
  float dist = length(xc - xb);
  if (!(dist < r)) return zero;
  float u = dist / r;
  float q = 1.0f - u * u;
  float kern = ((0.9375f * q) * q) / r;  // 15/16 (1 - u^2)^2 / r
  float rho = density_at(g, s, xc);
  ++lookups;
  float sigma_s = (s.albedo * s.k_sigma) * rho;
  const float* sl = v.slots + (size_t)beam * kSlotFloats;
  float sbeam = sb + B.w;  // distance from the beam origin
  uint32_t cb = 0, cc = 0;
  float tc = t - t_in;
  for (int i = 0; i < kBeamDists; ++i) {
    cb += sl[10 + i] >= sbeam ? 1u : 0u;
    cc += cam_d[i] >= tc ? 1u : 0u;
  }
  float tb = (float)cb * (1.0f / kBeamDists), tcam = (float)cc * (1.0f / kBeamDists);
  float ph = hg_pdf(s.ph, dot(bd, -rd));
  float w = ((((kern * sigma_s) * tcam) * tb) * ph) / sqrtf(den);
  return mk(sl[7] * w, sl[8] * w, sl[9] * w);
}

// Per-pixel gather with a warp-coherent traversal: a warp takes an 8x4
// pixel tile and walks the tree once for all its rays.  Each stack entry
// carries the mask of lanes whose rays hit the parent, and a lane tests and
// evaluates exactly the nodes and leaves its own single-ray depth-first walk
// would, in the same order (so its sum is the same); node data are loaded
// once for the warp (one broadcast transaction instead of one per lane).
// A visit of internal node b loads b's and its children's boxes together
// (node2) and tests both levels: the right child's part goes onto the stack
// first (its leaf, or its two children with the lanes that hit it), then
// the left child's (its right child), and the walk continues at the left
// child's left child (or the left leaf) — the binary walk's order.
constexpr int kGatherThreads = 128;
constexpr int kGatherStack2 = 128;  // up to 3 entries a visit of two levels (depth <= 64)

__global__ void __launch_bounds__(kGatherThreads) ppb_gather_kernel(GridView g, SceneView s, CamView cam, PassView pv,
                                                                    PpbGatherView v, double* __restrict__ sum,
                                                                    Counters cnt,
                                                                    unsigned long long* __restrict__ evaluated) {
  __shared__ uint2 s_stack[kGatherThreads / 32][kGatherStack2];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t tiles_x = (pv.cw + 7u) / 8u;
  const uint32_t cx = (wid % tiles_x) * 8u + (lane & 7u), cy = (wid / tiles_x) * 4u + (lane >> 3);
  const bool valid = cx < pv.cw && cy < pv.ch;
  uint32_t lookups = 0, cells = 0, segs = 0;
  uint32_t pix = 0;
  f3 o = mk(0.f, 0.f, 0.f), rd = mk(0.f, 0.f, 1.f), L = mk(0.f, 0.f, 0.f);
  float t_in = 0.0f, t_out = 0.0f;
  float cam_d[kBeamDists];
  bool trav = false;
  if (valid) {
    int x = (int)(pv.x0 + cx), y = (int)(pv.y0 + cy);
    pix = (uint32_t)y * pv.width + (uint32_t)x;
    camera_ray(cam, x, y, o, rd);
    float tmin, tmax;
    if (!slab(o, rd, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
      L = sky(s, rd);
    } else {
      t_in = fmaxf(tmin, 0.0f);
      t_out = tmax;
      f3 entry = along(o, rd, t_in);
      Rng rng = rng_pcg(v.seed ^ kGatherSalt, pix, v.pass);
      for (int i = 0; i < kBeamDists; ++i) {
        float t;
        cam_d[i] = free_flight(g, s, entry, rd, rng, t, lookups, cells) ? t : kEscaped;
      }
      uint32_t cexit = 0;
      for (int i = 0; i < kBeamDists; ++i) cexit += cam_d[i] >= (t_out - t_in) ? 1u : 0u;
      L = sky(s, rd) * ((float)cexit * (1.0f / kBeamDists));
      trav = v.n > 0;
    }
  }
  uint32_t active = __ballot_sync(0xffffffffu, trav);
  if (active) {
    uint2* stk = s_stack[threadIdx.x >> 5];
    const f3 inv = mk(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
    int sp = 0;  // warp-uniform, as are node and active
    uint32_t node = v.n == 1 ? (0u | kLeafBit) : 0u;
    while (true) {
      const bool mine = (active >> lane) & 1u;
      if (node & kLeafBit) {
        // the leaf's box and its segment (leaf order) in one round of loads
        const uint32_t lf = node & ~kLeafBit;
        const float4 lo = v.leaf_lo[lf], hi = v.leaf_hi[lf];
        const float4 A = v.seg_a[lf], B = v.seg_b[lf];
        const uint32_t beam = v.seg_beam[lf];
        if (mine && ray_box(o, inv, t_in, t_out, lo, hi)) {
          L = L + beam_contribution(g, s, v, A, B, beam, o, rd, t_in, t_out, cam_d, lookups);
          ++segs;
        }
      } else {
        const float4* q = v.node2 + 6 * (size_t)node;
        const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3], q4 = q[4], q5 = q[5];
        const uint32_t hit = __ballot_sync(0xffffffffu, mine && ray_box(o, inv, t_in, t_out, q0, q1));
        if (hit) {
          const bool hb = (hit >> lane) & 1u;
          const uint32_t l = __float_as_uint(q0.w), r = __float_as_uint(q1.w);
          // at most 3 pushes a visit of two levels: below kGatherStack2 for
          // depth <= 64 (30-bit keys + index bits); the guard only keeps a
          // deeper tree in bounds
          if (r & kLeafBit) {
            if (sp < kGatherStack2) {
              if (lane == 0) stk[sp] = make_uint2(r, hit);
              ++sp;
            }
          } else {
            const uint32_t h1 = __ballot_sync(0xffffffffu, hb && ray_box(o, inv, t_in, t_out, q4, q5));
            if (h1 && sp + 2 <= kGatherStack2) {
              if (lane == 0) {
                stk[sp] = make_uint2(__float_as_uint(q5.w), h1);
                stk[sp + 1] = make_uint2(__float_as_uint(q4.w), h1);
              }
              sp += 2;
            }
          }
          if (l & kLeafBit) {
            node = l;
            active = hit;
            continue;
          }
          const uint32_t h0 = __ballot_sync(0xffffffffu, hb && ray_box(o, inv, t_in, t_out, q2, q3));
          if (h0) {
            if (sp < kGatherStack2) {
              if (lane == 0) stk[sp] = make_uint2(__float_as_uint(q3.w), h0);
              ++sp;
            }
            node = __float_as_uint(q2.w);
            active = h0;
            continue;
          }
        }
      }
      if (sp == 0) break;
      --sp;
      __syncwarp();
      const uint2 e = stk[sp];
      __syncwarp();
      node = e.x;
      active = e.y;
    }
  }
  if (valid) write_result(pv, sum, pix, L);
  flush_counters(cnt, valid ? 1ull : 0ull, lookups, 0, cells);
  warp_count(evaluated, segs);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static void ppb_release(PpbState* st) {
  void* ptrs[] = {st->slots,      st->nbeams,      st->slot_segs,   st->slot_off,   st->photon_segs,
                  st->photon_off, st->scan_sums,   st->total,       st->seg_a,      st->seg_b,
                  st->leaf_a,     st->leaf_b,      st->leaf_beam,   st->node_pk,    st->seg_beam,
                  st->codes,      st->idx,         st->codes_sorted, st->idx_sorted, st->left,
                  st->right,      st->parent_int,  st->parent_leaf, st->flags,      st->leaf_lo,
                  st->leaf_hi,    st->node_lo,     st->node_hi,     st->node2};
  for (void* p : ptrs) cudaFree(p);
  probe_free(st->gather);
}

void ppb_free(vcr_ctx* ctx) {
  if (!ctx->ppb) return;
  ppb_release(ctx->ppb);
  delete ctx->ppb;
  ctx->ppb = nullptr;
}

// r_k = r_0 prod_{i=1..k} (i + alpha) / (i + 1), in double (the intended
// per-pass reduction of RenderTechniquePPB::UpdateRadius).
float ppb_radius_at(float r0, float alpha, uint32_t pass) {
  double r = r0;
  for (uint32_t i = 1; i <= pass; ++i) r *= ((double)i + (double)alpha) / ((double)i + 1.0);
  return (float)r;
}

vcr_status ppb_setup(vcr_ctx* ctx, const vcr_ppb_params* p) {
  if (!p || p->photons == 0 || p->photons > (1u << 21) || p->capacity < 2 || p->capacity > (1u << 26) ||
      !(p->radius > 0.0f) || !(p->alpha > 0.0f && p->alpha <= 1.0f))
    return fail(ctx, VCR_ERR_INVALID, "ppb params: photons 1..2^21, capacity 2..2^26, radius > 0, alpha in (0,1]");
  ppb_free(ctx);
  PpbState* st = new PpbState();
  ctx->ppb = st;
  st->prm = *p;
  uint32_t K = ctx->params.max_events ? std::min<uint32_t>(ctx->params.max_events + 1u, kMaxBeamsPerPhoton)
                                      : kMaxBeamsPerPhoton;
  st->K = K;
  size_t P = p->photons, C = p->capacity;
#define VCR_ALLOC(ptr, bytes) VCR_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(&(ptr)), (bytes)))
  VCR_ALLOC(st->slots, P * K * kSlotFloats * sizeof(float));
  VCR_ALLOC(st->nbeams, P * 4);
  VCR_ALLOC(st->slot_segs, P * K * 4);
  VCR_ALLOC(st->slot_off, P * K * 4);
  VCR_ALLOC(st->photon_segs, P * 4);
  VCR_ALLOC(st->photon_off, P * 4);
  VCR_ALLOC(st->scan_sums, 4096 * 4);
  VCR_ALLOC(st->total, 4);
  VCR_ALLOC(st->seg_a, C * sizeof(float4));
  VCR_ALLOC(st->seg_b, C * sizeof(float4));
  VCR_ALLOC(st->node_pk, 2 * C * sizeof(float4));
  VCR_ALLOC(st->node2, 6 * C * sizeof(float4));
  VCR_ALLOC(st->leaf_a, C * sizeof(float4));
  VCR_ALLOC(st->leaf_b, C * sizeof(float4));
  VCR_ALLOC(st->leaf_beam, C * 4);
  VCR_ALLOC(st->seg_beam, C * 4);
  VCR_ALLOC(st->codes, C * 4);
  VCR_ALLOC(st->idx, C * 4);
  VCR_ALLOC(st->codes_sorted, C * 4);
  VCR_ALLOC(st->idx_sorted, C * 4);
  VCR_ALLOC(st->left, C * 4);
  VCR_ALLOC(st->right, C * 4);
  VCR_ALLOC(st->parent_int, C * 4);
  VCR_ALLOC(st->parent_leaf, C * 4);
  VCR_ALLOC(st->flags, C * 4);
  VCR_ALLOC(st->leaf_lo, C * sizeof(float4));
  VCR_ALLOC(st->leaf_hi, C * sizeof(float4));
  VCR_ALLOC(st->node_lo, C * sizeof(float4));
  VCR_ALLOC(st->node_hi, C * sizeof(float4));
#undef VCR_ALLOC
  return ensure_scratch(ctx, sort_scratch_bytes(p->capacity));
}

// node2 (two tree levels per internal node, lbvh_node2_kernel) of a refit tree of n leaves.
vcr_status lbvh_node2(vcr_ctx* ctx, const float4* node_pk, const float4* leaf_lo, const float4* leaf_hi, int n,
                      float4* node2, cudaStream_t st) {
  if (n <= 1) return VCR_OK;
  lbvh_node2_kernel<<<ctx->sm_count * 8, 256, 0, st>>>(node_pk, leaf_lo, leaf_hi, (uint32_t)(n - 1), node2);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

vcr_status lbvh_build_refit(vcr_ctx* ctx, const uint32_t* codes, const uint32_t* order, const float4* seg_a,
                            const float4* seg_b, int n, uint32_t* left, uint32_t* right, uint32_t* parent_int,
                            uint32_t* parent_leaf, uint32_t* flags, float4* leaf_lo, float4* leaf_hi,
                            float4* node_lo, float4* node_hi, cudaStream_t st, float4* node_pk) {
  if (n <= 0) return VCR_OK;
  if (n > 1) {
    lbvh_build_kernel<<<(n - 1 + 255) / 256, 256, 0, st>>>(codes, n, left, right, parent_int, parent_leaf);
    VCR_CUDA(ctx, cudaGetLastError());
    VCR_CUDA(ctx, cudaMemsetAsync(flags, 0, (size_t)(n - 1) * 4, st));
  }
  lbvh_refit_kernel<<<(n + 255) / 256, 256, 0, st>>>(seg_a, seg_b, order, n, left, right, parent_int, parent_leaf,
                                                     flags, leaf_lo, leaf_hi, node_lo, node_hi, node_pk);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

vcr_status ppb_pass_launch(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t st_) {
  PpbState* st = ctx->ppb;
  if (!st) return fail(ctx, VCR_ERR_STATE, "vcr_ppb_pass needs vcr_ppb_setup");
  if (!ctx->has_grid || !ctx->has_cloud || !ctx->has_cam || !ctx->has_params || !ctx->d_sum)
    return fail(ctx, VCR_ERR_STATE, "vcr_ppb_pass needs a grid, cloud, camera, params and frame");
  if (ctx->params.rng_mode != VCR_RNG_PCG) return fail(ctx, VCR_ERR_UNSUPPORTED, "photon beams use PCG streams");
  PassView pv;
  vcr_status vs = make_pass_view(ctx, pass, pv);
  if (vs) return vs;
  if (pv.spp != 1) return fail(ctx, VCR_ERR_UNSUPPORTED, "photon beams gather one estimate per pixel and pass");
  GridView g = grid_view(ctx);
  SceneView s = scene_view(ctx);
  const uint32_t P = st->prm.photons, K = st->K, C = st->prm.capacity;
  st->radius = ppb_radius_at(st->prm.radius, st->prm.alpha, pass->pass_index);
  Counters cnt{ctx->d_counters};
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 5 * sizeof(unsigned long long), st_));
  PpbEmitView ev{st->slots, st->nbeams, st->slot_segs, st->slot_off, st->photon_segs, P, K, st->radius,
                 pass->seed, pass->pass_index};
  ppb_emit_kernel<<<(P + 127) / 128, 128, 0, st_>>>(g, s, ev, cnt);
  VCR_CUDA(ctx, cudaGetLastError());
  VCR_CUDA(ctx, exclusive_scan_u32(st->photon_segs, st->photon_off, P, st->scan_sums, st->total, st_));
  uint32_t total = 0;
  VCR_CUDA(ctx, cudaMemcpyAsync(&total, st->total, 4, cudaMemcpyDeviceToHost, st_));
  VCR_CUDA(ctx, cudaStreamSynchronize(st_));
  uint32_t n = std::min(total, C);
  st->segments = n;
  st->dropped = total - n;
  uint64_t threads = (uint64_t)P * K;
  ppb_segment_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st_>>>(
      s, st->slots, st->nbeams, st->slot_segs, st->slot_off, st->photon_off, P, K, st->radius, C, st->seg_a, st->seg_b,
      st->seg_beam, st->codes, st->idx);
  VCR_CUDA(ctx, cudaGetLastError());
  VCR_CUDA(ctx, sort_pairs_enqueue(ctx->sm_count, ctx->d_error, ctx->d_scratch, st->codes, st->idx, st->codes_sorted,
                                   st->idx_sorted, n, 0, 30, st_));
  vs = lbvh_build_refit(ctx, st->codes_sorted, st->idx_sorted, st->seg_a, st->seg_b, (int)n, st->left, st->right,
                        st->parent_int, st->parent_leaf, st->flags, st->leaf_lo, st->leaf_hi, st->node_lo,
                        st->node_hi, st_, st->node_pk);
  if (vs) return vs;
  if (n) {
    ppb_leaf_order_kernel<<<ctx->sm_count * 8, 256, 0, st_>>>(st->idx_sorted, st->seg_a, st->seg_b, st->seg_beam, n,
                                                              st->leaf_a, st->leaf_b, st->leaf_beam);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  vs = lbvh_node2(ctx, st->node_pk, st->leaf_lo, st->leaf_hi, (int)n, st->node2, st_);
  if (vs) return vs;
  PpbGatherView gv{st->leaf_a,  st->leaf_b, st->leaf_beam, st->slots,      st->leaf_lo,
                   st->leaf_hi, st->node2, (int)n,        pass->seed, pass->pass_index};
  // one warp per 8x4 pixel tile
  uint32_t tiles = ((pv.cw + 7u) / 8u) * ((pv.ch + 3u) / 4u);
  uint32_t warps_per_block = kGatherThreads / 32;
  vcr_status ps = probe_begin(ctx, st->gather, st_);
  if (ps) return ps;
  ppb_gather_kernel<<<(tiles + warps_per_block - 1) / warps_per_block, kGatherThreads, 0, st_>>>(
      g, s, cam_view(ctx->cam), pv, gv, ctx->d_sum, cnt, st->gather.d_count);
  VCR_CUDA(ctx, cudaGetLastError());
  ps = probe_end(ctx, st->gather, st_);
  if (ps) return ps;
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, st_));
  if (!(pv.flags & VCR_PASS_NO_ACCUMULATE)) {
    ctx->passes += 1;
    ctx->samples += 1;
  }
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_ppb_setup(vcr_ctx* ctx, const vcr_ppb_params* p) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  return ppb_setup(ctx, p);
}

extern "C" VCR_API vcr_status vcr_ppb_free(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaDeviceSynchronize();
  ppb_free(ctx);
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_ppb_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  return ppb_pass_launch(ctx, pass, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_ppb_info(vcr_ctx* ctx, vcr_ppb_info_t* out) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  if (!ctx->ppb) return fail(ctx, VCR_ERR_STATE, "no photon-beam state");
  out->segments = ctx->ppb->segments;
  out->dropped = ctx->ppb->dropped;
  out->radius = ctx->ppb->radius;
  out->beam_slots = ctx->ppb->K;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_ppb_gather_stats(vcr_ctx* ctx, uint64_t* count, float* ms) {
  if (!ctx || !count || !ms) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->ppb) return fail(ctx, VCR_ERR_STATE, "no photon-beam state");
  return probe_read(ctx, ctx->ppb->gather, *count, *ms);
}

// Copies of the last pass's beam data (test and debug access).
extern "C" VCR_API vcr_status vcr_ppb_read(vcr_ctx* ctx, vcr_ppb_buffer which, void* host, size_t bytes) {
  if (!ctx || !host) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  PpbState* st = ctx->ppb;
  if (!st) return fail(ctx, VCR_ERR_STATE, "no photon-beam state");
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  size_t n = st->segments, P = st->prm.photons, K = st->K;
  const void* src = nullptr;
  size_t want = 0;
  switch (which) {
    case VCR_PPB_SLOTS: src = st->slots; want = P * K * kSlotFloats * 4; break;
    case VCR_PPB_NBEAMS: src = st->nbeams; want = P * 4; break;
    case VCR_PPB_SEG_A: src = st->seg_a; want = n * 16; break;
    case VCR_PPB_SEG_B: src = st->seg_b; want = n * 16; break;
    case VCR_PPB_SEG_BEAM: src = st->seg_beam; want = n * 4; break;
    case VCR_PPB_CODES: src = st->codes; want = n * 4; break;
    case VCR_PPB_ORDER: src = st->idx_sorted; want = n * 4; break;
    case VCR_PPB_LEFT: src = st->left; want = n > 1 ? (n - 1) * 4 : 0; break;
    case VCR_PPB_RIGHT: src = st->right; want = n > 1 ? (n - 1) * 4 : 0; break;
    case VCR_PPB_NODE_LO: src = st->node_lo; want = n > 1 ? (n - 1) * 16 : 0; break;
    case VCR_PPB_NODE_HI: src = st->node_hi; want = n > 1 ? (n - 1) * 16 : 0; break;
    case VCR_PPB_LEAF_LO: src = st->leaf_lo; want = n * 16; break;
    case VCR_PPB_LEAF_HI: src = st->leaf_hi; want = n * 16; break;
    default: return fail(ctx, VCR_ERR_INVALID, "unknown beam buffer %d", (int)which);
  }
  if (bytes != want) return fail(ctx, VCR_ERR_INVALID, "beam buffer %d is %zu bytes, not %zu", (int)which, want, bytes);
  if (want) VCR_CUDA(ctx, cudaMemcpy(host, src, want, cudaMemcpyDeviceToHost));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_lbvh_build(vcr_ctx* ctx, const uint32_t* d_sorted_codes, const uint32_t* d_order,
                                             const float* d_seg_a, const float* d_seg_b, uint32_t n,
                                             uint32_t* d_left, uint32_t* d_right, float* d_node_lo, float* d_node_hi,
                                             float* d_leaf_lo, float* d_leaf_hi, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (n == 0) return VCR_OK;
  if (n > (1u << 30)) return fail(ctx, VCR_ERR_UNSUPPORTED, "LBVH of %u leaves", n);
  if (!d_sorted_codes || !d_order || !d_seg_a || !d_seg_b || !d_leaf_lo || !d_leaf_hi ||
      (n > 1 && (!d_left || !d_right || !d_node_lo || !d_node_hi)))
    return fail(ctx, VCR_ERR_INVALID, "null LBVH buffer");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  size_t need = (size_t)3 * n * 4;  // parent_int, parent_leaf, flags
  vcr_status vs = ensure_scratch(ctx, need);
  if (vs) return vs;
  uint32_t* pi = reinterpret_cast<uint32_t*>(ctx->d_scratch);
  uint32_t* pl = pi + n;
  uint32_t* fl = pl + n;
  cudaStream_t st = (cudaStream_t)stream;
  vs = lbvh_build_refit(ctx, d_sorted_codes, d_order, reinterpret_cast<const float4*>(d_seg_a),
                        reinterpret_cast<const float4*>(d_seg_b), (int)n, d_left, d_right, pi, pl, fl,
                        reinterpret_cast<float4*>(d_leaf_lo), reinterpret_cast<float4*>(d_leaf_hi),
                        reinterpret_cast<float4*>(d_node_lo), reinterpret_cast<float4*>(d_node_hi), st, nullptr);
  if (vs) return vs;
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, st));
  return VCR_OK;
}
