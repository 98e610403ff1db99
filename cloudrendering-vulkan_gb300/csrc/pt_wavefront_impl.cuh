// Persistent DDA wavefront path tracer: kernel and launcher.
//
// Same light transport as the per-pixel tracker (PathTracer.comp:366-425)
// with two changes of method the target asks for: free flights walk a
// pyramid level of per-cell majorants with a 3D DDA (instead of one global
// majorant, PathTracer.comp:338), and sun NEE is unbiased ratio tracking
// (instead of the shadow-volume lookup, PathTracer.comp:406-411).
//
// Schedule: persistent CTAs; every lane owns one path at a time and refills
// itself from a global cursor with one atomic per warp (ballot + popc), so
// lanes never idle while paths remain.  One launch may render several
// consecutive passes (pv.passes): its work items run through the passes in
// order, each with its pass's random streams, so the lanes that would sit
// idle while a pass's longest paths finish (a third of a pass on a dense
// cloud) already run the next pass's paths.  A wavefront step is one bounded DDA
// walk (at most `dda_steps` majorant cells, resumable: the optical depth
// left over is kept) followed by at most one density lookup, so a lane
// crossing many empty cells cannot hold its warp for a whole flight.  The
// step runs as warp-converged phases with __syncwarp() between them: DDA
// set-up of new rays, then every live lane's walk (a ray set up this step
// walks this step), then the density lookups of all candidate lanes at
// once, then the collision / escape bookkeeping.  Without the explicit
// reconvergence, lanes leaving the walk loop after different cell counts
// reached the lookup in separate groups (1.4x slower on the C5 pass).  When
// the selected majorant level fits, one thread stages it into shared memory
// with a TMA bulk copy (cp.async.bulk + mbarrier) at CTA start and every
// DDA cell visit reads shared memory.  The arithmetic per path is identical
// to the oracle's sequential loop, so results are bit-exact with it.
//
// This file is compiled twice: by pt_wavefront.cu into namespace
// vcr::exact (device code built with -fmad=false and the library's own
// transcendental series, bit-exact with the oracle) and by
// pt_wavefront_fast.cu into vcr::fast (contracted multiply-adds and the
// hardware approximations of log, exp and sincos; selected by
// vcr_tuning.fast_math).  VCR_WF_NS names the namespace.
#include "track.cuh"
#include "nrc.cuh"

#ifndef VCR_WF_NS
#error "VCR_WF_NS must name the namespace of this instantiation"
#endif

namespace vcr {
namespace VCR_WF_NS {

// Where paths that end in the radiance cache leave their query.
struct NrcSink {
  NrcRecord* rec;
  uint32_t* count;
  uint32_t capacity;
};

constexpr uint32_t kMbarDrain = kDefaultStageWait;  // wait for a copy in flight after a timeout

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0u;
}

// Copy `bytes` (multiple of 16, 16-byte aligned both sides) from global to
// this CTA's shared memory with one bulk copy; every thread waits (at most
// `polls` polls).  Returns false (error word set) if the copy did not
// complete in time; the copy in flight is then waited for once more (at
// most kMbarDrain polls) so that no copy lands after the CTA stops using
// the buffer, and the caller reads the majorants from global memory.
__device__ bool stage_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint32_t polls, int* err) {
  const uint32_t b = smem_u32(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(b)
                 : "memory");
  }
  bool ok = false;
  for (uint32_t i = 0; i < polls; ++i) {
    if (mbar_try_wait(b, 0u)) {
      ok = true;
      break;
    }
  }
  if (!ok) {
    atomicExch(err, 3);  // staging wait ran out; wait (bounded) once more for the copy in flight
    for (uint32_t i = 0; i < kMbarDrain; ++i)
      if (mbar_try_wait(b, 0u)) break;
  }
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

enum : uint32_t { kIdle = 0, kScatter = 1, kNee = 2 };

// Adds one path's count to a lane's 32-bit total; a total that could pass
// 2^31 goes to the 64-bit launch counter first (a path adds < 2^27, the
// work cap, so this is rare and never wraps).
__device__ __forceinline__ void tally(unsigned long long* dst, uint32_t& acc, uint32_t add) {
  if (acc + add >= 0x80000000u) {
    atomicAdd(dst, (unsigned long long)acc);
    acc = 0;
  }
  acc += add;
}

// Rarely-taken bodies live out of line: the persistent loop then stays small
// enough for the instruction cache (a fully inlined loop stalled on
// instruction fetch more than on memory).  They take and return values, not
// references, so the path state they touch stays in registers instead of
// being stored to the stack around each call; the kernel's struct
// parameters are __grid_constant__ so that passing them by const reference
// does not copy them to local memory.
struct DirRng {
  f3 d;
  Rng r;
};
__device__ __noinline__ DirRng sample_direction(const Phase& ph, f3 dir, Rng rng) {
  DirRng o;
  o.d = hg_sample(ph, dir, rng, true);
  o.r = rng;
  return o;
}

__device__ __noinline__ f3 escape_radiance(const SceneView& s, f3 dir) { return sky(s, dir); }

// Camera ray of a path; returns false (L = sky) if it misses the cloud.
struct PathStart {
  f3 pos, dir, L;
  bool hit;
};
__device__ __noinline__ PathStart start_path(const CamView& cam, const SceneView& s, int x, int y) {
  PathStart o;
  camera_ray(cam, x, y, o.pos, o.dir);
  o.L = mk(0.f, 0.f, 0.f);
  float tmin, tmax;
  if (!slab(o.pos, o.dir, s.b0, s.b1, tmin, tmax) || tmax < 0.0f || !(s.ds > 0.0f)) {
    o.L = sky(s, o.dir);
    o.hit = false;
    return o;
  }
  o.pos = along(o.pos, o.dir, tmax < tmin ? tmax : tmin);
  o.hit = true;
  return o;
}
__device__ __forceinline__ bool begin(const PathStart& o, f3& pos, f3& dir, f3& L) {
  pos = o.pos;
  dir = o.dir;
  L = o.L;
  return o.hit;
}

// A training path's radiance is final: turn the recorded radiance-before
// and throughput-before of each of its vertices into the target
// (L - L_before) / beta_before, walking the chain of its record slots.
__device__ __noinline__ void finish_training(const NrcTrainSink& ts, uint32_t slot, f3 L) {
  for (int i = 0; i < kNrcRecordEvents && slot != kNrcNoSlot; ++i) {
    NrcRecord* r = ts.rec + slot;
    float inv = 1.0f / __uint_as_float(r->pad[0]);
    r->w0 = (L.x - r->w0) * inv;
    r->w1 = (L.y - r->w1) * inv;
    r->w2 = (L.z - r->w2) * inv;
    slot = r->pad[1];
  }
}

// Append a training vertex; returns the slot (or the previous one if full).
__device__ __noinline__ uint32_t record_training(const NrcTrainSink& ts, const SceneView& s, f3 pos, f3 dir, f3 L,
                                                 float beta, uint32_t prev) {
  uint32_t q = atomicAdd(ts.count, 1u);
  if (q >= ts.capacity) return prev;
  NrcRecord r;
  r.px = pos.x; r.py = pos.y; r.pz = pos.z;
  r.vx = -dir.x; r.vy = -dir.y; r.vz = -dir.z;
  r.sx = s.sun.x; r.sy = s.sun.y; r.sz = s.sun.z;
  r.w0 = L.x; r.w1 = L.y; r.w2 = L.z;
  r.pix = kNrcNoSlot;
  r.pad[0] = __float_as_uint(beta);
  r.pad[1] = prev;
  r.pad[2] = 0u;
  ts.rec[q] = r;
  return q;
}

constexpr uint32_t kTrainPath = 0x80000000u;  // pid flag of a training path

// Russian roulette of a training path's continuation: survive with
// probability p and carry weight 1/p.
struct Roulette {
  Rng r;
  float beta;
  bool alive;
};
__device__ __noinline__ Roulette roulette(Rng rng, float p, float beta) {
  Roulette o;
  o.alive = rng_next(rng) < p;
  o.r = rng;
  o.beta = o.alive ? beta / p : beta;
  return o;
}
__device__ __forceinline__ bool roulette_survives(Rng& rng, float p, float& beta) {
  Roulette o = roulette(rng, p, beta);
  rng = o.r;
  beta = o.beta;
  return o.alive;
}

// 1024 threads per SM: 64 registers a thread (a few spill to L1).  On the
// 1024x512x1024 scene this measured 6% faster than 768 threads at 80
// registers (no spills) and 18% faster than 1280 threads at 48 registers.
// Work items [0, ts.paths) are training paths (their pid carries kTrainPath
// and their pix the slot of their last record); the pass's camera paths
// follow.  kBatch: the camera paths are those of bt's views (pid holds the
// view, whose sun the path uses), the view table sits in shared memory
// after the staged majorants, and the pass index adds *bt.pass_ctr (so a
// replayed graph renders consecutive passes).
__host__ __device__ constexpr uint32_t align16(uint32_t b) { return (b + 15u) & ~15u; }

template <int kThreads, bool kStage, bool kBatch>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads)
    pt_wavefront_kernel(const __grid_constant__ GridView g, const __grid_constant__ SceneView s,
                        const __grid_constant__ CamView cam, const __grid_constant__ PassView pv,
                        double* __restrict__ sum, uint32_t* __restrict__ stats, Counters cnt, uint32_t total,
                        uint32_t dda_steps, uint32_t maj_bytes, uint32_t stage_polls,
                        const __grid_constant__ NrcSink nq,
                        const __grid_constant__ NrcTrainSink ts, const __grid_constant__ BatchSink bt,
                        int* __restrict__ err) {
  extern __shared__ __align__(16) float s_maj[];
  __shared__ __align__(8) uint64_t s_bar;
  const float* maj = g.majorants;
  if (kStage) {
    if (stage_to_smem(s_maj, g.majorants, maj_bytes, &s_bar, stage_polls, err)) maj = s_maj;
  }
  BatchView* s_views = reinterpret_cast<BatchView*>(reinterpret_cast<char*>(s_maj) + (kStage ? align16(maj_bytes) : 0u));
  uint32_t pass = pv.pass;
  if (kBatch) {
    const uint2* src = reinterpret_cast<const uint2*>(bt.views);
    uint2* dst = reinterpret_cast<uint2*>(s_views);
    const uint32_t words = bt.count * (uint32_t)(sizeof(BatchView) / 8);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    pass += *bt.pass_ctr;
    __syncthreads();
  }
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t per_pass = pv.cw * pv.ch * pv.spp;  // camera paths of one pass
  const float k = s.k_sigma;
  const f3 lsun0 = -s.sun;
  uint32_t mode = kIdle;
  bool exhausted = false, flying = false, need_init = false;
  float tau = 0.0f;
  uint32_t pid = 0, pix = 0, events = 0, lookups = 0, cells = 0;
  uint32_t n_paths = 0, n_look = 0, n_ev = 0, n_cells = 0;  // this lane's totals (see tally)
  Rng rng{0u, 0u};
  f3 pos = mk(0.f, 0.f, 0.f), dir = pos, L = pos;
  float beta = 1.0f, T = 1.0f;
  Track tr;

  while (true) {
    // ---- warp-aggregated refill of idle lanes ---------------------------
    bool need = (mode == kIdle) && !exhausted;
    uint32_t mask = __ballot_sync(0xffffffffu, need);
    if (mask) {
      uint32_t leader = __ffs(mask) - 1;
      uint32_t base = 0;
      if (lane == leader) base = (uint32_t)atomicAdd(cnt.c + 4, (unsigned long long)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        uint32_t id = base + __popc(mask & ((1u << lane) - 1u));
        if (id >= total + ts.paths) {
          exhausted = true;
        } else if (kBatch) {  // camera path of a view: the last view with path0 <= id
          uint32_t lo = 0, hi = bt.count - 1u;
          while (lo < hi) {
            uint32_t mid = (lo + hi + 1u) >> 1;
            if (s_views[mid].path0 <= id) lo = mid;
            else hi = mid - 1u;
          }
          const BatchView& bv = s_views[lo];
          uint32_t local = id - bv.path0;
          uint32_t per_row = bv.width * pv.spp;
          uint32_t cy = local / per_row, rem = local - cy * per_row;
          uint32_t cx = rem / pv.spp, sp = rem - cx * pv.spp;
          uint32_t lp = cy * bv.width + cx;
          pid = lo;
          pix = bv.pix0 + lp;
          rng = rng_pcg(pv.seed + kViewSeedStep * lo, lp * pv.spp + sp, pass);
          L = mk(0.f, 0.f, 0.f);
          beta = 1.0f;
          events = lookups = cells = 0;
          ++n_paths;
          if (begin(start_path(bv.cam, s, (int)cx, (int)cy), pos, dir, L)) {
            mode = kScatter;
            need_init = true;
          } else {
            write_result(pv, sum, pix, L);
          }
        } else if (id < ts.paths) {  // training path from a uniformly drawn pixel of the crop
          rng = rng_pcg(pv.seed ^ kNrcTrainSalt, id, pass);
          uint32_t pp = (uint32_t)(rng_next(rng) * (float)(pv.cw * pv.ch));
          pp = min(pp, pv.cw * pv.ch - 1u);
          pid = kTrainPath;
          pix = kNrcNoSlot;
          L = mk(0.f, 0.f, 0.f);
          beta = 1.0f;
          events = lookups = cells = 0;
          ++n_paths;
          if (begin(start_path(cam, s, (int)(pv.x0 + pp % pv.cw), (int)(pv.y0 + pp / pv.cw)), pos, dir, L)) {
            mode = kScatter;
            need_init = true;
          }
        } else {
          id -= ts.paths;
          uint32_t pq = pass;  // a launch of several passes: item id / per_pass is the pass offset
          if (pv.passes > 1u) {
            const uint32_t q = id / per_pass;
            id -= q * per_pass;
            pq += q;
          }
          pid = id;
          uint32_t per_row = pv.cw * pv.spp;
          uint32_t cy = id / per_row, rem = id - cy * per_row;
          uint32_t cx = rem / pv.spp, sp = rem - cx * pv.spp;
          int x = (int)(pv.x0 + cx), y = (int)(pv.y0 + cy);
          pix = (uint32_t)y * pv.width + (uint32_t)x;
          rng = rng_pcg(pv.seed, pix * pv.spp + sp, pq);
          L = mk(0.f, 0.f, 0.f);
          beta = 1.0f;
          events = lookups = cells = 0;
          ++n_paths;
          if (begin(start_path(cam, s, x, y), pos, dir, L)) {
            mode = kScatter;
            need_init = true;
          } else {
            write_result(pv, sum, pix, L);
            if (stats && sp == 0) {
              uint32_t* st = stats + 4 * (size_t)pix;
              st[0] = 0; st[1] = 0; st[2] = pv.pass; st[3] = 0;
            }
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, exhausted && mode == kIdle)) break;

    // ---- the one DDA set-up site (camera ray, NEE ray, scattered ray) ------
    const f3 lsun = kBatch ? -s_views[pid].sun : lsun0;
    if (need_init) {  // a NEE ray runs towards the sun, a scattering ray along dir
      track_init(tr, g, s, maj, pos, mode == kNee ? lsun : dir, cells);
      need_init = false;
    }
    __syncwarp();
    // ---- one bounded walk ---------------------------------------------------
    const bool act = mode != kIdle;
    int r = kPending;
    if (act) {
      if (!flying) {
        tau = -vlog(rng_next(rng));
        flying = true;
      }
      r = track_walk(tr, g, maj, k, tau, cells, dda_steps);
    }
    __syncwarp();
    // ---- at most one density lookup (the candidate lanes together) ---------
    f3 p = pos;
    float rho = 0.0f;
    if (r == kCandidate) {
      f3 rd = mode == kScatter ? dir : lsun;
      p = along(pos, rd, tr.t);
      rho = density_at(g, s, p);
    }
    __syncwarp();
    // ---- collision, escape and path bookkeeping -----------------------------
    // Decisions first; the two costly continuations (a new scattering
    // direction, a finished path) then run as converged groups below.
    bool want_dir = false, finish = false, escaped = false;
    if (act) {
      if (r != kPending) {
        flying = false;
        bool nee_done = false;
        if (r == kCandidate) {
          ++lookups;
          if (mode == kScatter) {
            float xi = rng_next(rng);
            if (xi * tr.m < rho) {  // real collision (xi < rho / m): start the NEE ray
              pos = p;
              ++events;
              const bool training = (pid & kTrainPath) != 0u;
              if (training && events <= (uint32_t)kNrcRecordEvents)
                pix = record_training(ts, s, pos, dir, L, beta, pix);
              if (s.nrc_events && events == s.nrc_events && !training) {
                // end in the radiance cache: it predicts what leaves this vertex
                finish = true;
                uint32_t q = atomicAdd(nq.count, 1u);
                if (q < nq.capacity) {
                  NrcRecord r;
                  r.px = pos.x; r.py = pos.y; r.pz = pos.z;
                  r.vx = -dir.x; r.vy = -dir.y; r.vz = -dir.z;
                  r.sx = s.sun.x; r.sy = s.sun.y; r.sz = s.sun.z;
                  r.w0 = beta; r.w1 = beta; r.w2 = beta;
                  r.pix = pix;
                  r.pad[0] = r.pad[1] = r.pad[2] = 0u;
                  nq.rec[q] = r;
                }
              } else {
                beta = beta * s.albedo;
                T = 1.0f;
                mode = kNee;
                need_init = true;
              }
            }
          } else {
            T = T * (1.0f - rho / tr.m);
            if (T < 0.05f) {
              if (rng_next(rng) >= 0.5f) {
                T = 0.0f;
                nee_done = true;
              } else {
                T = T * 2.0f;
              }
            }
          }
        } else if (mode == kScatter) {
          escaped = true;
          finish = true;
        } else {
          nee_done = true;
        }
        if (nee_done) {
          const float phase = hg_pdf(s.ph, dot(-dir, -lsun));
          float c = ((s.light * phase) * T) * beta;
          L = L + mk(c, c, c);
          if (s.max_events && events >= s.max_events) {
            finish = true;
          } else if ((pid & kTrainPath) && ts.survival > 0.0f && events >= (uint32_t)kNrcRecordEvents &&
                     !roulette_survives(rng, ts.survival, beta)) {
            finish = true;  // past the recorded vertices: Russian roulette
          } else {
            want_dir = true;
          }
        }
        if (lookups + cells > kPathWorkCap) {  // runaway guard (non-finite input)
          finish = true;
          want_dir = false;
        }
      }
    }
    __syncwarp();
    if (want_dir) {
      DirRng nd = sample_direction(s.ph, dir, rng);
      dir = nd.d;
      rng = nd.r;
      mode = kScatter;
      need_init = true;
    }
    __syncwarp();
    if (finish) {
      if (escaped) L = L + escape_radiance(s, dir) * beta;
      if (pid & kTrainPath) {
        finish_training(ts, pix, L);
      } else {
        write_result(pv, sum, pix, L);
        if (stats && (pid % pv.spp) == 0) {
          uint32_t* st = stats + 4 * (size_t)pix;
          st[0] = events; st[1] = lookups; st[2] = pv.pass; st[3] = cells;
        }
      }
      tally(cnt.c + 1, n_look, lookups);
      tally(cnt.c + 2, n_ev, events);
      tally(cnt.c + 3, n_cells, cells);
      mode = kIdle;
      need_init = false;
    }
    __syncwarp();
  }
  flush_counters(cnt, n_paths, n_look, n_ev, n_cells);  // widened to 64 bits
}

constexpr uint32_t kMaxStagedBytes = 96u * 1024u;

template <int kThreads, bool kStage, bool kBatch>
static vcr_status launch_t(vcr_ctx* ctx, const GridView& g, const SceneView& s, const CamView& cam,
                           const PassView& pv, uint32_t* stats, Counters cnt, uint32_t total, uint32_t maj_bytes,
                           const NrcTrainSink& ts, const BatchSink& bt, double* sum, cudaStream_t st) {
  auto kern = pt_wavefront_kernel<kThreads, kStage, kBatch>;
  size_t smem = (kStage ? align16(maj_bytes) : 0u) + (kBatch ? bt.count * sizeof(BatchView) : 0u);
  if (kStage || kBatch)  // the attribute is per device, so it is set on every launch (a host-side call)
    VCR_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(kMaxStagedBytes + kMaxBatchViews * sizeof(BatchView))));
  int per_sm = 0;
  VCR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = (uint32_t)(ctx->sm_count * per_sm);
  uint32_t need = (total + ts.paths + kThreads - 1) / kThreads;
  if (blocks > need) blocks = need;
  if (blocks == 0) return VCR_OK;
  NrcSink nq{nullptr, nullptr, 0u};
  if (s.nrc_events && ctx->nrc) nq = NrcSink{ctx->nrc->query, ctx->nrc->query_count, ctx->nrc->query_capacity};
  kern<<<blocks, kThreads, smem, st>>>(g, s, cam, pv, sum, stats, cnt, total, ctx->tuning.dda_steps, maj_bytes,
                                       wait_limits().stage_wait, nq, ts, bt, ctx->d_error);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

template <bool kBatch>
static vcr_status launch_b(vcr_ctx* ctx, const GridView& g, const SceneView& s, const CamView& cam,
                           const PassView& pv, uint32_t* stats, Counters cnt, uint32_t total, uint32_t bytes,
                           bool stage, const NrcTrainSink& ts, const BatchSink& bt, double* sum, cudaStream_t st) {
  if (ctx->tuning.block_threads == 128)
    return stage ? launch_t<128, true, kBatch>(ctx, g, s, cam, pv, stats, cnt, total, bytes, ts, bt, sum, st)
                 : launch_t<128, false, kBatch>(ctx, g, s, cam, pv, stats, cnt, total, bytes, ts, bt, sum, st);
  return stage ? launch_t<256, true, kBatch>(ctx, g, s, cam, pv, stats, cnt, total, bytes, ts, bt, sum, st)
               : launch_t<256, false, kBatch>(ctx, g, s, cam, pv, stats, cnt, total, bytes, ts, bt, sum, st);
}

vcr_status wavefront_launch(vcr_ctx* ctx, const GridView& g, const SceneView& s, const CamView& cam,
                            const PassView& pv, uint32_t* stats, Counters cnt, uint32_t total, cudaStream_t st,
                            const NrcTrainSink* train, const BatchSink* batch, double* sum) {
  const vcr_tuning& t = ctx->tuning;
  NrcTrainSink ts{nullptr, nullptr, 0u, 0u, 0.0f};
  if (train) ts = *train;
  BatchSink bt{nullptr, 0u, nullptr};
  if (batch) bt = *batch;
  if ((uint64_t)total + ts.paths >= (uint64_t)kTrainPath)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "more than 2^31 paths in one launch");
  if (batch && (train || bt.count == 0 || bt.count > kMaxBatchViews || !bt.views || !bt.pass_ctr))
    return fail(ctx, VCR_ERR_INVALID, "a batch launch needs 1..%u views and no training paths", kMaxBatchViews);
  size_t cells = (size_t)g.mnb[0] * g.mnb[1] * g.mnb[2];
  uint32_t bytes = (uint32_t)(((cells + 3) & ~(size_t)3) * sizeof(float));  // padded level: 16-byte multiple
  bool stage = t.stage_majorants && bytes <= kMaxStagedBytes;
  if (!sum) sum = ctx->d_sum;
  return batch ? launch_b<true>(ctx, g, s, cam, pv, stats, cnt, total, bytes, stage, ts, bt, sum, st)
               : launch_b<false>(ctx, g, s, cam, pv, stats, cnt, total, bytes, stage, ts, bt, sum, st);
}

}  // namespace VCR_WF_NS
}  // namespace vcr
