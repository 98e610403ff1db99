// Host-side context of the vcr C-ABI and the launch helpers each kernel file
// exports to the ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/vcr/abi.h"
#include "vcr_device.cuh"

namespace vcr {
struct PpbState;
struct PpmState;
struct NrcState;
struct BatchState;
}  // namespace vcr

struct vcr_ctx {
  int device = 0;
  int sm_count = 0;
  std::string err;

  // density grid (bricks) + majorants
  vcr_grid_desc gdesc{};
  bool has_grid = false;
  int precision = 0;
  void* d_bricks = nullptr;
  float* d_scales = nullptr;
  float* d_majorants = nullptr;  // pyramid levels 0..3, each 16-byte aligned
  size_t grid_bytes[3] = {0, 0, 0};  // allocated bytes of bricks, scales, majorants (kept for a same-size grid)
  float max_density = 0.0f;
  int nb[3] = {0, 0, 0};
  int mnb[4][3] = {};            // cells per axis of each majorant level
  size_t moff[4] = {};           // float offset of each level in d_majorants
  vcr_tuning tuning{2u, 4u, 1u, 256u, 1u, 0u};
  // per-cell blocks of the 8 decoded trilinear corners (tuning.corner_blocks)
  float4* d_corners = nullptr;
  int corner_tiles[3] = {0, 0, 0};  // 8^3-cell tiles per axis over cells -1 .. n-1
  bool corners_valid = false;       // built from the bound grid (the buffer outlives a re-upload)

  vcr_cloud cloud{};
  bool has_cloud = false;
  vcr_camera cam{};
  bool has_cam = false;
  vcr_params params{};
  bool has_params = false;

  // frame target: FP64 RGB sums
  uint32_t width = 0, height = 0;
  double* d_sum = nullptr;
  uint32_t* d_stats = nullptr;
  uint32_t passes = 0;
  uint64_t samples = 0;  // camera samples per pixel summed over passes
  // recorded on the stream of every queued pass; synchronous reads wait on
  // it (a caller's non-blocking stream does not synchronise with stream 0)
  cudaEvent_t work_done = nullptr;
  // stream-ordered read back (vcr_readback_async): two device staging slots
  // copied out on the context's copy stream
  struct Readback {
    cudaStream_t copy = nullptr;
    cudaEvent_t staged[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    void* stage[2] = {nullptr, nullptr};
    size_t bytes = 0;
    int slot = 0;
  } rb;

  // device counters: [0] paths [1] lookups [2] events [3] dda cells [4] work cursor
  // [5] grid max (u32 bits) [7] relRMSE accumulator (double bits)
  unsigned long long* d_counters = nullptr;
  int* d_error = nullptr;  // device error word (bounded waits, index checks)

  // shadow volume
  float* d_sv = nullptr;
  vcr_shadow_volume sv{};
  bool has_sv = false;

  // reusable scratch
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;

  // technique state (allocated by the technique's setup call)
  vcr::PpbState* ppb = nullptr;
  vcr::PpmState* ppm = nullptr;
  vcr::NrcState* nrc = nullptr;
  vcr::BatchState* batch = nullptr;
};

namespace vcr {

// Error helpers: record a message on the context and return a status.
vcr_status fail(vcr_ctx* ctx, vcr_status st, const char* fmt, ...);
vcr_status cuda_fail(vcr_ctx* ctx, cudaError_t e, const char* what);

#define VCR_CUDA(ctx, call)                                        \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return ::vcr::cuda_fail((ctx), e_, #call); \
  } while (0)

// Process-wide limits of the device-side waits (vcr_set_wait_limits).
constexpr uint32_t kDefaultSortLookback = 1u << 22;
constexpr uint32_t kDefaultStageWait = 1u << 24;
vcr_wait_limits wait_limits();

// What a gather launch tested (a device counter) and its device time (two
// events recorded around the launch on its stream), for the techniques'
// info calls.
struct GatherProbe {
  unsigned long long* d_count = nullptr;
  cudaEvent_t start = nullptr, stop = nullptr;
  bool recorded = false;
};
vcr_status probe_begin(vcr_ctx* ctx, GatherProbe& p, cudaStream_t s);  // allocates on first use
vcr_status probe_end(vcr_ctx* ctx, GatherProbe& p, cudaStream_t s);
vcr_status probe_read(vcr_ctx* ctx, GatherProbe& p, uint64_t& count, float& ms);  // waits for the launch
void probe_free(GatherProbe& p);

// Adds a thread's count to a launch counter, one atomic per warp (every
// lane of the warp must call it).
#if defined(__CUDACC__)
__device__ __forceinline__ void warp_count(unsigned long long* dst, uint32_t v) {
  unsigned long long t = v;
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31u) == 0 && t) atomicAdd(dst, t);
}
#endif

// Scratch buffer owned by the context (grown, never shrunk).
vcr_status ensure_scratch(vcr_ctx* ctx, size_t bytes);

GridView grid_view(const vcr_ctx* ctx);
SceneView scene_view(const vcr_ctx* ctx);

// grid.cu
// A host grid, uploaded and bricked one brick layer at a time.
vcr_status grid_upload_host(vcr_ctx* ctx, const float* host, const vcr_grid_desc* desc, int precision);
vcr_status grid_build(vcr_ctx* ctx, const float* d_dense, const vcr_grid_desc* desc, int precision,
                      cudaStream_t s);
// The corner blocks of the bound grid (after the bricks are written).
vcr_status corner_build(vcr_ctx* ctx, cudaStream_t s);
vcr_status grid_fbm_device(vcr_ctx* ctx, float* d_dense, const vcr_grid_desc* desc,
                           const vcr_fbm_desc* fbm, cudaStream_t s);
void fbm_permutation(uint64_t seed, uint8_t perm[256]);
vcr_status grid_sample_launch(vcr_ctx* ctx, const float* d_pos, float* d_out, uint32_t n,
                              cudaStream_t s);
vcr_status dda_trace_launch(vcr_ctx* ctx, const float* d_o, const float* d_d, uint32_t n,
                            uint32_t max_cells, uint32_t* d_cells, float* d_t, uint32_t* d_count,
                            cudaStream_t s);

// pt_global.cu: one pass; with `train`, the radiance cache's training
// paths run in the same wavefront launch ahead of the camera paths
struct NrcTrainSink;
// `count` consecutive passes (pass_index, pass_index + 1, ...) in one DDA
// wavefront launch when count > 1.
vcr_status pt_pass_launch(vcr_ctx* ctx, const vcr_pass_desc* pass, cudaStream_t s,
                          const NrcTrainSink* train = nullptr, uint32_t count = 1);

// ppb.cu / ppm.cu / nrc.cu: release technique state (vcr_destroy)
void ppb_free(vcr_ctx* ctx);
void ppm_free(vcr_ctx* ctx);
void nrc_free(vcr_ctx* ctx);
void batch_free(vcr_ctx* ctx);

// nrc.cu: queries of paths that end in the radiance cache
uint32_t nrc_query_capacity(const vcr_ctx* ctx);
vcr_status nrc_reset_queries(vcr_ctx* ctx, cudaStream_t s);
vcr_status nrc_infer_queries(vcr_ctx* ctx, cudaStream_t s);
vcr_status nrc_refresh_copies(vcr_ctx* ctx);

// sv.cu
vcr_status sv_build_launch(vcr_ctx* ctx, const vcr_shadow_volume* sv, cudaStream_t s);

}  // namespace vcr
