// The C-ABI layer: context lifecycle, parameter helpers that restate the
// reference's host-side struct logic, .xyz I/O, scene state and read back.
#include <cstdarg>
#include <cstring>
#include <fstream>
#include <cmath>
#include <atomic>
#include <thread>

#include "vcr_internal.h"
#include "vcr_fbm.cuh"

namespace vcr {

static thread_local std::string g_create_error;

vcr_status fail(vcr_ctx* ctx, vcr_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  else g_create_error = buf;
  return st;
}

vcr_status cuda_fail(vcr_ctx* ctx, cudaError_t e, const char* what) {
  vcr_status st = e == cudaErrorMemoryAllocation ? VCR_ERR_OOM : VCR_ERR_CUDA;
  if (e == cudaErrorMemoryAllocation) cudaGetLastError();  // clear the sticky-free error
  return fail(ctx, st, "%s: %s", what, cudaGetErrorString(e));
}

vcr_status ensure_scratch(vcr_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->scratch_bytes) return VCR_OK;
  cudaFree(ctx->d_scratch);
  ctx->d_scratch = nullptr;
  ctx->scratch_bytes = 0;
  VCR_CUDA(ctx, cudaMalloc(&ctx->d_scratch, bytes));
  ctx->scratch_bytes = bytes;
  return VCR_OK;
}

GridView grid_view(const vcr_ctx* ctx) {
  GridView g;
  g.bricks = ctx->d_bricks;
  g.scales = ctx->d_scales;
  int lv = (int)ctx->tuning.majorant_level;
  g.majorants = ctx->d_majorants ? ctx->d_majorants + ctx->moff[lv] : nullptr;
  g.level = lv;
  for (int a = 0; a < 3; ++a) {
    g.n[a] = (int)ctx->gdesc.size[a];
    g.nb[a] = ctx->nb[a];
    g.mnb[a] = ctx->mnb[lv][a];
  }
  g.precision = ctx->precision;
  g.corners = (ctx->tuning.corner_blocks && ctx->d_corners && ctx->corners_valid) ? ctx->d_corners : nullptr;
  for (int a = 0; a < 3; ++a) g.ctiles[a] = ctx->corner_tiles[a];
  return g;
}

SceneView scene_view(const vcr_ctx* ctx) {
  SceneView s{};
  const vcr_cloud& c = ctx->cloud;
  s.b0 = mk(c.bounds_min[0], c.bounds_min[1], c.bounds_min[2]);
  s.b1 = mk(c.bounds_max[0], c.bounds_max[1], c.bounds_max[2]);
  s.max_ext = c.max_extinction;
  s.ds = c.density_scaling;
  s.bs = c.base_scaling;
  s.k_sigma = c.density_scaling / c.base_scaling;
  f3 ext = s.b1 - s.b0;
  const float cv = (float)(kBrick << ctx->tuning.majorant_level);  // voxels per majorant cell
  s.cell.x = (ext.x / (float)ctx->gdesc.size[0]) * cv;
  s.cell.y = (ext.y / (float)ctx->gdesc.size[1]) * cv;
  s.cell.z = (ext.z / (float)ctx->gdesc.size[2]) * cv;
  s.icell = mk(1.0f / s.cell.x, 1.0f / s.cell.y, 1.0f / s.cell.z);
  s.iext = mk(1.0f / ext.x, 1.0f / ext.y, 1.0f / ext.z);
  const vcr_params& p = ctx->params;
  s.ph.g = p.phase_g;
  s.ph.opg2 = p.phase_one_plus_g2;
  s.ph.omg2 = p.phase_one_minus_g2;
  s.ph.o2g = p.phase_one_over_2g;
  s.ph.iso = p.isotropic;
  s.albedo = p.albedo;
  s.light = p.light_intensity;
  s.sun = mk(p.sun_dir[0], p.sun_dir[1], p.sun_dir[2]);
  s.sky = mk(p.sky[0], p.sky[1], p.sky[2]);
  s.sky_mode = (int)p.sky_mode;
  s.rng_mode = (int)p.rng_mode;
  s.nee_mode = (int)p.nee_mode;
  s.tracker = (int)p.tracker;
  s.max_events = p.max_events;
  s.nrc_events = ctx->nrc ? p.nrc_events : 0u;
  return s;
}

__global__ void mean_kernel(const double* __restrict__ sum, float* __restrict__ out, size_t n, double inv) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)(sum[i] * inv);
}

// sum over pixels of sum_c (sum*inv - ref)^2 / (ref^2 + 1e-2); block partials
// into acc (zeroed by the caller), finished by rel_rmse_finish.
__global__ void rel_rmse_kernel(const double* __restrict__ sum, const double* __restrict__ ref, size_t n, double inv,
                                double* __restrict__ acc) {
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double r = ref[i], d = sum[i] * inv - r;
    s += d * d / (r * r + 1e-2);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ double part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(acc, s);
  }
}

__global__ void rel_rmse_finish(const double* __restrict__ acc, double px, double* __restrict__ out) {
  *out = sqrt(*acc / px);
}

}  // namespace vcr

using namespace vcr;

// ---------------------------------------------------------------------------
// lifecycle
// ---------------------------------------------------------------------------
extern "C" VCR_API uint32_t vcr_version(void) { return 0x000100u; }

extern "C" VCR_API const char* vcr_last_error(const vcr_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

extern "C" VCR_API vcr_status vcr_create(vcr_ctx** out, const vcr_device_desc* desc) {
  if (!out) return fail(nullptr, VCR_ERR_INVALID, "vcr_create: null output pointer");
  *out = nullptr;
  int dev = desc ? desc->device : 0;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(nullptr, VCR_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= count) return fail(nullptr, VCR_ERR_INVALID, "device %d of %d", dev, count);
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return fail(nullptr, VCR_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  vcr_ctx* ctx = new vcr_ctx();
  ctx->device = dev;
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, dev);
  e = cudaMalloc(&ctx->d_counters, 8 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_error, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_counters, 0, 8 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_error, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->work_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->work_done, 0);
  if (e != cudaSuccess) {
    vcr_status st = fail(nullptr, VCR_ERR_CUDA, "context allocation: %s", cudaGetErrorString(e));
    cudaFree(ctx->d_counters);
    cudaFree(ctx->d_error);
    delete ctx;
    return st;
  }
  *out = ctx;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_destroy(vcr_ctx* ctx) {
  if (!ctx) return VCR_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  void* ptrs[] = {ctx->d_bricks, ctx->d_scales, ctx->d_majorants, ctx->d_sum, ctx->d_stats,
                  ctx->d_counters, ctx->d_error, ctx->d_sv, ctx->d_scratch, ctx->d_corners};
  for (void* p : ptrs) cudaFree(p);
  ppb_free(ctx);
  ppm_free(ctx);
  nrc_free(ctx);
  batch_free(ctx);
  if (ctx->work_done) cudaEventDestroy(ctx->work_done);
  for (int i = 0; i < 2; ++i) {
    cudaFree(ctx->rb.stage[i]);
    if (ctx->rb.staged[i]) cudaEventDestroy(ctx->rb.staged[i]);
    if (ctx->rb.copied[i]) cudaEventDestroy(ctx->rb.copied[i]);
  }
  if (ctx->rb.copy) cudaStreamDestroy(ctx->rb.copy);
  delete ctx;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_synchronize(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  int err = 0;
  VCR_CUDA(ctx, cudaMemcpy(&err, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(ctx->d_error, 0, sizeof(int));
    return fail(ctx, VCR_ERR_TIMEOUT, "device error word %d (bounded wait ran out)", err);
  }
  return VCR_OK;
}

namespace vcr {
vcr_status probe_begin(vcr_ctx* ctx, GatherProbe& p, cudaStream_t s) {
  if (!p.d_count) {
    VCR_CUDA(ctx, cudaMalloc(&p.d_count, sizeof(unsigned long long)));
    VCR_CUDA(ctx, cudaEventCreate(&p.start));
    VCR_CUDA(ctx, cudaEventCreate(&p.stop));
  }
  VCR_CUDA(ctx, cudaMemsetAsync(p.d_count, 0, sizeof(unsigned long long), s));
  VCR_CUDA(ctx, cudaEventRecord(p.start, s));
  return VCR_OK;
}

vcr_status probe_end(vcr_ctx* ctx, GatherProbe& p, cudaStream_t s) {
  VCR_CUDA(ctx, cudaEventRecord(p.stop, s));
  p.recorded = true;
  return VCR_OK;
}

vcr_status probe_read(vcr_ctx* ctx, GatherProbe& p, uint64_t& count, float& ms) {
  count = 0;
  ms = 0.0f;
  if (!p.recorded) return VCR_OK;
  VCR_CUDA(ctx, cudaEventSynchronize(p.stop));
  VCR_CUDA(ctx, cudaEventElapsedTime(&ms, p.start, p.stop));
  unsigned long long c = 0;
  VCR_CUDA(ctx, cudaMemcpy(&c, p.d_count, sizeof c, cudaMemcpyDeviceToHost));
  count = c;
  return VCR_OK;
}

void probe_free(GatherProbe& p) {
  cudaFree(p.d_count);
  if (p.start) cudaEventDestroy(p.start);
  if (p.stop) cudaEventDestroy(p.stop);
  p = GatherProbe{};
}

static std::atomic<uint32_t> g_sort_lookback{kDefaultSortLookback};
static std::atomic<uint32_t> g_stage_wait{kDefaultStageWait};

vcr_wait_limits wait_limits() { return vcr_wait_limits{g_sort_lookback.load(), g_stage_wait.load()}; }
}  // namespace vcr

extern "C" VCR_API vcr_status vcr_set_wait_limits(const vcr_wait_limits* limits) {
  g_sort_lookback.store(limits ? limits->sort_lookback : kDefaultSortLookback);
  g_stage_wait.store(limits ? limits->stage_wait : kDefaultStageWait);
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_get_wait_limits(vcr_wait_limits* out) {
  if (!out) return fail(nullptr, VCR_ERR_INVALID, "null wait limits");
  *out = wait_limits();
  return VCR_OK;
}

// ---------------------------------------------------------------------------
// parameter helpers (host restatements of UniformBuffers.h / main.cpp logic)
// ---------------------------------------------------------------------------
extern "C" VCR_API vcr_status vcr_params_set_phase_g(vcr_params* p, float value) {
  if (!p) return fail(nullptr, VCR_ERR_INVALID, "null params");
  if (value > 1.0f || value < -1.0f) return VCR_OK;  // ignored, as SetPhaseG does
  float g = std::min(std::max(value, -0.95f), 0.95f);
  p->phase_g = g;
  p->isotropic = std::fabs(g) < 0.0001f ? 1 : 0;
  if (!p->isotropic) {
    p->phase_one_plus_g2 = 1.0f + g * g;
    p->phase_one_minus_g2 = 1.0f - g * g;
    p->phase_one_over_2g = 0.5f / g;
  }
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_cloud_from_grid(const vcr_grid_desc* grid, float base_scaling,
                                                  float density_scaling, vcr_cloud* out) {
  if (!grid || !out) return fail(nullptr, VCR_ERR_INVALID, "null argument");
  float size[3];
  for (int a = 0; a < 3; ++a)
    size[a] = (float)(grid->voxel_size[a] * (double)grid->size[a] * (double)base_scaling);
  out->bounds_min[0] = -size[0] / 2.0f;
  out->bounds_min[1] = -size[1] / 2.0f;
  out->bounds_min[2] = 0.0f;
  out->bounds_max[0] = size[0] / 2.0f;
  out->bounds_max[1] = size[1] / 2.0f;
  out->bounds_max[2] = size[2];
  out->max_extinction = 0.0f;  // filled from the grid by vcr_set_cloud
  out->base_scaling = base_scaling;
  out->density_scaling = density_scaling;
  return VCR_OK;
}

static void orthonormal_basis(const float n[3], float xp[3], float yp[3]) {
  float sz = n[2] >= 0.0f ? 1.0f : -1.0f;
  float a = n[1] / (1.0f + std::fabs(n[2]));
  float b = n[1] * a;
  float c = -n[0] * a;
  xp[0] = n[2] + sz * b; xp[1] = sz * c; xp[2] = -n[0];
  yp[0] = c; yp[1] = 1.0f - b; yp[2] = -sz * n[1];
}

extern "C" VCR_API vcr_status vcr_camera_look(vcr_camera* cam, const float position[3], const float forward[3],
                                              float fov_y_deg, float near_plane, int32_t width, int32_t height) {
  if (!cam || !position || !forward || width < 2 || height < 2 || !(near_plane > 0.0f))
    return fail(nullptr, VCR_ERR_INVALID, "vcr_camera_look: bad argument");
  double l = std::sqrt((double)forward[0] * forward[0] + (double)forward[1] * forward[1] +
                       (double)forward[2] * forward[2]);
  if (!(l > 0.0)) return fail(nullptr, VCR_ERR_INVALID, "vcr_camera_look: zero forward vector");
  for (int a = 0; a < 3; ++a) {
    cam->position[a] = position[a];
    cam->forward[a] = (float)(forward[a] / l);
  }
  orthonormal_basis(cam->forward, cam->right, cam->up);
  cam->near_plane = near_plane;
  cam->half_width = width / 2;
  cam->half_height = height / 2;
  float fov = std::min(std::max(fov_y_deg, 60.0f), 150.0f);  // SetFOV clamp (UniformBuffers.h:54)
  float h = 2.0f * std::tan(fov / 2.0f * 3.14159265358979f / 180.0f) * near_plane;
  cam->pixel_size_y = h / (float)(cam->half_height * 2);
  cam->pixel_size_x = cam->pixel_size_y * (float)cam->half_height / (float)cam->half_width;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_shadow_volume_setup(vcr_shadow_volume* sv, const float light_dir[3],
                                                      const float bounds_min[3], const float bounds_max[3],
                                                      uint32_t voxel_axis_count) {
  if (!sv || !light_dir || !bounds_min || !bounds_max || voxel_axis_count < 2)
    return fail(nullptr, VCR_ERR_INVALID, "vcr_shadow_volume_setup: bad argument");
  double l = std::sqrt((double)light_dir[0] * light_dir[0] + (double)light_dir[1] * light_dir[1] +
                       (double)light_dir[2] * light_dir[2]);
  if (!(l > 0.0)) return fail(nullptr, VCR_ERR_INVALID, "zero light direction");
  float d[3] = {(float)(light_dir[0] / l), (float)(light_dir[1] / l), (float)(light_dir[2] / l)};
  float r[3], u[3];
  orthonormal_basis(d, r, u);  // SetLightDirection (UniformBuffers.h:131-143)
  // SetOrigin (UniformBuffers.h:145-151): sphere around the AABB
  double dx = bounds_max[0] - bounds_min[0], dy = bounds_max[1] - bounds_min[1], dz = bounds_max[2] - bounds_min[2];
  float radius = (float)(std::sqrt(dx * dx + dy * dy + dz * dz) / 2.0);
  sv->voxel_axis_count = voxel_axis_count;
  sv->voxel_size = (2.0f * radius) / (float)(voxel_axis_count - 1);
  float center[3];
  for (int a = 0; a < 3; ++a) center[a] = (bounds_min[a] + bounds_max[a]) / 2.0f;
  // UpdateOrigin (UniformBuffers.h:159-166)
  for (int a = 0; a < 3; ++a) {
    float corner = radius * (-d[a] - r[a] - u[a]);
    sv->bounds_min[a] = center[a] + corner;
    sv->bounds_max[a] = center[a] - corner;
    sv->light_dir[a] = d[a];
    sv->right[a] = r[a];
    sv->up[a] = u[a];
  }
  // basisChange = inverse([right | up | light]) computed in double
  double M[3][3] = {{r[0], u[0], d[0]}, {r[1], u[1], d[1]}, {r[2], u[2], d[2]}};
  double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
               M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
  if (std::fabs(det) < 1e-12) return fail(nullptr, VCR_ERR_INVALID, "degenerate light basis");
  double inv[3][3];
  inv[0][0] = (M[1][1] * M[2][2] - M[1][2] * M[2][1]) / det;
  inv[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
  inv[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
  inv[1][0] = (M[1][2] * M[2][0] - M[1][0] * M[2][2]) / det;
  inv[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
  inv[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
  inv[2][0] = (M[1][0] * M[2][1] - M[1][1] * M[2][0]) / det;
  inv[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
  inv[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) sv->basis_change[3 * i + j] = (float)inv[i][j];
  return VCR_OK;
}

// ---------------------------------------------------------------------------
// grid
// ---------------------------------------------------------------------------
static vcr_status check_grid_desc(vcr_ctx* ctx, const vcr_grid_desc* desc, vcr_precision precision) {
  if (!desc) return fail(ctx, VCR_ERR_INVALID, "null grid descriptor");
  for (int a = 0; a < 3; ++a)
    if (desc->size[a] == 0 || desc->size[a] > 8192)
      return fail(ctx, VCR_ERR_INVALID, "grid axis %d has %u voxels (1..8192)", a, desc->size[a]);
  if ((int)precision < 0 || (int)precision > 2) return fail(ctx, VCR_ERR_INVALID, "bad precision %d", (int)precision);
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_grid_upload(vcr_ctx* ctx, const vcr_grid_desc* desc, const float* host,
                                              vcr_precision precision) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  vcr_status st = check_grid_desc(ctx, desc, precision);
  if (st) return st;
  if (!host) return fail(ctx, VCR_ERR_INVALID, "null host density");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  return grid_upload_host(ctx, host, desc, (int)precision);
}

extern "C" VCR_API vcr_status vcr_grid_generate(vcr_ctx* ctx, const vcr_grid_desc* desc, const vcr_fbm_desc* fbm,
                                                vcr_precision precision) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  vcr_status st = check_grid_desc(ctx, desc, precision);
  if (st) return st;
  if (!fbm || fbm->octaves == 0 || fbm->octaves > 16) return fail(ctx, VCR_ERR_INVALID, "fbm octaves must be 1..16");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  size_t bytes = (size_t)desc->size[0] * desc->size[1] * desc->size[2] * sizeof(float);
  float* d_dense = nullptr;
  VCR_CUDA(ctx, cudaMalloc(&d_dense, bytes));
  st = grid_fbm_device(ctx, d_dense, desc, fbm, 0);
  if (!st) st = grid_build(ctx, d_dense, desc, (int)precision, 0);
  cudaFree(d_dense);
  return st;
}

extern "C" VCR_API vcr_status vcr_grid_info(vcr_ctx* ctx, float* out_max, uint32_t out_bricks[3]) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->has_grid) return fail(ctx, VCR_ERR_STATE, "no grid");
  if (out_max) *out_max = ctx->max_density;
  if (out_bricks)
    for (int a = 0; a < 3; ++a) out_bricks[a] = (uint32_t)ctx->nb[a];
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_grid_read_majorants(vcr_ctx* ctx, uint32_t level, float* host, size_t count) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->has_grid) return fail(ctx, VCR_ERR_STATE, "no grid");
  if (level > 3) return fail(ctx, VCR_ERR_INVALID, "majorant level %u (0..3)", level);
  const int* m = ctx->mnb[level];
  size_t nb = (size_t)m[0] * m[1] * m[2];
  if (!host || count != nb) return fail(ctx, VCR_ERR_INVALID, "majorant count %zu != %zu", count, nb);
  VCR_CUDA(ctx, cudaMemcpy(host, ctx->d_majorants + ctx->moff[level], nb * sizeof(float), cudaMemcpyDeviceToHost));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_set_tuning(vcr_ctx* ctx, const vcr_tuning* t) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!t || t->majorant_level > 3 || t->dda_steps == 0 || t->dda_steps > 4096 ||
      (t->block_threads != 128 && t->block_threads != 256) || t->corner_blocks > 1 || t->fast_math > 1)
    return fail(ctx, VCR_ERR_INVALID,
                "tuning: level 0..3, dda_steps 1..4096, block_threads 128 or 256, corner_blocks and fast_math 0 "
                "or 1");
  ctx->tuning = *t;
  if (!t->corner_blocks && ctx->d_corners) {  // switched off: the memory goes back (cudaFree waits for the device)
    cudaFree(ctx->d_corners);
    ctx->d_corners = nullptr;
    ctx->corners_valid = false;
  }
  if (t->corner_blocks && ctx->has_grid && !ctx->corners_valid) {  // switched on after the grid was bound
    vcr_status st = corner_build(ctx, 0);
    if (st) return st;
    VCR_CUDA(ctx, cudaStreamSynchronize(0));
  }
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_get_tuning(vcr_ctx* ctx, vcr_tuning* out) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  *out = ctx->tuning;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_grid_sample(vcr_ctx* ctx, const float* d_pos, float* d_out, uint32_t n,
                                              void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->has_grid || !ctx->has_cloud) return fail(ctx, VCR_ERR_STATE, "sampling needs a grid and a cloud");
  if (n && (!d_pos || !d_out)) return fail(ctx, VCR_ERR_INVALID, "null buffer");
  return grid_sample_launch(ctx, d_pos, d_out, n, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_fbm_fill_host(const vcr_grid_desc* desc, const vcr_fbm_desc* fbm, float* out) {
  if (!desc || !fbm || !out) return fail(nullptr, VCR_ERR_INVALID, "null argument");
  FbmConst c{};
  fbm_make_perm(fbm->seed, c.perm);
  for (int a = 0; a < 3; ++a) c.n[a] = desc->size[a];
  c.octaves = fbm->octaves;
  c.lacunarity = fbm->lacunarity;
  c.gain = fbm->gain;
  c.f0 = fbm->base_frequency;
  size_t nx = desc->size[0], ny = desc->size[1], nz = desc->size[2];
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([&, t]() {
      for (size_t k = t; k < nz; k += nt)
        for (size_t j = 0; j < ny; ++j)
          for (size_t i = 0; i < nx; ++i)
            out[i + nx * (j + ny * k)] = fbm_density(c, (uint32_t)i, (uint32_t)j, (uint32_t)k);
    });
  for (auto& th : pool) th.join();
  return VCR_OK;
}

// .xyz: 3 x u32 counts, 3 x f64 voxel size, then floats with z fastest
// (GridData::save, GridData.h:12-25); loaded into x-fastest memory as
// Grid3D::Load does (Grid3D.h:73-85).
extern "C" VCR_API vcr_status vcr_xyz_read(const char* path, vcr_grid_desc* desc, float* out, size_t capacity) {
  if (!path || !desc) return fail(nullptr, VCR_ERR_INVALID, "null argument");
  std::ifstream in(path, std::ios::binary);
  if (!in.good()) return fail(nullptr, VCR_ERR_IO, "cannot open %s", path);
  uint32_t n[3];
  double vs[3];
  in.read(reinterpret_cast<char*>(n), sizeof(n));
  in.read(reinterpret_cast<char*>(vs), sizeof(vs));
  if (!in.good()) return fail(nullptr, VCR_ERR_IO, "%s: short header", path);
  for (int a = 0; a < 3; ++a) {
    desc->size[a] = n[a];
    desc->voxel_size[a] = vs[a];
  }
  desc->_pad = 0;
  if (!out) return VCR_OK;
  size_t total = (size_t)n[0] * n[1] * n[2];
  if (capacity < total) return fail(nullptr, VCR_ERR_CAPACITY, "%s: %zu voxels, capacity %zu", path, total, capacity);
  std::vector<float> file(total);
  in.read(reinterpret_cast<char*>(file.data()), (std::streamsize)(total * sizeof(float)));
  if ((size_t)in.gcount() != total * sizeof(float)) return fail(nullptr, VCR_ERR_IO, "%s: short data", path);
  size_t f = 0;
  for (size_t x = 0; x < n[0]; ++x)
    for (size_t y = 0; y < n[1]; ++y)
      for (size_t z = 0; z < n[2]; ++z) out[x + n[0] * (y + n[1] * z)] = file[f++];
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_xyz_write(const char* path, const vcr_grid_desc* desc, const float* data) {
  if (!path || !desc || !data) return fail(nullptr, VCR_ERR_INVALID, "null argument");
  std::ofstream out(path, std::ios::binary);
  if (!out.good()) return fail(nullptr, VCR_ERR_IO, "cannot create %s", path);
  uint32_t n[3] = {desc->size[0], desc->size[1], desc->size[2]};
  out.write(reinterpret_cast<const char*>(n), sizeof(n));
  out.write(reinterpret_cast<const char*>(desc->voxel_size), 3 * sizeof(double));
  std::vector<float> file((size_t)n[0] * n[1] * n[2]);
  size_t f = 0;
  for (size_t x = 0; x < n[0]; ++x)
    for (size_t y = 0; y < n[1]; ++y)
      for (size_t z = 0; z < n[2]; ++z) file[f++] = data[x + n[0] * (y + n[1] * z)];
  out.write(reinterpret_cast<const char*>(file.data()), (std::streamsize)(file.size() * sizeof(float)));
  if (!out.good()) return fail(nullptr, VCR_ERR_IO, "write failed: %s", path);
  return VCR_OK;
}

// ---------------------------------------------------------------------------
// scene state
// ---------------------------------------------------------------------------
extern "C" VCR_API vcr_status vcr_set_cloud(vcr_ctx* ctx, const vcr_cloud* cloud) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!cloud) return fail(ctx, VCR_ERR_INVALID, "null cloud");
  for (int a = 0; a < 3; ++a)
    if (!(cloud->bounds_max[a] > cloud->bounds_min[a])) return fail(ctx, VCR_ERR_INVALID, "empty cloud bounds");
  if (!(cloud->base_scaling > 0.0f)) return fail(ctx, VCR_ERR_INVALID, "base_scaling must be > 0");
  ctx->cloud = *cloud;
  if (!(ctx->cloud.max_extinction > 0.0f)) {
    if (!ctx->has_grid) return fail(ctx, VCR_ERR_STATE, "max_extinction <= 0 needs a grid to derive it");
    ctx->cloud.max_extinction = std::max(ctx->max_density, 0.01f);  // main.cpp:152
  }
  ctx->has_cloud = true;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_set_camera(vcr_ctx* ctx, const vcr_camera* cam) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!cam) return fail(ctx, VCR_ERR_INVALID, "null camera");
  ctx->cam = *cam;
  ctx->has_cam = true;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_set_params(vcr_ctx* ctx, const vcr_params* p) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!p) return fail(ctx, VCR_ERR_INVALID, "null params");
  if (p->rng_mode > 1 || p->nee_mode > 1 || p->sky_mode > 1 || p->tracker > 1)
    return fail(ctx, VCR_ERR_INVALID, "bad mode enum");
  ctx->params = *p;
  ctx->has_params = true;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_set_frame(vcr_ctx* ctx, uint32_t width, uint32_t height) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 28))
    return fail(ctx, VCR_ERR_INVALID, "frame %ux%u", width, height);
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (width != ctx->width || height != ctx->height) {
    cudaFree(ctx->d_sum);
    cudaFree(ctx->d_stats);
    ctx->d_sum = nullptr;
    ctx->d_stats = nullptr;
    ctx->width = ctx->height = 0;
    size_t px = (size_t)width * height;
    VCR_CUDA(ctx, cudaMalloc(&ctx->d_sum, px * 3 * sizeof(double)));
    VCR_CUDA(ctx, cudaMalloc(&ctx->d_stats, px * 4 * sizeof(uint32_t)));
    ctx->width = width;
    ctx->height = height;
  }
  return vcr_reset_accumulation(ctx);
}

extern "C" VCR_API vcr_status vcr_reset_accumulation(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "no frame");
  size_t px = (size_t)ctx->width * ctx->height;
  VCR_CUDA(ctx, cudaMemset(ctx->d_sum, 0, px * 3 * sizeof(double)));
  VCR_CUDA(ctx, cudaMemset(ctx->d_stats, 0, px * 4 * sizeof(uint32_t)));
  ctx->passes = 0;
  ctx->samples = 0;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_shadow_volume_build(vcr_ctx* ctx, const vcr_shadow_volume* sv, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!sv) return fail(ctx, VCR_ERR_INVALID, "null shadow volume");
  return sv_build_launch(ctx, sv, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_pt_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  return pt_pass_launch(ctx, pass, (cudaStream_t)stream);
}

extern "C" VCR_API vcr_status vcr_pt_passes(vcr_ctx* ctx, const vcr_pass_desc* first, uint32_t count,
                                            void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!first) return fail(ctx, VCR_ERR_INVALID, "null pass");
  return pt_pass_launch(ctx, first, (cudaStream_t)stream, nullptr, count);
}

extern "C" VCR_API vcr_status vcr_pt_counters(vcr_ctx* ctx, uint64_t out[4]) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  unsigned long long c[4];
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  VCR_CUDA(ctx, cudaMemcpy(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; ++i) out[i] = c[i];
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_dda_trace(vcr_ctx* ctx, const float* d_o, const float* d_d, uint32_t n,
                                            uint32_t max_cells, uint32_t* d_cells, float* d_t, uint32_t* d_count,
                                            void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->has_grid || !ctx->has_cloud) return fail(ctx, VCR_ERR_STATE, "DDA needs a grid and a cloud");
  if (n && (!d_o || !d_d || !d_cells || !d_t || !d_count || max_cells == 0))
    return fail(ctx, VCR_ERR_INVALID, "bad DDA buffers");
  return dda_trace_launch(ctx, d_o, d_d, n, max_cells, d_cells, d_t, d_count, (cudaStream_t)stream);
}

// The copy stream, events and `bytes`-sized staging slots of the
// stream-ordered read back (created on first use).
static vcr_status readback_ring(vcr_ctx* ctx, size_t bytes) {
  vcr_ctx::Readback& r = ctx->rb;
  if (!r.copy) {
    VCR_CUDA(ctx, cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
      VCR_CUDA(ctx, cudaEventCreateWithFlags(&r.staged[i], cudaEventDisableTiming));
      VCR_CUDA(ctx, cudaEventCreateWithFlags(&r.copied[i], cudaEventDisableTiming));
      VCR_CUDA(ctx, cudaEventRecord(r.copied[i], r.copy));
    }
  }
  if (r.bytes < bytes) {
    VCR_CUDA(ctx, cudaStreamSynchronize(r.copy));
    for (int i = 0; i < 2; ++i) {
      cudaFree(r.stage[i]);
      r.stage[i] = nullptr;
    }
    r.bytes = 0;
    for (int i = 0; i < 2; ++i) VCR_CUDA(ctx, cudaMalloc(&r.stage[i], bytes));
    r.bytes = bytes;
  }
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_readback_async(vcr_ctx* ctx, vcr_buffer_id id, void* host, size_t bytes,
                                                 void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!host) return fail(ctx, VCR_ERR_INVALID, "null host buffer");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "no frame");
  const size_t n = (size_t)ctx->width * ctx->height * 3;
  if (id == VCR_BUF_IMAGE_MEAN) {
    if (bytes != n * sizeof(float)) return fail(ctx, VCR_ERR_INVALID, "mean image is %zu bytes", n * 4);
  } else if (id == VCR_BUF_IMAGE_SUM) {
    if (bytes != n * sizeof(double)) return fail(ctx, VCR_ERR_INVALID, "sum image is %zu bytes", n * 8);
  } else {
    return fail(ctx, VCR_ERR_UNSUPPORTED, "buffer id %d has no stream-ordered read back", (int)id);
  }
  vcr_status rs = readback_ring(ctx, bytes);
  if (rs) return rs;
  vcr_ctx::Readback& r = ctx->rb;
  const int k = r.slot;
  r.slot ^= 1;
  cudaStream_t st = (cudaStream_t)stream;
  VCR_CUDA(ctx, cudaStreamWaitEvent(st, r.copied[k], 0));  // the slot's previous copy has landed
  if (id == VCR_BUF_IMAGE_MEAN) {
    const double inv = ctx->samples ? 1.0 / (double)ctx->samples : 0.0;  // passes queued so far
    mean_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ctx->d_sum, (float*)r.stage[k], n, inv);
    VCR_CUDA(ctx, cudaGetLastError());
  } else {
    VCR_CUDA(ctx, cudaMemcpyAsync(r.stage[k], ctx->d_sum, bytes, cudaMemcpyDeviceToDevice, st));
  }
  VCR_CUDA(ctx, cudaEventRecord(r.staged[k], st));
  VCR_CUDA(ctx, cudaStreamWaitEvent(r.copy, r.staged[k], 0));
  VCR_CUDA(ctx, cudaMemcpyAsync(host, r.stage[k], bytes, cudaMemcpyDeviceToHost, r.copy));
  VCR_CUDA(ctx, cudaEventRecord(r.copied[k], r.copy));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_readback_wait(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (ctx->rb.copy) VCR_CUDA(ctx, cudaStreamSynchronize(ctx->rb.copy));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_readback(vcr_ctx* ctx, vcr_buffer_id id, void* host, size_t bytes) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!host) return fail(ctx, VCR_ERR_INVALID, "null host buffer");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));  // after the last queued pass
  size_t px = (size_t)ctx->width * ctx->height;
  switch (id) {
    case VCR_BUF_IMAGE_MEAN: {
      if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "no frame");
      if (bytes != px * 3 * sizeof(float)) return fail(ctx, VCR_ERR_INVALID, "mean image is %zu bytes", px * 3 * 4);
      vcr_status st = ensure_scratch(ctx, px * 3 * sizeof(float));
      if (st) return st;
      double inv = ctx->samples ? 1.0 / (double)ctx->samples : 0.0;
      size_t n = px * 3;
      mean_kernel<<<(unsigned)((n + 255) / 256), 256>>>(ctx->d_sum, (float*)ctx->d_scratch, n, inv);
      VCR_CUDA(ctx, cudaGetLastError());
      VCR_CUDA(ctx, cudaMemcpy(host, ctx->d_scratch, bytes, cudaMemcpyDefault));
      return VCR_OK;
    }
    case VCR_BUF_IMAGE_SUM:
      if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "no frame");
      if (bytes != px * 3 * sizeof(double)) return fail(ctx, VCR_ERR_INVALID, "sum image is %zu bytes", px * 24);
      VCR_CUDA(ctx, cudaMemcpy(host, ctx->d_sum, bytes, cudaMemcpyDefault));
      return VCR_OK;
    case VCR_BUF_PATH_STATS:
      if (!ctx->d_stats) return fail(ctx, VCR_ERR_STATE, "no frame");
      if (bytes != px * 4 * sizeof(uint32_t)) return fail(ctx, VCR_ERR_INVALID, "stats are %zu bytes", px * 16);
      VCR_CUDA(ctx, cudaMemcpy(host, ctx->d_stats, bytes, cudaMemcpyDefault));
      return VCR_OK;
    case VCR_BUF_SHADOW_VOLUME: {
      if (!ctx->has_sv) return fail(ctx, VCR_ERR_STATE, "no shadow volume");
      size_t n = (size_t)ctx->sv.voxel_axis_count;
      if (bytes != n * n * n * sizeof(float)) return fail(ctx, VCR_ERR_INVALID, "shadow volume is %zu bytes", n * n * n * 4);
      VCR_CUDA(ctx, cudaMemcpy(host, ctx->d_sv, bytes, cudaMemcpyDefault));
      return VCR_OK;
    }
    default:
      return fail(ctx, VCR_ERR_UNSUPPORTED, "buffer id %d not readable here", (int)id);
  }
}

extern "C" VCR_API vcr_status vcr_image_rel_rmse(vcr_ctx* ctx, const double* d_ref, double* d_out, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!d_ref || !d_out) return fail(ctx, VCR_ERR_INVALID, "null reference or output");
  if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "no frame");
  cudaStream_t s = (cudaStream_t)stream;
  size_t px = (size_t)ctx->width * ctx->height;
  double inv = ctx->samples ? 1.0 / (double)ctx->samples : 0.0;
  double* acc = reinterpret_cast<double*>(ctx->d_counters + 7);
  VCR_CUDA(ctx, cudaMemsetAsync(acc, 0, sizeof(double), s));
  unsigned blocks = (unsigned)std::min<size_t>((px * 3 + 255) / 256, (size_t)ctx->sm_count * 8);
  rel_rmse_kernel<<<blocks, 256, 0, s>>>(ctx->d_sum, d_ref, px * 3, inv, acc);
  VCR_CUDA(ctx, cudaGetLastError());
  rel_rmse_finish<<<1, 1, 0, s>>>(acc, (double)px, d_out);
  VCR_CUDA(ctx, cudaGetLastError());
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_pass_count(vcr_ctx* ctx, uint32_t* out) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  *out = ctx->passes;
  return VCR_OK;
}
