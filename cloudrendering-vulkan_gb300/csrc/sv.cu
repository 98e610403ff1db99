// Shadow volume: a light-aligned n^3 grid of approximate sun transmittance,
// exp(-(z+1) * voxelSize * mean density along the column), the
// reference-parity NEE term.
//
// Reference: ShadowVolume.comp:77-93 (one thread per (x,y) column marching z),
// calculateVoxelPosition (Tests.cpp:104-110 restates it on the CPU),
// dispatch RenderTechniqueSV.cpp:102-113.
#include "vcr_internal.h"

namespace vcr {

struct SvBuild {
  f3 b0, right, up, light;
  float vs;
  int n;
};

// One thread per column; consecutive threads take consecutive x so every
// z-slice store is coalesced.
__global__ void __launch_bounds__(256) sv_build_kernel(GridView g, SceneView s, SvBuild b, float* __restrict__ out) {
  uint32_t col = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t n = (uint32_t)b.n;
  if (col >= n * n) return;
  uint32_t x = col % n, y = col / n;
  float acc = 0.0f, dist = 0.0f;
  size_t plane = (size_t)n * n;
  for (uint32_t z = 0; z < n; ++z) {
    float fx = (float)x * b.vs, fy = (float)y * b.vs, fz = (float)z * b.vs;
    f3 p;
    p.x = ((b.b0.x + fx * b.right.x) + fy * b.up.x) + fz * b.light.x;
    p.y = ((b.b0.y + fx * b.right.y) + fy * b.up.y) + fz * b.light.y;
    p.z = ((b.b0.z + fx * b.right.z) + fy * b.up.z) + fz * b.light.z;
    if (in_box(p, s.b0, s.b1)) acc = acc + (density_at(g, s, p) * s.ds) / s.bs;
    dist = dist + b.vs;
    out[(size_t)col + plane * z] = vexp(((-dist) * acc) / (float)(z + 1));
  }
}

vcr_status sv_build_launch(vcr_ctx* ctx, const vcr_shadow_volume* sv, cudaStream_t st) {
  if (!ctx->has_grid || !ctx->has_cloud) return fail(ctx, VCR_ERR_STATE, "shadow volume needs a grid and a cloud");
  uint32_t n = sv->voxel_axis_count;
  if (n < 2 || n > 1024) return fail(ctx, VCR_ERR_INVALID, "shadow volume axis count %u outside [2, 1024]", n);
  size_t bytes = (size_t)n * n * n * sizeof(float);
  if (!ctx->has_sv || ctx->sv.voxel_axis_count != n) {
    cudaFree(ctx->d_sv);
    ctx->d_sv = nullptr;
    ctx->has_sv = false;
    VCR_CUDA(ctx, cudaMalloc(&ctx->d_sv, bytes));
  }
  SvBuild b;
  b.b0 = mk(sv->bounds_min[0], sv->bounds_min[1], sv->bounds_min[2]);
  b.right = mk(sv->right[0], sv->right[1], sv->right[2]);
  b.up = mk(sv->up[0], sv->up[1], sv->up[2]);
  b.light = mk(sv->light_dir[0], sv->light_dir[1], sv->light_dir[2]);
  b.vs = sv->voxel_size;
  b.n = (int)n;
  uint32_t cols = n * n;
  sv_build_kernel<<<(cols + 255) / 256, 256, 0, st>>>(grid_view(ctx), scene_view(ctx), b, ctx->d_sv);
  VCR_CUDA(ctx, cudaGetLastError());
  ctx->sv = *sv;
  ctx->has_sv = true;
  return VCR_OK;
}

}  // namespace vcr
