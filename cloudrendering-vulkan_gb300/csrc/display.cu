// Display image: the headless form of the reference's blit of its RGBA32F
// result into the B8G8R8A8_SRGB swapchain (RenderTechniquePT.cpp:143-167,
// VulkanSwapchain.cpp:72).  One thread per pixel reads the pixel's three
// FP64 sums (24 B) and writes one packed 8-bit pixel (4 B): an HBM-bound
// streaming kernel.
#include "pt_common.cuh"

namespace vcr {

__global__ void display_kernel(const double* __restrict__ sum, size_t npx, double inv, float exposure,
                               uint32_t order, uint32_t* __restrict__ out) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npx) return;
  uint32_t q[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v = (float)(sum[3 * p + c] * inv) * exposure;
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    q[c] = (uint32_t)(srgb_encode(v) * 255.0f + 0.5f);
  }
  const uint32_t r = order ? q[2] : q[0], b = order ? q[0] : q[2];
  out[p] = r | (q[1] << 8) | (b << 16) | (255u << 24);
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_display(vcr_ctx* ctx, const vcr_display_desc* desc, void* out, size_t bytes,
                                          void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!desc || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  if (!ctx->d_sum) return fail(ctx, VCR_ERR_STATE, "no frame");
  if (desc->order > VCR_ORDER_BGRA || !(desc->exposure >= 0.0f))
    return fail(ctx, VCR_ERR_INVALID, "bad display description");
  const size_t npx = (size_t)ctx->width * ctx->height;
  if (bytes != npx * 4) return fail(ctx, VCR_ERR_INVALID, "display image is %zu bytes", npx * 4);
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  cudaPointerAttributes at{};
  VCR_CUDA(ctx, cudaPointerGetAttributes(&at, out));
  const bool on_device = (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == ctx->device;
  uint32_t* dst = reinterpret_cast<uint32_t*>(out);
  if (!on_device) {
    vcr_status vs = ensure_scratch(ctx, bytes);
    if (vs) return vs;
    dst = reinterpret_cast<uint32_t*>(ctx->d_scratch);
  }
  const double inv = ctx->samples ? 1.0 / (double)ctx->samples : 0.0;
  if (npx) {
    display_kernel<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(ctx->d_sum, npx, inv, desc->exposure, desc->order,
                                                                  dst);
    VCR_CUDA(ctx, cudaGetLastError());
  }
  if (!on_device) {
    VCR_CUDA(ctx, cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, st));
    VCR_CUDA(ctx, cudaStreamSynchronize(st));
  }
  return VCR_OK;
}
