// Persistent DDA wavefront path tracer: the bit-exact instantiation of the
// kernel (pt_wavefront_impl.cuh), the dispatch between it and the
// fast-math one (pt_wavefront_fast.cu), and the autotuner.
#define VCR_WF_NS exact
#include "pt_wavefront_impl.cuh"

namespace vcr {
namespace fast {
vcr_status wavefront_launch(vcr_ctx* ctx, const GridView& g, const SceneView& s, const CamView& cam,
                            const PassView& pv, uint32_t* stats, Counters cnt, uint32_t total, cudaStream_t st,
                            const NrcTrainSink* train, const BatchSink* batch, double* sum);
}  // namespace fast

vcr_status wavefront_launch(vcr_ctx* ctx, const GridView& g, const SceneView& s, const CamView& cam,
                            const PassView& pv, uint32_t* stats, Counters cnt, uint32_t total, cudaStream_t st,
                            const NrcTrainSink* train, const BatchSink* batch, double* sum) {
  return ctx->tuning.fast_math ? fast::wavefront_launch(ctx, g, s, cam, pv, stats, cnt, total, st, train, batch, sum)
                               : exact::wavefront_launch(ctx, g, s, cam, pv, stats, cnt, total, st, train, batch, sum);
}

}  // namespace vcr

using namespace vcr;

// Times one pass per candidate tuning and keeps the fastest.  The passes
// render into the sums, which are reset afterwards.
extern "C" VCR_API vcr_status vcr_autotune_pt(vcr_ctx* ctx, const vcr_pass_desc* pass, vcr_tuning* out,
                                              void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  if (ctx->params.tracker != VCR_TRACKER_DDA) return fail(ctx, VCR_ERR_STATE, "autotune applies to the DDA tracker");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t a, b;
  VCR_CUDA(ctx, cudaEventCreate(&a));
  VCR_CUDA(ctx, cudaEventCreate(&b));
  vcr_tuning saved = ctx->tuning, best = saved;
  float best_ms = 1e30f;
  const uint32_t levels[] = {0, 1, 2, 3};
  const uint32_t steps[] = {2, 8, 16};
  const uint32_t threads[] = {128, 256};
  vcr_status status = VCR_OK;
  for (uint32_t lv : levels)
    for (uint32_t sp : steps)
      for (uint32_t th : threads) {
        ctx->tuning = vcr_tuning{lv, sp, 1u, th, saved.corner_blocks, saved.fast_math};
        for (int rep = 0; rep < 2 && !status; ++rep) {  // first run warms up
          cudaEventRecord(a, st);
          status = pt_pass_launch(ctx, pass, st);
          cudaEventRecord(b, st);
        }
        if (status) break;
        cudaEventSynchronize(b);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best_ms) {
          best_ms = ms;
          best = ctx->tuning;
        }
      }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->tuning = status ? saved : best;
  if (status) return status;
  vcr_status r = vcr_reset_accumulation(ctx);
  if (r) return r;
  if (out) *out = best;
  return VCR_OK;
}
