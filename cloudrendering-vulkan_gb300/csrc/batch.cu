// Batched multi-view tracking: many views (cameras of uneven resolution,
// each with its own sun direction) rendered by one persistent wavefront
// launch over one work range, so the SMs stay full across views instead of
// draining at the end of each view.  A pass can be recorded once as a CUDA
// graph and replayed; each replay renders the next pass index (a device
// counter the graph increments).  The reference renders one camera per
// RenderTechnique dispatch (RenderTechniquePT.cpp:129-168); this extends
// that dispatch, with the path arithmetic of each view unchanged.
#include <algorithm>

#include "batch.cuh"

namespace vcr {

__global__ void batch_advance_kernel(uint32_t* ctr) { *ctr += 1u; }

void batch_free(vcr_ctx* ctx) {
  BatchState* b = ctx->batch;
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture) cudaStreamDestroy(b->capture);
  cudaFree(b->d_views);
  cudaFree(b->d_sum);
  cudaFree(b->d_ctr);
  delete b;
  ctx->batch = nullptr;
}

static vcr_status batch_check(vcr_ctx* ctx, const vcr_pass_desc* pass, PassView& pv) {
  BatchState* b = ctx->batch;
  if (!b) return fail(ctx, VCR_ERR_STATE, "no batch (vcr_batch_setup)");
  if (!pass) return fail(ctx, VCR_ERR_INVALID, "null pass");
  if (!ctx->has_grid || !ctx->has_cloud || !ctx->has_params)
    return fail(ctx, VCR_ERR_STATE, "a batch pass needs a grid, cloud and params");
  const vcr_params& P = ctx->params;
  if (P.tracker != VCR_TRACKER_DDA || P.rng_mode != VCR_RNG_PCG || P.nee_mode != VCR_NEE_RATIO || P.nrc_events)
    return fail(ctx, VCR_ERR_UNSUPPORTED, "batches run the DDA tracker with PCG streams, ratio NEE, no cache");
  if (pass->flags) return fail(ctx, VCR_ERR_UNSUPPORTED, "batch passes take no pass flags");
  pv = PassView{};
  pv.seed = pass->seed;
  pv.pass = pass->pass_index;
  pv.spp = pass->spp ? pass->spp : 1;
  if (b->pixels * pv.spp >= (1ull << 31)) return fail(ctx, VCR_ERR_UNSUPPORTED, "more than 2^31 paths in one pass");
  return VCR_OK;
}

static vcr_status batch_launch(vcr_ctx* ctx, const PassView& pv, const uint32_t* ctr, cudaStream_t s) {
  BatchState* b = ctx->batch;
  VCR_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 5 * sizeof(unsigned long long), s));
  BatchSink bt{b->d_views, (uint32_t)b->views.size(), ctr};
  CamView unused{};
  return wavefront_launch(ctx, grid_view(ctx), scene_view(ctx), unused, pv, nullptr, Counters{ctx->d_counters},
                          (uint32_t)(b->pixels * pv.spp), s, nullptr, &bt, b->d_sum);
}

static vcr_status batch_clear(vcr_ctx* ctx) {
  BatchState* b = ctx->batch;
  VCR_CUDA(ctx, cudaMemset(b->d_sum, 0, b->pixels * 3 * sizeof(double)));
  VCR_CUDA(ctx, cudaMemset(b->d_ctr, 0, 2 * sizeof(uint32_t)));
  b->passes = 0;
  b->samples = 0;
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_batch_setup(vcr_ctx* ctx, const vcr_view_desc* views, uint32_t count) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!views || count == 0 || count > kMaxBatchViews)
    return fail(ctx, VCR_ERR_INVALID, "a batch has 1..%u views", kMaxBatchViews);
  uint64_t pixels = 0;
  for (uint32_t v = 0; v < count; ++v) {
    const vcr_view_desc& d = views[v];
    if (d.width == 0 || d.height == 0 || (uint64_t)d.width * d.height > (1ull << 28))
      return fail(ctx, VCR_ERR_INVALID, "view %u: frame %ux%u", v, d.width, d.height);
    pixels += (uint64_t)d.width * d.height;
  }
  if (pixels >= (1ull << 31)) return fail(ctx, VCR_ERR_INVALID, "more than 2^31 pixels in a batch");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  batch_free(ctx);
  BatchState* b = new BatchState();
  ctx->batch = b;
  b->views.assign(views, views + count);
  b->pixels = pixels;
  uint64_t p0 = 0;
  for (uint32_t v = 0; v < count; ++v) {
    const vcr_view_desc& d = views[v];
    BatchView t{};
    t.cam = cam_view(d.camera);
    t.sun = mk(d.sun_dir[0], d.sun_dir[1], d.sun_dir[2]);
    t.width = d.width;
    t.height = d.height;
    t.pix0 = (uint32_t)p0;
    t.path0 = 0;  // set per spp at launch time: path0 = pix0 * spp
    b->table.push_back(t);
    b->pix0.push_back(p0);
    p0 += (uint64_t)d.width * d.height;
  }
  VCR_CUDA(ctx, cudaMalloc(&b->d_views, count * sizeof(BatchView)));
  VCR_CUDA(ctx, cudaMalloc(&b->d_sum, pixels * 3 * sizeof(double)));
  VCR_CUDA(ctx, cudaMalloc(&b->d_ctr, 2 * sizeof(uint32_t)));
  VCR_CUDA(ctx, cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
  return batch_clear(ctx);
}

// The view table holds path0 = pix0 * spp, so it is rewritten when the spp
// of the passes changes; a recorded graph (which reads the table when it
// runs) is then dropped.
static vcr_status batch_table(vcr_ctx* ctx, uint32_t spp, cudaStream_t s) {
  BatchState* b = ctx->batch;
  if (b->table_spp == spp) return VCR_OK;
  if (b->exec) {
    VCR_CUDA(ctx, cudaDeviceSynchronize());
    cudaGraphExecDestroy(b->exec);
    cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
  }
  for (size_t v = 0; v < b->table.size(); ++v) b->table[v].path0 = (uint32_t)(b->pix0[v] * spp);
  VCR_CUDA(ctx, cudaMemcpyAsync(b->d_views, b->table.data(), b->table.size() * sizeof(BatchView),
                                cudaMemcpyHostToDevice, s));
  VCR_CUDA(ctx, cudaStreamSynchronize(s));  // the host table is rewritten by the next call
  b->table_spp = spp;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_batch_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  PassView pv;
  vcr_status vs = batch_check(ctx, pass, pv);
  if (vs) return vs;
  BatchState* b = ctx->batch;
  cudaStream_t s = (cudaStream_t)stream;
  vs = batch_table(ctx, pv.spp, s);
  if (vs) return vs;
  vs = batch_launch(ctx, pv, b->d_ctr + 1, s);  // direct passes add the constant 0
  if (vs) return vs;
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  b->passes += 1;
  b->samples += pv.spp;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_batch_graph_record(vcr_ctx* ctx, const vcr_pass_desc* pass) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  PassView pv;
  vcr_status vs = batch_check(ctx, pass, pv);
  if (vs) return vs;
  BatchState* b = ctx->batch;
  vs = batch_table(ctx, pv.spp, b->capture);
  if (vs) return vs;
  VCR_CUDA(ctx, cudaDeviceSynchronize());  // no replay of the old graph in flight
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  VCR_CUDA(ctx, cudaMemset(b->d_ctr, 0, sizeof(uint32_t)));
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  VCR_CUDA(ctx, cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeRelaxed));
  vs = batch_launch(ctx, pv, b->d_ctr, b->capture);
  if (!vs) {
    batch_advance_kernel<<<1, 1, 0, b->capture>>>(b->d_ctr);
    if (cudaGetLastError() != cudaSuccess) vs = fail(ctx, VCR_ERR_CUDA, "pass counter launch");
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->capture, &g);
  if (vs) {
    if (g) cudaGraphDestroy(g);
    return vs;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
  b->graph = g;
  VCR_CUDA(ctx, cudaGraphInstantiate(&b->exec, g, 0));
  b->graph_spp = pv.spp;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_batch_graph_replay(vcr_ctx* ctx, uint32_t count, void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  BatchState* b = ctx->batch;
  if (!b || !b->exec) return fail(ctx, VCR_ERR_STATE, "no recorded batch graph");
  cudaStream_t s = (cudaStream_t)stream;
  for (uint32_t i = 0; i < count; ++i) VCR_CUDA(ctx, cudaGraphLaunch(b->exec, s));
  VCR_CUDA(ctx, cudaEventRecord(ctx->work_done, s));
  b->passes += count;
  b->samples += (uint64_t)b->graph_spp * count;
  return VCR_OK;
}

// Times one batch pass per candidate tuning (majorant level x DDA cells per
// step x CTA size) and keeps the fastest; the sums are cleared afterwards.
extern "C" VCR_API vcr_status vcr_batch_autotune(vcr_ctx* ctx, const vcr_pass_desc* pass, vcr_tuning* out,
                                                 void* stream) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  PassView pv;
  vcr_status vs = batch_check(ctx, pass, pv);
  if (vs) return vs;
  BatchState* b = ctx->batch;
  cudaStream_t s = (cudaStream_t)stream;
  vs = batch_table(ctx, pv.spp, s);
  if (vs) return vs;
  cudaEvent_t e0, e1;
  VCR_CUDA(ctx, cudaEventCreate(&e0));
  VCR_CUDA(ctx, cudaEventCreate(&e1));
  vcr_tuning saved = ctx->tuning, best = saved;
  float best_ms = 1e30f;
  const uint32_t levels[] = {0, 1, 2, 3}, steps[] = {2, 8, 16}, threads[] = {128, 256};
  for (uint32_t lv : levels)
    for (uint32_t sp : steps)
      for (uint32_t th : threads) {
        ctx->tuning = vcr_tuning{lv, sp, 1u, th, saved.corner_blocks, saved.fast_math};
        for (int rep = 0; rep < 2 && !vs; ++rep) {  // the first run warms up
          cudaEventRecord(e0, s);
          vs = batch_launch(ctx, pv, b->d_ctr + 1, s);
          cudaEventRecord(e1, s);
        }
        if (vs) break;
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
          best_ms = ms;
          best = ctx->tuning;
        }
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tuning = vs ? saved : best;
  if (vs) return vs;
  vs = batch_clear(ctx);
  if (vs) return vs;
  if (out) *out = best;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_batch_read(vcr_ctx* ctx, uint32_t view, double* out, size_t bytes) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  BatchState* b = ctx->batch;
  if (!b) return fail(ctx, VCR_ERR_STATE, "no batch");
  if (view >= b->views.size()) return fail(ctx, VCR_ERR_INVALID, "view %u of %zu", view, b->views.size());
  size_t px = (size_t)b->views[view].width * b->views[view].height;
  if (bytes != px * 3 * sizeof(double)) return fail(ctx, VCR_ERR_INVALID, "view %u sums are %zu bytes", view, px * 24);
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  VCR_CUDA(ctx, cudaMemcpy(out, b->d_sum + 3 * b->pix0[view], bytes, cudaMemcpyDefault));
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_batch_info(vcr_ctx* ctx, vcr_batch_info_t* out) {
  if (!ctx || !out) return fail(ctx, VCR_ERR_INVALID, "null argument");
  BatchState* b = ctx->batch;
  if (!b) return fail(ctx, VCR_ERR_STATE, "no batch");
  out->views = (uint32_t)b->views.size();
  out->passes = b->passes;
  out->pixels = b->pixels;
  out->samples = b->samples;
  return VCR_OK;
}

extern "C" VCR_API vcr_status vcr_batch_reset(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->batch) return fail(ctx, VCR_ERR_STATE, "no batch");
  VCR_CUDA(ctx, cudaEventSynchronize(ctx->work_done));
  return batch_clear(ctx);
}

extern "C" VCR_API vcr_status vcr_batch_free(vcr_ctx* ctx) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaDeviceSynchronize();
  batch_free(ctx);
  return VCR_OK;
}
