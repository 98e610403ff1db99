// Checkpoint / resume of the progressive state: a long render (thousands
// of passes, hours of a PPM estimate, an online-trained cache) survives a
// restart.  The reference keeps this state only in GPU memory for the life
// of the process (frameCount and the accumulated image, main.cpp:262,
// PathTracer.comp:420-424; pmRadius, RenderTechniquePPM.cpp:302-312).
//
// File: "VCRCKPT\0", u32 version (2), u32 section count, then sections of
// { char tag[4]; u32 zero; u64 bytes; payload }:
//   SCEN  u64 scene hash (always first): FNV-1a over the grid description
//         and precision, the level-0 majorants (per-brick maxima of the
//         density, a fingerprint of its content), the cloud, camera and
//         parameter structs, and the batch's views and the photon-map
//         parameters when those are set up
//   FRAM  u32 width, height, passes, 0; u64 samples; f64 sums [w*h*3]
//   PPMS  u64 pixels; f64 statistics [pixels*8] (N, R, tau rgb, bg rgb)
//   NRCW  u32 step, has_average, training paths per step, weight count;
//         f32 weights, Adam m, Adam v [, moving average]
//   NRCG  (grid encoding) u64 table values, u32 has_average; f32 tables,
//         Adam m, Adam v [, moving average]
//   BTCH  u64 pixels; u32 passes, 0; u64 samples; f64 sums [pixels*3]
// Loading checks every section against the context's current setup (the
// same scene hash, frame size, the technique set up with the same sizes)
// and leaves the rest of the context as it is; unknown tags are skipped.
// Section lengths are checked against the bytes left in the file, so a
// truncated or corrupt file is an I/O error, not an allocation failure.
#include <cstring>
#include <fstream>
#include <new>

#include "batch.cuh"
#include "nrc.cuh"
#include "ppm.cuh"

namespace vcr {

static const char kMagic[8] = {'V', 'C', 'R', 'C', 'K', 'P', 'T', '\0'};
constexpr uint32_t kCkptVersion = 2;

struct Section {
  char tag[4];
  std::vector<uint8_t> data;
};

template <typename T>
static void put(std::vector<uint8_t>& v, const T& x) {
  const uint8_t* p = reinterpret_cast<const uint8_t*>(&x);
  v.insert(v.end(), p, p + sizeof(T));
}

static vcr_status put_device(vcr_ctx* ctx, std::vector<uint8_t>& v, const void* d, size_t bytes) {
  size_t at = v.size();
  v.resize(at + bytes);
  VCR_CUDA(ctx, cudaMemcpy(v.data() + at, d, bytes, cudaMemcpyDeviceToHost));
  return VCR_OK;
}

// FNV-1a, 64 bits.
struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void add(const void* p, size_t n) {
    const uint8_t* b = static_cast<const uint8_t*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  }
  template <typename T>
  void add(const T& x) { add(&x, sizeof(T)); }
};

// Hash of what the progressive state was rendered from (see the file
// header).  A part not bound hashes as a marker, so "no camera" differs
// from any camera.
static vcr_status scene_hash(vcr_ctx* ctx, uint64_t& out) {
  Fnv f;
  f.add((uint32_t)ctx->has_grid);
  if (ctx->has_grid) {
    for (int a = 0; a < 3; ++a) {
      f.add(ctx->gdesc.size[a]);
      f.add(ctx->gdesc.voxel_size[a]);
    }
    f.add(ctx->precision);
    const size_t cells = (size_t)ctx->mnb[0][0] * ctx->mnb[0][1] * ctx->mnb[0][2];
    std::vector<float> maj(cells);
    VCR_CUDA(ctx, cudaMemcpy(maj.data(), ctx->d_majorants + ctx->moff[0], cells * sizeof(float),
                             cudaMemcpyDeviceToHost));
    f.add(maj.data(), cells * sizeof(float));
  }
  f.add((uint32_t)ctx->has_cloud);
  if (ctx->has_cloud) f.add(ctx->cloud);
  f.add((uint32_t)ctx->has_cam);
  if (ctx->has_cam) f.add(ctx->cam);
  f.add((uint32_t)ctx->has_params);
  if (ctx->has_params) f.add(ctx->params);
  f.add((uint32_t)(ctx->batch != nullptr));
  if (ctx->batch) f.add(ctx->batch->views.data(), ctx->batch->views.size() * sizeof(vcr_view_desc));
  f.add((uint32_t)(ctx->ppm != nullptr));
  if (ctx->ppm) f.add(ctx->ppm->prm);
  out = f.h;
  return VCR_OK;
}

static vcr_status save_sections(vcr_ctx* ctx, std::vector<Section>& out) {
  {
    Section s{{'S', 'C', 'E', 'N'}, {}};
    uint64_t h = 0;
    vcr_status vs = scene_hash(ctx, h);
    if (vs) return vs;
    put(s.data, h);
    out.push_back(std::move(s));
  }
  if (ctx->d_sum) {
    Section s{{'F', 'R', 'A', 'M'}, {}};
    put(s.data, ctx->width);
    put(s.data, ctx->height);
    put(s.data, ctx->passes);
    put(s.data, 0u);
    put(s.data, (uint64_t)ctx->samples);
    vcr_status vs = put_device(ctx, s.data, ctx->d_sum, (size_t)ctx->width * ctx->height * 3 * sizeof(double));
    if (vs) return vs;
    out.push_back(std::move(s));
  }
  if (ctx->ppm) {
    Section s{{'P', 'P', 'M', 'S'}, {}};
    put(s.data, (uint64_t)ctx->ppm->pixels);
    vcr_status vs = put_device(ctx, s.data, ctx->ppm->stats, ctx->ppm->pixels * 8 * sizeof(double));
    if (vs) return vs;
    out.push_back(std::move(s));
  }
  if (ctx->nrc) {
    NrcState* st = ctx->nrc;
    Section s{{'N', 'R', 'C', 'W'}, {}};
    put(s.data, st->step);
    put(s.data, st->ema ? 1u : 0u);
    put(s.data, st->npaths);
    put(s.data, (uint32_t)kNrcWeightCount);
    const size_t nb = (size_t)kNrcWeightCount * sizeof(float);
    const float* parts[] = {st->w, st->m, st->v, st->ema};
    for (const float* d : parts)
      if (d) {
        vcr_status vs = put_device(ctx, s.data, d, nb);
        if (vs) return vs;
      }
    out.push_back(std::move(s));
    if (st->gw) {  // the grid encoding's tables: values, Adam moments, moving average
      Section g{{'N', 'R', 'C', 'G'}, {}};
      put(g.data, (uint64_t)kNrcGridParams);
      put(g.data, st->gema ? 1u : 0u);
      const float* gparts[] = {st->gw, st->gm, st->gv, st->gema};
      for (const float* d : gparts)
        if (d) {
          vcr_status vs = put_device(ctx, g.data, d, kNrcGridParams * sizeof(float));
          if (vs) return vs;
        }
      out.push_back(std::move(g));
    }
  }
  if (ctx->batch) {
    BatchState* b = ctx->batch;
    Section s{{'B', 'T', 'C', 'H'}, {}};
    put(s.data, (uint64_t)b->pixels);
    put(s.data, b->passes);
    put(s.data, 0u);
    put(s.data, (uint64_t)b->samples);
    vcr_status vs = put_device(ctx, s.data, b->d_sum, b->pixels * 3 * sizeof(double));
    if (vs) return vs;
    out.push_back(std::move(s));
  }
  return VCR_OK;
}

}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_checkpoint_save(vcr_ctx* ctx, const char* path) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!path) return fail(ctx, VCR_ERR_INVALID, "null path");
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  std::vector<Section> secs;
  vcr_status vs = save_sections(ctx, secs);
  if (vs) return vs;
  std::string tmp = std::string(path) + ".partial";
  {
    std::ofstream f(tmp, std::ios::binary | std::ios::trunc);
    if (!f) return fail(ctx, VCR_ERR_IO, "cannot write %s", tmp.c_str());
    f.write(kMagic, 8);
    uint32_t hdr[2] = {kCkptVersion, (uint32_t)secs.size()};
    f.write(reinterpret_cast<const char*>(hdr), sizeof hdr);
    for (const Section& s : secs) {
      uint32_t zero = 0;
      uint64_t n = s.data.size();
      f.write(s.tag, 4);
      f.write(reinterpret_cast<const char*>(&zero), 4);
      f.write(reinterpret_cast<const char*>(&n), 8);
      f.write(reinterpret_cast<const char*>(s.data.data()), (std::streamsize)n);
    }
    if (!f) return fail(ctx, VCR_ERR_IO, "write to %s failed", tmp.c_str());
  }
  // the checkpoint replaces the old one only once it is complete
  if (std::rename(tmp.c_str(), path) != 0) return fail(ctx, VCR_ERR_IO, "cannot rename %s to %s", tmp.c_str(), path);
  return VCR_OK;
}

namespace {

// Reads fixed-size fields from a section payload, failing on a short one.
struct Reader {
  const uint8_t* p;
  size_t left;
  template <typename T>
  bool get(T& x) {
    if (left < sizeof(T)) return false;
    std::memcpy(&x, p, sizeof(T));
    p += sizeof(T);
    left -= sizeof(T);
    return true;
  }
};

}  // namespace

extern "C" VCR_API vcr_status vcr_checkpoint_load(vcr_ctx* ctx, const char* path) {
  if (!ctx) return fail(nullptr, VCR_ERR_INVALID, "null context");
  if (!path) return fail(ctx, VCR_ERR_INVALID, "null path");
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(ctx, VCR_ERR_IO, "cannot open %s", path);
  char magic[8];
  uint32_t hdr[2];
  if (!f.read(magic, 8) || std::memcmp(magic, kMagic, 8) != 0 || !f.read(reinterpret_cast<char*>(hdr), 8))
    return fail(ctx, VCR_ERR_IO, "%s is not a vcr checkpoint", path);
  if (hdr[0] != kCkptVersion) return fail(ctx, VCR_ERR_UNSUPPORTED, "checkpoint version %u", hdr[0]);
  const std::streamoff here = f.tellg();
  f.seekg(0, std::ios::end);
  const std::streamoff end = f.tellg();
  f.seekg(here);
  if (here < 0 || end < here || !f) return fail(ctx, VCR_ERR_IO, "cannot size %s", path);
  uint64_t left = (uint64_t)(end - here);
  std::vector<Section> secs;
  for (uint32_t i = 0; i < hdr[1]; ++i) {
    Section s;
    uint32_t zero;
    uint64_t n;
    if (left < 16 || !f.read(s.tag, 4) || !f.read(reinterpret_cast<char*>(&zero), 4) ||
        !f.read(reinterpret_cast<char*>(&n), 8) || n > left - 16)
      return fail(ctx, VCR_ERR_IO, "truncated checkpoint %s", path);
    left -= 16 + n;
    try {
      s.data.resize(n);
    } catch (const std::bad_alloc&) {
      return fail(ctx, VCR_ERR_IO, "checkpoint section of %llu bytes does not fit in host memory", (unsigned long long)n);
    }
    if (!f.read(reinterpret_cast<char*>(s.data.data()), (std::streamsize)n))
      return fail(ctx, VCR_ERR_IO, "truncated checkpoint %s", path);
    secs.push_back(std::move(s));
  }
  VCR_CUDA(ctx, cudaSetDevice(ctx->device));
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  // validate every section before changing anything
  if (secs.empty() || std::memcmp(secs[0].tag, "SCEN", 4) != 0 || secs[0].data.size() != sizeof(uint64_t))
    return fail(ctx, VCR_ERR_IO, "%s has no scene hash", path);
  {
    uint64_t saved = 0, now = 0;
    std::memcpy(&saved, secs[0].data.data(), sizeof saved);
    vcr_status vs = scene_hash(ctx, now);
    if (vs) return vs;
    if (saved != now)
      return fail(ctx, VCR_ERR_STATE,
                  "checkpoint %s was saved for another scene (grid, cloud, camera, parameters, batch views or "
                  "photon-map parameters differ)",
                  path);
  }
  bool has_nrcw = false, has_nrcg = false;
  for (const Section& s : secs) {
    Reader r{s.data.data(), s.data.size()};
    has_nrcw = has_nrcw || !std::memcmp(s.tag, "NRCW", 4);
    has_nrcg = has_nrcg || !std::memcmp(s.tag, "NRCG", 4);
    if (!std::memcmp(s.tag, "FRAM", 4)) {
      uint32_t w, h, passes, z;
      uint64_t samples;
      if (!r.get(w) || !r.get(h) || !r.get(passes) || !r.get(z) || !r.get(samples)) return fail(ctx, VCR_ERR_IO, "bad FRAM");
      if (!ctx->d_sum || w != ctx->width || h != ctx->height)
        return fail(ctx, VCR_ERR_STATE, "checkpoint frame %ux%u, context frame %ux%u", w, h, ctx->width, ctx->height);
      if (r.left != (size_t)w * h * 3 * sizeof(double)) return fail(ctx, VCR_ERR_IO, "bad FRAM size");
    } else if (!std::memcmp(s.tag, "PPMS", 4)) {
      uint64_t px;
      if (!r.get(px)) return fail(ctx, VCR_ERR_IO, "bad PPMS");
      if (!ctx->ppm || ctx->ppm->pixels != px) return fail(ctx, VCR_ERR_STATE, "checkpoint holds PPM statistics: vcr_ppm_setup first");
      if (r.left != px * 8 * sizeof(double)) return fail(ctx, VCR_ERR_IO, "bad PPMS size");
    } else if (!std::memcmp(s.tag, "NRCW", 4)) {
      uint32_t step, has_avg, npaths, count;
      if (!r.get(step) || !r.get(has_avg) || !r.get(npaths) || !r.get(count)) return fail(ctx, VCR_ERR_IO, "bad NRCW");
      if (!ctx->nrc || count != (uint32_t)kNrcWeightCount || (has_avg != 0) != (ctx->nrc->ema != nullptr))
        return fail(ctx, VCR_ERR_STATE, "checkpoint holds a radiance cache: vcr_nrc_setup with the same ema_decay first");
      if (r.left != (size_t)count * sizeof(float) * (3u + has_avg)) return fail(ctx, VCR_ERR_IO, "bad NRCW size");
    } else if (!std::memcmp(s.tag, "NRCG", 4)) {
      uint64_t count;
      uint32_t has_avg;
      if (!r.get(count) || !r.get(has_avg)) return fail(ctx, VCR_ERR_IO, "bad NRCG");
      if (!ctx->nrc || !ctx->nrc->gw || count != kNrcGridParams || (has_avg != 0) != (ctx->nrc->gema != nullptr))
        return fail(ctx, VCR_ERR_STATE,
                    "checkpoint holds a grid-encoded radiance cache: vcr_nrc_setup with the grid encoding and the "
                    "same ema_decay first");
      if (r.left != (size_t)count * sizeof(float) * (3u + has_avg)) return fail(ctx, VCR_ERR_IO, "bad NRCG size");
    } else if (!std::memcmp(s.tag, "BTCH", 4)) {
      uint64_t px, samples;
      uint32_t passes, z;
      if (!r.get(px) || !r.get(passes) || !r.get(z) || !r.get(samples)) return fail(ctx, VCR_ERR_IO, "bad BTCH");
      if (!ctx->batch || ctx->batch->pixels != px) return fail(ctx, VCR_ERR_STATE, "checkpoint holds a batch: vcr_batch_setup with the same views first");
      if (r.left != px * 3 * sizeof(double)) return fail(ctx, VCR_ERR_IO, "bad BTCH size");
    }
  }
  if (has_nrcw && !has_nrcg && ctx->nrc && ctx->nrc->gw)
    return fail(ctx, VCR_ERR_STATE, "checkpoint holds a frequency-encoded radiance cache; this one has the grid encoding");
  // apply
  for (const Section& s : secs) {
    Reader r{s.data.data(), s.data.size()};
    if (!std::memcmp(s.tag, "FRAM", 4)) {
      uint32_t w, h, passes, z;
      uint64_t samples;
      r.get(w); r.get(h); r.get(passes); r.get(z); r.get(samples);
      VCR_CUDA(ctx, cudaMemcpy(ctx->d_sum, r.p, r.left, cudaMemcpyHostToDevice));
      ctx->passes = passes;
      ctx->samples = samples;
    } else if (!std::memcmp(s.tag, "PPMS", 4)) {
      uint64_t px;
      r.get(px);
      VCR_CUDA(ctx, cudaMemcpy(ctx->ppm->stats, r.p, r.left, cudaMemcpyHostToDevice));
    } else if (!std::memcmp(s.tag, "NRCW", 4)) {
      NrcState* st = ctx->nrc;
      uint32_t step, has_avg, npaths, count;
      r.get(step); r.get(has_avg); r.get(npaths); r.get(count);
      const size_t nb = (size_t)count * sizeof(float);
      float* parts[] = {st->w, st->m, st->v, st->ema};
      for (int i = 0; i < 3 + (int)has_avg; ++i) VCR_CUDA(ctx, cudaMemcpy(parts[i], r.p + i * nb, nb, cudaMemcpyHostToDevice));
      st->step = step;
      st->records = false;  // the records are not part of a checkpoint
      // the calibrated training-path count applies to the scene bound now
      st->npaths = npaths;
      st->calib_cam = ctx->cam;
      st->calib_cloud = ctx->cloud;
      st->calib_w = ctx->width;
      st->calib_h = ctx->height;
      vcr_status vs = nrc_refresh_copies(ctx);
      if (vs) return vs;
    } else if (!std::memcmp(s.tag, "NRCG", 4)) {
      NrcState* st = ctx->nrc;
      uint64_t count;
      uint32_t has_avg;
      r.get(count);
      r.get(has_avg);
      const size_t nb = (size_t)count * sizeof(float);
      float* gparts[] = {st->gw, st->gm, st->gv, st->gema};
      for (int i = 0; i < 3 + (int)has_avg; ++i)
        VCR_CUDA(ctx, cudaMemcpy(gparts[i], r.p + i * nb, nb, cudaMemcpyHostToDevice));
    } else if (!std::memcmp(s.tag, "BTCH", 4)) {
      BatchState* b = ctx->batch;
      uint64_t px, samples;
      uint32_t passes, z;
      r.get(px); r.get(passes); r.get(z); r.get(samples);
      VCR_CUDA(ctx, cudaMemcpy(b->d_sum, r.p, r.left, cudaMemcpyHostToDevice));
      b->passes = passes;
      b->samples = samples;
    }
  }
  VCR_CUDA(ctx, cudaDeviceSynchronize());
  return VCR_OK;
}
