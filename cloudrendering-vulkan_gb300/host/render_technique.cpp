// C++ host layer over the C-ABI: Device, Grid and the RenderTechnique
// family (RenderTechnique.h:15-67, RenderTechniquePT/PPM/PPB.h), headless.
#include "../../include/vcr/render_technique.hpp"

#include <algorithm>
#include <cmath>

namespace vcr {

void Check(vcr_status status, const vcr_ctx* ctx) {
  if (status == VCR_OK) return;
  const char* msg = vcr_last_error(ctx);
  static const char* names[] = {"OK", "INVALID", "CUDA", "OOM", "TIMEOUT", "STATE", "IO", "UNSUPPORTED", "CAPACITY"};
  std::string name = (status >= 0 && status < 9) ? names[status] : std::to_string((int)status);
  throw Error(status, "vcr " + name + ": " + (msg ? msg : ""));
}

// ---------------------------------------------------------------------------
// Device
// ---------------------------------------------------------------------------
Device::Device(int device) {
  vcr_device_desc d{};
  d.device = device;
  Check(vcr_create(&ctx_, &d), nullptr);
}

Device::~Device() { vcr_destroy(ctx_); }

void Device::Synchronize() { Check(vcr_synchronize(ctx_), ctx_); }

// ---------------------------------------------------------------------------
// Grid (Grid3D<float>)
// ---------------------------------------------------------------------------
Grid Grid::Load(const std::string& path) {
  Grid g;
  Check(vcr_xyz_read(path.c_str(), &g.desc, nullptr, 0));
  size_t n = (size_t)g.desc.size[0] * g.desc.size[1] * g.desc.size[2];
  g.data.resize(n);
  Check(vcr_xyz_read(path.c_str(), &g.desc, g.data.data(), n));
  return g;
}

void Grid::Save(const std::string& path) const { Check(vcr_xyz_write(path.c_str(), &desc, data.data())); }

Grid Grid::Generate(uint32_t x, uint32_t y, uint32_t z, const vcr_fbm_desc& fbm) {
  Grid g;
  g.desc.size[0] = x;
  g.desc.size[1] = y;
  g.desc.size[2] = z;
  double v = 1.0 / (double)std::max(x, std::max(y, z));  // the cloud spans one unit along its longest axis
  for (int a = 0; a < 3; ++a) g.desc.voxel_size[a] = v;
  g.data.resize((size_t)x * y * z);
  Check(vcr_fbm_fill_host(&g.desc, &fbm, g.data.data()));
  return g;
}

float Grid::GetMajorant() const {
  float m = 0.0f;
  for (float d : data) m = std::max(m, d);
  return m;
}

// ---------------------------------------------------------------------------
// RenderTechnique
// ---------------------------------------------------------------------------
RenderTechnique::RenderTechnique(Device& device, PushConstants* pushConstants)
    : device_(&device), pushConstants_(pushConstants) {}

void RenderTechnique::Require(bool condition, const char* what) const {
  if (!condition) throw Error(VCR_ERR_STATE, std::string("vcr STATE: ") + what);
}

void RenderTechnique::BindCloud(const Grid& grid, const vcr_cloud& cloud, int precision) {
  pendingGrid_ = &grid;
  pendingCloud_ = cloud;
  pendingPrecision_ = precision;
  hasPendingCloud_ = true;
}

void RenderTechnique::BindCloudProperties(const vcr_cloud& cloud) {
  pendingCloudProps_ = cloud;
  hasPendingCloudProps_ = true;
}

void RenderTechnique::BindCamera(const vcr_camera& camera) {
  pendingCamera_ = camera;
  hasPendingCamera_ = true;
}

void RenderTechnique::BindParameters(const vcr_params& params) {
  pendingParams_ = params;
  hasPendingParams_ = true;
}

void RenderTechnique::BindShadowVolume(const vcr_shadow_volume& shadowVolume) {
  pendingShadowVolume_ = shadowVolume;
  hasPendingShadowVolume_ = true;
}

void RenderTechnique::Commit() {
  vcr_ctx* c = Context();
  bool restart = false;
  if (hasPendingCloud_) {
    Check(vcr_grid_upload(c, &pendingGrid_->desc, pendingGrid_->data.data(), (vcr_precision)pendingPrecision_), c);
    vcr_cloud cl = pendingCloud_;
    if (!(cl.max_extinction > 0.0f)) {  // SetCloudProperties: max(grid max, 0.01) (main.cpp:152)
      float mx = 0.0f;
      uint32_t nb[3];
      Check(vcr_grid_info(c, &mx, nb), c);
      cl.max_extinction = std::max(mx, 0.01f);
    }
    Check(vcr_set_cloud(c, &cl), c);
    hasPendingCloud_ = false;
    pendingGrid_ = nullptr;
    restart = true;
  }
  if (hasPendingCloudProps_) {
    Check(vcr_set_cloud(c, &pendingCloudProps_), c);
    hasPendingCloudProps_ = false;
    restart = true;
  }
  if (hasPendingCamera_) {
    Check(vcr_set_camera(c, &pendingCamera_), c);
    hasPendingCamera_ = false;
    restart = true;
  }
  if (hasPendingParams_) {
    Check(vcr_set_params(c, &pendingParams_), c);
    hasPendingParams_ = false;
    restart = true;
  }
  if (hasPendingShadowVolume_) {
    Check(vcr_shadow_volume_build(c, &pendingShadowVolume_, nullptr), c);
    hasPendingShadowVolume_ = false;
    restart = true;
  }
  if (restart && frameSet_) {
    Check(vcr_reset_accumulation(c), c);
    if (pushConstants_) pushConstants_->frameCount = 1;
  }
}

void RenderTechnique::SetFrameTarget(uint32_t width, uint32_t height) {
  Check(vcr_set_frame(Context(), width, height), Context());
  frameSet_ = true;
  width_ = width;
  height_ = height;
  if (pushConstants_) pushConstants_->frameCount = 1;
}

vcr_pass_desc RenderTechnique::PassDesc(uint32_t passIndex, uint32_t spp) const {
  Require(frameSet_, "no frame target (SetFrameTarget)");
  vcr_pass_desc p{};
  p.seed = pushConstants_ ? (uint32_t)pushConstants_->seed : 0u;
  p.pass_index = passIndex;
  p.spp = spp;
  return p;
}

void RenderTechnique::Advance() {
  if (pushConstants_) pushConstants_->frameCount += 1;
}

void RenderTechnique::ClearFrameTarget() {
  // The sums stay allocated until the next SetFrameTarget or the device's
  // end; the technique only stops rendering into them.
  frameSet_ = false;
}

std::vector<float> RenderTechnique::ReadMean() const {
  Require(frameSet_, "no frame target");
  std::vector<float> out((size_t)width_ * height_ * 3);
  Check(vcr_readback(Context(), VCR_BUF_IMAGE_MEAN, out.data(), out.size() * sizeof(float)), Context());
  return out;
}

std::vector<uint8_t> RenderTechnique::ReadDisplay(float exposure, bool bgra) const {
  Require(frameSet_, "no frame target");
  std::vector<uint8_t> out((size_t)width_ * height_ * 4);
  vcr_display_desc d{};
  d.exposure = exposure;
  d.order = bgra ? VCR_ORDER_BGRA : VCR_ORDER_RGBA;
  Check(vcr_display(Context(), &d, out.data(), out.size(), nullptr), Context());
  return out;
}

void RenderTechnique::WriteExr(const std::string& path, bool half) const {
  std::vector<float> rgb = ReadMean();
  Check(vcr_write_exr(path.c_str(), width_, height_, rgb.data(), half ? VCR_EXR_HALF : VCR_EXR_FLOAT), nullptr);
}

void RenderTechnique::WritePng(const std::string& path, float exposure) const {
  std::vector<uint8_t> rgba = ReadDisplay(exposure, false);
  Check(vcr_write_png(path.c_str(), width_, height_, rgba.data()), nullptr);
}

uint32_t RenderTechnique::PassCount() const {
  uint32_t n = 0;
  Check(vcr_pass_count(Context(), &n), Context());
  return n;
}

// ---------------------------------------------------------------------------
// TechniquePT (RenderTechniquePT::RecordDrawCommands, RenderTechniquePT.cpp:129-168)
// ---------------------------------------------------------------------------
void TechniquePT::RecordPass(void* stream, uint32_t passIndex) {
  vcr_pass_desc p = PassDesc(passIndex, samplesPerPass);
  Check(vcr_pt_pass(Context(), &p, stream), Context());
  Advance();
}

// ---------------------------------------------------------------------------
// TechniquePPM (RenderTechniquePPM.cpp: AllocateResources :115-156,
// RecordDrawCommands :229-300, UpdateRadius :302-312)
// ---------------------------------------------------------------------------
TechniquePPM::TechniquePPM(Device& device, PushConstants* pushConstants, const vcr_ppm_params& photonMap)
    : RenderTechnique(device, pushConstants), photonMap_(photonMap) {
  if (pushConstants_) pushConstants_->pmRadius = photonMap_.radius;
}

TechniquePPM::~TechniquePPM() {
  if (allocated_) vcr_ppm_free(Context());
}

void TechniquePPM::AllocateResources() {
  Check(vcr_ppm_setup(Context(), &photonMap_), Context());
  allocated_ = true;
}

void TechniquePPM::FreeResources() {
  if (allocated_) Check(vcr_ppm_free(Context()), Context());
  allocated_ = false;
}

void TechniquePPM::RecordPass(void* stream, uint32_t passIndex) {
  Require(allocated_, "TechniquePPM::AllocateResources first");
  vcr_pass_desc p = PassDesc(passIndex);
  Check(vcr_ppm_pass(Context(), &p, stream), Context());
  // the per-pixel radii shrink independently; pmRadius keeps the reference's
  // global schedule r_k = r_{k-1} ((k - 1 + alpha) / k)^(1/3) for display
  if (pushConstants_) {
    float k = (float)pushConstants_->frameCount;
    pushConstants_->pmRadius *= std::cbrt((k - 1.0f + photonMap_.alpha) / k);
  }
  Advance();
}

// ---------------------------------------------------------------------------
// TechniquePPB (RenderTechniquePPB.cpp: AllocateResources :282-355,
// UpdatePhotonMapProperties :357-363, RecordDrawCommands :436-519)
// ---------------------------------------------------------------------------
TechniquePPB::TechniquePPB(Device& device, PushConstants* pushConstants, const vcr_ppb_params& beams)
    : RenderTechnique(device, pushConstants), beams_(beams) {
  if (pushConstants_) pushConstants_->pmRadius = beams_.radius;
}

TechniquePPB::~TechniquePPB() {
  if (allocated_) vcr_ppb_free(Context());
}

void TechniquePPB::AllocateResources() {
  Check(vcr_ppb_setup(Context(), &beams_), Context());
  allocated_ = true;
}

void TechniquePPB::FreeResources() {
  if (allocated_) Check(vcr_ppb_free(Context()), Context());
  allocated_ = false;
}

void TechniquePPB::UpdatePhotonMapProperties(const vcr_ppb_params& beams) {
  beams_ = beams;
  if (allocated_) {
    FreeResources();
    AllocateResources();
  }
  if (frameSet_) Check(vcr_reset_accumulation(Context()), Context());
}

void TechniquePPB::RecordPass(void* stream, uint32_t passIndex) {
  Require(allocated_, "TechniquePPB::AllocateResources first");
  vcr_pass_desc p = PassDesc(passIndex);
  Check(vcr_ppb_pass(Context(), &p, stream), Context());
  if (pushConstants_) {
    vcr_ppb_info_t info{};
    Check(vcr_ppb_info(Context(), &info), Context());
    pushConstants_->pmRadius = info.radius;
  }
  Advance();
}

// ---------------------------------------------------------------------------
// TechniqueNRC
// ---------------------------------------------------------------------------
TechniqueNRC::TechniqueNRC(Device& device, PushConstants* pushConstants, const vcr_nrc_params& cache,
                           const NrcSchedule& schedule)
    : RenderTechnique(device, pushConstants), cache_(cache), schedule_(schedule) {}

namespace {
// Seeds of the training-set launches: a stream of their own, apart from
// the camera passes' and from each other's (pass index = launch count).
constexpr uint32_t kTrainSetSeedSalt = 0x6A09E667u;
}  // namespace

TechniqueNRC::~TechniqueNRC() {
  if (allocated_) vcr_nrc_free(Context());
}

void TechniqueNRC::AllocateResources() {
  Check(vcr_nrc_setup(Context(), &cache_), Context());
  allocated_ = true;
  passes_ = 0;
  launches_ = 0;
}

void TechniqueNRC::Warmup(void* stream, uint32_t steps, uint32_t sets, uint32_t batch) {
  Require(allocated_, "TechniqueNRC::AllocateResources first");
  Require(sets >= 1, "TechniqueNRC::Warmup needs sets >= 1");
  const uint32_t records = batch ? batch : cache_.train_samples;
  // steps per launch: every set walked about as often as the bench's warm-up walks it
  const uint32_t perLaunch = std::max(1u, sets * (cache_.train_samples / std::max(records, 1u)) * 5u);
  for (uint32_t done = 0; done < steps;) {
    vcr_pass_desc t = PassDesc(launches_++, sets);
    t.seed ^= kTrainSetSeedSalt;
    Check(vcr_nrc_train_step(Context(), &t, stream), Context());
    const uint32_t more = std::min(perLaunch, steps - done) - 1u;
    if (more) Check(vcr_nrc_train_more(Context(), more, records, stream), Context());
    done += more + 1u;
  }
}

void TechniqueNRC::FreeResources() {
  if (allocated_) Check(vcr_nrc_free(Context()), Context());
  allocated_ = false;
}

void TechniqueNRC::RecordPass(void* stream, uint32_t passIndex) {
  Require(allocated_, "TechniqueNRC::AllocateResources first");
  vcr_pass_desc p = PassDesc(passIndex, std::max(schedule_.spp, 1u));
  if (schedule_.poolSets == 0) {
    Check(vcr_nrc_frame(Context(), &p, stream), Context());
  } else {
    Check(vcr_pt_pass(Context(), &p, stream), Context());
    if (passes_ % std::max(schedule_.poolEvery, 1u) == 0) {
      vcr_pass_desc t = PassDesc(launches_++, schedule_.poolSets);
      t.seed ^= kTrainSetSeedSalt;
      Check(vcr_nrc_train_step(Context(), &t, stream), Context());
    } else {
      const uint32_t records = schedule_.batch ? schedule_.batch : cache_.train_samples;
      Check(vcr_nrc_train_more(Context(), 1, records, stream), Context());
    }
  }
  ++passes_;
  Advance();
}

}  // namespace vcr
