// vcr::Renderer: the reference's main.cpp orchestration of its techniques
// (technique switch main.cpp:197-221, UpdateShadowVolume :223-264,
// UpdateCloudData :266-335, the Apply button :545-596), headless.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "vcr/render_technique.hpp"

namespace vcr {

namespace {

template <class T>
bool same(const T& a, const T& b) {
  return std::memcmp(&a, &b, sizeof(T)) == 0;
}

// CameraProperties::SetRotation (UniformBuffers.h:31-37): forward =
// Rx(pitch) * Ry(yaw) * (0, 0, 1), right-handed rotations (glm::rotate).
void forward_of(const float rotation[2], float out[3]) {
  const float pi = 3.14159265358979f;
  const float p = rotation[0] * (pi / 180.0f), y = rotation[1] * (pi / 180.0f);
  out[0] = std::sin(y);
  out[1] = -std::sin(p) * std::cos(y);
  out[2] = std::cos(p) * std::cos(y);
}

}  // namespace

Renderer::Renderer(Device& device, PushConstants* pushConstants, const vcr_params& params,
                   const vcr_ppm_params& photonMap, const vcr_ppb_params& beams, uint32_t shadowVolumeSize)
    : device_(&device),
      pushConstants_(pushConstants),
      pt_(device, pushConstants),
      ppm_(device, pushConstants, photonMap),
      ppb_(device, pushConstants, beams),
      params_(params),
      shadowVolumeSize_(shadowVolumeSize) {}

Renderer::~Renderer() = default;

RenderTechnique& Renderer::Active() {
  switch (current_) {
    case Technique::PhotonMapping: return ppm_;
    case Technique::PhotonBeams: return ppb_;
    default: return pt_;
  }
}

uint32_t Renderer::PassCount() const {
  uint32_t n = 0;
  Check(vcr_pass_count(device_->Handle(), &n), device_->Handle());
  return n;
}

void Renderer::Restart() {
  if (!hasSettings_) return;  // no frame yet: nothing has accumulated
  Check(vcr_reset_accumulation(device_->Handle()), device_->Handle());
  if (pushConstants_) pushConstants_->frameCount = 1;
}

void Renderer::LoadCloud(const Grid& grid, int precision, float baseScaling) {
  // SetCloudProperties (main.cpp:145-163): bounds from the grid, the global
  // majorant with its 0.01 floor (:152)
  Check(vcr_cloud_from_grid(&grid.desc, baseScaling, settings_.densityScaling, &cloud_));
  cloud_.max_extinction = std::max(grid.GetMajorant(), 0.01f);
  RenderTechnique& t = Active();
  t.BindCloud(grid, cloud_, precision);
  t.Commit();
  hasCloud_ = true;
  hasShadowVolume_ = false;  // its box follows the cloud's (SetOrigin)
  if (hasSettings_) {
    Settings s = settings_;
    Apply(s);
  }
  Restart();
}

bool Renderer::Apply(Settings& s) {
  // SetFOV / SetRotation clamp the caller's values (UniformBuffers.h:31-48)
  s.fov = std::clamp(s.fov, 60.0f, 150.0f);
  s.rotation[0] = std::clamp(s.rotation[0], -80.0f, 80.0f);
  RenderTechnique& t = Active();
  bool changed = false;
  if (!hasSettings_ || s.width != settings_.width || s.height != settings_.height) {
    pt_.SetFrameTarget(s.width, s.height);
    ppm_.SetFrameTarget(s.width, s.height);
    ppb_.SetFrameTarget(s.width, s.height);
    if (current_ != Technique::PathTracing) {  // per-pixel state follows the frame
      t.FreeResources();
      t.AllocateResources();
    }
    changed = true;
  }
  float fwd[3];
  forward_of(s.rotation, fwd);
  vcr_camera cam{};
  Check(vcr_camera_look(&cam, s.position, fwd, s.fov, s.nearPlane, (int32_t)s.width, (int32_t)s.height));
  if (!hasSettings_ || !same(cam, camera_)) {
    camera_ = cam;
    t.BindCamera(camera_);
    changed = true;
  }
  vcr_params p = params_;
  Check(vcr_params_set_phase_g(&p, s.phaseG));
  const float n = std::sqrt(s.sunDirection[0] * s.sunDirection[0] + s.sunDirection[1] * s.sunDirection[1] +
                            s.sunDirection[2] * s.sunDirection[2]);
  if (!(n > 0.0f)) throw Error(VCR_ERR_INVALID, "sun direction of zero length");
  for (int a = 0; a < 3; ++a) p.sun_dir[a] = s.sunDirection[a] / n;
  if (!hasSettings_ || !same(p, params_)) {
    params_ = p;
    t.BindParameters(params_);
    changed = true;
  }
  if (hasCloud_ && cloud_.density_scaling != s.densityScaling) {
    cloud_.density_scaling = s.densityScaling;
    t.BindCloudProperties(cloud_);
    changed = true;
  }
  if (hasCloud_ && params_.nee_mode == VCR_NEE_SHADOW_VOLUME) {
    // UpdateShadowVolume: lit along the camera's forward for photon beams
    // (main.cpp:226-229), else along the light
    vcr_shadow_volume sv{};
    Check(vcr_shadow_volume_setup(&sv, current_ == Technique::PhotonBeams ? fwd : params_.sun_dir,
                                  cloud_.bounds_min, cloud_.bounds_max, shadowVolumeSize_));
    if (!hasShadowVolume_ || !same(sv, shadowVolume_)) {
      shadowVolume_ = sv;
      t.BindShadowVolume(shadowVolume_);
      hasShadowVolume_ = true;
      changed = true;
    }
  }
  t.Commit();
  settings_ = s;
  hasSettings_ = true;
  if (changed) Restart();
  return changed;
}

void Renderer::SetTechnique(Technique technique) {
  if (technique == current_) return;
  Active().FreeResources();
  current_ = technique;
  RenderTechnique& t = Active();
  if (hasSettings_) {  // otherwise Apply sets the frame and allocates
    t.SetFrameTarget(settings_.width, settings_.height);
    t.AllocateResources();
  }
  if (hasSettings_ && params_.nee_mode == VCR_NEE_SHADOW_VOLUME) {  // the light may follow the camera now
    hasShadowVolume_ = false;
    Settings s = settings_;
    Apply(s);
  }
  Restart();
}

void Renderer::Render(void* stream) {
  if (!hasCloud_ || !hasSettings_) throw Error(VCR_ERR_STATE, "Renderer::Render needs LoadCloud and Apply");
  Active().RecordPass(stream, PassCount());
}

}  // namespace vcr
