/* C++ host layer over the vcr C-ABI: the reference's RenderTechnique
 * lifecycle (RenderTechnique.h:15-67) for a headless GB300 device.
 *
 *   reference (Vulkan)                           here
 *   RenderTechnique(VulkanDevice*, PushConstants*)  RenderTechnique(Device&, PushConstants*)
 *   QueueUpdateCloudData / ...Sampler             BindCloud(grid, cloud, precision)
 *   QueueUpdateCameraProperties                   BindCamera
 *   QueueUpdateParameters                         BindParameters
 *   QueueUpdateShadowVolume / ...Sampler          BindShadowVolume
 *   UpdateDescriptorSets (RenderTechnique.cpp:14-18)  Commit: applies the queued bindings
 *   SetFrameReferences / ClearFrameReferences     SetFrameTarget / ClearFrameTarget (device sums)
 *   RecordDrawCommands(VkCommandBuffer, image)    RecordPass(stream, passIndex)
 *   RenderTechniquePPM/PPB::AllocateResources /   AllocateResources / FreeResources
 *   FreeResources
 *   RenderTechniquePPB::UpdatePhotonMapProperties UpdatePhotonMapProperties
 *
 * Errors: the reference aborts (Validation.cpp:4-10) or throws
 * std::runtime_error; every failing vcr call here throws vcr::Error with the
 * status and the context's message.  Ownership: as in the reference, a
 * technique holds non-owning pointers to the device and the push
 * constants, and updates pushConstants->pmRadius (RenderTechniquePPM.cpp:
 * 306-310) and frameCount.  Streams are cudaStream_t passed as void*.
 * One host thread drives a device (the reference's single recording
 * thread, main.cpp:603-712). */
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "abi.h"

namespace vcr {

class VCR_API Error : public std::runtime_error {
 public:
  Error(vcr_status status, const std::string& msg) : std::runtime_error(msg), status_(status) {}
  vcr_status status() const { return status_; }

 private:
  vcr_status status_;
};

/* Throws vcr::Error for a status other than VCR_OK. */
VCR_API void Check(vcr_status status, const vcr_ctx* ctx = nullptr);

/* PushConstants (UniformBuffers.h:6-13). */
struct PushConstants {
  double time = 0;
  int seed = 100;
  uint32_t frameCount = 1;
  float pmRadius = 0;
  uint32_t currentBuffer = 0;
};

/* A GPU context (stands for VulkanDevice). */
class VCR_API Device {
 public:
  explicit Device(int device = 0);
  ~Device();
  Device(const Device&) = delete;
  Device& operator=(const Device&) = delete;
  vcr_ctx* Handle() const { return ctx_; }
  void Synchronize();

 private:
  vcr_ctx* ctx_ = nullptr;
};

/* Grid3D<float> (Grid3D.h:5-192): a dense x-fastest grid with its voxel
 * size; Load / Save use the .xyz format (Grid3D.h:44-90, 166-178). */
struct VCR_API Grid {
  vcr_grid_desc desc{};
  std::vector<float> data;

  static Grid Load(const std::string& path);
  void Save(const std::string& path) const;
  /* Seeded Perlin fBm of the given size (the synthetic cloud). */
  static Grid Generate(uint32_t x, uint32_t y, uint32_t z, const vcr_fbm_desc& fbm);
  float GetMajorant() const; /* max density (Grid3D.h:180-192) */
};

class VCR_API RenderTechnique {
 public:
  RenderTechnique(Device& device, PushConstants* pushConstants);
  virtual ~RenderTechnique() = default;
  RenderTechnique(const RenderTechnique&) = delete;
  RenderTechnique& operator=(const RenderTechnique&) = delete;

  /* Queue updates; nothing reaches the device before Commit. */
  void BindCloud(const Grid& grid, const vcr_cloud& cloud, int precision = VCR_PREC_FP32);
  /* The cloud properties alone (QueueUpdateCloudData without the sampler):
   * bounds and scalings change, the stored grid stays. */
  void BindCloudProperties(const vcr_cloud& cloud);
  void BindCamera(const vcr_camera& camera);
  void BindParameters(const vcr_params& params);
  void BindShadowVolume(const vcr_shadow_volume& shadowVolume);
  /* Apply the queued updates (UpdateDescriptorSets).  A changed cloud,
   * camera, parameters or frame restarts the progressive accumulation. */
  void Commit();

  void SetFrameTarget(uint32_t width, uint32_t height);
  void ClearFrameTarget();

  /* One progressive pass on `stream` (RecordDrawCommands).  Increments
   * pushConstants->frameCount. */
  virtual void RecordPass(void* stream, uint32_t passIndex) = 0;
  virtual void AllocateResources() {}
  virtual void FreeResources() {}

  /* The accumulated mean image, float RGB, width * height * 3. */
  std::vector<float> ReadMean() const;
  /* What the swapchain blit would show (RenderTechniquePT.cpp:143-167 into
   * the B8G8R8A8_SRGB swapchain): 8-bit sRGB pixels, width * height * 4
   * bytes, R G B A or (bgra) B G R A, alpha 255. */
  std::vector<uint8_t> ReadDisplay(float exposure = 1.0f, bool bgra = false) const;
  /* The mean image as an OpenEXR file (FLOAT or, with half, HALF channels;
   * vcr_write_exr) and the display bytes as a PNG file (vcr_write_png):
   * the headless stand-in for presenting the frame. */
  void WriteExr(const std::string& path, bool half = false) const;
  void WritePng(const std::string& path, float exposure = 1.0f) const;
  uint32_t PassCount() const;
  uint32_t Width() const { return width_; }
  uint32_t Height() const { return height_; }
  vcr_ctx* Context() const { return device_->Handle(); }

 protected:
  void Require(bool condition, const char* what) const;
  vcr_pass_desc PassDesc(uint32_t passIndex, uint32_t spp = 1) const;
  void Advance();  // after a recorded pass: frameCount += 1

  Device* device_ = nullptr;
  PushConstants* pushConstants_ = nullptr;
  bool frameSet_ = false;
  uint32_t width_ = 0, height_ = 0;

 private:
  const Grid* pendingGrid_ = nullptr;
  vcr_cloud pendingCloud_{};
  int pendingPrecision_ = VCR_PREC_FP32;
  bool hasPendingCloud_ = false;
  vcr_cloud pendingCloudProps_{};
  bool hasPendingCloudProps_ = false;
  vcr_camera pendingCamera_{};
  bool hasPendingCamera_ = false;
  vcr_params pendingParams_{};
  bool hasPendingParams_ = false;
  vcr_shadow_volume pendingShadowVolume_{};
  bool hasPendingShadowVolume_ = false;
};

/* RenderTechniquePT (RenderTechniquePT.h:11): delta/ratio tracking. */
class VCR_API TechniquePT : public RenderTechnique {
 public:
  using RenderTechnique::RenderTechnique;
  void RecordPass(void* stream, uint32_t passIndex) override;
  uint32_t samplesPerPass = 1;
};

/* RenderTechniquePPM (RenderTechniquePPM.h:19): progressive photon mapping
 * with per-pixel FP64 statistics. */
class VCR_API TechniquePPM : public RenderTechnique {
 public:
  TechniquePPM(Device& device, PushConstants* pushConstants, const vcr_ppm_params& photonMap);
  ~TechniquePPM() override;
  void AllocateResources() override;
  void FreeResources() override;
  void RecordPass(void* stream, uint32_t passIndex) override;

 private:
  vcr_ppm_params photonMap_;
  bool allocated_ = false;
};

/* RenderTechniquePPB (RenderTechniquePPB.h:10): progressive photon beams. */
class VCR_API TechniquePPB : public RenderTechnique {
 public:
  TechniquePPB(Device& device, PushConstants* pushConstants, const vcr_ppb_params& beams);
  ~TechniquePPB() override;
  void AllocateResources() override;
  void FreeResources() override;
  /* UpdatePhotonMapProperties (RenderTechniquePPB.cpp:357-363): new beam
   * parameters; reallocates if resources are live. */
  void UpdatePhotonMapProperties(const vcr_ppb_params& beams);
  void RecordPass(void* stream, uint32_t passIndex) override;

 private:
  vcr_ppb_params beams_;
  bool allocated_ = false;
};

/* How TechniqueNRC trains while it renders.  poolSets = 0: every pass is a
 * vcr_nrc_frame (its training paths run in the pass's own launch, whose
 * length their deepest path sets).  poolSets = S > 0: every pass is a
 * vcr_pt_pass ending in the cache plus one Adam step on the next `batch`
 * records (0: train_samples) of a pool of S training sets, traced in one
 * launch every poolEvery passes.  Training paths never read the weights, so
 * pooled records train as well as per-pass ones, and one launch of S sets
 * costs about as much as three of one set. */
struct NrcSchedule {
  uint32_t poolSets = 0;
  uint32_t poolEvery = 96;
  uint32_t batch = 0;
  uint32_t spp = 1;  // camera samples per pixel of each pass (the query capacity must cover width x height x spp)
};

/* The DDA tracker with the learned radiance cache: paths end in the cache
 * after params.nrc_events events; every pass also trains it. */
class VCR_API TechniqueNRC : public RenderTechnique {
 public:
  TechniqueNRC(Device& device, PushConstants* pushConstants, const vcr_nrc_params& cache,
               const NrcSchedule& schedule = NrcSchedule());
  ~TechniqueNRC() override;
  void AllocateResources() override;
  void FreeResources() override;
  void RecordPass(void* stream, uint32_t passIndex) override;
  /* Training before the first pass: at least `steps` Adam steps, from
   * launches of `sets` training sets (vcr_nrc_train_step with pass.spp =
   * sets), each walked by vcr_nrc_train_more in batches of `batch` records
   * (0: train_samples).  Needs the camera, cloud and frame bound. */
  void Warmup(void* stream, uint32_t steps, uint32_t sets, uint32_t batch);

 private:
  vcr_nrc_params cache_;
  NrcSchedule schedule_;
  uint32_t passes_ = 0;    // passes since AllocateResources
  uint32_t launches_ = 0;  // training-set launches since AllocateResources
  bool allocated_ = false;
};

/* The state the reference's window edits (main.cpp:500-596).  Apply clamps
 * fov and pitch the way CameraProperties::SetFOV / SetRotation clamp the
 * caller's values (UniformBuffers.h:29-58). */
struct Settings {
  uint32_t width = 800, height = 600;
  float position[3] = {0.0f, 0.0f, -0.4f};
  float rotation[2] = {0.0f, 0.0f};  /* degrees: pitch about x (|pitch| <= 80), then yaw about y */
  float fov = 90.0f;                 /* vertical, degrees, [60, 150] */
  float nearPlane = 0.1f;
  float phaseG = 0.857f;             /* Parameters::SetPhaseG */
  float densityScaling = 8.0f;       /* CloudProperties.densityScaling */
  float sunDirection[3] = {0.0f, -0.5f, 0.866f}; /* direction the sunlight travels (normalised) */
};

enum class Technique { PathTracing = 0, PhotonMapping = 1, PhotonBeams = 2 };

/* The reference's main.cpp around its techniques, headless: one device, the
 * three techniques, the current one (the switch of main.cpp:197-221), and
 * the updates each edit needs.  Every edit that changes the image restarts
 * the progressive accumulation (frameCount = 1, main.cpp:262).
 *   LoadCloud  ≙ UpdateCloudData (main.cpp:266-335): grid, bounds, majorant
 *   Apply      ≙ the Apply button (main.cpp:545-596) + UpdateShadowVolume
 *                (:223-264): resolution, camera, phase, density, light;
 *                the shadow volume is rebuilt when the parameters use it,
 *                lit along the camera's forward for photon beams
 *   Render     ≙ one frame's RecordDrawCommands of the current technique */
class VCR_API Renderer {
 public:
  Renderer(Device& device, PushConstants* pushConstants, const vcr_params& params,
           const vcr_ppm_params& photonMap, const vcr_ppb_params& beams, uint32_t shadowVolumeSize = 128);
  ~Renderer();
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;

  void LoadCloud(const Grid& grid, int precision = VCR_PREC_FP32, float baseScaling = 1.0f);
  /* Returns whether the accumulation restarted; `settings` receives the
   * clamped fov and pitch. */
  bool Apply(Settings& settings);
  void SetTechnique(Technique technique);
  void Render(void* stream);

  Technique Current() const { return current_; }
  RenderTechnique& Active();
  const vcr_camera& Camera() const { return camera_; }
  const vcr_params& Parameters() const { return params_; }
  const vcr_cloud& Cloud() const { return cloud_; }
  uint32_t PassCount() const;

 private:
  void Restart();

  Device* device_;
  PushConstants* pushConstants_;
  TechniquePT pt_;
  TechniquePPM ppm_;
  TechniquePPB ppb_;
  Technique current_ = Technique::PathTracing;
  vcr_params params_{};
  vcr_camera camera_{};
  vcr_cloud cloud_{};
  vcr_shadow_volume shadowVolume_{};
  uint32_t shadowVolumeSize_;
  bool hasCloud_ = false, hasSettings_ = false, hasShadowVolume_ = false;
  Settings settings_{};
};

}  // namespace vcr
