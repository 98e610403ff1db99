// Test infrastructure: the reference's own compute shaders run on the CPU.
// PathTracer.comp and ShadowVolume.comp are transliterated by
// oracle/build_ref.py (parameter qualifiers, descriptor declarations,
// float literals and main's name: nothing of their bodies) into
// oracle/_ref/, and included here inside one namespace each, over the GLSL
// pieces of glsl_shim.h; the uniform blocks, images and samplers they name
// are set through the entry points below.  Built into
// oracle/_ref/libref_shaders.so only where the reference tree exists.
//
// Entry points (C ABI, all single invocations unless named *_image):
//   ref_set_scene       cloud texture + CloudProperties, CameraProperties,
//                       Parameters, ShadowVolumeProperties + its texture
//   ref_pt_image        PathTracer.comp main for every pixel (dispatch
//                       (W / 32 + 1, H / 32 + 1) as RenderTechniquePT
//                       records it), into an RGBA float image
//   ref_sv_build        ShadowVolume.comp main for every column
//   ref_* functions     single shader functions, the RNG state in / out
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "../include/vcr/abi.h"

namespace ref_pt {
#include "glsl_shim.h"
CameraPropertiesBlock cameraProperties;
CloudPropertiesBlock cloudProperties;
ParametersBlock parameters;
ShadowVolumePropertiesBlock shadowVolumeProperties;
PushConstantsBlock pushConstants;
image2D resultImage;
sampler3D cloudSampler;
sampler3D shadowSampler;
#include "_ref/PathTracer.comp.cpp"
}  // namespace ref_pt

namespace ref_sv {
#include "glsl_shim.h"
ShadowVolumePropertiesBlock shadowVolumeProperties;
CloudPropertiesBlock cloudProperties;
image3D shadowVolume;
sampler3D cloudSampler;
#include "_ref/ShadowVolume.comp.cpp"
}  // namespace ref_sv

namespace {

template <class V>
V v3(const float* p) {
  return V(p[0], p[1], p[2]);
}

// ShadowVolumeProperties as UniformBuffers.h:114-166 lays it out: bounds
// with w = 1, directions with w = 0, basisChange the inverse of the basis
// (right, up, light) — for an orthonormal basis its transpose, which is
// the row-major world -> (right, up, light) matrix the C-ABI struct holds.
template <class NS_SV>
void fill_sv(NS_SV& b, const vcr_shadow_volume& sv) {
  using vec4 = decltype(b.lightDirection);
  b.bounds[0] = vec4(sv.bounds_min[0], sv.bounds_min[1], sv.bounds_min[2], 1.0f);
  b.bounds[1] = vec4(sv.bounds_max[0], sv.bounds_max[1], sv.bounds_max[2], 1.0f);
  b.lightDirection = vec4(sv.light_dir[0], sv.light_dir[1], sv.light_dir[2], 0.0f);
  b.right = vec4(sv.right[0], sv.right[1], sv.right[2], 0.0f);
  b.up = vec4(sv.up[0], sv.up[1], sv.up[2], 0.0f);
  for (int c = 0; c < 3; ++c) b.basisChange.c[c] = vec4(sv.basis_change[c], sv.basis_change[3 + c], sv.basis_change[6 + c], 0.0f);
  b.basisChange.c[3] = vec4(0.0f, 0.0f, 0.0f, 1.0f);
  b.voxelAxisCount = sv.voxel_axis_count;
  b.voxelSize = sv.voxel_size;
}

template <class NS_CL>
void fill_cloud(NS_CL& b, const vcr_cloud& cl, const uint32_t n[3]) {
  using vec4 = decltype(b.bounds[0]);
  using V4 = typename std::remove_reference<vec4>::type;
  b.bounds[0] = V4(cl.bounds_min[0], cl.bounds_min[1], cl.bounds_min[2], 1.0f);
  b.bounds[1] = V4(cl.bounds_max[0], cl.bounds_max[1], cl.bounds_max[2], 1.0f);
  b.voxelCount.x = n[0];
  b.voxelCount.y = n[1];
  b.voxelCount.z = n[2];
  b.voxelCount.w = 0;
  b.maxExtinction = cl.max_extinction;
  b.baseScaling = cl.base_scaling;
  b.densityScaling = cl.density_scaling;
}

}  // namespace

extern "C" {

// Everything the two shaders read.  `dense` (x fastest, n[0] x n[1] x n[2]
// floats) is the cloud texture; `sv_tex` (sv->voxel_axis_count^3, x fastest)
// the shadow-volume texture the path tracer samples (may be null for the
// shadow-volume build itself).  The pointers are kept, not copied.
void ref_set_scene(const float* dense, const uint32_t n[3], const vcr_cloud* cl, const vcr_camera* cam,
                   const vcr_params* prm, const vcr_shadow_volume* sv, const float* sv_tex) {
  for (int a = 0; a < 3; ++a) {
    ref_pt::cloudSampler.n[a] = (int)n[a];
    ref_sv::cloudSampler.n[a] = (int)n[a];
  }
  ref_pt::cloudSampler.texels = dense;
  ref_sv::cloudSampler.texels = dense;
  fill_cloud(ref_pt::cloudProperties, *cl, n);
  fill_cloud(ref_sv::cloudProperties, *cl, n);
  if (cam) {
    auto& c = ref_pt::cameraProperties;
    c.position = v3<ref_pt::vec3>(cam->position);
    c.halfWidth = cam->half_width;
    c.forward = v3<ref_pt::vec3>(cam->forward);
    c.halfHeight = cam->half_height;
    c.right = v3<ref_pt::vec3>(cam->right);
    c.nearPlane = cam->near_plane;
    c.up = v3<ref_pt::vec3>(cam->up);
    c.pixelSizeY = cam->pixel_size_y;
    c.pixelSizeX = cam->pixel_size_x;
  }
  if (prm) {
    auto& p = ref_pt::parameters;
    p.maxRayBounces = prm->max_events;
    p.lightIntensity = prm->light_intensity;
    p.phaseG = prm->phase_g;
    p.phaseOnePlusG2 = prm->phase_one_plus_g2;
    p.phaseOneMinusG2 = prm->phase_one_minus_g2;
    p.phaseOneOver2G = prm->phase_one_over_2g;
    p.isotropic = prm->isotropic != 0;
  }
  if (sv) {
    fill_sv(ref_pt::shadowVolumeProperties, *sv);
    fill_sv(ref_sv::shadowVolumeProperties, *sv);
    const int m = (int)sv->voxel_axis_count;
    for (int a = 0; a < 3; ++a) ref_pt::shadowSampler.n[a] = m;
    ref_pt::shadowSampler.texels = sv_tex;
  }
}

// PathTracer.comp main over a W x H image: `rgba` holds the previous
// result (imageLoad) and receives the new one; frameCount as the push
// constant (0: the result is this pass's radiance).
void ref_pt_image(uint32_t W, uint32_t H, int seed, uint32_t frame_count, float* rgba, int threads) {
  using namespace ref_pt;
  resultImage.rgba = rgba;
  resultImage.width = (int)W;
  pushConstants.seed = seed;
  pushConstants.frameCount = frame_count;
  gl_NumWorkGroups = uvec3(W / 32u + 1u, H / 32u + 1u, 1u);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
  for (int64_t y = 0; y < (int64_t)H; ++y)
    for (uint32_t x = 0; x < W; ++x) {
      gl_GlobalInvocationID = uvec3(x, (uint32_t)y, 0u);
      shader_main();
    }
}

// ShadowVolume.comp main for every (x, y) column of an n^3 volume.
void ref_sv_build(float* out, int threads) {
  using namespace ref_sv;
  const uint32_t n = shadowVolumeProperties.voxelAxisCount;
  shadowVolume.r = out;
  shadowVolume.n = (int)n;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
  for (int64_t y = 0; y < (int64_t)n; ++y)
    for (uint32_t x = 0; x < n; ++x) {
      gl_GlobalInvocationID = uvec3(x, (uint32_t)y, 0u);
      shader_main();
    }
}

// ---- single functions of PathTracer.comp ----------------------------------
void ref_sample_background(const float dir[3], float out[4]) {
  ref_pt::vec4 c = ref_pt::sampleBackground(v3<ref_pt::vec3>(dir));
  for (int i = 0; i < 4; ++i) out[i] = c[i];
}

int ref_intersect_cloud(const float pos[3], const float dir[3], float* tmin, float* tmax) {
  ref_pt::Ray r;
  r.pos = v3<ref_pt::vec3>(pos);
  r.dir = v3<ref_pt::vec3>(dir);
  return ref_pt::intersectCloud(r, *tmax, *tmin) ? 1 : 0;
}

void ref_camera_ray(int x, int y, float pos[3], float dir[3]) {
  ref_pt::Ray r;
  ref_pt::getCameraRay(ref_pt::ivec2(x, y), r);
  for (int i = 0; i < 3; ++i) {
    pos[i] = r.pos[i];
    dir[i] = r.dir[i];
  }
}

uint32_t ref_initialize_random(uint32_t seed) {
  ref_pt::initializeRandom(seed);
  return ref_pt::rng_state;
}

// n numbers of generateRandomNumber from `state`; returns the state after.
uint32_t ref_random_numbers(uint32_t state, uint32_t n, float* out) {
  ref_pt::rng_state = state;
  for (uint32_t i = 0; i < n; ++i) out[i] = ref_pt::generateRandomNumber();
  return ref_pt::rng_state;
}

float ref_sample_phase(const float in[3], const float out[3]) {
  return ref_pt::samplePhase(v3<ref_pt::vec3>(in), v3<ref_pt::vec3>(out));
}

void ref_onb(const float n[3], float xp[3], float yp[3]) {
  ref_pt::vec3 a, b;
  ref_pt::createOrthonormalBasis(v3<ref_pt::vec3>(n), a, b);
  for (int i = 0; i < 3; ++i) {
    xp[i] = a[i];
    yp[i] = b[i];
  }
}

uint32_t ref_scatter_ray(const float in[3], uint32_t state, float out[3]) {
  ref_pt::rng_state = state;
  ref_pt::vec3 d(0.0f);
  ref_pt::scatterRay(v3<ref_pt::vec3>(in), d);
  for (int i = 0; i < 3; ++i) out[i] = d[i];
  return ref_pt::rng_state;
}

float ref_sample_cloud(const float pos[3]) { return ref_pt::sampleCloud(v3<ref_pt::vec3>(pos)); }

float ref_sample_shadow_volume(const float pos[3]) {
  return ref_pt::sampleShadowVolume(v3<ref_pt::vec3>(pos));
}

// findScatterPoint from (pos, dir): returns 1 with pos moved to the
// collision, 0 on leaving the cloud; *state carries the RNG.
int ref_find_scatter_point(float pos[3], const float dir[3], uint32_t* state) {
  ref_pt::rng_state = *state;
  ref_pt::Ray r;
  r.pos = v3<ref_pt::vec3>(pos);
  r.dir = v3<ref_pt::vec3>(dir);
  const bool hit = ref_pt::findScatterPoint(r);
  for (int i = 0; i < 3; ++i) pos[i] = r.pos[i];
  *state = ref_pt::rng_state;
  return hit ? 1 : 0;
}

}  // extern "C"
