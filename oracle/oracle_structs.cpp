// ORACLE — test infrastructure only (see oracle_math.h).  The reference's
// host-side set-up of the uniform structs a render reads, restated so the
// CPU reference leg of the benchmark builds its scene without the product
// library:
//   Parameters::SetPhaseG            UniformBuffers.h:93-106
//   SetCloudProperties               main.cpp:145-163 (bounds from the grid)
//   CameraProperties::SetResolution  UniformBuffers.h:46-50
//   CameraProperties::SetFOV         UniformBuffers.h:52-58 (60..150 deg clamp)
//   utilities::GetOrthonormalBasis   Utilities.cpp:7-16 (right and up from forward)
// The camera is given by a position and a forward vector instead of the
// reference's pitch/yaw rotation (UniformBuffers.h:29-35); the basis built
// from the forward vector is the reference's.
#include <algorithm>
#include <cmath>

#include "../include/vcr/abi.h"

namespace {

void orthonormal_basis(const float n[3], float xp[3], float yp[3]) {
  float sz = n[2] >= 0.0f ? 1.0f : -1.0f;
  float a = n[1] / (1.0f + std::fabs(n[2]));
  float b = n[1] * a;
  float c = -n[0] * a;
  xp[0] = n[2] + sz * b;
  xp[1] = sz * c;
  xp[2] = -n[0];
  yp[0] = c;
  yp[1] = 1.0f - b;
  yp[2] = -sz * n[1];
}

}  // namespace

extern "C" {

int oracle_params_set_phase_g(vcr_params* p, float value) {
  if (!p) return 1;
  if (value > 1.0f || value < -1.0f) return 0;  // SetPhaseG ignores values outside [-1, 1]
  float g = std::min(std::max(value, -0.95f), 0.95f);
  p->phase_g = g;
  p->isotropic = std::fabs(g) < 0.0001f ? 1 : 0;
  if (!p->isotropic) {
    p->phase_one_plus_g2 = 1.0f + g * g;
    p->phase_one_minus_g2 = 1.0f - g * g;
    p->phase_one_over_2g = 0.5f / g;
  }
  return 0;
}

// Cloud bounds: x and y centred, z from 0 (main.cpp:147-160); the global
// majorant is the caller's (GetMajorant of the grid, clamped to >= 0.01).
int oracle_cloud_from_grid(const vcr_grid_desc* grid, float base_scaling, float density_scaling, vcr_cloud* out) {
  if (!grid || !out) return 1;
  float size[3];
  for (int a = 0; a < 3; ++a) size[a] = (float)(grid->voxel_size[a] * (double)grid->size[a] * (double)base_scaling);
  out->bounds_min[0] = -size[0] / 2.0f;
  out->bounds_min[1] = -size[1] / 2.0f;
  out->bounds_min[2] = 0.0f;
  out->bounds_max[0] = size[0] / 2.0f;
  out->bounds_max[1] = size[1] / 2.0f;
  out->bounds_max[2] = size[2];
  out->max_extinction = 0.0f;
  out->base_scaling = base_scaling;
  out->density_scaling = density_scaling;
  return 0;
}

int oracle_camera_look(vcr_camera* cam, const float position[3], const float forward[3], float fov_y_deg,
                       float near_plane, int32_t width, int32_t height) {
  if (!cam || !position || !forward || width < 2 || height < 2 || !(near_plane > 0.0f)) return 1;
  double l = std::sqrt((double)forward[0] * forward[0] + (double)forward[1] * forward[1] +
                       (double)forward[2] * forward[2]);
  if (!(l > 0.0)) return 1;
  for (int a = 0; a < 3; ++a) {
    cam->position[a] = position[a];
    cam->forward[a] = (float)(forward[a] / l);
  }
  orthonormal_basis(cam->forward, cam->right, cam->up);
  cam->near_plane = near_plane;
  cam->half_width = width / 2;
  cam->half_height = height / 2;
  float fov = std::min(std::max(fov_y_deg, 60.0f), 150.0f);
  float h = 2.0f * std::tan(fov / 2.0f * 3.14159265358979f / 180.0f) * near_plane;
  cam->pixel_size_y = h / (float)(cam->half_height * 2);
  cam->pixel_size_x = cam->pixel_size_y * (float)cam->half_height / (float)cam->half_width;
  return 0;
}

}  // extern "C"
