// Drives vcr::Renderer through an edit session the way the reference's
// window does (load a cloud, Apply, render frames, edit camera / density /
// technique, Apply again) and checks the progressive state after each step.
// Prints "renderer checks <n>" with the number of checks that held, the
// camera forward after a (20, 30) degree rotation, and writes
//   [vcr_params][vcr_camera][vcr_cloud][vcr_grid_desc][u32 w][u32 h]
//   [u32 passes][f32 mean image w*h*3]
// for the final path-traced frame, so a test can re-render the same structs
// through the C-ABI and compare.
//   renderer_driver <out>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vcr/render_technique.hpp"

static vcr_params scene_params() {
  vcr_params p{};
  p.max_events = 64;
  p.light_intensity = 1.0f;
  vcr_params_set_phase_g(&p, 0.857f);
  p.albedo = 0.99f;
  for (int i = 0; i < 3; ++i) p.sky[i] = 0.1f;
  p.sky_mode = VCR_SKY_CONSTANT;
  p.rng_mode = VCR_RNG_PCG;
  p.nee_mode = VCR_NEE_RATIO;
  p.tracker = VCR_TRACKER_DDA;
  return p;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <out>\n", argv[0]);
    return 2;
  }
  int ok = 0, total = 0;
  auto expect = [&](bool c, const char* what) {
    ++total;
    if (c) ++ok;
    else std::printf("failed: %s\n", what);
  };
  try {
    vcr::Device device(0);
    vcr::PushConstants pc;
    pc.seed = 23;
    vcr_ppm_params pm{1u << 13, 1u << 16, 0.02f, 0.7f};
    vcr_ppb_params pb{1u << 9, 1u << 15, 0.02f, 0.8f};
    vcr::Renderer r(device, &pc, scene_params(), pm, pb, 64);
    vcr_fbm_desc fbm{};
    fbm.seed = 3;
    fbm.octaves = 4;
    fbm.lacunarity = 2.0f;
    fbm.gain = 0.5f;
    fbm.base_frequency = 4.0f;
    vcr::Grid grid = vcr::Grid::Generate(64, 32, 64, fbm);

    vcr::Settings s;
    s.width = 64;
    s.height = 48;
    s.densityScaling = 16.0f;
    const vcr::Settings start = s;
    r.LoadCloud(grid);
    expect(r.Apply(s), "first Apply restarts");
    for (int k = 0; k < 3; ++k) r.Render(nullptr);
    device.Synchronize();
    expect(r.PassCount() == 3 && pc.frameCount == 4, "three frames accumulate");
    expect(!r.Apply(s), "an unchanged Apply keeps the accumulation");
    r.Render(nullptr);
    device.Synchronize();
    expect(r.PassCount() == 4, "and the next frame adds to it");

    s.rotation[0] = 120.0f;
    s.fov = 200.0f;
    expect(r.Apply(s), "a camera edit restarts");
    expect(s.rotation[0] == 80.0f && s.fov == 150.0f, "pitch and fov are clamped like SetRotation / SetFOV");
    expect(r.PassCount() == 0 && pc.frameCount == 1, "the restart clears the sums (frameCount = 1)");
    s.densityScaling = 24.0f;
    expect(r.Apply(s) && r.Cloud().density_scaling == 24.0f, "a density edit reaches the cloud");

    r.SetTechnique(vcr::Technique::PhotonMapping);
    r.Render(nullptr);
    r.Render(nullptr);
    device.Synchronize();
    expect(r.PassCount() == 2, "photon mapping renders after the switch");
    r.SetTechnique(vcr::Technique::PhotonBeams);
    r.Render(nullptr);
    device.Synchronize();
    expect(r.PassCount() == 1, "photon beams render after the switch");

    vcr::Settings rot = start;
    rot.rotation[0] = 20.0f;
    rot.rotation[1] = 30.0f;
    r.SetTechnique(vcr::Technique::PathTracing);
    r.Apply(rot);
    const vcr_camera& c = r.Camera();
    std::printf("forward %.9g %.9g %.9g\n", c.forward[0], c.forward[1], c.forward[2]);

    s = start;
    expect(r.Apply(s), "back to the first settings");
    for (int k = 0; k < 4; ++k) r.Render(nullptr);
    device.Synchronize();
    expect(r.PassCount() == 4, "four frames");
    std::vector<float> img = r.Active().ReadMean();

    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    vcr_params prm = r.Parameters();
    vcr_camera cam = r.Camera();
    vcr_cloud cl = r.Cloud();
    std::fwrite(&prm, sizeof prm, 1, f);
    std::fwrite(&cam, sizeof cam, 1, f);
    std::fwrite(&cl, sizeof cl, 1, f);
    std::fwrite(&grid.desc, sizeof grid.desc, 1, f);
    const uint32_t hdr[3] = {s.width, s.height, r.PassCount()};
    std::fwrite(hdr, sizeof hdr, 1, f);
    std::fwrite(img.data(), sizeof(float), img.size(), f);
    std::fclose(f);
  } catch (const vcr::Error& e) {
    std::printf("error %d: %s\n", (int)e.status(), e.what());
    return 1;
  }
  std::printf("renderer checks %d of %d\n", ok, total);
  return ok == total ? 0 : 1;
}
