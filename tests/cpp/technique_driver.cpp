// Drives the C++ RenderTechnique layer the way the reference's main.cpp
// drives its techniques (construction :811-814, bindings :859-883, frame
// references :842-844, per-frame RecordDrawCommands :631): builds a small
// fBm cloud, binds it with a camera and parameters, renders `passes`
// passes with the named technique, and writes
//   [vcr_params][vcr_camera][vcr_cloud][vcr_grid_desc][u32 w][u32 h]
//   [u32 passes][f32 pmRadius][f32 mean image w*h*3]
// to the output file, so a test can re-render the same structs through
// the C-ABI and compare.  The PT mode also writes the frame through
// WriteExr / WritePng next to it.
//   technique_driver <pt|ppm|ppb|nrc|nrcpool|misuse> <out> [passes]
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "vcr/render_technique.hpp"

static vcr_params scene_params() {
  vcr_params p{};
  p.max_events = 64;
  p.light_intensity = 1.0f;
  vcr_params_set_phase_g(&p, 0.857f);
  p.albedo = 0.99f;
  const double e = 30.0 * M_PI / 180.0, a = M_PI;  // sun at 30 deg, light travelling +x and down
  p.sun_dir[0] = (float)-(std::cos(e) * std::cos(a));
  p.sun_dir[1] = (float)-std::sin(e);
  p.sun_dir[2] = 0.0f;
  for (int i = 0; i < 3; ++i) p.sky[i] = 0.1f;
  p.sky_mode = VCR_SKY_CONSTANT;
  p.rng_mode = VCR_RNG_PCG;
  p.nee_mode = VCR_NEE_RATIO;
  p.tracker = VCR_TRACKER_DDA;
  return p;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <pt|ppm|ppb|nrc|nrcpool|misuse> <out> [passes]\n", argv[0]);
    return 2;
  }
  const std::string mode = argv[1];
  const int passes = argc > 3 ? std::atoi(argv[3]) : 4;
  const uint32_t W = 64, H = 48;
  try {
    vcr::Device device(0);
    vcr::PushConstants pc;
    pc.seed = 17;

    vcr_fbm_desc fbm{};
    fbm.seed = 3;
    fbm.octaves = 4;
    fbm.lacunarity = 2.0f;
    fbm.gain = 0.5f;
    fbm.base_frequency = 4.0f;
    vcr::Grid grid = vcr::Grid::Generate(64, 32, 64, fbm);
    vcr_cloud cloud{};
    vcr::Check(vcr_cloud_from_grid(&grid.desc, 1.0f, 16.0f, &cloud));
    cloud.max_extinction = std::fmax(grid.GetMajorant(), 0.01f);
    vcr_camera cam{};
    const float pos[3] = {0.0f, 0.0f, -0.4f}, fwd[3] = {0.0f, 0.0f, 1.0f};
    vcr::Check(vcr_camera_look(&cam, pos, fwd, 90.0f, 0.1f, (int)W, (int)H));
    vcr_params prm = scene_params();

    vcr::RenderTechnique* tech = nullptr;
    vcr::TechniquePT pt(device, &pc);
    vcr_ppm_params pm{1u << 14, 1u << 16, 0.02f, 0.7f};
    vcr::TechniquePPM ppm(device, &pc, pm);
    vcr_ppb_params pb{1u << 10, 1u << 15, 0.02f, 0.8f};
    vcr::TechniquePPB ppb(device, &pc, pb);
    vcr_nrc_params nc{4096, 1e-3f, W * H, 1, 0.0f};
    vcr::TechniqueNRC nrc(device, &pc, nc);
    vcr::NrcSchedule pool;  // a pool of 4 sets re-traced every 2nd pass, 1,024-record steps
    pool.poolSets = 4;
    pool.poolEvery = 2;
    pool.batch = 1024;
    vcr::TechniqueNRC nrcpool(device, &pc, nc, pool);
    if (mode == "pt") tech = &pt;
    else if (mode == "ppm") tech = &ppm;
    else if (mode == "ppb") tech = &ppb;
    else if (mode == "nrc") tech = &nrc;
    else if (mode == "nrcpool") tech = &nrcpool;
    else if (mode == "misuse") {
      // a pass before the frame target and before AllocateResources must
      // throw vcr::Error (the reference aborts instead)
      int thrown = 0;
      try { pt.RecordPass(nullptr, 0); } catch (const vcr::Error& e) { thrown += e.status() == VCR_ERR_STATE; }
      ppm.SetFrameTarget(W, H);
      try { ppm.RecordPass(nullptr, 0); } catch (const vcr::Error& e) { thrown += e.status() == VCR_ERR_STATE; }
      try { vcr::Grid::Load("/nonexistent/cloud.xyz"); } catch (const vcr::Error& e) { thrown += e.status() == VCR_ERR_IO; }
      std::printf("misuse errors %d\n", thrown);
      return thrown == 3 ? 0 : 1;
    } else {
      std::fprintf(stderr, "unknown technique %s\n", mode.c_str());
      return 2;
    }
    if (mode == "nrc" || mode == "nrcpool") prm.nrc_events = 2;

    tech->BindCloud(grid, cloud, VCR_PREC_FP32);
    tech->BindCamera(cam);
    tech->BindParameters(prm);
    tech->SetFrameTarget(W, H);
    tech->Commit();
    tech->AllocateResources();
    if (mode == "nrcpool") nrcpool.Warmup(nullptr, 40, 4, 1024);  // 40 steps from 4-set launches
    for (int k = 0; k < passes; ++k) tech->RecordPass(nullptr, (uint32_t)k);
    device.Synchronize();
    std::vector<float> img = tech->ReadMean();
    if (tech->PassCount() != (uint32_t)passes || pc.frameCount != (uint32_t)passes + 1u) {
      std::fprintf(stderr, "pass count %u frameCount %u\n", tech->PassCount(), pc.frameCount);
      return 1;
    }
    if (mode == "pt") {  // the frame as files: <out>.exr (FLOAT), <out>.half.exr, <out>.png
      const std::string base = argv[2];
      tech->WriteExr(base + ".exr");
      tech->WriteExr(base + ".half.exr", true);
      tech->WritePng(base + ".png");
    }
    tech->FreeResources();

    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 1;
    uint32_t hdr[3] = {W, H, (uint32_t)passes};
    std::fwrite(&prm, sizeof prm, 1, f);
    std::fwrite(&cam, sizeof cam, 1, f);
    std::fwrite(&cloud, sizeof cloud, 1, f);
    std::fwrite(&grid.desc, sizeof grid.desc, 1, f);
    std::fwrite(hdr, sizeof hdr, 1, f);
    std::fwrite(&pc.pmRadius, sizeof(float), 1, f);
    std::fwrite(img.data(), sizeof(float), img.size(), f);
    std::fclose(f);
    std::printf("%s passes %d pmRadius %g\n", mode.c_str(), passes, pc.pmRadius);
  } catch (const vcr::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
