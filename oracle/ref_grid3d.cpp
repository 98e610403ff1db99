// Test infrastructure: drives the reference's own Grid3D<float>
// (CloudRendering-Vulkan/Grid3D.h: Load :44-90, Save :166-178, GetMajorant
// :180-192), compiled from its header where it lies, so the project's .xyz
// reader/writer and majorant can be checked against it.  Built by
// oracle/build_ref.py into oracle/_ref/ only when the reference tree exists.
//
//   ref_grid3d load <in.xyz> <out.bin>  : Grid3D::Load, then write
//        u32 X Y Z, f64 voxel x y z, f32 majorant, f32 data in memory order
//   ref_grid3d save <in.bin> <out.xyz>  : a Grid3D built from
//        u32 X Y Z, f64 voxel x y z, f32 data (memory order), then Save
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include <glm/glm.hpp>

#include "Grid3D.h"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  const std::string mode = argv[1];
  if (mode == "load") {
    Grid3D<float>* g = Grid3D<float>::Load(argv[2]);
    if (!g) return 3;
    glm::uvec3 n = g->GetVoxelCount();
    glm::dvec3 v = g->GetVoxelSize();
    std::ofstream out(argv[3], std::ios::binary);
    uint32_t dims[3] = {n.x, n.y, n.z};
    double vs[3] = {v.x, v.y, v.z};
    float maj = g->GetMajorant();
    out.write(reinterpret_cast<const char*>(dims), sizeof dims);
    out.write(reinterpret_cast<const char*>(vs), sizeof vs);
    out.write(reinterpret_cast<const char*>(&maj), sizeof maj);
    out.write(reinterpret_cast<const char*>(g->GetData()), (std::streamsize)g->GetByteSize());
    delete g;
    return out ? 0 : 4;
  }
  if (mode == "save") {
    std::ifstream in(argv[2], std::ios::binary);
    uint32_t dims[3];
    double vs[3];
    if (!in.read(reinterpret_cast<char*>(dims), sizeof dims) || !in.read(reinterpret_cast<char*>(vs), sizeof vs))
      return 3;
    size_t n = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<float> data(n);
    if (!in.read(reinterpret_cast<char*>(data.data()), (std::streamsize)(n * sizeof(float)))) return 3;
    Grid3D<float> g(dims[0], dims[1], dims[2], vs[0], vs[1], vs[2]);
    g.Copy(data.data(), n * sizeof(float));
    g.Save(argv[3]);
    return 0;
  }
  return 2;
}
