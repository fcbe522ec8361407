// The reference app's shape import written against the facade
// (seepage_flows/src/seepageflow/main.cpp:121-167): ReadBgeoFileForGPU of a
// shape file, then CudaVolumeEmitter::BuildSeepageflowShapeMultiVolume (sand
// object) or CudaBoundaryEmitter::BuildBoundaryShapeVolume (shape boundary).
// Host only; links libsf_gb300.so for the .bgeo reader and needs no GPU.
// Compile with -DDB_PBR_PATH="<root>/" and put the file at
// <root>/bgeo/<folder>/<name>.bgeo.
//   shape_import volume <folder> <name> <offset 0|1> <lowest_y> <times>
//   shape_import boundary <folder> <name>
// Writes raw float32 to stdout: volume -> sandMinRadius, then per particle
// pos(3) col(3) cda0asat(3) radius mass amcamcp(2) label; boundary -> per
// particle pos(3) label.
#include <cstdio>
#include <cstdlib>

#include "sf_kiri_facade.hpp"

using namespace KIRI;

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::string mode = argv[1];
    const Vec_Float4 shape = ReadBgeoFileForGPU(argv[2], argv[3]);
    if (shape.empty()) return 3;
    std::vector<float> out;
    if (mode == "volume" && argc == 7) {
        SeepageflowMultiVolumeData data;
        CudaVolumeEmitter em;
        for (int k = 0; k < std::atoi(argv[6]); ++k)  // one call per object, as the app's loop over shapes
            em.BuildSeepageflowShapeMultiVolume(data, shape, make_float3(0.88f, 0.79f, 0.62f), 2650.f,
                                                make_float3(0.5f, 0.6f, 0.8f), make_float2(0.7f, 0.3f),
                                                std::atoi(argv[4]) != 0, float(std::atof(argv[5])));
        out.push_back(data.sandMinRadius);
        for (size_t i = 0; i < data.pos.size(); ++i)
            out.insert(out.end(), {data.pos[i].x, data.pos[i].y, data.pos[i].z, data.col[i].x, data.col[i].y,
                                   data.col[i].z, data.cda0asat[i].x, data.cda0asat[i].y, data.cda0asat[i].z,
                                   data.radius[i], data.mass[i], data.amcamcp[i].x, data.amcamcp[i].y,
                                   float(data.label[i])});
    } else if (mode == "boundary" && argc == 4) {
        BoundaryData data;
        CudaBoundaryEmitter().BuildBoundaryShapeVolume(data, shape);
        for (size_t i = 0; i < data.pos.size(); ++i)
            out.insert(out.end(), {data.pos[i].x, data.pos[i].y, data.pos[i].z, float(data.label[i])});
    } else {
        return 2;
    }
    std::fwrite(out.data(), sizeof(float), out.size(), stdout);
    return 0;
}
