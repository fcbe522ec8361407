// Prints the sample points of the facade's emitters (include/sf_kiri_facade.hpp)
// as raw float32 to stdout, for comparison with the reference emitters'
// fixtures (tests/golden/emitters.npz). Host only; needs no GPU.
//   emitter_points world <lx ly lz hx hy hz r>
//   emitter_points emit <type 0|1|2> <r> <a> <b>   (position (0.9,0.9,1.25), velocity (0,0,-5))
#include <cstdio>
#include <cstdlib>

#include "sf_kiri_facade.hpp"

using namespace KIRI;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string mode = argv[1];
    std::vector<float> out;
    if (mode == "world" && argc == 9) {
        BoundaryData data;
        CudaBoundaryEmitter().BuildWorldBoundary(
            data, make_float3(float(std::atof(argv[2])), float(std::atof(argv[3])), float(std::atof(argv[4]))),
            make_float3(float(std::atof(argv[5])), float(std::atof(argv[6])), float(std::atof(argv[7]))),
            float(std::atof(argv[8])));
        for (const float3& p : data.pos) out.insert(out.end(), {p.x, p.y, p.z});
    } else if (mode == "emit" && argc == 6) {
        CudaEmitter em(make_float3(0.9f, 0.9f, 1.25f), make_float3(0.f, 0.f, -5.f), true);
        const int type = std::atoi(argv[2]);
        const float r = float(std::atof(argv[3])), a = float(std::atof(argv[4])), b = float(std::atof(argv[5]));
        if (type == 0) em.BuildSquareEmitter(r, a);
        else if (type == 1) em.BuildCircleEmitter(r, a);
        else em.BuildRectangleEmitter(r, a, b);
        for (const float3& p : em.Emit()) out.insert(out.end(), {p.x, p.y, p.z});
    } else {
        return 2;
    }
    std::fwrite(out.data(), sizeof(float), out.size(), stdout);
    return 0;
}
