// Drop-in check of include/sf_kiri_facade.hpp: the scene set-up and frame
// loop of seepage_flows/src/seepageflow/main.cpp:25-283, written against the
// facade, on a seeded box scene (the app's bunny asset is not distributed).
// Writes the initial and final particle states (creation order) to the file
// named by argv[1] so the test can replay them through the CPU oracle.
#include <cstdio>
#include <cstdlib>

#include "facade_scene.hpp"

using namespace KIRI;

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: facade_main <dump> <frames> [<bgeo export folder>]\n");
        return 2;
    }
    const int frames = std::atoi(argv[2]);
    const float3 lowest = make_float3(0.f, 0.f, 0.f), highest = make_float3(0.4f, 0.4f, 0.4f);
    facade_test::setReferenceParams(WCSPH_SOLVER);
    CUDA_SPH_EMITTER_PARAMS.enable = false;

    auto emitter = std::make_shared<CudaEmitter>(make_float3(0.2f, 0.3f, 0.2f), make_float3(0.f, -1.f, 0.f), false);
    BoundaryData boundary;
    CudaBoundaryEmitter().BuildWorldBoundary(boundary, lowest, highest, CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius);

    // sand block + water column (the two box volumes of a seepage scene)
    Vec_Float3 cda;
    Vec_Float2 amc;
    SeepageflowVolumeData vol = facade_test::buildVolume(cda, amc);
    auto particles = std::make_shared<CudaSFParticles>(vol.pos.size() + 64, vol.pos, vol.col, vol.label, vol.mass,
                                                       vol.radius, cda, amc);
    auto searcher = std::make_shared<CudaGNSearcher>(lowest, highest, particles->MaxSize(),
                                                     CUDA_BOUNDARY_PARAMS.kernel_radius, SEEPAGE_MULTI);
    auto boundaryParticles = std::make_shared<CudaBoundaryParticles>(boundary.pos, boundary.label);
    CudaSphSFSolverPtr solver = std::make_shared<CudaWCSphSFSolver>(particles->MaxSize());
    auto boundarySearcher = std::make_shared<CudaGNBoundarySearcher>(lowest, highest, boundaryParticles->MaxSize(),
                                                                     CUDA_BOUNDARY_PARAMS.kernel_radius);
    CudaSFParticlesPtr pp = particles;
    CudaBoundaryParticlesPtr bb = boundaryParticles;
    CudaGNSearcherPtr ss = searcher;
    CudaGNBoundarySearcherPtr bs = boundarySearcher;
    CudaEmitterPtr ee = emitter;
    CudaSFSystem system(pp, bb, solver, ss, bs, ee, true);
    if (!system.Handle()) return 3;

    const size_t n = particles->Size();
    FILE* f = std::fopen(argv[1], "wb");
    auto dump = [&](const Vec_Float3& pos, const std::vector<int32_t>* ids) {
        std::fwrite(pos.data(), sizeof(float3), pos.size(), f);
        (void)ids;
    };
    dump(vol.pos, nullptr);
    const float renderInterval = 1.f / 30.f;
    size_t calls = 0;
    for (int frame = 0; frame < frames; ++frame) {  // main.cpp:235-247
        float remaining = renderInterval;
        while (remaining > 1e-6f) {
            if (!system.UpdateSystemChecked(remaining, nullptr)) return 4;
            remaining -= remaining / float(system.GetNumOfSubTimeSteps());
            ++calls;
        }
    }
    std::vector<float> out(3 * n);
    if (sf_get_field(system.Handle(), 0, SF_FIELD_POS, SF_ORDER_ID, out.data(), int64_t(n), 0) != SF_OK) return 5;
    std::fwrite(out.data(), sizeof(float), out.size(), f);
    std::fclose(f);
    const float3* dpos = particles->GetPosPtr();
    // the searchers' cell tables (GetCellStartPtr): G + 1 monotone entries
    // ending with the particle / boundary count
    for (int which = 0; which < 2; ++which) {
        const CudaGNBaseSearcher& se = which ? static_cast<const CudaGNBaseSearcher&>(*boundarySearcher)
                                             : static_cast<const CudaGNBaseSearcher&>(*searcher);
        const int3 g = se.GetGridSize();
        std::vector<size_t> t(size_t(g.x) * g.y * g.z + 1);
        const size_t* d = se.GetCellStartPtr();
        if (!d || cudaMemcpy(t.data(), d, t.size() * sizeof(size_t), cudaMemcpyDeviceToHost) != cudaSuccess) return 7;
        bool mono = true;
        for (size_t c = 1; c < t.size(); ++c) mono = mono && t[c] >= t[c - 1];
        std::printf("cell table %d: entries=%zu last=%zu monotone=%d\n", which, t.size(), t.back(), int(mono));
    }
    if (argc > 3) {  // the app's per-frame export (main.cpp:265-276) and a read-back
        ExportBgeoFileCUDA(argv[3], UInt2Str4Digit(unsigned(frames)), particles->GetPosPtr(), particles->GetColPtr(),
                           particles->GetRadiusPtr(), particles->GetLabelPtr(), particles->Size());
        const Vec_Float4 back = ReadBgeoFileForGPU("out", UInt2Str4Digit(unsigned(frames)));
        std::printf("bgeo read back: %zu points, first pscale %.6g\n", back.size(),
                    back.empty() ? -1.0 : double(back[0].w));
    }
    std::printf("facade ok: particles=%zu boundary=%zu frames=%d calls=%zu n_sub=%zu device_pos=%p\n", n,
                boundary.pos.size(), frames, calls, system.GetNumOfSubTimeSteps(), static_cast<const void*>(dpos));
    return dpos ? 0 : 6;
}
