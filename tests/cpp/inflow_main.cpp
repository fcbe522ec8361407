// Inflow check of include/sf_kiri_facade.hpp: the facade scene with the SPH
// emitter switched on (CUDA_SPH_EMITTER_PARAMS and an enabled CudaEmitter, a
// square emitter 0.2 m above the floor shooting water downwards), advanced by
// `calls` UpdateSystem(1/30 s) calls under the WCSPH or the SPH emission
// schedule of CudaSFSystem::OnUpdateSolver (cuda_sf_system.cu:86-115). The
// particle arrays have 32 slots of headroom (three emissions of the 9-point
// emitter), so the capacity cut-off (Size() + emitted < MaxSize(), else the
// emitter switches off) is reached at the fourth.
//
// Writes to argv[1], little-endian: int64 n0, npts, calls; float32 initial
// positions (n0 x 3, creation order); float32 emitter points (npts x 3);
// int64 particle count after every call; int64 sub-step count of every call;
// int64 n; float32 final positions and velocities (n x 3 each, creation order).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "facade_scene.hpp"

using namespace KIRI;

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: inflow_main <dump> <wcsph|sph> <calls>\n");
        return 2;
    }
    const bool wcsph = std::strcmp(argv[2], "sph") != 0;
    const int calls = std::atoi(argv[3]);
    const float3 lowest = make_float3(0.f, 0.f, 0.f), highest = make_float3(0.4f, 0.4f, 0.4f);
    facade_test::setReferenceParams(wcsph ? WCSPH_SOLVER : SPH_SOLVER);
    CUDA_SPH_EMITTER_PARAMS.enable = true;
    CUDA_SPH_EMITTER_PARAMS.run = true;
    CUDA_SPH_EMITTER_PARAMS.emit_type = CudaSphEmitterType::SQUARE;
    CUDA_SPH_EMITTER_PARAMS.emit_radius = 0.03f;
    CUDA_SPH_EMITTER_PARAMS.emit_pos = make_float3(0.2f, 0.2f, 0.2f);
    CUDA_SPH_EMITTER_PARAMS.emit_vel = make_float3(0.f, -1.f, 0.f);
    CUDA_SPH_EMITTER_PARAMS.emit_col = make_float3(0.3f, 0.6f, 1.f);

    auto emitter = std::make_shared<CudaEmitter>(CUDA_SPH_EMITTER_PARAMS.emit_pos, CUDA_SPH_EMITTER_PARAMS.emit_vel,
                                                 true);
    BoundaryData boundary;
    CudaBoundaryEmitter().BuildWorldBoundary(boundary, lowest, highest, CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius);
    Vec_Float3 cda;
    Vec_Float2 amc;
    SeepageflowVolumeData vol = facade_test::buildVolume(cda, amc);
    auto particles = std::make_shared<CudaSFParticles>(vol.pos.size() + 32, vol.pos, vol.col, vol.label, vol.mass,
                                                       vol.radius, cda, amc);
    auto searcher = std::make_shared<CudaGNSearcher>(lowest, highest, particles->MaxSize(),
                                                     CUDA_BOUNDARY_PARAMS.kernel_radius, SEEPAGE_MULTI);
    auto boundaryParticles = std::make_shared<CudaBoundaryParticles>(boundary.pos, boundary.label);
    CudaSphSFSolverPtr solver;
    if (wcsph)
        solver = std::make_shared<CudaWCSphSFSolver>(particles->MaxSize());
    else
        solver = std::make_shared<CudaSphSFSolver>(particles->MaxSize());
    auto boundarySearcher = std::make_shared<CudaGNBoundarySearcher>(lowest, highest, boundaryParticles->MaxSize(),
                                                                     CUDA_BOUNDARY_PARAMS.kernel_radius);
    CudaSFParticlesPtr pp = particles;
    CudaBoundaryParticlesPtr bb = boundaryParticles;
    CudaGNSearcherPtr ss = searcher;
    CudaGNBoundarySearcherPtr bs = boundarySearcher;
    CudaEmitterPtr ee = emitter;
    CudaSFSystem system(pp, bb, solver, ss, bs, ee, true);
    if (!system.Handle()) return 3;

    const Vec_Float3 points = emitter->Emit();
    const int64_t n0 = int64_t(vol.pos.size()), npts = int64_t(points.size()), nc = calls;
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 4;
    std::fwrite(&n0, sizeof(int64_t), 1, f);
    std::fwrite(&npts, sizeof(int64_t), 1, f);
    std::fwrite(&nc, sizeof(int64_t), 1, f);
    std::fwrite(vol.pos.data(), sizeof(float3), vol.pos.size(), f);
    std::fwrite(points.data(), sizeof(float3), points.size(), f);
    std::vector<int64_t> counts, nsubs;
    const float renderInterval = 1.f / 30.f;
    for (int k = 0; k < calls; ++k) {
        if (!system.UpdateSystemChecked(renderInterval, nullptr)) return 5;
        counts.push_back(int64_t(particles->Size()));
        nsubs.push_back(int64_t(system.GetNumOfSubTimeSteps()));
    }
    std::fwrite(counts.data(), sizeof(int64_t), counts.size(), f);
    std::fwrite(nsubs.data(), sizeof(int64_t), nsubs.size(), f);
    const int64_t n = int64_t(particles->Size());
    std::fwrite(&n, sizeof(int64_t), 1, f);
    std::vector<float> out(3 * size_t(n));
    for (int field : {int(SF_FIELD_POS), int(SF_FIELD_VEL)}) {
        if (sf_get_field(system.Handle(), 0, field, SF_ORDER_ID, out.data(), n, 0) != SF_OK) return 6;
        std::fwrite(out.data(), sizeof(float), out.size(), f);
    }
    std::fclose(f);
    std::printf("inflow ok: %s calls=%d particles %lld -> %lld (capacity %zu) points=%lld emitter=%d\n",
                wcsph ? "wcsph" : "sph", calls, static_cast<long long>(n0), static_cast<long long>(n),
                particles->MaxSize(), static_cast<long long>(npts), int(emitter->GetEmitterStatus()));
    return 0;
}
