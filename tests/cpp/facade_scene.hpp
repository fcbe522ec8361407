// Scene set-up shared by the facade test programs (facade_main.cpp,
// inflow_main.cpp): the reference app's parameter block
// (seepage_flows/src/seepageflow/main.cpp:40-83) for a 0.4 m box with
// h = 0.04, written against the facade's global parameter structs.
#pragma once

#include "sf_kiri_facade.hpp"

namespace facade_test {

using namespace KIRI;

inline void setReferenceParams(CudaSphSolverType solver) {
    const float3 lowest = make_float3(0.f, 0.f, 0.f), highest = make_float3(0.4f, 0.4f, 0.4f);
    CUDA_SEEPAGEFLOW_PARAMS.sph_density = 1000.f;
    CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius = 0.01f;
    CUDA_SEEPAGEFLOW_PARAMS.sph_kernel_radius = 4.f * 0.01f;
    const float diam = 2.f * 0.01f;
    CUDA_SEEPAGEFLOW_PARAMS.sph_mass = 0.8f * diam * diam * diam * 1000.f;
    const float visc = 0.05f, c = 100.f;
    CUDA_SEEPAGEFLOW_PARAMS.sph_nu = (visc + visc) * CUDA_SEEPAGEFLOW_PARAMS.sph_kernel_radius * c;
    CUDA_SEEPAGEFLOW_PARAMS.sph_bnu = 0.2f * CUDA_SEEPAGEFLOW_PARAMS.sph_kernel_radius * c;
    CUDA_SEEPAGEFLOW_PARAMS.sph_stiff = 0.001f * c * c * 1000.f / 7.f;
    CUDA_SEEPAGEFLOW_PARAMS.sph_visc = visc;
    CUDA_SEEPAGEFLOW_PARAMS.dem_density = 2650.f;
    CUDA_SEEPAGEFLOW_PARAMS.dem_particle_radius = 0.01f;
    CUDA_SEEPAGEFLOW_PARAMS.dem_young = 1e5f;
    CUDA_SEEPAGEFLOW_PARAMS.dem_poisson = 0.3f;
    CUDA_SEEPAGEFLOW_PARAMS.dem_tan_friction_angle = 0.5f;
    CUDA_SEEPAGEFLOW_PARAMS.dem_damping = 0.4f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_c0 = 0.7f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_cd = 0.5f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_csat = 0.f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_cmc = 1.f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_cmc_p = 0.01f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_a0 = 0.f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_asat = 0.8f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_amc = 1.5f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_amc_p = 0.5f;
    CUDA_SEEPAGEFLOW_PARAMS.sf_dry_sand_color = make_float3(0.88f, 0.79552f, 0.5984f);
    CUDA_SEEPAGEFLOW_PARAMS.sf_wet_sand_color = make_float3(0.38f, 0.29f, 0.14f);
    CUDA_SEEPAGEFLOW_PARAMS.dt = 0.5f * 0.01f / std::sqrt(1e5f / 2650.f);
    CUDA_SEEPAGEFLOW_PARAMS.gravity = make_float3(0.f, -9.81f, 0.f);
    CUDA_SEEPAGEFLOW_PARAMS.sf_type = MULTI_SF;
    CUDA_SEEPAGEFLOW_PARAMS.solver_type = solver;
    CUDA_BOUNDARY_PARAMS.lowest_point = lowest;
    CUDA_BOUNDARY_PARAMS.highest_point = highest;
    CUDA_BOUNDARY_PARAMS.world_size = make_float3(0.4f, 0.4f, 0.4f);
    CUDA_BOUNDARY_PARAMS.world_center = make_float3(0.2f, 0.2f, 0.2f);
    CUDA_BOUNDARY_PARAMS.kernel_radius = CUDA_SEEPAGEFLOW_PARAMS.sph_kernel_radius;
    const float3 q = make_float3(0.4f / 0.04f, 0.4f / 0.04f, 0.4f / 0.04f);
    CUDA_BOUNDARY_PARAMS.grid_size = make_int3(int(q.x), int(q.y), int(q.z));
}

// The sand block and water column of the facade scenes (seeded jitter).
inline SeepageflowVolumeData buildVolume(Vec_Float3& cda, Vec_Float2& amc) {
    SeepageflowVolumeData vol;
    CudaVolumeEmitter ve;
    const float sandMass = 2650.f * ((4.f / 3.f) * kKiriPi * std::pow(0.01f, 3.f));
    ve.BuildSeepageflowBoxVolume(vol, make_float3(0.22f, 0.02f, 0.08f), make_int3(8, 6, 8), 0.01f,
                                 CUDA_SEEPAGEFLOW_PARAMS.sf_dry_sand_color, sandMass, 1, 0.0002f, 11u);
    ve.BuildSeepageflowBoxVolume(vol, make_float3(0.06f, 0.02f, 0.08f), make_int3(7, 10, 8), 0.01f,
                                 make_float3(0.5f, 0.8f, 1.f), CUDA_SEEPAGEFLOW_PARAMS.sph_mass, 0, 0.0002f, 12u);
    cda.assign(vol.pos.size(), make_float3(0.f, 0.f, 0.f));
    amc.assign(vol.pos.size(), make_float2(0.f, 0.f));
    for (size_t i = 0; i < vol.pos.size(); ++i)
        if (vol.label[i] == 1) {
            cda[i] = make_float3(0.5f, 0.f, 0.8f);
            amc[i] = make_float2(1.5f, 0.5f);
        }
    return vol;
}

}  // namespace facade_test
