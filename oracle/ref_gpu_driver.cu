// REFERENCE GPU DRIVER -- test and measurement infrastructure, not product code.
//
// Runs the reference's own CUDA library (seepage_flows_cuda, built for this
// GPU with its own -use_fast_math flags by oracle/build_ref_cuda.sh) through
// its public classes, the way the reference app does
// (seepage_flows/src/main.cpp:173-220 construction, :244/:257 UpdateSystem,
// the Get*Ptr getters): the global parameter structs are set, then
// CudaSFParticles, CudaBoundaryParticles, CudaGNSearcher,
// CudaGNBoundarySearcher, the WCSPH or SPH seepage solver, a CudaEmitter
// (disabled unless one is described) and CudaSFSystem are constructed, and
// every step is one CudaBaseSystem::UpdateSystem(renderInterval) call (one
// substep of renderInterval / N_sub, N_sub from the CFL of the previous
// substep).
//
// Particle ids: the per-particle radius array is carried through the sort
// (cuda_neighbor_searcher.cu:81,100) and read by no kernel of the solver
// (the DEM uses the uniform dem_particle_radius), so the driver stores each
// particle's creation index in it (exact in float below 2^24) and reads it
// back as the id; the reference's code is unchanged.
//
// Emitter: sfrg_create takes an optional emitter description (position,
// velocity, colour, type, radius, width, height); the driver then sets
// CUDA_SPH_EMITTER_PARAMS (enable, run) and hands the system an enabled
// CudaEmitter, whose samples the system constructor builds
// (cuda_sf_system.cu:46-70) and whose schedule OnUpdateSolver runs.
//
// C ABI for oracle/__init__.py (ctypes); results are copied to host doubles.
#include "sf_capi.h"

#include <kiri_pbs_cuda/data/cuda_boundary_params.h>
#include <kiri_pbs_cuda/data/cuda_seepageflow_params.h>
#include <kiri_pbs_cuda/data/cuda_sph_params.h>
#include <kiri_pbs_cuda/system/cuda_sf_system.cuh>

#include <cstring>
#include <memory>
#include <vector>

using namespace KIRI;

namespace {

struct RefGpu {
    CudaSFParticlesPtr particles;
    CudaBoundaryParticlesPtr boundary;
    CudaGNSearcherPtr searcher;
    CudaGNBoundarySearcherPtr bsearcher;
    CudaSFSystemPtr system;
    size_t nb = 0;
    size_t cells = 0;
    CudaSeepageflowParams P{};
    CudaBoundaryParams B{};
    CudaSphEmitterParams E{};
};

float3 f3(const float* v) { return make_float3(v[0], v[1], v[2]); }

template <typename T> bool copyDown(std::vector<T>& h, const T* d, size_t n) {
    h.resize(n);
    return n == 0 || cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost) == cudaSuccess;
}

}  // namespace

extern "C" {

// Cell keys of the last sort in the current (sorted) order: the searchers
// sort a copy of the particles' cell keys (mGridIdxArray,
// cuda_neighbor_searcher.cu:70-111; particle2cell keeps the order before the
// sort), whose first Size() entries are the sorted keys.
enum { kFieldKey = SF_FIELD_KEY, kBFieldKey = 35 };

// Creates the reference system for one scene; null on a CUDA error.
// emit: null, or 13 floats: position[3], velocity[3], colour[3], type
// (0 square, 1 circle, 2 rectangle), radius, width, height.
void* sfrg_create(const sf_params* p, const sf_boundary_params* b, const sf_solver_params* s,
                  const sf_scene_init* in, int64_t capacity, int sort_multi, const float* emit) {
    if (!p || !b || !s || !in || in->n <= 0 || capacity < in->n) return nullptr;
    cudaGetLastError();
    auto* r = new RefGpu();
    CudaSeepageflowParams& P = r->P;
    P.sph_mass = p->sph_mass;
    P.sph_density = p->sph_density;
    P.sph_particle_radius = p->sph_particle_radius;
    P.sph_kernel_radius = p->sph_kernel_radius;
    P.sph_stiff = p->sph_stiff;
    P.sph_visc = p->sph_visc;
    P.sph_nu = p->sph_nu;
    P.sph_bnu = p->sph_bnu;
    P.dem_mass = p->dem_mass;
    P.dem_density = p->dem_density;
    P.dem_particle_radius = p->dem_particle_radius;
    P.dem_kernel_radius = p->dem_kernel_radius;
    P.dem_young = p->dem_young;
    P.dem_poisson = p->dem_poisson;
    P.dem_tan_friction_angle = p->dem_tan_friction_angle;
    P.dem_damping = p->dem_damping;
    P.sf_c0 = p->sf_c0;
    P.sf_csat = p->sf_csat;
    P.sf_cmc = p->sf_cmc;
    P.sf_cmc_p = p->sf_cmc_p;
    P.sf_cd = p->sf_cd;
    P.sf_a0 = p->sf_a0;
    P.sf_asat = p->sf_asat;
    P.sf_amc = p->sf_amc;
    P.sf_amc_p = p->sf_amc_p;
    P.sf_dry_sand_color = f3(p->sf_dry_sand_color);
    P.sf_wet_sand_color = f3(p->sf_wet_sand_color);
    P.gravity = f3(p->gravity);
    P.dt = p->dt;
    P.solver_type = p->solver_type == SF_SOLVER_WCSPH ? WCSPH_SOLVER : SPH_SOLVER;
    P.sf_type = p->sf_type == SF_TYPE_MULTI_SF ? MULTI_SF : SF;
    CudaBoundaryParams& B = r->B;
    B.kernel_radius = b->kernel_radius;
    B.lowest_point = f3(b->lowest_point);
    B.highest_point = f3(b->highest_point);
    B.world_size = B.highest_point - B.lowest_point;
    B.world_center = (B.highest_point + B.lowest_point) / 2.f;
    B.grid_size = make_int3(b->grid_size[0], b->grid_size[1], b->grid_size[2]);
    // the reference reads its globals at construction and at every UpdateSystem
    CUDA_SEEPAGEFLOW_PARAMS = P;
    CUDA_BOUNDARY_PARAMS = B;
    CUDA_SPH_EMITTER_PARAMS.enable = emit != nullptr;
    CUDA_SPH_EMITTER_PARAMS.run = emit != nullptr;
    if (emit) {
        CUDA_SPH_EMITTER_PARAMS.emit_pos = f3(emit);
        CUDA_SPH_EMITTER_PARAMS.emit_vel = f3(emit + 3);
        CUDA_SPH_EMITTER_PARAMS.emit_col = f3(emit + 6);
        CUDA_SPH_EMITTER_PARAMS.emit_type =
            emit[9] == 1.f ? CudaSphEmitterType::CIRCLE
                           : (emit[9] == 2.f ? CudaSphEmitterType::RECTANGLE : CudaSphEmitterType::SQUARE);
        CUDA_SPH_EMITTER_PARAMS.emit_radius = emit[10];
        CUDA_SPH_EMITTER_PARAMS.emit_width = emit[11];
        CUDA_SPH_EMITTER_PARAMS.emit_height = emit[12];
    }
    r->E = CUDA_SPH_EMITTER_PARAMS;

    const size_t n = size_t(in->n);
    Vec_Float3 pos(n), col(n), cda(n);
    Vec_SizeT label(n);
    Vec_Float mass(n), ids(n);
    Vec_Float2 amc(n);
    for (size_t i = 0; i < n; ++i) {
        pos[i] = f3(in->pos + 3 * i);
        col[i] = f3(in->col + 3 * i);
        label[i] = size_t(in->label[i]);
        mass[i] = in->mass[i];
        ids[i] = float(i);
        cda[i] = in->cda0asat ? f3(in->cda0asat + 3 * i) : make_float3(0.f);
        amc[i] = in->amcamcp ? make_float2(in->amcamcp[2 * i], in->amcamcp[2 * i + 1]) : make_float2(0.f, 0.f);
    }
    r->nb = size_t(in->nb);
    Vec_Float3 bpos(r->nb);
    Vec_SizeT blabel(r->nb);
    for (size_t i = 0; i < r->nb; ++i) {
        bpos[i] = f3(in->bpos + 3 * i);
        blabel[i] = in->blabel ? size_t(in->blabel[i]) : 0;
    }
    r->particles = std::make_shared<CudaSFParticles>(size_t(capacity), pos, col, label, mass, ids, cda, amc);
    if (in->vel)
        cudaMemcpy(r->particles->GetVelPtr(), in->vel, sizeof(float3) * n, cudaMemcpyHostToDevice);
    r->boundary = std::make_shared<CudaBoundaryParticles>(bpos, blabel);
    r->searcher = std::make_shared<CudaGNSearcher>(B.lowest_point, B.highest_point, size_t(capacity), B.kernel_radius,
                                                   sort_multi ? SEEPAGE_MULTI : SEEPAGE);
    r->bsearcher = std::make_shared<CudaGNBoundarySearcher>(B.lowest_point, B.highest_point, r->nb, B.kernel_radius);
    CudaSphSFSolverPtr solver;
    if (P.solver_type == WCSPH_SOLVER)
        solver = std::make_shared<CudaWCSphSFSolver>(size_t(capacity), s->negative_scale, s->time_step_limit_scale,
                                                     s->speed_of_sound);
    else
        solver = std::make_shared<CudaSphSFSolver>(size_t(capacity));
    CudaEmitterPtr emitter = emit ? std::make_shared<CudaEmitter>(f3(emit), f3(emit + 3), true)
                                  : std::make_shared<CudaEmitter>();
    // the system constructor moves from its arguments: hand it copies
    CudaSFParticlesPtr pArg = r->particles;
    CudaBoundaryParticlesPtr bArg = r->boundary;
    CudaGNSearcherPtr sArg = r->searcher;
    CudaGNBoundarySearcherPtr bsArg = r->bsearcher;
    r->system = std::make_shared<CudaSFSystem>(pArg, bArg, solver, sArg, bsArg, emitter, true);
    const int3 g = r->searcher->GetGridSize();
    r->cells = size_t(g.x) * size_t(g.y) * size_t(g.z);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        delete r;
        return nullptr;
    }
    return r;
}

void sfrg_destroy(void* h) { delete static_cast<RefGpu*>(h); }

// One UpdateSystem(render_interval) call; returns its own event-timed ms.
float sfrg_update(void* h, float render_interval) {
    auto* r = static_cast<RefGpu*>(h);
    CUDA_SEEPAGEFLOW_PARAMS = r->P;
    CUDA_BOUNDARY_PARAMS = r->B;
    CUDA_SPH_EMITTER_PARAMS = r->E;
    return r->system->UpdateSystem(render_interval);
}

// `calls` UpdateSystem calls; returns the wall milliseconds of all of them
// (each call ends with a device synchronisation in the reference).
double sfrg_run(void* h, float render_interval, int64_t calls) {
    auto* r = static_cast<RefGpu*>(h);
    CUDA_SEEPAGEFLOW_PARAMS = r->P;
    CUDA_BOUNDARY_PARAMS = r->B;
    CUDA_SPH_EMITTER_PARAMS = r->E;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaDeviceSynchronize();
    cudaEventRecord(a, 0);
    for (int64_t k = 0; k < calls; ++k) r->system->UpdateSystem(render_interval);
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return double(ms);
}

int sfrg_cuda_error(void) { return int(cudaGetLastError()); }

int64_t sfrg_num_substeps(void* h) { return int64_t(static_cast<RefGpu*>(h)->system->GetNumOfSubTimeSteps()); }

int64_t sfrg_size(void* h) { return int64_t(static_cast<RefGpu*>(h)->particles->Size()); }

// Field `field` (SF_FIELD_* / SF_BFIELD_*, or kBFieldKey) in the reference's
// current order as doubles (n x width); SF_FIELD_ID is the creation index
// (emitted particles carry their radius there instead), SF_FIELD_KEY the
// cell key of the last sort.
int sfrg_get_field(void* h, int field, double* out, int64_t count) {
    auto* r = static_cast<RefGpu*>(h);
    const CudaSFParticlesPtr& P = r->particles;
    const size_t n = P->Size();
    auto put3 = [&](const float3* d, size_t m) {
        std::vector<float3> v;
        if (!copyDown(v, d, m)) return 2;
        for (size_t i = 0; i < m; ++i) {
            out[3 * i] = v[i].x;
            out[3 * i + 1] = v[i].y;
            out[3 * i + 2] = v[i].z;
        }
        return 0;
    };
    auto put1 = [&](const float* d, size_t m) {
        std::vector<float> v;
        if (!copyDown(v, d, m)) return 2;
        for (size_t i = 0; i < m; ++i) out[i] = v[i];
        return 0;
    };
    auto putS = [&](const size_t* d, size_t m) {
        std::vector<size_t> v;
        if (!copyDown(v, d, m)) return 2;
        for (size_t i = 0; i < m; ++i) out[i] = double(v[i]);
        return 0;
    };
    const bool bfield = field >= SF_BFIELD_POS;
    if (count != int64_t(bfield ? r->nb : n)) return 1;
    switch (field) {
    case SF_FIELD_POS: return put3(P->GetPosPtr(), n);
    case SF_FIELD_VEL: return put3(P->GetVelPtr(), n);
    case SF_FIELD_ACC: return put3(P->GetAccPtr(), n);
    case SF_FIELD_COL: return put3(P->GetColPtr(), n);
    case SF_FIELD_LABEL: return putS(P->GetLabelPtr(), n);
    case SF_FIELD_ID: return put1(P->GetRadiusPtr(), n);
    case SF_FIELD_MASS: return put1(P->GetMassPtr(), n);
    case SF_FIELD_DENSITY: return put1(P->GetDensityPtr(), n);
    case SF_FIELD_PRESSURE: return put1(P->GetPressurePtr(), n);
    case SF_FIELD_VOIDAGE: return put1(P->GetVoidagePtr(), n);
    case SF_FIELD_SATURATION: return put1(P->GetSaturationPtr(), n);
    case SF_FIELD_MAX_SATURATION: return put1(P->GetMaxSaturationPtr(), n);
    case SF_FIELD_AVG_FLOW: return put3(P->GetAvgFlowVelPtr(), n);
    case SF_FIELD_AVG_DRAG: return put3(P->GetAvgDragForcePtr(), n);
    case SF_FIELD_ADHESION: return put3(P->GetAdhesionForcePtr(), n);
    case SF_FIELD_AVG_ADHESION: return put3(P->GetAvgAdhesionForcePtr(), n);
    case SF_FIELD_CDA0ASAT: return put3(P->GetCdA0AsatPtr(), n);
    case kFieldKey: return putS(r->searcher->GetGridIdxArrayPtr(), n);
    case kBFieldKey: return putS(r->bsearcher->GetGridIdxArrayPtr(), r->nb);
    case SF_BFIELD_POS: return put3(r->boundary->GetPosPtr(), r->nb);
    case SF_BFIELD_LABEL: return putS(r->boundary->GetLabelPtr(), r->nb);
    case SF_BFIELD_VOLUME: return put1(r->boundary->GetVolumePtr(), r->nb);
    default: return 1;
    }
}

// Cell-start table of the particles (which = 0) or of the boundary (1): G + 1 entries.
int sfrg_get_cell_table(void* h, int which, int64_t* out, int64_t count) {
    auto* r = static_cast<RefGpu*>(h);
    if (count != int64_t(r->cells) + 1) return 1;
    std::vector<size_t> v;
    if (!copyDown(v, which ? r->bsearcher->GetCellStartPtr() : r->searcher->GetCellStartPtr(), r->cells + 1))
        return 2;
    for (size_t i = 0; i <= r->cells; ++i) out[i] = int64_t(v[i]);
    return 0;
}

}  // extern "C"
