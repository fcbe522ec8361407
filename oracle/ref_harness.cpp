// REFERENCE HARNESS -- test infrastructure, not product code.
//
// Runs the reference's own seepage-flow kernels on the CPU. The reference
// headers are compiled in place (oracle/build_ref.sh points the include path
// at the sph_seepage_flows sources; nothing is copied) with the forced-include
// prelude oracle/ref_shim/host_prelude.h, which turns each __global__ kernel
// into a host function and supplies blockIdx/threadIdx. Each "launch" below
// calls the kernel body once per thread index, exactly as the reference's
// <<<grid, 256>>> launches do (grid over the particle count).
//
// The Thrust glue of the reference (sort_by_key, fill, exclusive_scan,
// transform, max_element) and the AccDampingForSand functor (which does not
// compile against current CCCL tuples) are restated here with the cited
// reference lines. The physics arithmetic is the reference's own code.
//
// Output goes to oracle/_ref/libsfref.so; tests use it to pin the oracle and
// tests/golden/make_golden.py uses it to write the committed fixtures.

#include "../include/sf_capi.h"

#include <kiri_pbs_cuda/kernel/cuda_sph_kernel.cuh>
#include <kiri_pbs_cuda/solver/seepageflow/cuda_sph_sf_solver_gpu.cuh>
#include <kiri_pbs_cuda/solver/seepageflow/cuda_wcsph_sf_solver_gpu.cuh>
#include <kiri_pbs_cuda/system/cuda_sph_system_gpu.cuh>
#include <kiri_pbs_cuda/thrust_helper/helper_thrust.cuh>
#include <kiri_pbs_cuda/emitter/cuda_boundary_emitter.cuh>
#include <kiri_pbs_cuda/emitter/cuda_emitter.cuh>
#include <kiri_pbs_cuda/emitter/cuda_volume_emitter.cuh>
#include <kiri_pbs_cuda/data/cuda_seepageflow_params.h>
#include <kiri_pbs_cuda/data/cuda_boundary_params.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

thread_local sfref_dim3 sfref_blockIdx, sfref_blockDim, sfref_threadIdx;

namespace {

using namespace KIRI;

constexpr unsigned kBlock = KIRI_CUBLOCKSIZE;

// Emulates kernel<<<ceil(num/256), 256>>>: one body call per thread.
template <typename F> void launch(size_t num, F&& body) {
    const long blocks = long((num + kBlock - 1) / kBlock);
#pragma omp parallel for schedule(dynamic, 4)
    for (long b = 0; b < blocks; ++b) {
        sfref_blockDim = sfref_dim3{kBlock, 1, 1};
        sfref_blockIdx = sfref_dim3{unsigned(b), 0, 0};
        for (unsigned t = 0; t < kBlock; ++t) {
            sfref_threadIdx = sfref_dim3{t, 0, 0};
            body();
        }
    }
}

struct Ref {
    CudaSeepageflowParams P{};
    CudaBoundaryParams B{};
    sf_solver_params S{};
    size_t n = 0, nb = 0;
    int3 gsize;
    size_t G;
    std::vector<size_t> label, id, key;
    std::vector<float3> pos, vel, acc, col, avgFlow, avgDrag, adh, avgAdh, cda0asat;
    std::vector<float2> amcamcp;
    std::vector<float> radius, mass, density, pressure, voidage, saturation, maxSat;
    std::vector<float3> bpos;
    std::vector<size_t> blabel;
    std::vector<float> bvolume;
    std::vector<size_t> cellStart, bcellStart;
    size_t numSub = 1;

    ThrustHelper::Pos2GridXYZ<float3> p2xyz() const {
        return ThrustHelper::Pos2GridXYZ<float3>(B.lowest_point, B.kernel_radius, B.grid_size);
    }
    ThrustHelper::GridXYZ2GridHash xyz2hash() const { return ThrustHelper::GridXYZ2GridHash(B.grid_size); }

    // Stable sort permutation by integer key + count/exclusive-scan cell table
    // (cuda_neighbor_searcher.cu:36-51,64-116; CountingInCell_CUDA in
    // searcher/cuda_neighbor_searcher_gpu.cuh:18-25).
    std::vector<size_t> sortAndCount(std::vector<size_t>& keys, std::vector<size_t>& start) {
        std::vector<size_t> order(keys.size());
        std::iota(order.begin(), order.end(), size_t(0));
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return keys[a] < keys[b]; });
        start.assign(G + 1, 0);
        for (size_t k : keys) start[k]++;
        size_t run = 0;
        for (size_t c = 0; c <= G; ++c) {
            size_t v = start[c];
            start[c] = run;
            run += v;
        }
        return order;
    }
    template <typename V> static void permute(std::vector<V>& a, const std::vector<size_t>& order) {
        std::vector<V> t(a.size());
        for (size_t i = 0; i < order.size(); ++i) t[i] = a[order[i]];
        a.swap(t);
    }

    void init(const sf_params* p, const sf_boundary_params* b, const sf_solver_params* s, const sf_scene_init* in) {
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
        P.sf_dry_sand_color = make_float3(p->sf_dry_sand_color[0], p->sf_dry_sand_color[1], p->sf_dry_sand_color[2]);
        P.sf_wet_sand_color = make_float3(p->sf_wet_sand_color[0], p->sf_wet_sand_color[1], p->sf_wet_sand_color[2]);
        P.gravity = make_float3(p->gravity[0], p->gravity[1], p->gravity[2]);
        P.dt = p->dt;
        P.solver_type = p->solver_type == SF_SOLVER_WCSPH ? WCSPH_SOLVER : SPH_SOLVER;
        P.sf_type = p->sf_type == SF_TYPE_MULTI_SF ? MULTI_SF : SF;
        B.kernel_radius = b->kernel_radius;
        B.lowest_point = make_float3(b->lowest_point[0], b->lowest_point[1], b->lowest_point[2]);
        B.highest_point = make_float3(b->highest_point[0], b->highest_point[1], b->highest_point[2]);
        B.grid_size = make_int3(b->grid_size[0], b->grid_size[1], b->grid_size[2]);
        S = *s;
        gsize = B.grid_size;
        G = size_t(gsize.x) * gsize.y * gsize.z;
        n = size_t(in->n);
        nb = size_t(in->nb);
        label.resize(n);
        id.resize(n);
        key.assign(n, 0);
        pos.resize(n);
        vel.assign(n, make_float3(0.f));
        col.resize(n);
        cda0asat.assign(n, make_float3(0.f));
        amcamcp.assign(n, make_float2(0.f, 0.f));
        radius.resize(n);
        mass.resize(n);
        for (size_t i = 0; i < n; ++i) {
            label[i] = size_t(in->label[i]);
            id[i] = i;
            pos[i] = make_float3(in->pos[3 * i], in->pos[3 * i + 1], in->pos[3 * i + 2]);
            if (in->vel) vel[i] = make_float3(in->vel[3 * i], in->vel[3 * i + 1], in->vel[3 * i + 2]);
            col[i] = make_float3(in->col[3 * i], in->col[3 * i + 1], in->col[3 * i + 2]);
            if (in->cda0asat)
                cda0asat[i] = make_float3(in->cda0asat[3 * i], in->cda0asat[3 * i + 1], in->cda0asat[3 * i + 2]);
            if (in->amcamcp) amcamcp[i] = make_float2(in->amcamcp[2 * i], in->amcamcp[2 * i + 1]);
            radius[i] = in->radius[i];
            mass[i] = in->mass[i];
        }
        acc.assign(n, make_float3(0.f));
        avgFlow = avgDrag = adh = avgAdh = acc;
        density.assign(n, 0.f);
        pressure = voidage = saturation = maxSat = density;
        bpos.resize(nb);
        blabel.resize(nb);
        for (size_t i = 0; i < nb; ++i) {
            bpos[i] = make_float3(in->bpos[3 * i], in->bpos[3 * i + 1], in->bpos[3 * i + 2]);
            blabel[i] = in->blabel ? size_t(in->blabel[i]) : 0;
        }
        // boundary searcher (cuda_base_system.cu:26) + boundary volume (cuda_sf_system.cu:121-136)
        std::vector<size_t> bk(nb);
        ThrustHelper::Pos2GridHash<float3> hsh(B.lowest_point, B.kernel_radius, B.grid_size);
        for (size_t i = 0; i < nb; ++i) bk[i] = hsh(bpos[i]);
        std::vector<size_t> order = sortAndCount(bk, bcellStart);
        permute(bpos, order);
        permute(blabel, order);
        bvolume.assign(nb, 0.f);
        launch(nb, [&] {
            ComputeBoundaryVolume_CUDA(bpos.data(), bvolume.data(), nb, bcellStart.data(), gsize, p2xyz(),
                                       xyz2hash(), Poly6Kernel(B.kernel_radius));
        });
    }

    // BuildGNSearcher + SortData(SEEPAGE_MULTI) (cuda_neighbor_searcher.cu:36-51, 85-112)
    void sortStage() {
        ThrustHelper::Pos2GridHash<float3> hsh(B.lowest_point, B.kernel_radius, B.grid_size);
        for (size_t i = 0; i < n; ++i) key[i] = hsh(pos[i]);
        std::vector<size_t> order = sortAndCount(key, cellStart);
        permute(label, order);
        permute(pos, order);
        permute(vel, order);
        permute(col, order);
        permute(radius, order);
        permute(mass, order);
        permute(maxSat, order);
        permute(cda0asat, order);
        permute(amcamcp, order);
        permute(id, order);
        permute(key, order);
    }

    void substep(float timeArg, bool adaptive) {
        sortStage();
        // ExtraForces (cuda_sph_sf_solver.cu:390-402)
        for (size_t i = 0; i < n; ++i) acc[i] = make_float3(0.f) + P.gravity;
        const float h = B.kernel_radius;
        launch(n, [&] {
            ComputeSFDensity_CUDA(label.data(), pos.data(), mass.data(), density.data(), P.sph_density,
                                  P.dem_density, n, cellStart.data(), bpos.data(), bvolume.data(),
                                  bcellStart.data(), gsize, p2xyz(), xyz2hash(), Poly6Kernel(h));
        });
        if (P.solver_type == WCSPH_SOLVER) {
            launch(n, [&] {
                ComputeSFPressureByTait_CUDA(label.data(), density.data(), pressure.data(), n, P.sph_density,
                                             P.sph_stiff, S.negative_scale);
            });
        } else {
            launch(n, [&] {
                ComputeSFPressure_CUDA(label.data(), density.data(), pressure.data(), n, P.sph_density, P.sph_stiff,
                                       1.f);
            });
        }
        launch(n, [&] {
            ComputeSFAvgFlow_CUDA(label.data(), pos.data(), vel.data(), mass.data(), density.data(), avgFlow.data(),
                                  voidage.data(), saturation.data(), n, cellStart.data(), gsize, p2xyz(),
                                  xyz2hash(), Poly6Kernel(h));
        });
        launch(n, [&] {
            ComputeSFSandVoidage_CUDA(label.data(), pos.data(), mass.data(), density.data(), voidage.data(), n,
                                      cellStart.data(), gsize, p2xyz(), xyz2hash(), Poly6Kernel(h));
        });
        const float grav = std::fabs(P.gravity.y);
        if (P.sf_type == SF) {
            launch(n, [&] {
                ComputeSFWaterAdhesionForces_CUDA(
                    label.data(), pos.data(), mass.data(), density.data(), saturation.data(), adh.data(),
                    avgAdh.data(), n, cellStart.data(), gsize, p2xyz(), xyz2hash(),
                    QuadraticBezierCoeff(P.sf_a0, P.sf_amc, P.sf_amc_p, P.sf_asat), Poly6Kernel(h),
                    AdhesionAkinci13(h));
            });
            launch(n, [&] {
                ComputeSFSandLinearMomentum_CUDA(
                    label.data(), pos.data(), vel.data(), acc.data(), mass.data(), density.data(), pressure.data(),
                    voidage.data(), saturation.data(), avgFlow.data(), avgDrag.data(), avgAdh.data(),
                    P.dem_particle_radius, P.sph_particle_radius, P.dem_young, P.dem_poisson,
                    P.dem_tan_friction_angle, P.sf_cd, grav, P.sph_density, n, B.lowest_point, B.highest_point,
                    cellStart.data(), bpos.data(), blabel.data(), bcellStart.data(), gsize, p2xyz(), xyz2hash(),
                    QuadraticBezierCoeff(P.sf_c0, P.sf_cmc, P.sf_cmc_p, P.sf_csat), Poly6Kernel(h),
                    SpikyKernelGrad(h));
            });
        } else {
            launch(n, [&] {
                ComputeMultiSFWaterAdhesionForces_CUDA(label.data(), pos.data(), mass.data(), density.data(),
                                                       saturation.data(), adh.data(), avgAdh.data(),
                                                       cda0asat.data(), amcamcp.data(), n, cellStart.data(), gsize,
                                                       p2xyz(), xyz2hash(), Poly6Kernel(h), AdhesionAkinci13(h));
            });
            launch(n, [&] {
                ComputeMultiSFSandLinearMomentum_CUDA(
                    label.data(), pos.data(), vel.data(), acc.data(), mass.data(), density.data(), pressure.data(),
                    voidage.data(), saturation.data(), avgFlow.data(), avgDrag.data(), avgAdh.data(),
                    P.dem_particle_radius, P.sph_particle_radius, P.dem_young, P.dem_poisson,
                    P.dem_tan_friction_angle, cda0asat.data(), grav, P.sph_density, n, B.lowest_point,
                    B.highest_point, cellStart.data(), bpos.data(), blabel.data(), bcellStart.data(), gsize, p2xyz(),
                    xyz2hash(), QuadraticBezierCoeff(P.sf_c0, P.sf_cmc, P.sf_cmc_p, P.sf_csat), Poly6Kernel(h),
                    SpikyKernelGrad(h));
            });
        }
        launch(n, [&] {
            ComputeSFWaterLinearMomentum_CUDA(label.data(), pos.data(), vel.data(), acc.data(), mass.data(),
                                              density.data(), pressure.data(), voidage.data(), avgDrag.data(),
                                              adh.data(), P.sph_density, P.sph_nu, P.sph_bnu, n, cellStart.data(),
                                              bpos.data(), bvolume.data(), bcellStart.data(), gsize, p2xyz(),
                                              xyz2hash(), Poly6Kernel(h), SpikyKernelGrad(h));
        });
        launch(n, [&] {
            ComputeSFWetSandColor_CUDA(label.data(), saturation.data(), maxSat.data(), col.data(), n,
                                       P.sf_dry_sand_color, P.sf_wet_sand_color);
        });
        float dt = timeArg;
        if (adaptive) {
            if (P.solver_type == WCSPH_SOLVER) {
                // ComputeSubTimeStepsByCFL (cuda_wcsph_sf_solver.cu:35-58)
                size_t best = 0;
                for (size_t i = 1; i < n; ++i)
                    if (length(acc[best]) < length(acc[i])) best = i;
                float3 maxAcc = acc[best];
                float maxForceMagnitude = length(maxAcc) * P.sph_mass;
                float bySpeed = 0.4f * h / S.speed_of_sound;
                float byForce = 0.25f * std::sqrt(h * P.sph_mass / maxForceMagnitude);
                float desired = std::min(S.time_step_limit_scale * std::min(bySpeed, byForce), P.dt);
                numSub = static_cast<size_t>(timeArg / desired);
            } else {
                numSub = static_cast<size_t>(timeArg / P.dt);  // cuda_sph_sf_solver.cpp:23
            }
            // WCSPH advects by renderInterval / N_sub (cuda_wcsph_sf_solver.cpp:168-172),
            // plain SPH by params.dt (cuda_sph_sf_solver.cpp:141-146)
            dt = P.solver_type == WCSPH_SOLVER ? timeArg / static_cast<float>(numSub) : P.dt;
        }
        // CudaSFParticles::Advect (cuda_sf_particles.cu:18-48) with AccDampingForSand
        // (cuda_sf_particles.cuh:19-40)
        for (size_t i = 0; i < n; ++i)
            if (label[i] == 1) {
                float3 a = acc[i];
                acc[i] = a * (make_float3(1.f) - P.dem_damping * sgn(a * (vel[i] + 0.5f * dt * a)));
            }
        for (size_t i = 0; i < n; ++i) vel[i] = vel[i] + dt * acc[i];
        for (size_t i = 0; i < n; ++i) pos[i] = pos[i] + dt * vel[i];
        launch(n, [&] {
            SFWaterBoundaryConstrain_CUDA(label.data(), pos.data(), vel.data(), n, B.lowest_point, B.highest_point,
                                          P.sph_particle_radius, bpos.data(), blabel.data(), bcellStart.data(),
                                          gsize, p2xyz(), xyz2hash());
        });
        for (size_t i = 0; i < n; ++i) {
            adh[i] = make_float3(0.f);
            avgAdh[i] = make_float3(0.f);
        }
    }
};

void put3(const std::vector<float3>& a, double* d) {
    for (size_t i = 0; i < a.size(); ++i) {
        d[3 * i] = a[i].x;
        d[3 * i + 1] = a[i].y;
        d[3 * i + 2] = a[i].z;
    }
}
template <typename V> void put1(const std::vector<V>& a, double* d) {
    for (size_t i = 0; i < a.size(); ++i) d[i] = double(a[i]);
}

}  // namespace

extern "C" {

void* sfref_create(const sf_params* p, const sf_boundary_params* b, const sf_solver_params* s,
                   const sf_scene_init* in) {
    auto* r = new Ref();
    r->init(p, b, s, in);
    return r;
}

void sfref_destroy(void* h) { delete static_cast<Ref*>(h); }

int sfref_substeps(void* h, double time_arg, int adaptive, int64_t n) {
    auto* r = static_cast<Ref*>(h);
    for (int64_t k = 0; k < n; ++k) r->substep(float(time_arg), adaptive != 0);
    return SF_OK;
}

int64_t sfref_num_substeps(void* h) { return int64_t(static_cast<Ref*>(h)->numSub); }

int sfref_get_field(void* h, int field, double* d, int64_t count) {
    auto* r = static_cast<Ref*>(h);
    const size_t n = field >= SF_BFIELD_POS ? r->nb : r->n;
    if (size_t(count) != n) return SF_ERR_INVALID;
    switch (field) {
    case SF_FIELD_POS: put3(r->pos, d); break;
    case SF_FIELD_VEL: put3(r->vel, d); break;
    case SF_FIELD_ACC: put3(r->acc, d); break;
    case SF_FIELD_COL: put3(r->col, d); break;
    case SF_FIELD_LABEL: put1(r->label, d); break;
    case SF_FIELD_RADIUS: put1(r->radius, d); break;
    case SF_FIELD_MASS: put1(r->mass, d); break;
    case SF_FIELD_DENSITY: put1(r->density, d); break;
    case SF_FIELD_PRESSURE: put1(r->pressure, d); break;
    case SF_FIELD_VOIDAGE: put1(r->voidage, d); break;
    case SF_FIELD_SATURATION: put1(r->saturation, d); break;
    case SF_FIELD_MAX_SATURATION: put1(r->maxSat, d); break;
    case SF_FIELD_AVG_FLOW: put3(r->avgFlow, d); break;
    case SF_FIELD_AVG_DRAG: put3(r->avgDrag, d); break;
    case SF_FIELD_ADHESION: put3(r->adh, d); break;
    case SF_FIELD_AVG_ADHESION: put3(r->avgAdh, d); break;
    case SF_FIELD_CDA0ASAT: put3(r->cda0asat, d); break;
    case SF_FIELD_AMCAMCP:
        for (size_t i = 0; i < n; ++i) {
            d[2 * i] = r->amcamcp[i].x;
            d[2 * i + 1] = r->amcamcp[i].y;
        }
        break;
    case SF_FIELD_ID: put1(r->id, d); break;
    case SF_FIELD_KEY: put1(r->key, d); break;
    case SF_BFIELD_POS: put3(r->bpos, d); break;
    case SF_BFIELD_LABEL: put1(r->blabel, d); break;
    case SF_BFIELD_VOLUME: put1(r->bvolume, d); break;
    default: return SF_ERR_INVALID;
    }
    return SF_OK;
}

int sfref_get_cell_table(void* h, int which, int64_t* d, int64_t count) {
    auto* r = static_cast<Ref*>(h);
    const std::vector<size_t>& t = which ? r->bcellStart : r->cellStart;
    if (size_t(count) != t.size()) return SF_ERR_INVALID;
    for (size_t i = 0; i < t.size(); ++i) d[i] = int64_t(t[i]);
    return SF_OK;
}

// CudaBoundaryEmitter::BuildWorldBoundary (cuda_boundary_emitter.cpp:12-80),
// the reference's own code. Returns the particle count; writes at most cap.
int64_t sfref_world_boundary(const float lp[3], const float hp[3], float particle_radius, float* out_pos,
                             int32_t* out_label, int64_t cap) {
    BoundaryData data;
    CudaBoundaryEmitter em;
    em.BuildWorldBoundary(data, make_float3(lp[0], lp[1], lp[2]), make_float3(hp[0], hp[1], hp[2]),
                          particle_radius);
    const int64_t cnt = int64_t(data.pos.size());
    for (int64_t i = 0; i < std::min(cnt, cap); ++i) {
        out_pos[3 * i] = data.pos[i].x;
        out_pos[3 * i + 1] = data.pos[i].y;
        out_pos[3 * i + 2] = data.pos[i].z;
        out_label[i] = int32_t(data.label[i]);
    }
    return cnt;
}

// CudaEmitter (cuda_emitter.cpp:12-95): builds the emitter of the given type
// (0 square, 1 circle, 2 rectangle) and returns the Emit() points.
int64_t sfref_emitter_points(const float pos[3], const float vel[3], int type, float particle_radius, float r_or_w,
                             float h, float* out, int64_t cap) {
    CudaEmitter em(make_float3(pos[0], pos[1], pos[2]), make_float3(vel[0], vel[1], vel[2]), true);
    if (type == 0) em.BuildSquareEmitter(particle_radius, r_or_w);
    else if (type == 1) em.BuildCircleEmitter(particle_radius, r_or_w);
    else em.BuildRectangleEmitter(particle_radius, r_or_w, h);
    if (em.GetNumOfEmitterPoints() == 0) return 0;
    Vec_Float3 pts = em.Emit();
    const int64_t cnt = int64_t(pts.size());
    for (int64_t i = 0; i < std::min(cnt, cap); ++i) {
        out[3 * i] = pts[i].x;
        out[3 * i + 1] = pts[i].y;
        out[3 * i + 2] = pts[i].z;
    }
    return cnt;
}

// CudaVolumeEmitter::BuildSeepageflowShapeMultiVolume (cuda_volume_emitter.cpp:
// 137-175), the reference's own code, on n shape points (x, y, z, radius),
// called twice when `twice` (two objects gathered into one volume, as the
// app's loop over shape files does). Writes per particle pos, col, cda0asat
// (3 floats), radius, mass (1), amcamcp (2), label; returns the count (at most
// cap written) and the data's sandMinRadius.
int64_t sfref_shape_multi_volume(const float* shape, int64_t n, const float color[3], float density,
                                 const float cda0asat[3], const float amcamcp[2], int offset_y, float lowest_y,
                                 int twice, float* out_pos, float* out_col, float* out_cda, float* out_radius,
                                 float* out_mass, float* out_amc, int32_t* out_label, int64_t cap,
                                 float* sand_min_radius) {
    Vec_Float4 sh;
    for (int64_t i = 0; i < n; ++i) sh.push_back(make_float4(shape[4 * i], shape[4 * i + 1], shape[4 * i + 2], shape[4 * i + 3]));
    SeepageflowMultiVolumeData data;
    CudaVolumeEmitter em;
    for (int k = 0; k < (twice ? 2 : 1); ++k)
        em.BuildSeepageflowShapeMultiVolume(data, sh, make_float3(color[0], color[1], color[2]), density,
                                            make_float3(cda0asat[0], cda0asat[1], cda0asat[2]),
                                            make_float2(amcamcp[0], amcamcp[1]), offset_y != 0, lowest_y);
    const int64_t cnt = int64_t(data.pos.size());
    for (int64_t i = 0; i < std::min(cnt, cap); ++i) {
        const float3 v3[3] = {data.pos[i], data.col[i], data.cda0asat[i]};
        float* o3[3] = {out_pos, out_col, out_cda};
        for (int a = 0; a < 3; ++a) {
            o3[a][3 * i] = v3[a].x;
            o3[a][3 * i + 1] = v3[a].y;
            o3[a][3 * i + 2] = v3[a].z;
        }
        out_radius[i] = data.radius[i];
        out_mass[i] = data.mass[i];
        out_amc[2 * i] = data.amcamcp[i].x;
        out_amc[2 * i + 1] = data.amcamcp[i].y;
        out_label[i] = int32_t(data.label[i]);
    }
    *sand_min_radius = data.sandMinRadius;
    return cnt;
}

// CudaBoundaryEmitter::BuildBoundaryShapeVolume (cuda_boundary_emitter.cpp:82-92).
int64_t sfref_boundary_shape_volume(const float* shape, int64_t n, float* out_pos, int32_t* out_label, int64_t cap) {
    Vec_Float4 sh;
    for (int64_t i = 0; i < n; ++i) sh.push_back(make_float4(shape[4 * i], shape[4 * i + 1], shape[4 * i + 2], shape[4 * i + 3]));
    BoundaryData data;
    CudaBoundaryEmitter em;
    em.BuildBoundaryShapeVolume(data, sh);
    const int64_t cnt = int64_t(data.pos.size());
    for (int64_t i = 0; i < std::min(cnt, cap); ++i) {
        out_pos[3 * i] = data.pos[i].x;
        out_pos[3 * i + 1] = data.pos[i].y;
        out_pos[3 * i + 2] = data.pos[i].z;
        out_label[i] = int32_t(data.label[i]);
    }
    return cnt;
}

}  // extern "C"
