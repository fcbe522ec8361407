// sf_kiri_facade.hpp -- C++ drop-in for the seepage_flows_cuda host API.
//
// Header-only C++17 layer over sf_capi.h that keeps the class names,
// constructor arguments and call sequence of the reference library, so an
// application written against it (seepage_flows/src/seepageflow/main.cpp:
// 25-297) compiles against this header and libsf_gb300.so instead:
//
//   CudaSFParticles        include/kiri_pbs_cuda/particle/cuda_sf_particles.cuh:42-219
//   CudaBoundaryParticles  include/kiri_pbs_cuda/particle/cuda_boundary_particles.cuh:19-48
//   CudaGNSearcher, CudaGNBoundarySearcher
//                          include/kiri_pbs_cuda/searcher/cuda_neighbor_searcher.cuh:25-113
//   CudaSphSFSolver, CudaWCSphSFSolver
//                          include/kiri_pbs_cuda/solver/seepageflow/cuda_{sph,wcsph}_sf_solver.cuh
//   CudaSFSystem           include/kiri_pbs_cuda/system/cuda_sf_system.cuh, src/.../cuda_sf_system.cu:17-119
//   CudaEmitter, CudaBoundaryEmitter, CudaVolumeEmitter
//                          include/kiri_pbs_cuda/emitter/*.cuh, src/kiri_pbs_cuda/emitter/*.cpp
//   global parameter structs CUDA_SEEPAGEFLOW_PARAMS, CUDA_BOUNDARY_PARAMS,
//   CUDA_SPH_EMITTER_PARAMS, CUDA_SEEPAGEFLOW_APP_PARAMS (include/kiri_pbs_cuda/data/*.h)
//
// Differences a caller can observe:
//   * the particle getters (GetPosPtr, ...) return device float3/float/size_t
//     arrays in the current cell-sorted order like the reference, but they are
//     copies made on demand from the internal float4 layout: a pointer stays
//     valid until the next UpdateSystem or getter call of the same field, and
//     writes through it are not seen by the solver;
//   * errors are reported on stderr and as a false return of UpdateSystemChecked
//     instead of being swallowed.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "sf_capi.h"

namespace KIRI {

template <class T> using Vector = std::vector<T>;
using Vec_Float = Vector<float>;
using Vec_Float2 = Vector<float2>;
using Vec_Float3 = Vector<float3>;
using Vec_Float4 = Vector<float4>;
using Vec_SizeT = Vector<size_t>;
template <class T> using SharedPtr = std::shared_ptr<T>;

constexpr float kKiriPi = 3.141592653589793238462643383279502884197f;

// ------------------------------------------------------------- parameters
enum CudaSphSolverType { SPH_SOLVER, WCSPH_SOLVER, IISPH_SOLVER };
enum CudaSeepageflowType { SF, MULTI_SF };
enum CudaSphEmitterType { SQUARE, CIRCLE, RECTANGLE };
enum SearcherParticleType { SEEPAGE = 0, SEEPAGE_MULTI = 1 };

struct CudaSeepageflowParams {
    float sph_mass, sph_density, sph_particle_radius, sph_kernel_radius;
    float sph_stiff, sph_visc, sph_nu, sph_bnu;
    float dem_mass, dem_density, dem_particle_radius, dem_kernel_radius;
    float dem_young, dem_poisson, dem_tan_friction_angle, dem_damping;
    float sf_c0, sf_csat, sf_cmc, sf_cmc_p, sf_cd;
    float sf_a0, sf_asat, sf_amc, sf_amc_p;
    float3 sf_dry_sand_color, sf_wet_sand_color;
    float3 gravity;
    float dt;
    CudaSphSolverType solver_type;
    CudaSeepageflowType sf_type;
};

struct CudaSeepageflowAppParams {
    size_t max_num = 100000;
    bool run = false;
    bool run_offline = false;
    int scene_data_idx = 0;
    char bgeo_export_folder[320] = "default";
    bool bgeo_export = false;
};

struct CudaBoundaryParams {
    float kernel_radius;
    float3 lowest_point, highest_point, world_size, world_center;
    int3 grid_size;
};

struct CudaSphEmitterParams {
    bool enable = false;
    bool run = false;
    float3 emit_pos, emit_vel, emit_col;
    CudaSphEmitterType emit_type = CudaSphEmitterType::SQUARE;
    float emit_radius = 0.0f, emit_width = 0.0f, emit_height = 0.0f;
};

inline CudaSeepageflowParams CUDA_SEEPAGEFLOW_PARAMS{};
inline CudaSeepageflowAppParams CUDA_SEEPAGEFLOW_APP_PARAMS{};
inline CudaBoundaryParams CUDA_BOUNDARY_PARAMS{};
inline CudaSphEmitterParams CUDA_SPH_EMITTER_PARAMS{};

namespace detail {
inline float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
inline float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 mul(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float3 a) { return std::sqrt(dot(a, a)); }
inline float3 normalize(float3 v) { return mul(v, 1.f / std::sqrt(dot(v, v))); }
inline float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

inline sf_params toC(const CudaSeepageflowParams& p) {
    sf_params c;
    c.sph_mass = p.sph_mass;
    c.sph_density = p.sph_density;
    c.sph_particle_radius = p.sph_particle_radius;
    c.sph_kernel_radius = p.sph_kernel_radius;
    c.sph_stiff = p.sph_stiff;
    c.sph_visc = p.sph_visc;
    c.sph_nu = p.sph_nu;
    c.sph_bnu = p.sph_bnu;
    c.dem_mass = p.dem_mass;
    c.dem_density = p.dem_density;
    c.dem_particle_radius = p.dem_particle_radius;
    c.dem_kernel_radius = p.dem_kernel_radius;
    c.dem_young = p.dem_young;
    c.dem_poisson = p.dem_poisson;
    c.dem_tan_friction_angle = p.dem_tan_friction_angle;
    c.dem_damping = p.dem_damping;
    c.sf_c0 = p.sf_c0;
    c.sf_csat = p.sf_csat;
    c.sf_cmc = p.sf_cmc;
    c.sf_cmc_p = p.sf_cmc_p;
    c.sf_cd = p.sf_cd;
    c.sf_a0 = p.sf_a0;
    c.sf_asat = p.sf_asat;
    c.sf_amc = p.sf_amc;
    c.sf_amc_p = p.sf_amc_p;
    const float3 cols[2] = {p.sf_dry_sand_color, p.sf_wet_sand_color};
    float* dst[2] = {c.sf_dry_sand_color, c.sf_wet_sand_color};
    for (int k = 0; k < 2; ++k) {
        dst[k][0] = cols[k].x;
        dst[k][1] = cols[k].y;
        dst[k][2] = cols[k].z;
    }
    c.gravity[0] = p.gravity.x;
    c.gravity[1] = p.gravity.y;
    c.gravity[2] = p.gravity.z;
    c.dt = p.dt;
    c.solver_type = p.solver_type == WCSPH_SOLVER ? SF_SOLVER_WCSPH : SF_SOLVER_SPH;
    c.sf_type = p.sf_type == MULTI_SF ? SF_TYPE_MULTI_SF : SF_TYPE_SF;
    return c;
}

inline sf_boundary_params toC(const CudaBoundaryParams& b) {
    sf_boundary_params c;
    c.kernel_radius = b.kernel_radius;
    const float3 v[4] = {b.lowest_point, b.highest_point, b.world_size, b.world_center};
    float* d[4] = {c.lowest_point, c.highest_point, c.world_size, c.world_center};
    for (int k = 0; k < 4; ++k) {
        d[k][0] = v[k].x;
        d[k][1] = v[k].y;
        d[k][2] = v[k].z;
    }
    c.grid_size[0] = b.grid_size.x;
    c.grid_size[1] = b.grid_size.y;
    c.grid_size[2] = b.grid_size.z;
    return c;
}

// Device staging buffer for one getter.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    void* reserve(size_t b) {
        if (b > bytes) {
            if (ptr) cudaFree(ptr);
            ptr = nullptr;
            bytes = 0;
            if (cudaMalloc(&ptr, b) != cudaSuccess) return nullptr;
            bytes = b;
        }
        return ptr;
    }
    ~DeviceBuffer() {
        if (ptr) cudaFree(ptr);
    }
};
}  // namespace detail

// -------------------------------------------------------------- particles
class CudaSFSystem;

class CudaParticles {
public:
    virtual ~CudaParticles() = default;
    size_t Size() const;
    size_t MaxSize() const { return mMaxNum; }

protected:
    size_t mMaxNum = 0;
    size_t mInitialNum = 0;
    CudaSFSystem* mSystem = nullptr;
    friend class CudaSFSystem;
};

class CudaSFParticles final : public CudaParticles {
public:
    CudaSFParticles(const size_t numOfMaxParticles, const Vec_Float3& p, const Vec_Float3& col,
                    const Vec_SizeT& label, const Vec_Float& mass, const Vec_Float& radius)
        : CudaSFParticles(numOfMaxParticles, p, col, label, mass, radius, Vec_Float3(), Vec_Float2()) {}
    CudaSFParticles(const size_t numOfMaxParticles, const Vec_Float3& p, const Vec_Float3& col,
                    const Vec_SizeT& label, const Vec_Float& mass, const Vec_Float& radius,
                    const Vec_Float3& cda0asat, const Vec_Float2& amcamcp)
        : pos(p), colv(col), mass_(mass), radius_(radius), cda(cda0asat), amc(amcamcp) {
        mMaxNum = numOfMaxParticles;
        mInitialNum = p.size();
        labels.assign(label.begin(), label.end());
    }
    CudaSFParticles(const Vec_Float3& p, const Vec_Float3& col, const Vec_SizeT& label, const Vec_Float& mass,
                    const Vec_Float& radius)
        : CudaSFParticles(p.size(), p, col, label, mass, radius) {}

    // CudaSFParticles getters (cuda_sf_particles.cuh:170-190): device copies in
    // sorted order, refreshed by each call. The reference returns writable
    // pointers into its own arrays; these are copies, so they are const: code
    // that writes through a getter (which would change nothing here) fails to
    // compile instead of silently doing nothing. Change a field with
    // sf_set_field on Handle().
    const float3* GetPosPtr() const { return static_cast<const float3*>(field(SF_FIELD_POS, 12)); }
    const float3* GetVelPtr() const { return static_cast<const float3*>(field(SF_FIELD_VEL, 12)); }
    const float3* GetAccPtr() const { return static_cast<const float3*>(field(SF_FIELD_ACC, 12)); }
    const float3* GetColPtr() const { return static_cast<const float3*>(field(SF_FIELD_COL, 12)); }
    const float* GetRadiusPtr() const { return static_cast<const float*>(field(SF_FIELD_RADIUS, 4)); }
    const float* GetMassPtr() const { return static_cast<const float*>(field(SF_FIELD_MASS, 4)); }
    const float* GetDensityPtr() const { return static_cast<const float*>(field(SF_FIELD_DENSITY, 4)); }
    const float* GetPressurePtr() const { return static_cast<const float*>(field(SF_FIELD_PRESSURE, 4)); }
    const float* GetVoidagePtr() const { return static_cast<const float*>(field(SF_FIELD_VOIDAGE, 4)); }
    const float* GetSaturationPtr() const { return static_cast<const float*>(field(SF_FIELD_SATURATION, 4)); }
    const float* GetMaxSaturationPtr() const { return static_cast<const float*>(field(SF_FIELD_MAX_SATURATION, 4)); }
    const float3* GetAvgFlowVelPtr() const { return static_cast<const float3*>(field(SF_FIELD_AVG_FLOW, 12)); }
    const float3* GetAvgDragForcePtr() const { return static_cast<const float3*>(field(SF_FIELD_AVG_DRAG, 12)); }
    const float3* GetAdhesionForcePtr() const { return static_cast<const float3*>(field(SF_FIELD_ADHESION, 12)); }
    const float3* GetAvgAdhesionForcePtr() const { return static_cast<const float3*>(field(SF_FIELD_AVG_ADHESION, 12)); }
    const float3* GetCdA0AsatPtr() const { return static_cast<const float3*>(field(SF_FIELD_CDA0ASAT, 12)); }
    const float2* GetAmcAmcpPtr() const { return static_cast<const float2*>(field(SF_FIELD_AMCAMCP, 8)); }
    const size_t* GetLabelPtr() const;

    // CudaSFParticles::AddSphParticles (cuda_sf_particles.cu:50-68)
    void AddSphParticles(Vec_Float3 pos, float3 col, float3 vel, float mass, float radius);

private:
    void* field(int id, size_t elemBytes) const;
    Vec_Float3 pos, colv;
    Vec_Float mass_, radius_;
    Vec_Float3 cda;
    Vec_Float2 amc;
    std::vector<int32_t> labels;
    mutable detail::DeviceBuffer bufs[SF_FIELD_COUNT];
    mutable detail::DeviceBuffer labelBuf;
    friend class CudaSFSystem;
};
using CudaSFParticlesPtr = SharedPtr<CudaSFParticles>;

class CudaBoundaryParticles final : public CudaParticles {
public:
    explicit CudaBoundaryParticles(const Vec_Float3& p) : pos(p), labels(p.size(), 0) {
        mMaxNum = mInitialNum = p.size();
    }
    CudaBoundaryParticles(const Vec_Float3& p, const Vec_SizeT& label) : pos(p), labels(label.begin(), label.end()) {
        mMaxNum = mInitialNum = p.size();
    }

private:
    Vec_Float3 pos;
    std::vector<int32_t> labels;
    friend class CudaSFSystem;
};
using CudaBoundaryParticlesPtr = SharedPtr<CudaBoundaryParticles>;

// --------------------------------------------------------------- searchers
// The grid of a searcher (cuda_neighbor_searcher.cu:19-34). The cell tables
// themselves live in the handle; GetCellStart copies them out.
class CudaGNBaseSearcher {
public:
    CudaGNBaseSearcher(const float3 lowestPoint, const float3 highestPoint, const size_t maxNumOfParticles,
                       const float cellSize)
        : mLowestPoint(lowestPoint), mHighestPoint(highestPoint), mCellSize(cellSize),
          mMaxNumOfParticles(maxNumOfParticles) {
        const float3 q = f3div(detail::sub(highestPoint, lowestPoint), cellSize);
        mGridSize = make_int3(int(q.x), int(q.y), int(q.z));
    }
    virtual ~CudaGNBaseSearcher() = default;
    float3 GetLowestPoint() const { return mLowestPoint; }
    float3 GetHighestPoint() const { return mHighestPoint; }
    float GetCellSize() const { return mCellSize; }
    int3 GetGridSize() const { return mGridSize; }
    // CudaGNBaseSearcher::GetCellStartPtr (cuda_neighbor_searcher.cuh:35-44):
    // device array of G + 1 size_t, the start of every cell in the sorted
    // particles (boundary particles for the boundary searcher) and the count
    // at entry G. A copy of the table of the last sort, refreshed by each
    // call; nullptr before the searcher's system exists.
    const size_t* GetCellStartPtr() const;

protected:
    static float3 f3div(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
    float3 mLowestPoint, mHighestPoint;
    float mCellSize;
    size_t mMaxNumOfParticles;
    int3 mGridSize;
    CudaSFSystem* mSystem = nullptr;
    int mTable = 0;  // 0: particle cell table, 1: boundary cell table
    mutable detail::DeviceBuffer mCellBuf;
    friend class CudaSFSystem;
};

class CudaGNSearcher final : public CudaGNBaseSearcher {
public:
    CudaGNSearcher(const float3 lp, const float3 hp, const size_t num, const float cellSize,
                   const SearcherParticleType type)
        : CudaGNBaseSearcher(lp, hp, num, cellSize), mType(type) {}
    SearcherParticleType GetType() const { return mType; }

private:
    SearcherParticleType mType;
};
using CudaGNSearcherPtr = SharedPtr<CudaGNSearcher>;

class CudaGNBoundarySearcher final : public CudaGNBaseSearcher {
public:
    CudaGNBoundarySearcher(const float3 lp, const float3 hp, const size_t num, const float cellSize)
        : CudaGNBaseSearcher(lp, hp, num, cellSize) {
        mTable = 1;
    }
};
using CudaGNBoundarySearcherPtr = SharedPtr<CudaGNBoundarySearcher>;

// ------------------------------------------------------------------ solvers
class CudaSphSFSolver {
public:
    explicit CudaSphSFSolver(const size_t num) : mMaxNum(num) {}
    virtual ~CudaSphSFSolver() = default;
    size_t GetNumOfSubTimeSteps() const { return mNumOfSubTimeSteps; }
    virtual sf_solver_params SolverParams() const { return sf_solver_params{1.f, 3.f, 100.f}; }

protected:
    size_t mMaxNum;
    size_t mNumOfSubTimeSteps = 1;
    friend class CudaSFSystem;
};
using CudaSphSFSolverPtr = SharedPtr<CudaSphSFSolver>;

class CudaWCSphSFSolver final : public CudaSphSFSolver {
public:
    explicit CudaWCSphSFSolver(const size_t num, const float negativeScale = 0.f,
                               const float timeStepLimitScale = 3.f, const float speedOfSound = 100.f)
        : CudaSphSFSolver(num), mNegativeScale(negativeScale), mTimeStepLimitScale(timeStepLimitScale),
          mSpeedOfSound(speedOfSound) {}
    float GetSpeedOfSound() const { return mSpeedOfSound; }
    float GetTimeStepLimitScale() const { return mTimeStepLimitScale; }
    void SetTimeStepLimitScale(float s) { mTimeStepLimitScale = std::max(s, 0.f); }
    void SetSpeedOfSound(float c) { mSpeedOfSound = std::max(c, 1e-6f); }
    sf_solver_params SolverParams() const override {
        return sf_solver_params{mNegativeScale, mTimeStepLimitScale, mSpeedOfSound};
    }

private:
    float mNegativeScale, mTimeStepLimitScale, mSpeedOfSound;
};
using CudaWCSphSFSolverPtr = SharedPtr<CudaWCSphSFSolver>;

// ----------------------------------------------------------------- emitters
// CudaEmitter (include/kiri_pbs_cuda/emitter/cuda_emitter.cuh, src/.../cuda_emitter.cpp)
class CudaEmitter {
public:
    CudaEmitter() : CudaEmitter(make_float3(0.f, 0.f, 0.f), make_float3(1.f, 0.f, 0.f), false) {}
    CudaEmitter(float3 emitPosition, float3 emitVelocity, bool enable)
        : bEnable(enable), mEmitPosition(emitPosition) {
        UpdateEmitterVelocity(emitVelocity);
    }
    Vec_Float3 Emit() const {
        Vec_Float3 out;
        out.reserve(mSamples.size());
        for (const float2& s : mSamples)
            out.push_back(detail::add(detail::add(mEmitPosition, detail::mul(mEmitAxis1, s.x)),
                                      detail::mul(mEmitAxis2, s.y)));
        return out;
    }
    void SetEmitterStatus(const bool enable) { bEnable = enable; }
    void UpdateEmitterVelocity(float3 v) {
        mEmitVelocity = v;
        const float3 axis = detail::normalize(v);
        if (std::fabs(axis.x) == 1.f && std::fabs(axis.y) == 0.f && std::fabs(axis.z) == 0.f)
            mEmitAxis1 = detail::normalize(detail::cross(axis, make_float3(0.f, 1.f, 0.f)));
        else
            mEmitAxis1 = detail::normalize(detail::cross(axis, make_float3(1.f, 0.f, 0.f)));
        mEmitAxis2 = detail::normalize(detail::cross(axis, mEmitAxis1));
    }
    void BuildSquareEmitter(float particleRadius, float emitterRadius) {
        build(particleRadius, -emitterRadius, emitterRadius, -emitterRadius, emitterRadius, -1.f);
    }
    void BuildCircleEmitter(float particleRadius, float emitterRadius) {
        build(particleRadius, -emitterRadius, emitterRadius, -emitterRadius, emitterRadius, emitterRadius);
    }
    void BuildRectangleEmitter(float particleRadius, float emitterWidth, float emitterHeight) {
        build(particleRadius, -emitterWidth, emitterWidth, -emitterHeight, emitterHeight, -1.f);
    }
    bool GetEmitterStatus() const { return bEnable; }
    size_t GetNumOfEmitterPoints() const { return mSamples.size(); }
    float3 GetEmitterPosition() const { return mEmitPosition; }
    float3 GetEmitterVelocity() const { return mEmitVelocity; }

private:
    // Float loop counters stepping by the particle diameter, as the reference's emitters do.
    void build(float r, float i0, float i1, float j0, float j1, float circle) {
        mSamples.clear();
        const float offset = r * 2.f;
        for (float i = i0; i < i1; i += offset)
            for (float j = j0; j < j1; j += offset)
                if (circle < 0.f || std::sqrt(i * i + j * j) <= circle) mSamples.push_back(make_float2(i, j));
        bBuild = !mSamples.empty();
    }
    bool bEnable = false, bBuild = false;
    Vec_Float2 mSamples;
    float3 mEmitPosition{}, mEmitVelocity{}, mEmitAxis1{}, mEmitAxis2{};
};
using CudaEmitterPtr = SharedPtr<CudaEmitter>;

struct BoundaryData {
    Vec_Float3 pos;
    Vec_SizeT label;
};

// CudaBoundaryEmitter (src/kiri_pbs_cuda/emitter/cuda_boundary_emitter.cpp:12-92)
class CudaBoundaryEmitter {
public:
    explicit CudaBoundaryEmitter(bool enable = true) : bEnable(enable) {}
    // Six lattice planes at pitch 2r; the loop bounds compare the integer
    // counter with the float extent, as the reference does.
    void BuildWorldBoundary(BoundaryData& data, const float3& lowest, const float3& highest,
                            const float particleRadius) const {
        if (!bEnable) return;
        const float spacing = particleRadius * 2.f;
        const float3 sides = make_float3((highest.x - lowest.x) / spacing, (highest.y - lowest.y) / spacing,
                                         (highest.z - lowest.z) / spacing);
        auto plane = [&](float na, float nb, auto point) {
            for (size_t i = 0; float(i) <= na; ++i)
                for (size_t j = 0; float(j) <= nb; ++j) {
                    data.pos.push_back(point(float(i) * spacing, float(j) * spacing));
                    data.label.push_back(0);
                }
        };
        plane(sides.x, sides.z, [&](float a, float b) { return make_float3(lowest.x + a, lowest.y, lowest.z + b); });
        plane(sides.x, sides.z, [&](float a, float b) { return make_float3(lowest.x + a, highest.y, lowest.z + b); });
        plane(sides.x, sides.y, [&](float a, float b) { return make_float3(lowest.x + a, lowest.y + b, lowest.z); });
        plane(sides.x, sides.y, [&](float a, float b) { return make_float3(lowest.x + a, lowest.y + b, highest.z); });
        plane(sides.y, sides.z, [&](float a, float b) { return make_float3(lowest.x, lowest.y + a, lowest.z + b); });
        plane(sides.y, sides.z, [&](float a, float b) { return make_float3(highest.x, lowest.y + a, lowest.z + b); });
    }
    void BuildBoundaryShapeVolume(BoundaryData& data, const Vec_Float4& shape) const {
        if (!bEnable) return;
        for (const float4& s : shape) {
            data.pos.push_back(make_float3(s.x, s.y, s.z));
            data.label.push_back(1);
        }
    }

private:
    bool bEnable;
};

struct SeepageflowVolumeData {
    float sandMinRadius;
    Vec_Float3 pos, col;
    Vec_Float mass, radius;
    Vec_SizeT label;
};
struct SeepageflowMultiVolumeData {
    float sandMinRadius;
    Vec_Float3 pos, col;
    Vec_Float mass, radius;
    Vec_SizeT label;
    Vec_Float3 cda0asat;
    Vec_Float2 amcamcp;
};

// CudaVolumeEmitter (src/kiri_pbs_cuda/emitter/cuda_volume_emitter.cpp:79-175).
// The box builder jitters by jitter * normalize(uniform(-1,1)^3); pass a seed
// for a reproducible scene (the reference seeds from std::random_device).
class CudaVolumeEmitter {
public:
    explicit CudaVolumeEmitter(bool enable = true) : bEnable(enable) {}
    void BuildSeepageflowBoxVolume(SeepageflowVolumeData& data, float3 lowest, int3 vsize, float particleRadius,
                                   float3 color, float mass, size_t label, float jitter,
                                   unsigned seed = std::random_device{}()) const {
        if (!bEnable) return;
        data.sandMinRadius = particleRadius;
        std::default_random_engine eng(seed);
        std::uniform_real_distribution<> dist(-1.f, 1.f);
        const float offset = 2.f * particleRadius;
        for (int i = 0; i < vsize.x; ++i)
            for (int j = 0; j < vsize.y; ++j)
                for (int k = 0; k < vsize.z; ++k) {
                    float3 p = make_float3(lowest.x + float(i) * offset, lowest.y + float(j) * offset,
                                           lowest.z + float(k) * offset);
                    const float x = float(dist(eng)), y = float(dist(eng)), z = float(dist(eng));
                    data.pos.push_back(detail::add(p, detail::mul(detail::normalize(make_float3(x, y, z)), jitter)));
                    data.col.push_back(color);
                    data.label.push_back(label);
                    data.radius.push_back(particleRadius);
                    data.mass.push_back(mass);
                }
    }
    void BuildSeepageflowShapeMultiVolume(SeepageflowMultiVolumeData& data, const Vec_Float4& shape, float3 color,
                                          float sandDensity, float3 cda0asat, float2 amcamcp, bool offsetY,
                                          float worldLowestY) const {
        if (!bEnable) return;
        // Huge<size_t>() of the reference, as a float
        const float huge = static_cast<float>(std::numeric_limits<size_t>::max());
        if (data.pos.empty()) data.sandMinRadius = huge;
        float minY = huge;
        for (const float4& s : shape) {
            data.pos.push_back(make_float3(s.x, s.y, s.z));
            data.col.push_back(color);
            data.label.push_back(1);
            data.radius.push_back(s.w);
            data.mass.push_back(sandDensity * ((4.f / 3.f) * kKiriPi * std::pow(s.w, 3.f)));
            data.sandMinRadius = std::min(s.w, data.sandMinRadius);
            data.cda0asat.push_back(cda0asat);
            data.amcamcp.push_back(amcamcp);
            minY = std::min(minY, s.y);
        }
        if (offsetY) {
            const float off = minY - (worldLowestY + data.sandMinRadius * 5.f);
            // every particle gathered so far, as cuda_volume_emitter.cpp:169-173 does
            for (size_t i = 0; i < data.pos.size(); ++i) data.pos[i].y -= off;
        }
    }

private:
    bool bEnable;
};

// ------------------------------------------------------------------ system
// CudaSFSystem (src/kiri_pbs_cuda/system/cuda_sf_system.cu:17-119) with the
// UpdateSystem of CudaBaseSystem (cuda_base_system.cu:29-56).
class CudaSFSystem {
public:
    CudaSFSystem(CudaSFParticlesPtr& particles, CudaBoundaryParticlesPtr& boundaryParticles,
                 CudaSphSFSolverPtr& solver, CudaGNSearcherPtr& searcher, CudaGNBoundarySearcherPtr& boundarySearcher,
                 CudaEmitterPtr& emitter, const bool adaptiveSubTimeStep)
        : mParticles(particles), mBoundaries(boundaryParticles), mSolver(solver), mSearcher(searcher),
          mBoundarySearcher(boundarySearcher), mEmitter(emitter), bAdaptive(adaptiveSubTimeStep) {
        if (CUDA_SPH_EMITTER_PARAMS.enable && mEmitter) {
            switch (CUDA_SPH_EMITTER_PARAMS.emit_type) {
            case SQUARE:
                mEmitter->BuildSquareEmitter(CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius,
                                             CUDA_SPH_EMITTER_PARAMS.emit_radius);
                break;
            case CIRCLE:
                mEmitter->BuildCircleEmitter(CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius,
                                             CUDA_SPH_EMITTER_PARAMS.emit_radius);
                break;
            case RECTANGLE:
                mEmitter->BuildRectangleEmitter(CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius,
                                                CUDA_SPH_EMITTER_PARAMS.emit_width, CUDA_SPH_EMITTER_PARAMS.emit_height);
                break;
            }
        }
        const CudaSFParticles& P = *mParticles;
        const size_t n = P.pos.size();
        std::vector<float> pos(3 * n), col(3 * n), cda(3 * n, 0.f), amc(2 * n, 0.f);
        for (size_t i = 0; i < n; ++i) {
            pos[3 * i] = P.pos[i].x;
            pos[3 * i + 1] = P.pos[i].y;
            pos[3 * i + 2] = P.pos[i].z;
            col[3 * i] = P.colv[i].x;
            col[3 * i + 1] = P.colv[i].y;
            col[3 * i + 2] = P.colv[i].z;
            if (i < P.cda.size()) {
                cda[3 * i] = P.cda[i].x;
                cda[3 * i + 1] = P.cda[i].y;
                cda[3 * i + 2] = P.cda[i].z;
            }
            if (i < P.amc.size()) {
                amc[2 * i] = P.amc[i].x;
                amc[2 * i + 1] = P.amc[i].y;
            }
        }
        const CudaBoundaryParticles& Bp = *mBoundaries;
        std::vector<float> bpos(3 * Bp.pos.size());
        for (size_t i = 0; i < Bp.pos.size(); ++i) {
            bpos[3 * i] = Bp.pos[i].x;
            bpos[3 * i + 1] = Bp.pos[i].y;
            bpos[3 * i + 2] = Bp.pos[i].z;
        }
        sf_scene_init in{};
        in.n = int64_t(n);
        in.pos = pos.data();
        in.col = col.data();
        in.label = P.labels.data();
        in.mass = P.mass_.data();
        in.radius = P.radius_.data();
        in.cda0asat = cda.data();
        in.amcamcp = amc.data();
        in.nb = int64_t(Bp.pos.size());
        in.bpos = bpos.data();
        in.blabel = Bp.labels.data();
        const sf_params p = detail::toC(CUDA_SEEPAGEFLOW_PARAMS);
        const sf_boundary_params b = detail::toC(CUDA_BOUNDARY_PARAMS);
        const sf_solver_params s = mSolver->SolverParams();
        const sf_status st = sf_create(&p, &b, &s, &in, int64_t(P.MaxSize()), nullptr, &mHandle);
        if (st != SF_OK) {
            std::fprintf(stderr, "CudaSFSystem: sf_create failed (%d): %s\n", st, sf_last_error_string(nullptr));
            mHandle = nullptr;
        }
        mParticles->mSystem = this;
        mBoundaries->mSystem = this;
        if (mSearcher) mSearcher->mSystem = this;
        if (mBoundarySearcher) mBoundarySearcher->mSystem = this;
    }
    ~CudaSFSystem() {
        if (mHandle) sf_destroy(mHandle);
    }
    CudaSFSystem(const CudaSFSystem&) = delete;
    CudaSFSystem& operator=(const CudaSFSystem&) = delete;

    // One substep; returns the device time in ms like CudaBaseSystem::UpdateSystem.
    float UpdateSystem(float renderInterval) {
        float ms = 0.f;
        UpdateSystemChecked(renderInterval, &ms);
        return ms;
    }
    bool UpdateSystemChecked(float renderInterval, float* msOut) {
        if (!mHandle) return false;
        const sf_params p = detail::toC(CUDA_SEEPAGEFLOW_PARAMS);  // edit global, next step sees it
        if (std::memcmp(&p, &mLastParams, sizeof(p)) != 0) {
            if (sf_set_params(mHandle, 0, &p) != SF_OK) return report("sf_set_params");
            mLastParams = p;
        }
        int64_t nsub = 0;
        if (sf_step(mHandle, renderInterval, &nsub, msOut) != SF_OK) return report("sf_step");
        mSolver->mNumOfSubTimeSteps = size_t(nsub);
        return emit(renderInterval);
    }
    size_t GetNumOfSubTimeSteps() const { return mSolver->GetNumOfSubTimeSteps(); }
    bool GetAdaptiveSubTimeStep() const { return bAdaptive; }
    CudaSFParticlesPtr GetSFParticles() const { return mParticles; }
    sf_handle* Handle() const { return mHandle; }

private:
    bool report(const char* what) {
        std::fprintf(stderr, "CudaSFSystem: %s failed: %s\n", what, sf_last_error_string(mHandle));
        return false;
    }
    // The emitter schedule of CudaSFSystem::OnUpdateSolver (cuda_sf_system.cu:86-115).
    bool emit(float renderInterval) {
        if (!mEmitter || !mEmitter->GetEmitterStatus() || !CUDA_SPH_EMITTER_PARAMS.run) return true;
        const float3 v = mEmitter->GetEmitterVelocity();
        const float r = CUDA_SEEPAGEFLOW_PARAMS.sph_particle_radius;
        bool fire = false;
        if (CUDA_SEEPAGEFLOW_PARAMS.solver_type == SPH_SOLVER) {
            const size_t stepNum = size_t(2.f * r / (detail::length(v) * CUDA_SEEPAGEFLOW_PARAMS.dt));
            fire = stepNum == 0 || (mEmitterCounter++ % stepNum == 0);
        } else {
            mEmitterElapsedTime += renderInterval / float(GetNumOfSubTimeSteps());
            if ((detail::length(v) * mEmitterElapsedTime) / (2.f * r) >= float(mEmitterCounter)) {
                fire = true;
                mEmitterCounter++;
            }
        }
        if (!fire) return true;
        const Vec_Float3 pts = mEmitter->Emit();
        if (mParticles->Size() + pts.size() < mParticles->MaxSize())
            mParticles->AddSphParticles(pts, CUDA_SPH_EMITTER_PARAMS.emit_col, v, CUDA_SEEPAGEFLOW_PARAMS.sph_mass, r);
        else
            mEmitter->SetEmitterStatus(false);
        return true;
    }

    CudaSFParticlesPtr mParticles;
    CudaBoundaryParticlesPtr mBoundaries;
    CudaSphSFSolverPtr mSolver;
    CudaGNSearcherPtr mSearcher;
    CudaGNBoundarySearcherPtr mBoundarySearcher;
    CudaEmitterPtr mEmitter;
    bool bAdaptive;
    sf_handle* mHandle = nullptr;
    sf_params mLastParams{};
    size_t mEmitterCounter = 0;
    float mEmitterElapsedTime = 0.f;
    friend class CudaSFParticles;
};
using CudaSFSystemPtr = SharedPtr<CudaSFSystem>;

// ----------------------------------------------------- out-of-line members
inline size_t CudaParticles::Size() const {
    if (!mSystem || !mSystem->Handle()) return mInitialNum;
    int64_t n = 0, cap = 0;
    sf_size(mSystem->Handle(), 0, &n, &cap);
    return size_t(n);
}

inline const size_t* CudaGNBaseSearcher::GetCellStartPtr() const {
    if (!mSystem || !mSystem->Handle()) return nullptr;
    int32_t g[3];
    int64_t cells = 0;
    if (sf_get_grid(mSystem->Handle(), 0, g, &cells) != SF_OK) return nullptr;
    std::vector<int64_t> t(size_t(cells) + 1);
    if (sf_get_cell_table(mSystem->Handle(), 0, mTable, t.data(), int64_t(t.size())) != SF_OK) return nullptr;
    std::vector<size_t> ts(t.begin(), t.end());
    void* d = mCellBuf.reserve(ts.size() * sizeof(size_t));
    if (!d || cudaMemcpy(d, ts.data(), ts.size() * sizeof(size_t), cudaMemcpyHostToDevice) != cudaSuccess)
        return nullptr;
    return static_cast<size_t*>(d);
}

inline void* CudaSFParticles::field(int id, size_t elemBytes) const {
    if (!mSystem || !mSystem->Handle()) return nullptr;
    const size_t n = Size();
    void* d = bufs[id].reserve(std::max<size_t>(1, n) * elemBytes);
    if (!d) return nullptr;
    if (n > 0 && sf_get_field(mSystem->Handle(), 0, id, SF_ORDER_SORTED, d, int64_t(n), 1) != SF_OK) return nullptr;
    if (sf_synchronize(mSystem->Handle()) != SF_OK) return nullptr;  // the copy is complete on return
    return d;
}

inline const size_t* CudaSFParticles::GetLabelPtr() const {
    if (!mSystem || !mSystem->Handle()) return nullptr;
    const size_t n = Size();
    std::vector<int32_t> l(n);
    std::vector<size_t> ls(n);
    if (n > 0 && sf_get_field(mSystem->Handle(), 0, SF_FIELD_LABEL, SF_ORDER_SORTED, l.data(), int64_t(n), 0) != SF_OK)
        return nullptr;
    for (size_t i = 0; i < n; ++i) ls[i] = size_t(l[i]);
    void* d = labelBuf.reserve(std::max<size_t>(1, n) * sizeof(size_t));
    if (!d || cudaMemcpy(d, ls.data(), n * sizeof(size_t), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return static_cast<size_t*>(d);
}

inline void CudaSFParticles::AddSphParticles(Vec_Float3 p, float3 col, float3 vel, float mass, float radius) {
    if (!mSystem || !mSystem->Handle()) return;
    std::vector<float> flat(3 * p.size());
    for (size_t i = 0; i < p.size(); ++i) {
        flat[3 * i] = p[i].x;
        flat[3 * i + 1] = p[i].y;
        flat[3 * i + 2] = p[i].z;
    }
    const float c[3] = {col.x, col.y, col.z}, v[3] = {vel.x, vel.y, vel.z};
    const sf_status st = sf_add_sph_particles(mSystem->Handle(), 0, flat.data(), int64_t(p.size()), c, v, mass, radius);
    if (st == SF_ERR_CAPACITY) std::printf("Current SPH particles numbers exceed maximum particles. \n");
}


// ------------------------------------------------------------- bgeo files
// ReadBgeoFileForGPU, ReadMultiBgeoFilesForGPU and ExportBgeoFileCUDA
// (seepage_flows/include/kiri_utils.h:252-448), over sf_read_bgeo and
// sf_export_bgeo_device. DB_PBR_PATH is the reference's asset root (a compile
// definition there); the reader looks for DB_PBR_PATH "bgeo/<folder>/<name>.bgeo".
#ifndef DB_PBR_PATH
#define DB_PBR_PATH "./"
#endif
using String = std::string;
using Vec_String = Vector<std::string>;

inline String UInt2Str4Digit(unsigned int input) {  // frame names of the export (main.cpp:270)
    char buf[16];
    std::snprintf(buf, sizeof(buf), "%04u", input);
    return String(buf);
}

inline Vec_Float4 ReadBgeoFileForGPU(String Folder, String Name, bool flip_yz = false) {
    const String path = String(DB_PBR_PATH) + "bgeo/" + Folder + "/" + Name + ".bgeo";
    Vec_Float4 out;
    int64_t n = 0;
    if (sf_read_bgeo(path.c_str(), flip_yz ? 1 : 0, nullptr, 0, &n) == SF_OK) {
        out.resize(size_t(n));
        if (n == 0 || sf_read_bgeo(path.c_str(), flip_yz ? 1 : 0, reinterpret_cast<float*>(out.data()), n, &n) == SF_OK)
            return out;
    }
    std::fprintf(stderr, "%s\n", sf_last_error_string(nullptr));
    return Vec_Float4();
}

inline Vec_Float4 ReadMultiBgeoFilesForGPU(Vec_String folders, Vec_String file_names, bool flip_yz = false) {
    Vec_Float4 out;
    for (size_t k = 0; k < folders.size() && k < file_names.size(); ++k) {
        const Vec_Float4 one = ReadBgeoFileForGPU(folders[k], file_names[k], flip_yz);
        out.insert(out.end(), one.begin(), one.end());
    }
    return out;
}

inline void ExportBgeoFileCUDA(const std::string& folder_path, const std::string& file_name, const float3* positions,
                               const float3* colors, const float* radius, const size_t* labels,
                               const size_t particles_num) {
    static_assert(sizeof(size_t) == sizeof(uint64_t), "labels are read as 64-bit words");
    if (sf_export_bgeo_device(folder_path.c_str(), file_name.c_str(), reinterpret_cast<const float*>(positions),
                              reinterpret_cast<const float*>(colors), radius,
                              reinterpret_cast<const uint64_t*>(labels), int64_t(particles_num), nullptr) != SF_OK)
        std::fprintf(stderr, "%s\n", sf_last_error_string(nullptr));
}

}  // namespace KIRI
