// Device-side data layout and pair physics of the GB300 seepage-flow substep.
//
// Layout in HBM (one handle, any number of scenes; "slot" = array index):
//   * every scene owns a slot range [slot_off, slot_off + slot_cap) whose
//     length is a multiple of kSlotAlign, so each thread block of a pass
//     belongs to exactly one scene (blockScene[] maps block -> scene);
//   * live particles fill the front of the range after every sort; the rest
//     are parking slots (pos.w == 0) whose key is the scene's parking cell
//     (local index G), which sorts after every real cell;
//   * cells of all scenes share one global index space: scene s owns
//     [cell_off, cell_off + G + 1); cellStart has total_cells + 1 entries;
//   * per-slot float4 arrays (16-byte loads, cell-sorted):
//       pos4  = (x, y, z, w)  w = +mass (water), -mass (sand), 0 (parking)
//       vel4  = (vx, vy, vz, density)
//       aux4  = (pressure, fluid voidage, saturation, voidage)
//       flow4 = (average flow velocity, sand: adhesion Bezier factor of its saturation)
//       adh4  = (adhesion force, 0)      avgadh4 = (average adhesion force, 0)
//       drag4 = (average drag force, sand: density)  acc4 = (acceleration, 0)
//       col4  = (colour, max saturation) mat4    = (cd, a0, asat, radius)
//       amc2  = (amc, amcp)              pid     = creation index
//   * boundary particles: bpos4 = (x, y, z, v) with v = +volume (label 0) or
//     -volume (label 1), sorted by cell with their own cell table.
//
// The pair terms restate the reference device functions operation for
// operation (IEEE division and square root, no fused multiply-add: the
// library is built with --fmad=false), so that the results match the
// reference's FP32 arithmetic. Constants the reference computes from
// parameters only (kernel coefficients, capillary volume, ...) are computed
// on the host in the same float operations and passed in SceneDev.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sfg {

constexpr int kSlotAlign = 256;
constexpr float kEps = 1e-6f;  // KIRI_EPSILON (kiri_pbs_pch.cuh:52)

struct BezierDev {  // QuadraticBezierCoeff (cuda_sf_utils.cuh:36-83)
    float b, c, d, e, py0, py1, px1, py2;
};

struct SceneDev {
    // grid (CudaBoundaryParams: lowest_point, kernel_radius, grid_size)
    float lpx, lpy, lpz, hpx, hpy, hpz, cell;
    int gx, gy, gz, ncell;  // ncell = gx*gy*gz (the parking cell is local index ncell)
    int cell_off;           // global index of local cell 0
    int slot_off, slot_cap;
    int b_off, nb;
    // reach of any non-zero pair term, squared and widened by 1e-5 relative
    float reach2;
    // SPH kernels (Poly6Kernel, SpikyKernelGrad, AdhesionAkinci13; cuda_sph_kernel.cuh)
    float h, h2, poly6, spiky, adh_coef, W0;
    // water
    float rho0, stiff, neg_scale, nu, bnu, sph_radius, sph_mass;
    int tait;
    // sand
    float rho1, dem_radius, kn, ks, tan2, damping, wall_rij;
    float rij2;       // 2 * dem_radius
    float dem_reach2; // (2 * dem_radius + rupture distance)^2, widened: DEM and capillary vanish beyond
    // capillary bridge constants (cuda_dem_solver_common_gpu.cuh:53-90)
    float cap_vlb, cap_srupt, cap_vlb_pir, cap_pir, cap_cos, cap_sin, cap_m2pi;
    BezierDev capG, adhG;
    float cd;
    int multi;
    int shape_boundary;  // the scene has boundary particles with label 1
    float grav_abs;
    float gvx, gvy, gvz;
    float dry[3], wet[3];
    // CFL (cuda_wcsph_sf_solver.cu:35-58)
    float cfl_by_speed, cfl_hm, cfl_mass, cfl_scale, params_dt;
    int wcsph;
    // factor on the adjoint's seed cotangents (sf_set_adjoint_seed_scale; 1 by default)
    float adj_seed_scale;
};

// Per-scene device scalars written by the passes.
struct SceneState {
    unsigned int amax_bits;  // max |acc| of the substep (float bits, >= 0)
    int n;                   // live particle count
    long long n_sub;         // sub-step count of the last integrate
    float dt;                // dt of the last integrate
    unsigned int list_need;  // largest neighbour count above 7/8 of the list capacity (0: none)
};

// ---------------------------------------------------------------- float3 math
__device__ __forceinline__ float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ void operator+=(float3& a, float3 b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(float3 v) { return sqrtf(dot3(v, v)); }
__device__ __forceinline__ int sgn1(float v) { return (0.f < v) - (v < 0.f); }

// ThrustHelper::ComputeGridXYZByPos3 / Pos2GridXYZ (helper_thrust.cuh:56-64,92-114)
__device__ __forceinline__ int3 cellOf(const SceneDev& S, float3 p) {
    const float rx = p.x - S.lpx, ry = p.y - S.lpy, rz = p.z - S.lpz;
    int3 c;
    c.x = min(max((int)(rx / S.cell), 0), S.gx - 1);
    c.y = min(max((int)(ry / S.cell), 0), S.gy - 1);
    c.z = min(max((int)(rz / S.cell), 0), S.gz - 1);
    return c;
}
__device__ __forceinline__ int localHash(const SceneDev& S, int3 c) { return c.x * S.gy * S.gz + c.y * S.gz + c.z; }

// Pos2GridHash (helper_thrust.cuh:66-89) into the global cell space; parking
// slots (w = 0) get the scene's parking cell. A non-finite position sets bit 0
// of the error word.
__device__ __forceinline__ unsigned int slotKey(const SceneDev& S, float4 p, unsigned int* errWord) {
    if (p.w == 0.f) return unsigned(S.cell_off + S.ncell);
    const float3 q = make_float3(p.x, p.y, p.z);
    if (!(isfinite(q.x) && isfinite(q.y) && isfinite(q.z))) atomicOr(errWord, 1u);
    return unsigned(S.cell_off + localHash(S, cellOf(S, q)));
}

// Poly6Kernel::operator() (cuda_sph_kernel.cuh:90-97)
__device__ __forceinline__ float poly6(const SceneDev& S, float r) {
    float r2 = r * r;
    if (r2 >= S.h2) return 0.f;
    float d = S.h2 - r2;
    return S.poly6 * d * d * d;
}
// SpikyKernelGrad::operator() (cuda_sph_kernel.cuh:110-117)
__device__ __forceinline__ float3 spikyGrad(const SceneDev& S, float3 r) {
    float rlen = len3(r);
    if (rlen >= S.h || rlen < kEps) return mk3(0.f, 0.f, 0.f);
    float d = S.h - rlen;
    return S.spiky * d * d / rlen * r;
}
// AdhesionAkinci13::operator() (cuda_sph_kernel.cuh:196-202). The fourth
// root is taken as two IEEE square roots (within one ulp of x^(1/4), as close
// as powf(x, 0.25f) and a fraction of its cost); the water adhesion it feeds
// is checked against the reference arithmetic within a tolerance.
__device__ __forceinline__ float adhesionSpline(const SceneDev& S, float r) {
    if (2.f * r > S.h && r <= S.h) return S.adh_coef * sqrtf(sqrtf(-4.f * r * r / S.h + 6.f * r - 2.f * S.h));
    return 0.f;
}
// QuadraticBezierCoeff::operator() (cuda_sf_utils.cuh:57-82)
__device__ __forceinline__ float bezier(const BezierDev& G, float sr) {
    if (sr < 0.f) return G.py0;
    if (sr >= 1.f) return G.py2;
    if (sr <= G.px1) {
        const float t = sr / G.px1;
        const float omt = 1.f - t;
        return omt * omt * G.py0 + 2.f * t * omt * G.py1 + t * t * G.py1;
    }
    const float t = (G.b + sqrtf(G.c + G.d * (G.px1 - sr))) / G.e;
    const float omt = 1.f - t;
    return omt * omt * G.py1 + 2.f * t * omt * G.py1 + t * t * G.py2;
}

// ComputeDemForces (cuda_dem_solver_common_gpu.cuh:20-51); max_fs uses the
// host-computed powf(tanFrictionAngle, 2).
__device__ __forceinline__ float3 demForce(float3 dij, float3 vij, float rij, float kn, float ks, float tan2) {
    float3 f = mk3(0.f, 0.f, 0.f);
    float dist = len3(dij);
    float pen = rij - dist;
    if (pen > 0.f) {
        float3 n = dij / dist;
        float de = dot3(vij, n);
        float3 vt = vij - de * n;
        float3 fn = kn * pen * n;
        float3 fs = -ks * vt;
        float max_fs = dot3(fn, fn) * tan2;
        if (dot3(fs, fs) > max_fs) {
            float ratio = sqrtf(max_fs) / len3(fs);
            fs = fs * ratio;
        }
        f = -fn - fs;
    }
    return f;
}

// ComputeDemCapillaryForces (cuda_dem_solver_common_gpu.cuh:53-90) for the
// uniform sand radius; the radius-only constants come from SceneDev.
__device__ __forceinline__ float3 capillaryForce(const SceneDev& S, float3 dij, float sr) {
    float3 f = mk3(0.f, 0.f, 0.f);
    const float r = S.dem_radius;
    float dist = len3(dij);
    float H = dist - (r + r);
    if (H < S.cap_srupt && H > 0.f) {
        float3 N = dij / dist;
        float coeff = bezier(S.capG, sr);
        float d = -H + sqrtf(H * H + S.cap_vlb_pir);
        float phi = sqrtf(2.f * H / r * (-1.f + sqrtf(1.f + S.cap_vlb / (S.cap_pir * H * H))));
        float ncp = S.cap_m2pi * coeff * r * S.cap_cos / (1.f + H / (2.f * d));
        float stf = S.cap_m2pi * coeff * r * phi * S.cap_sin;
        f = -N * (ncp + stf);
    }
    return f;
}

}  // namespace sfg
