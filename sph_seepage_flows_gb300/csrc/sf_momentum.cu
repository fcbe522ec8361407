// Momentum passes of the GB300 seepage-flow substep (sand and water linear
// momentum, cuda_sph_sf_solver_gpu.cuh:723-950), in a translation unit of
// their own. Their per-neighbour terms are evaluated together, so their sums
// are in a different order from the reference's sub-loops and are checked
// against the reference arithmetic within a tolerance (1e-5 of the sum of
// term magnitudes), not bit for bit.
#include "sf_device.cuh"
#include "sf_kernels.h"
#include "sf_neighbors.cuh"

namespace sfg {

// ---------------------------------------------------------- sand momentum
// Both momentum passes run with a register budget of 48 (5 blocks of
// kSlotAlign threads per SM): their neighbour gathers are latency bound and
// gain more from the occupancy than they lose to the values moved to the stack.
// Compute[Multi]SFSandLinearMomentum_CUDA (cuda_sph_sf_solver_gpu.cuh:723-897):
// DEM and capillary terms of sand neighbours (21-50, 83-109), buoyancy and
// adhesion terms of water neighbours (240-273, 314-341), DEM against shape
// boundary particles (52-81) and ComputeDemWorldBoundaryForces
// (cuda_dem_solver_common_gpu.cuh:132-199). acc = g + 2 (f + df) / m.
template <int G>
__global__ void __launch_bounds__(kSlotAlign, 5) kSandMomentum(
    const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene, NbrLists L,
    const float4* __restrict__ pos4, const float4* __restrict__ vel4, const float4* __restrict__ aux4,
    const float4* __restrict__ flow4, const float4* __restrict__ avgadh4, const float4* __restrict__ mat4,
    const float4* __restrict__ bpos4, float2* __restrict__ dp, const float4* __restrict__ grec4,
    float4* __restrict__ drag4, float4* __restrict__ acc4) {
    SF_SLOT_PROLOGUE_G
    const float4 pi4 = pos4[slot];
    if (!(pi4.w < 0.f)) {
        if (pi4.w > 0.f && part == 0) drag4[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float3 pi = xyz(pi4);
    const float mi = -pi4.w;
    const float4 vi4 = vel4[slot];
    const float3 vi = xyz(vi4);
    const float di = vi4.w;
    const float4 ai = aux4[slot];
    const float vol_i = mi / fmaxf(kEps, di);
    float v_w = 0.f;
    float3 f = mk3(0.f, 0.f, 0.f), df = f;
    // DEM and capillary terms vanish beyond contact + liquid-bridge reach:
    // iterate the contact list (or the sand list when it overflowed)
    auto contact = [&](int j) {
        const float3 dij = xyz(pos4[j]) - pi;
        const float4 gj = grec4[j];  // (velocity, saturation)
        f += demForce(dij, xyz(gj) - vi, S.rij2, S.kn, S.ks, S.tan2);
        f += capillaryForce(S, dij, (ai.z + gj.w) / 2.f);
    };
    const int cc = L.ccnt[slot];
    if (cc <= kMaxContact) {
        const unsigned* __restrict__ p = L.cnbr + slot;
#pragma unroll 2
        for (int k = part; k < cc; k += G) contact(int(p[k * L.M]));
    } else {
        forSandNeighbors<G>(S, L, slot, pi, pos4, [&](int j) {
            if (j == slot) return;
            const float3 dij = xyz(pos4[j]) - pi;
            if (dot3(dij, dij) < S.dem_reach2) contact(j);
        }, part);
    }
    forWaterNeighbors<G, true>(S, L, slot, pi, pos4, [&](int j) {
        const float4 pj = pos4[j];
        const float3 dij = pi - xyz(pj);
        const float4 aj = aux4[j];
        const float4 gj = avgadh4[j];  // (average adhesion, D)
        const float wij = poly6(S, len3(dij));
        if (aj.w > 0.f && aj.w <= 1.f) {
            const float dj = gj.w;
            v_w += pj.w / dj * wij;
            f += -mi * pj.w * aj.x / fmaxf(kEps, di * dj) * spikyGrad(S, dij);
        }
        f += wij * vol_i * xyz(gj);
    }, part);
    if (S.shape_boundary) {
        forBoundaryNeighbors<G>(S, L, slot, pi, bpos4, [&](int b) {
            const float4 bj = bpos4[b];
            if (bj.w < 0.f) f += demForce(pi - xyz(bj), mk3(-vi.x, -vi.y, -vi.z), S.rij2, S.kn, S.ks, S.tan2);
        }, part);
    }
    f = groupSum3<G>(f);
    v_w = groupSum<G>(v_w);
    if (part != 0) return;
    // ComputeDemWorldBoundaryForces; the z-min wall tests 2 * rij (DEM:191)
    {
        const float rij = S.wall_rij;
        const float3 nv = -vi;
        if (pi.x > S.hpx - rij) f += demForce(mk3(1.f, 0.f, 0.f) * fabsf(pi.x - S.hpx), nv, rij, S.kn, S.ks, S.tan2);
        if (pi.x < S.lpx + rij) f += demForce(mk3(-1.f, 0.f, 0.f) * fabsf(pi.x - S.lpx), nv, rij, S.kn, S.ks, S.tan2);
        if (pi.y > S.hpy - rij) f += demForce(mk3(0.f, 1.f, 0.f) * fabsf(pi.y - S.hpy), nv, rij, S.kn, S.ks, S.tan2);
        if (pi.y < S.lpy + rij) f += demForce(mk3(0.f, -1.f, 0.f) * fabsf(pi.y - S.lpy), nv, rij, S.kn, S.ks, S.tan2);
        if (pi.z > S.hpz - rij) f += demForce(mk3(0.f, 0.f, 1.f) * fabsf(pi.z - S.hpz), nv, rij, S.kn, S.ks, S.tan2);
        if (pi.z < S.lpz + 2.f * rij)
            f += demForce(mk3(0.f, 0.f, -1.f) * fabsf(pi.z - S.lpz), nv, rij, S.kn, S.ks, S.tan2);
    }
    const float eps_i = ai.w;
    if (eps_i < 1.f && eps_i > 0.f) {
        const float cd = S.multi ? mat4[slot].x : S.cd;
        const float dragCoeff = cd * powf(eps_i, 3.f) / powf(1.f - eps_i, 2.f);
        if (dragCoeff != 0.f)
            df = S.grav_abs * S.rho0 * powf(eps_i, 2.f) / dragCoeff * (xyz(flow4[slot]) - vi) * mi / di;
    }
    const float3 avgDrag = v_w != 0.f ? df / v_w : mk3(0.f, 0.f, 0.f);
    // w: the density, which the water momentum pass gathers with the drag
    drag4[slot] = make_float4(avgDrag.x, avgDrag.y, avgDrag.z, di);
    reinterpret_cast<float*>(dp + slot)[1] = v_w;  // the average's denominator, for the adjoint
    const float3 g = mk3(0.f, 0.f, 0.f) + mk3(S.gvx, S.gvy, S.gvz);
    const float3 a = g + 2.f * (f + df) / mi;
    acc4[slot] = make_float4(a.x, a.y, a.z, 0.f);
}

// --------------------------------------------------------- water momentum
// ComputeSFWaterLinearMomentum_CUDA (cuda_sph_sf_solver_gpu.cuh:899-950):
// pressure and artificial viscosity of water neighbours (343-406), seepage
// terms of sand neighbours (275-312), boundary pressure and viscosity
// (cuda_sph_solver_common_gpu.cuh:89-139, called with rho0 as the particle
// density). acc = g + (a - F_adh / m). Every thread then contributes |acc|
// of its slot (sand included) to the scene maximum (cuda_wcsph_sf_solver.cu:43-47).
template <int G>
__global__ void __launch_bounds__(kSlotAlign, 5) kWaterMomentum(
    const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene, SceneState* __restrict__ state,
    NbrLists L, const float4* __restrict__ pos4, const float4* __restrict__ vel4, const float4* __restrict__ aux4,
    const float4* __restrict__ drag4, const float4* __restrict__ adh4, const float4* __restrict__ bpos4,
    const float2* __restrict__ dp, const float4* __restrict__ grec4, float4* __restrict__ acc4,
    unsigned int* errWord) {
    SF_SLOT_PROLOGUE_G
    const float4 pi4 = pos4[slot];
    float alen = 0.f;
    if (pi4.w > 0.f) {
        const float3 pi = xyz(pi4);
        const float4 vi4 = vel4[slot];
        const float3 vi = xyz(vi4);
        const float2 dpi = dp[slot];
        const float di = dpi.x;
        const float pri = aux4[slot].x;
        const float pterm_i = dpi.y;
        float3 a = mk3(0.f, 0.f, 0.f);
        forWaterNeighbors<G, true>(S, L, slot, pi, pos4, [&](int j) {
            if (j == slot) return;
            const float4 pj = pos4[j];
            const float4 gj = grec4[j];  // (velocity, P)
            // D of the neighbour, loaded with its position and record for
            // every pair (only approaching pairs use it): its latency then
            // overlaps the pressure term instead of stalling inside the
            // viscosity branch
            const float dj = dp[j].x;
            const float3 dij = pi - xyz(pj);
            const float3 nab = spikyGrad(S, dij);
            a += -pj.w * (pterm_i + gj.w) * nab;
            const float dd = dot3(vi - xyz(gj), dij);
            if (dd < 0.f) {
                const float pij = -S.nu / (di + dj) * (dd / (dot3(dij, dij) + kEps));
                a += -pj.w * pij * nab;
            }
        }, part);
        forSandNeighbors<G, true>(S, L, slot, pi, pos4, [&](int j) {
            const float4 pj = pos4[j];
            const float3 dij = pi - xyz(pj);
            const float4 dragj = drag4[j];  // (average drag, density)
            const float dj = dragj.w;
            const float wij = poly6(S, len3(dij));
            const float3 nab = spikyGrad(S, dij);
            const float3 buoy = pj.w * pri / fmaxf(kEps, di * dj) * nab;  // -m_j with m_j = -w
            const float3 drag = -wij / di * xyz(dragj);
            a += buoy + drag;
        }, part);
        const float bp = pri / fmaxf(kEps, S.rho0 * S.rho0);
        const float bvis = -S.bnu / (2.f * S.rho0);
        forBoundaryNeighbors<G>(S, L, slot, pi, bpos4, [&](int b) {
            const float4 bj = bpos4[b];
            const float3 dij = pi - xyz(bj);
            const float3 nab = spikyGrad(S, dij);
            a += -S.rho0 * fabsf(bj.w) * bp * nab;
            const float dd = dot3(vi, dij);
            if (dd < 0.f) {
                const float pij = bvis * (dd / (dot3(dij, dij) + kEps));
                a += -fabsf(bj.w) * S.rho0 * pij * nab;
            }
        }, part);
        a = groupSum3<G>(a);
        if (part == 0) {
            const float3 g = mk3(0.f, 0.f, 0.f) + mk3(S.gvx, S.gvy, S.gvz);
            const float3 acc = g + (a - xyz(adh4[slot]) / pi4.w);
            acc4[slot] = make_float4(acc.x, acc.y, acc.z, 0.f);
            alen = len3(acc);
        }
    } else if (pi4.w < 0.f && part == 0) {
        alen = len3(xyz(acc4[slot]));
    }
    if (!(alen <= 3.0e38f) && pi4.w != 0.f) atomicOr(errWord, 1u);
    // block max of |acc| (non-negative floats order like their bit patterns)
    float m = (alen == alen) ? alen : 0.f;
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wmax[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmax[warp] = m;
    __syncthreads();
    if (warp == 0) {
        m = lane < int(blockDim.x >> 5) ? wmax[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0 && m > 0.f) atomicMax(&state[sid].amax_bits, __float_as_uint(m));
    }
}

// ------------------------------------------------------------ launchers
// Blocks of a tuned pass over all slots.
static inline int grid(const LaunchCtx& c, int pass) { return c.slotBlocks * (kSlotAlign / c.block[pass]); }

template <int G> void launchSandMomentumG(const LaunchCtx& c, const PassBuffers& b) {
    kSandMomentum<G><<<grid(c, kPassSand) * G, c.block[kPassSand], 0, c.stream>>>(
        c.scenes, c.blockScene, b.lists, b.pos4, b.vel4, b.aux4, b.flow4, b.avgadh4, b.mat4, b.bpos4, b.dp, b.grec4,
        b.drag4, b.acc4);
}
void launchSandMomentum(const LaunchCtx& c, const PassBuffers& b) {
    switch (c.lanes) {
    case 2: launchSandMomentumG<2>(c, b); break;
    case 4: launchSandMomentumG<4>(c, b); break;
    case 8: launchSandMomentumG<8>(c, b); break;
    default: launchSandMomentumG<1>(c, b); break;
    }
}

template <int G> void launchWaterMomentumG(const LaunchCtx& c, const PassBuffers& b) {
    kWaterMomentum<G><<<grid(c, kPassWater) * G, c.block[kPassWater], 0, c.stream>>>(
        c.scenes, c.blockScene, c.state, b.lists, b.pos4, b.vel4, b.aux4, b.drag4, b.adh4, b.bpos4, b.dp, b.grec4,
        b.acc4, c.errWord);
}
void launchWaterMomentum(const LaunchCtx& c, const PassBuffers& b) {
    switch (c.lanes) {
    case 2: launchWaterMomentumG<2>(c, b); break;
    case 4: launchWaterMomentumG<4>(c, b); break;
    case 8: launchWaterMomentumG<8>(c, b); break;
    default: launchWaterMomentumG<1>(c, b); break;
    }
}

}  // namespace sfg
