// Reverse-mode adjoint of the fixed-dt substep.
//
// The adjoint of one substep runs after the forward stages sort .. water
// momentum of that substep were recomputed from its stored input state, so
// the neighbour lists and every intermediate field are those of the forward
// pass. It walks the dependency levels of the substep backwards:
//
//   A1 integrate        x' = x + dt v',  v' = v + dt a'  (sand: damped a)
//   A2 water momentum   a_w(x, v, rho, p, eps; sand drag, adhesion)
//   A3 sand momentum    a_s = g + 2 (f + df) / m, avg drag = df / v_w
//   A4 voidage/adhesion sand voidage, water adhesion and average adhesion
//   A5 average flow     sand average flow and saturation, fluid voidage
//   A6 density          water density (+ boundary) and pressure
//
// Every level is a gather: thread k collects every cotangent that lands on
// particle k, both from the terms of its own outputs and from the terms in
// which k is the neighbour of an output particle i. The latter are found by
// walking k's own neighbour list (the lists are symmetric), so no
// per-particle cotangent is written by two threads and no atomics are
// needed; a pair term is evaluated once from each end. Pair Jacobians come
// from forward-mode dual numbers (sf_dual.cuh) over the few inputs each pair
// term has; the vector-Jacobian product is their contraction with the
// output cotangent. Branch conditions (contact, friction cap, damping sign,
// positive voidage, water clamp) are taken from the forward values.
//
// Cotangents of positions and velocities between substeps are kept by
// particle id (scene slot_off + id), so the sort needs no bookkeeping.
// Parameter cotangents are reduced per block and summed by the host in
// block order. Parameters: tan friction angle, capillary scale (multiplies
// the capillary Bezier values c0, cmc, csat) and permeability scale
// (multiplies cd). The push-out of water from shape-boundary particles in
// the integrator is held constant (no cotangent through it).
#include "sf_adjoint.h"
#include "sf_dual.cuh"
#include "sf_neighbors.cuh"

namespace sfg {

#define SF_ADJ_PROLOGUE                                                    \
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;                \
    const int sid = blockScene[(blockIdx.x * blockDim.x) / kSlotAlign];    \
    const SceneDev& S = scenes[sid];

// ------------------------------------------------------- dual helpers
template <int K> __device__ __forceinline__ V3T<Dual<K>> dvec(float3 a, int k0) {
    return v3(dseed<K>(a.x, k0), dseed<K>(a.y, k0 + 1), dseed<K>(a.z, k0 + 2));
}
template <int K> __device__ __forceinline__ V3T<Dual<K>> dvecc(float3 a) {
    return v3(dconst<K>(a.x), dconst<K>(a.y), dconst<K>(a.z));
}
// u . (d out / d seed k) for a vector output
template <int K> __device__ __forceinline__ float vjp(float3 u, const V3T<Dual<K>>& o, int k) {
    return u.x * o.x.d[k] + u.y * o.y.d[k] + u.z * o.z.d[k];
}
template <int K> __device__ __forceinline__ float3 vjp3(float3 u, const V3T<Dual<K>>& o, int k0) {
    return mk3(vjp(u, o, k0), vjp(u, o, k0 + 1), vjp(u, o, k0 + 2));
}
template <int K> __device__ __forceinline__ float3 grad3(const Dual<K>& o, int k0) {
    return mk3(o.d[k0], o.d[k0 + 1], o.d[k0 + 2]);
}
__device__ __forceinline__ void add3(float4& a, float3 b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
}
__device__ __forceinline__ float4 f4(float3 a, float w = 0.f) { return make_float4(a.x, a.y, a.z, w); }

// Block sum of two values; every thread of the block must call it.
__device__ __forceinline__ float2 blockSum2(float a, float b) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __shared__ float2 w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = make_float2(a, b);
    __syncthreads();
    float2 s = make_float2(0.f, 0.f);
    if (threadIdx.x == 0)
        for (int k = 0; k < int(blockDim.x >> 5); ++k) {
            s.x += w[k].x;
            s.y += w[k].y;
        }
    return s;  // valid in thread 0
}

// ----------------------------------------------------------- pair terms
// The forward terms as templates on the scalar type (values identical to the
// forward kernels in sf_kernels.cu; only their derivatives are used here).

// Pressure + artificial viscosity on water i from water j
// (cuda_sph_sf_solver_gpu.cuh:343-406); d = x_i - x_j, dv = v_i - v_j.
template <typename T>
__device__ __forceinline__ V3T<T> waterPairT(const SceneDev& S, V3T<T> d, V3T<T> dv, T rhoI, T pI, T epsI, T rhoJ,
                                             T pJ, T epsJ, float mj) {
    const T di = rhoI / tmaxc(kEps, epsI);
    const T dj = rhoJ / tmaxc(kEps, epsJ);
    const V3T<T> nab = spikyGradT(S, d);
    V3T<T> a = (-mj * (pI / tmaxc(kEps, di * di) + pJ / tmaxc(kEps, dj * dj))) * nab;
    const T dd = dotT(dv, d);
    if (val(dd) < 0.f) {
        const T pij = (-S.nu / (di + dj)) * (dd / (dotT(d, d) + kEps));
        a = a + (-mj * pij) * nab;
    }
    return a;
}
// Buoyancy + drag on water i from sand j (275-312); d = x_i - x_j.
template <typename T>
__device__ __forceinline__ V3T<T> seepageT(const SceneDev& S, V3T<T> d, T pI, T rhoI, T epsI, float rhoJ,
                                           V3T<T> dragJ, float mj) {
    const T di = rhoI / tmaxc(kEps, epsI);
    const T wij = poly6T(S, lenT(d));
    const V3T<T> nab = spikyGradT(S, d);
    return (-mj * pI / tmaxc(kEps, di * rhoJ)) * nab + (-wij / di) * dragJ;
}
// Boundary pressure + viscosity on water i (cuda_sph_solver_common_gpu.cuh:
// 89-139 with rho0 as the density); d = x_i - x_b.
template <typename T>
__device__ __forceinline__ V3T<T> boundaryT(const SceneDev& S, V3T<T> d, V3T<T> vI, T pI, float vol) {
    const V3T<T> nab = spikyGradT(S, d);
    V3T<T> a = (-S.rho0 * vol * (pI / fmaxf(kEps, S.rho0 * S.rho0))) * nab;
    const T dd = dotT(vI, d);
    if (val(dd) < 0.f) {
        const T pij = (-S.bnu / (2.f * S.rho0)) * (dd / (dotT(d, d) + kEps));
        a = a + (-vol * S.rho0 * pij) * nab;
    }
    return a;
}
// DEM + capillary force on sand i from sand j (21-50, 83-109); d = x_j - x_i, dv = v_j - v_i.
template <typename T>
__device__ __forceinline__ V3T<T> contactT(const SceneDev& S, V3T<T> d, V3T<T> dv, T satI, T satJ, T tanPhi,
                                           T capScale) {
    return demForceT(d, dv, S.rij2, S.kn, S.ks, tanPhi * tanPhi) + capillaryForceT(S, d, (satI + satJ) / 2.f, capScale);
}
// Buoyancy + adhesion on sand i from water j (240-273, 314-341); d = x_i - x_j.
template <typename T>
__device__ __forceinline__ V3T<T> sandWaterT(const SceneDev& S, V3T<T> d, float mi, float rhoI, T pJ, T rhoJ, T epsJ,
                                             V3T<T> avgAdhJ, float mj) {
    const T wij = poly6T(S, lenT(d));
    V3T<T> f = d * 0.f;
    if (val(epsJ) > 0.f && val(epsJ) <= 1.f) {
        const T dj = rhoJ / tmaxc(kEps, epsJ);
        f = (-mi * mj * pJ / tmaxc(kEps, rhoI * dj)) * spikyGradT(S, d);
    }
    return f + (wij * (mi / fmaxf(kEps, rhoI))) * avgAdhJ;
}
// Water j's term of v_w of sand i; d = x_i - x_j.
template <typename T>
__device__ __forceinline__ T vwTermT(const SceneDev& S, V3T<T> d, T rhoJ, T epsJ, float mj) {
    if (!(val(epsJ) > 0.f && val(epsJ) <= 1.f)) return lenT(d) * 0.f;
    return (mj / (rhoJ / tmaxc(kEps, epsJ))) * poly6T(S, lenT(d));
}
// ComputeDemWorldBoundaryForces on sand i (cuda_dem_solver_common_gpu.cuh:132-199).
template <typename T>
__device__ __forceinline__ V3T<T> wallsT(const SceneDev& S, V3T<T> p, V3T<T> v, T tanPhi) {
    const float rij = S.wall_rij;
    const T tan2 = tanPhi * tanPhi;
    const V3T<T> nv = -v;
    const T z = p.x * 0.f;
    V3T<T> f = v3(z, z, z);
    if (val(p.x) > S.hpx - rij) f = f + demForceT(v3(tabs(p.x - S.hpx), z, z), nv, rij, S.kn, S.ks, tan2);
    if (val(p.x) < S.lpx + rij) f = f + demForceT(v3(-tabs(p.x - S.lpx), z, z), nv, rij, S.kn, S.ks, tan2);
    if (val(p.y) > S.hpy - rij) f = f + demForceT(v3(z, tabs(p.y - S.hpy), z), nv, rij, S.kn, S.ks, tan2);
    if (val(p.y) < S.lpy + rij) f = f + demForceT(v3(z, -tabs(p.y - S.lpy), z), nv, rij, S.kn, S.ks, tan2);
    if (val(p.z) > S.hpz - rij) f = f + demForceT(v3(z, z, tabs(p.z - S.hpz)), nv, rij, S.kn, S.ks, tan2);
    if (val(p.z) < S.lpz + 2.f * rij) f = f + demForceT(v3(z, z, -tabs(p.z - S.lpz)), nv, rij, S.kn, S.ks, tan2);
    return f;
}
// Drag df of sand i (cuda_sph_sf_solver_gpu.cuh:880-887).
template <typename T>
__device__ __forceinline__ V3T<T> dragT(const SceneDev& S, T eps, V3T<T> flow, V3T<T> v, float m, float rho, float cd,
                                        T permScale) {
    if (!(val(eps) < 1.f && val(eps) > 0.f)) return v * 0.f;
    const T dragCoeff = (cd * permScale) * tpow(eps, 3.f) / tpow(1.f - eps, 2.f);
    if (val(dragCoeff) == 0.f) return v * 0.f;
    return ((S.grav_abs * S.rho0) * tpow(eps, 2.f) / dragCoeff) * (flow - v) * m / rho;
}
// Adhesion on water i from sand j (175-207, 574-678); d = x_i - x_j.
template <typename T>
__device__ __forceinline__ V3T<T> adhesionT(const SceneDev& S, V3T<T> d, T satJ, float mi, float mj) {
    const T l = lenT(d);
    return (bezierT(S.adhG, satJ, 1.f) * mi * mj * adhesionSplineT(S, l)) * d / tmaxc(kEps, l);
}
// Gradient of W(|d|) with respect to d.
__device__ __forceinline__ float3 poly6Grad(const SceneDev& S, float3 d) {
    return grad3(poly6T(S, lenT(dvec<3>(d, 0))), 0);
}

// ------------------------------------------------------------- kernels
__global__ void kAdjSeed(const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene,
                         const float4* __restrict__ pos4, const int* __restrict__ pid,
                         const float* __restrict__ target, float4* __restrict__ adjX, float4* __restrict__ adjV,
                         float2* __restrict__ lossPartial) {
    SF_ADJ_PROLOGUE
    const float4 p = pos4[slot];
    float l = 0.f, ns = 0.f;
    if (p.w != 0.f) {
        const int id = S.slot_off + pid[slot];
        float3 g = mk3(0.f, 0.f, 0.f);
        if (p.w < 0.f) {
            const float3 d = xyz(p) - mk3(target[3 * id], target[3 * id + 1], target[3 * id + 2]);
            l = dot3(d, d);
            ns = 1.f;
            g = 2.f * d;
        }
        adjX[id] = f4(g);
        adjV[id] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float2 t = blockSum2(l, ns);
    if (threadIdx.x == 0) lossPartial[blockIdx.x] = t;
}

// A1: CudaSFParticles::Advect with the damping sign and the clamp of the forward values.
__global__ void kAdjIntegrate(const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene, AdjBuffers A,
                              PassBuffers b, const int* __restrict__ pid, float dt) {
    SF_ADJ_PROLOGUE
    const float4 p4 = b.pos4[slot];
    if (p4.w == 0.f) return;
    const int id = S.slot_off + pid[slot];
    float3 xb = xyz(A.adjX[id]), vb = xyz(A.adjV[id]);
    const float3 a = xyz(b.acc4[slot]), v = xyz(b.vel4[slot]);
    float3 damp = mk3(1.f, 1.f, 1.f);
    if (p4.w < 0.f) {
        const float3 q = a * (v + 0.5f * dt * a);
        damp = mk3(1.f, 1.f, 1.f) - S.damping * mk3(float(sgn1(q.x)), float(sgn1(q.y)), float(sgn1(q.z)));
    } else {  // SFWaterBoundaryConstrain_CUDA: clamped components carry no cotangent
        const float3 vn = v + dt * a;
        const float3 pn = xyz(p4) + dt * vn;
        const float r2 = 2.f * S.sph_radius;
        if (pn.x > S.hpx - r2) { xb.x = 0.f; if (vn.x > 0.f) vb.x = 0.f; }
        else if (pn.x < S.lpx + r2) { xb.x = 0.f; if (vn.x < 0.f) vb.x = 0.f; }
        if (pn.y > S.hpy - r2) { xb.y = 0.f; if (vn.y > 0.f) vb.y = 0.f; }
        else if (pn.y < S.lpy + r2) { xb.y = 0.f; if (vn.y < 0.f) vb.y = 0.f; }
        if (pn.z > S.hpz - r2) { xb.z = 0.f; if (vn.z > 0.f) vb.z = 0.f; }
        else if (pn.z < S.lpz + r2) { xb.z = 0.f; if (vn.z < 0.f) vb.z = 0.f; }
    }
    const float3 vnb = vb + dt * xb;  // cotangent of v'
    A.acc[slot] = f4((dt * vnb) * damp);
    A.x[slot] = f4(xb);
    A.v[slot] = f4(vnb);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    A.s[slot] = z;
    A.flow[slot] = z;
    A.adh[slot] = z;
    A.avgadh[slot] = z;
    A.drag[slot] = z;
}

// A2: water momentum (acc = g + a - F_adh / m).
__global__ void __launch_bounds__(kSlotAlign) kAdjWater(const SceneDev* __restrict__ scenes,
                                                        const int* __restrict__ blockScene, AdjBuffers A,
                                                        PassBuffers b) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const NbrLists& L = b.lists;
    const float3 xk = xyz(pk4), vk = xyz(b.vel4[slot]);
    const float rhoK = b.vel4[slot].w, pK = b.aux4[slot].x, epsK = b.aux4[slot].w;
    float3 gx = mk3(0.f, 0.f, 0.f), gv = gx;
    float grho = 0.f, gp = 0.f, geps = 0.f;
    if (pk4.w > 0.f) {
        const float mk = pk4.w;
        const float3 ak = xyz(A.acc[slot]);
        A.adh[slot] = f4(ak / -mk);
        forWaterNeighbors(S, L, slot, xk, b.pos4, [&](int j) {
            if (j == slot) return;
            const float4 pj4 = b.pos4[j];
            const float3 xj = xyz(pj4), vj = xyz(b.vel4[j]);
            const float rhoJ = b.vel4[j].w, pJ = b.aux4[j].x, epsJ = b.aux4[j].w;
            {   // own term a_k(k, j); seeds d 0-2, dv 3-5, rho_k 6, p_k 7, eps_k 8
                const auto o = waterPairT<Dual<9>>(S, dvec<9>(xk - xj, 0), dvec<9>(vk - vj, 3), dseed<9>(rhoK, 6),
                                                   dseed<9>(pK, 7), dseed<9>(epsK, 8), dconst<9>(rhoJ),
                                                   dconst<9>(pJ), dconst<9>(epsJ), pj4.w);
                gx += vjp3(ak, o, 0);
                gv += vjp3(ak, o, 3);
                grho += vjp(ak, o, 6);
                gp += vjp(ak, o, 7);
                geps += vjp(ak, o, 8);
            }
            {   // k as the neighbour in a_j(j, k): d = x_j - x_k, dv = v_j - v_k
                const float3 aj = xyz(A.acc[j]);
                const auto o = waterPairT<Dual<9>>(S, dvec<9>(xj - xk, 0), dvec<9>(vj - vk, 3), dconst<9>(rhoJ),
                                                   dconst<9>(pJ), dconst<9>(epsJ), dseed<9>(rhoK, 6),
                                                   dseed<9>(pK, 7), dseed<9>(epsK, 8), mk);
                gx += -vjp3(aj, o, 0);
                gv += -vjp3(aj, o, 3);
                grho += vjp(aj, o, 6);
                gp += vjp(aj, o, 7);
                geps += vjp(aj, o, 8);
            }
        });
        forSandNeighbors(S, L, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            // seeds d 0-2, p_k 3, rho_k 4, eps_k 5
            const auto o = seepageT<Dual<6>>(S, dvec<6>(xk - xyz(pj4), 0), dseed<6>(pK, 3), dseed<6>(rhoK, 4),
                                             dseed<6>(epsK, 5), b.vel4[j].w, dvecc<6>(xyz(b.drag4[j])), -pj4.w);
            gx += vjp3(ak, o, 0);
            gp += vjp(ak, o, 3);
            grho += vjp(ak, o, 4);
            geps += vjp(ak, o, 5);
        });
        forBoundaryNeighbors(S, L, slot, xk, b.bpos4, [&](int bb) {
            const float4 bj = b.bpos4[bb];
            const auto o = boundaryT<Dual<7>>(S, dvec<7>(xk - xyz(bj), 0), dvec<7>(vk, 3), dseed<7>(pK, 6), fabsf(bj.w));
            gx += vjp3(ak, o, 0);
            gv += vjp3(ak, o, 3);
            gp += vjp(ak, o, 6);
        });
    } else {
        // sand k in the seepage term of water i: d = x_i - x_k; seeds d 0-2, drag_k 3-5
        const float mk = -pk4.w;
        const float3 dragK = xyz(b.drag4[slot]);
        float3 gdrag = mk3(0.f, 0.f, 0.f);
        forWaterNeighbors(S, L, slot, xk, b.pos4, [&](int i) {
            const float4 pi4 = b.pos4[i];
            const float3 ai = xyz(A.acc[i]);
            const auto o = seepageT<Dual<6>>(S, dvec<6>(xyz(pi4) - xk, 0), dconst<6>(b.aux4[i].x),
                                             dconst<6>(b.vel4[i].w), dconst<6>(b.aux4[i].w), rhoK,
                                             dvec<6>(dragK, 3), mk);
            gx += -vjp3(ai, o, 0);
            gdrag += vjp3(ai, o, 3);
        });
        A.drag[slot] = f4(gdrag);
    }
    add3(A.x[slot], gx);
    add3(A.v[slot], gv);
    float4 s = A.s[slot];
    s.x += grho;
    s.y += gp;
    s.z += geps;
    A.s[slot] = s;
}

// A3a: per sand particle: v_w, drag, walls and shape-boundary DEM; writes
// (f-bar, v_w-bar) and adds the friction / permeability parameter partials.
__global__ void __launch_bounds__(kSlotAlign) kAdjSandSelf(const SceneDev* __restrict__ scenes,
                                                           const int* __restrict__ blockScene, AdjBuffers A,
                                                           PassBuffers b, float* __restrict__ paramPartial) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    float gTan = 0.f, gPerm = 0.f;
    if (pk4.w < 0.f) {
        const float mk = -pk4.w;
        const float3 xk = xyz(pk4), vk = xyz(b.vel4[slot]);
        const float rhoK = b.vel4[slot].w, epsK = b.aux4[slot].w;
        const float tanPhi = sqrtf(S.tan2);
        float vw = 0.f;
        forWaterNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            vw += vwTermT<float>(S, v3(d.x, d.y, d.z), b.vel4[j].w, b.aux4[j].w, pj4.w);
        });
        const float3 fb = (2.f / mk) * xyz(A.acc[slot]);
        const float3 dragB = xyz(A.drag[slot]);
        // df; seeds eps 0, flow 1-3, v 4-6, permeability scale 7
        const float cd = S.multi ? b.mat4[slot].x : S.cd;
        const auto df = dragT<Dual<8>>(S, dseed<8>(epsK, 0), dvec<8>(xyz(b.flow4[slot]), 1), dvec<8>(vk, 4), mk, rhoK,
                                       cd, dseed<8>(1.f, 7));
        float3 dfb = fb;
        float vwb = 0.f;
        if (vw != 0.f) {
            dfb = dfb + dragB / vw;
            vwb = -dot3(dragB, mk3(df.x.v, df.y.v, df.z.v)) / (vw * vw);
        }
        float4 s = A.s[slot];
        s.z += vjp(dfb, df, 0);
        A.s[slot] = s;
        A.flow[slot] = f4(vjp3(dfb, df, 1));
        float3 gv = vjp3(dfb, df, 4);
        gPerm = vjp(dfb, df, 7);
        // world walls; seeds x 0-2, v 3-5, tan phi 6
        const auto w = wallsT<Dual<7>>(S, dvec<7>(xk, 0), dvec<7>(vk, 3), dseed<7>(tanPhi, 6));
        float3 gx = vjp3(fb, w, 0);
        gv += vjp3(fb, w, 3);
        gTan = vjp(fb, w, 6);
        if (S.shape_boundary) {
            forBoundaryNeighbors(S, b.lists, slot, xk, b.bpos4, [&](int bb) {
                const float4 bj = b.bpos4[bb];
                if (!(bj.w < 0.f)) return;
                const auto tp = dseed<7>(tanPhi, 6);
                const auto o = demForceT(dvec<7>(xk - xyz(bj), 0), -dvec<7>(vk, 3), S.rij2, S.kn, S.ks, tp * tp);
                gx += vjp3(fb, o, 0);
                gv += vjp3(fb, o, 3);
                gTan += vjp(fb, o, 6);
            });
        }
        add3(A.x[slot], gx);
        add3(A.v[slot], gv);
        A.f[slot] = f4(fb, vwb);
    }
    const float2 t = blockSum2(gTan, gPerm);
    if (threadIdx.x == 0) {
        paramPartial[3 * blockIdx.x] += t.x;
        paramPartial[3 * blockIdx.x + 2] += t.y;
    }
}

// A3b: sand pair terms (contacts, buoyancy + adhesion, v_w) from both ends.
__global__ void __launch_bounds__(kSlotAlign) kAdjSandPairs(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene, AdjBuffers A,
                                                            PassBuffers b, float* __restrict__ paramPartial) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    float gTan = 0.f, gCap = 0.f;
    if (pk4.w != 0.f) {
        const float3 xk = xyz(pk4), vk = xyz(b.vel4[slot]);
        const float rhoK = b.vel4[slot].w, pK = b.aux4[slot].x, satK = b.aux4[slot].z, epsK = b.aux4[slot].w;
        float3 gx = mk3(0.f, 0.f, 0.f), gv = gx, gadh = gx;
        float gsat = 0.f, grho = 0.f, gp = 0.f, geps = 0.f;
        if (pk4.w < 0.f) {
            const float mk = -pk4.w;
            const float4 fk4 = A.f[slot];
            const float3 fb = xyz(fk4);
            const float tanPhi = sqrtf(S.tan2);
            forSandNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
                if (j == slot) return;
                const float4 pj4 = b.pos4[j];
                const float3 d = xyz(pj4) - xk;
                if (!(dot3(d, d) < S.dem_reach2)) return;
                const float3 vj = xyz(b.vel4[j]);
                const float satJ = b.aux4[j].z;
                {   // own f_k(k, j), d = x_j - x_k; seeds d 0-2, dv 3-5, sat_k 6, tan phi 7, capillary scale 8
                    const auto o = contactT<Dual<9>>(S, dvec<9>(d, 0), dvec<9>(vj - vk, 3), dseed<9>(satK, 6),
                                                     dconst<9>(satJ), dseed<9>(tanPhi, 7), dseed<9>(1.f, 8));
                    gx += -vjp3(fb, o, 0);
                    gv += -vjp3(fb, o, 3);
                    gsat += vjp(fb, o, 6);
                    gTan += vjp(fb, o, 7);
                    gCap += vjp(fb, o, 8);
                }
                {   // k as the neighbour in f_j(j, k), d = x_k - x_j; seeds d 0-2, dv 3-5, sat_k 6
                    const float3 fj = xyz(A.f[j]);
                    const auto o = contactT<Dual<7>>(S, dvec<7>(-1.f * d, 0), dvec<7>(vk - vj, 3), dconst<7>(satJ),
                                                     dseed<7>(satK, 6), dconst<7>(tanPhi), dconst<7>(1.f));
                    gx += vjp3(fj, o, 0);
                    gv += vjp3(fj, o, 3);
                    gsat += vjp(fj, o, 6);
                }
            });
            const float vwb = fk4.w;
            forWaterNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
                const float4 pj4 = b.pos4[j];
                const float3 d = xk - xyz(pj4);
                const float rhoJ = b.vel4[j].w, epsJ = b.aux4[j].w;
                const auto o = sandWaterT<Dual<3>>(S, dvec<3>(d, 0), mk, rhoK, dconst<3>(b.aux4[j].x),
                                                   dconst<3>(rhoJ), dconst<3>(epsJ), dvecc<3>(xyz(b.avgadh4[j])),
                                                   pj4.w);
                gx += vjp3(fb, o, 0);
                if (vwb != 0.f)
                    gx += vwb * grad3(vwTermT<Dual<3>>(S, dvec<3>(d, 0), dconst<3>(rhoJ), dconst<3>(epsJ), pj4.w), 0);
            });
        } else {
            // water k in the buoyancy / adhesion and v_w terms of sand i: d = x_i - x_k
            const float mk = pk4.w;
            const float3 avgAdhK = xyz(b.avgadh4[slot]);
            forSandNeighbors(S, b.lists, slot, xk, b.pos4, [&](int i) {
                const float4 pi4 = b.pos4[i];
                const float4 fi4 = A.f[i];
                const float3 d = xyz(pi4) - xk;
                // seeds d 0-2, p_k 3, rho_k 4, eps_k 5, avg adhesion_k 6-8
                const auto o = sandWaterT<Dual<9>>(S, dvec<9>(d, 0), -pi4.w, b.vel4[i].w, dseed<9>(pK, 3),
                                                   dseed<9>(rhoK, 4), dseed<9>(epsK, 5), dvec<9>(avgAdhK, 6), mk);
                const float3 fi = xyz(fi4);
                gx += -vjp3(fi, o, 0);
                gp += vjp(fi, o, 3);
                grho += vjp(fi, o, 4);
                geps += vjp(fi, o, 5);
                gadh += vjp3(fi, o, 6);
                if (fi4.w != 0.f) {  // seeds d 0-2, rho_k 3, eps_k 4
                    const auto t = vwTermT<Dual<5>>(S, dvec<5>(d, 0), dseed<5>(rhoK, 3), dseed<5>(epsK, 4), mk);
                    gx += -fi4.w * grad3(t, 0);
                    grho += fi4.w * t.d[3];
                    geps += fi4.w * t.d[4];
                }
            });
        }
        add3(A.x[slot], gx);
        add3(A.v[slot], gv);
        add3(A.avgadh[slot], gadh);
        float4 s = A.s[slot];
        s.x += grho;
        s.y += gp;
        s.z += geps;
        s.w += gsat;
        A.s[slot] = s;
    }
    const float2 t = blockSum2(gTan, gCap);
    if (threadIdx.x == 0) {
        paramPartial[3 * blockIdx.x] += t.x;
        paramPartial[3 * blockIdx.x + 1] += t.y;
    }
}

// A4a: sand: voidage = num / den -> (num-bar, den-bar); water: adhesion
// cotangent total (F_adh-bar + avg-bar / v_s) and v_s-bar.
__global__ void __launch_bounds__(kSlotAlign) kAdjVoidSelf(const SceneDev* __restrict__ scenes,
                                                           const int* __restrict__ blockScene, AdjBuffers A,
                                                           PassBuffers b) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const float3 xk = xyz(pk4);
    if (pk4.w < 0.f) {
        float num = 0.f, den = 0.f;
        forWaterNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            const float vj = pj4.w / b.vel4[j].w;
            const float wij = poly6(S, len3(xk - xyz(pj4)));
            num += b.aux4[j].y * vj * wij;
            den += vj * wij;
        });
        const float eb = A.s[slot].z;
        A.r[slot] = den != 0.f ? make_float4(eb / den, -eb * num / (den * den), 0.f, 0.f)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        float vs = 0.f;
        forSandNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            vs += -pj4.w / b.vel4[j].w * poly6(S, len3(xk - xyz(pj4)));
        });
        const float3 avgB = xyz(A.avgadh[slot]);
        float3 tot = xyz(A.adh[slot]);
        float vsb = 0.f;
        if (vs != 0.f) {
            tot = tot + avgB / vs;
            vsb = -dot3(avgB, xyz(b.adh4[slot])) / (vs * vs);
        }
        A.r[slot] = f4(tot, vsb);
    }
}

// A4b: voidage / adhesion pair terms from both ends.
__global__ void __launch_bounds__(kSlotAlign) kAdjVoidPairs(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene, AdjBuffers A,
                                                            PassBuffers b) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const float3 xk = xyz(pk4);
    const float rhoK = b.vel4[slot].w;
    float3 gx = mk3(0.f, 0.f, 0.f);
    float gsat = 0.f, grho = 0.f, geps = 0.f;
    if (pk4.w < 0.f) {
        const float mk = -pk4.w;
        const float4 rk = A.r[slot];
        const float satK = b.aux4[slot].z;
        const float vk = mk / rhoK;
        forWaterNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            // own num / den sums: d = x_k - x_j
            const float vj = pj4.w / b.vel4[j].w;
            gx += (rk.x * b.aux4[j].y * vj + rk.y * vj) * poly6Grad(S, xk - xyz(pj4));
            // k in the adhesion and v_s of water j: d = x_j - x_k; seeds d 0-2, sat_k 3
            const float4 rj = A.r[j];
            const float3 d = xyz(pj4) - xk;
            const auto o = adhesionT<Dual<4>>(S, dvec<4>(d, 0), dseed<4>(satK, 3), pj4.w, mk);
            gx += -vjp3(xyz(rj), o, 0);
            gsat += vjp(xyz(rj), o, 3);
            if (rj.w != 0.f) gx += (-rj.w * vk) * poly6Grad(S, d);
        });
    } else {
        const float mk = pk4.w;
        const float4 rk = A.r[slot];
        const float epsfK = b.aux4[slot].y;
        forSandNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            // own adhesion and v_s terms
            gx += vjp3(xyz(rk), adhesionT<Dual<3>>(S, dvec<3>(d, 0), dconst<3>(b.aux4[j].z), mk, -pj4.w), 0);
            if (rk.w != 0.f) gx += (rk.w * (-pj4.w / b.vel4[j].w)) * poly6Grad(S, d);
            // k in the num / den of sand j: d = x_j - x_k; seeds d 0-2, eps_f,k 3, rho_k 4
            const float4 rj = A.r[j];
            const auto w = poly6T<Dual<5>>(S, lenT(dvec<5>(-1.f * d, 0)));
            const auto vj = mk / dseed<5>(rhoK, 4);
            const auto t = rj.x * (dseed<5>(epsfK, 3) * vj * w) + rj.y * (vj * w);
            gx += -grad3(t, 0);
            geps += t.d[3];
            grho += t.d[4];
        });
    }
    add3(A.x[slot], gx);
    float4 s = A.s[slot];
    s.x += grho;
    s.z += geps;
    s.w += gsat;
    A.s[slot] = s;
}

// A5a: sand: average flow = num / sat, sat = sum V_j W -> (num-bar, sat-bar total).
__global__ void kAdjFlowSelf(AdjBuffers A, PassBuffers b) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    const float4 pk4 = b.pos4[slot];
    if (!(pk4.w < 0.f)) return;
    const float den = b.aux4[slot].z;
    const float3 fb = xyz(A.flow[slot]);
    float3 nb = mk3(0.f, 0.f, 0.f);
    float db = A.s[slot].w;
    if (den != 0.f) {
        nb = fb / den;
        db += -dot3(fb, xyz(b.flow4[slot])) / den;  // num / den^2 = flow / den
    }
    A.r[slot] = f4(nb, db);
}

// A5b: average flow / saturation / fluid voidage pair terms from both ends.
__global__ void __launch_bounds__(kSlotAlign) kAdjFlowPairs(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene, AdjBuffers A,
                                                            PassBuffers b) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const float3 xk = xyz(pk4);
    float3 gx = mk3(0.f, 0.f, 0.f), gv = gx;
    float grho = 0.f;
    if (pk4.w < 0.f) {
        const float4 rk = A.r[slot];
        const float vk = -pk4.w / b.vel4[slot].w;
        forWaterNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            const float4 vj4 = b.vel4[j];
            // own sums: v_j V_j W and V_j W, d = x_k - x_j
            const float vj = pj4.w / vj4.w;
            gx += (vj * (dot3(xyz(rk), xyz(vj4)) + rk.w)) * poly6Grad(S, xk - xyz(pj4));
            // k in the fluid voidage of water j: -V_k W(x_j - x_k)
            gx += (A.s[j].z * vk) * poly6Grad(S, xyz(pj4) - xk);
        });
    } else {
        const float mk = pk4.w;
        const float ek = A.s[slot].z;
        const float3 vk3 = xyz(b.vel4[slot]);
        const float rhoK = b.vel4[slot].w;
        forSandNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            // own fluid voidage 1 - sum V_j W(x_k - x_j)
            gx += (-ek * (-pj4.w / b.vel4[j].w)) * poly6Grad(S, d);
            // k in the flow / saturation sums of sand j: d = x_j - x_k; seeds d 0-2, rho_k 3
            const float4 rj = A.r[j];
            const auto t = (mk / dseed<4>(rhoK, 3)) * poly6T<Dual<4>>(S, lenT(dvec<4>(-1.f * d, 0)));
            const float s = dot3(xyz(rj), vk3) + rj.w;
            gx += -s * grad3(t, 0);
            grho += s * t.d[3];
            gv += t.v * xyz(rj);
        });
    }
    add3(A.x[slot], gx);
    add3(A.v[slot], gv);
    A.s[slot].x += grho;
}

// A6a: water: density cotangent including the pressure path.
__global__ void kAdjDensitySelf(const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene,
                                AdjBuffers A, PassBuffers b) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    if (!(pk4.w > 0.f)) return;
    const float rho = b.vel4[slot].w;
    float dp;
    if (S.tait) {  // ComputeSFPressureByTait_CUDA
        const float x = rho / S.rho0;
        const float p = S.stiff * (powf(x, 7.f) - 1.f);
        dp = S.stiff * 7.f * powf(x, 6.f) / S.rho0 * (p < 0.f ? S.neg_scale : 1.f);
    } else {
        dp = S.stiff;
    }
    const float4 s = A.s[slot];
    A.r[slot] = make_float4(s.x + s.y * dp, 0.f, 0.f, 0.f);
}

// A6b: density pair terms: own m_j W(x_k - x_j) and water j's m_k W(x_j - x_k),
// boundary terms rho0 V_b W(x_k - x_b).
__global__ void __launch_bounds__(kSlotAlign) kAdjDensityPairs(const SceneDev* __restrict__ scenes,
                                                               const int* __restrict__ blockScene, AdjBuffers A,
                                                               PassBuffers b) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    if (!(pk4.w > 0.f)) return;
    const float3 xk = xyz(pk4);
    const float mk = pk4.w;
    const float rk = A.r[slot].x;
    float3 gx = mk3(0.f, 0.f, 0.f);
    forWaterNeighbors(S, b.lists, slot, xk, b.pos4, [&](int j) {
        if (j == slot) return;
        const float4 pj4 = b.pos4[j];
        gx += (rk * pj4.w + A.r[j].x * mk) * poly6Grad(S, xk - xyz(pj4));
    });
    forBoundaryNeighbors(S, b.lists, slot, xk, b.bpos4, [&](int bb) {
        const float4 bj = b.bpos4[bb];
        gx += (rk * S.rho0 * fabsf(bj.w)) * poly6Grad(S, xk - xyz(bj));
    });
    add3(A.x[slot], gx);
}

// Cotangents of the substep's input positions and velocities, by id.
__global__ void kAdjFinish(const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene, AdjBuffers A,
                           const float4* __restrict__ pos4, const int* __restrict__ pid) {
    SF_ADJ_PROLOGUE
    if (pos4[slot].w == 0.f) return;
    const int id = S.slot_off + pid[slot];
    A.adjX[id] = A.x[slot];
    A.adjV[id] = A.v[slot];
}

// ------------------------------------------------------------ launchers
void launchAdjSeed(const LaunchCtx& c, const float4* pos4, const int* pid, const float* target, float4* adjX,
                   float4* adjV, float2* lossPartial) {
    kAdjSeed<<<c.slotBlocks, kSlotAlign, 0, c.stream>>>(c.scenes, c.blockScene, pos4, pid, target, adjX, adjV,
                                                        lossPartial);
}

int launchAdjSubstep(const LaunchCtx& c, const AdjBuffers& A, const PassBuffers& b, const int* pid, float dt,
                     float* paramPartial) {
    const dim3 g(c.slotBlocks), t(kSlotAlign);
    const cudaStream_t s = c.stream;
    kAdjIntegrate<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b, pid, dt);
    kAdjWater<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    kAdjSandSelf<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b, paramPartial);
    kAdjSandPairs<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b, paramPartial);
    kAdjVoidSelf<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    kAdjVoidPairs<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    kAdjFlowSelf<<<g, t, 0, s>>>(A, b);
    kAdjFlowPairs<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    kAdjDensitySelf<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    kAdjDensityPairs<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    kAdjFinish<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b.pos4, pid);
    return 11;
}

}  // namespace sfg
