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
// needed. Pair terms that are antisymmetric (water pressure + viscosity:
// a_j(j,k) = -(m_k / m_j) a_k(k,j); sand contacts: f_j(j,k) = -f_k(k,j))
// are evaluated once per thread with the combined cotangent of both ends.
//
// The vector-Jacobian products of the SPH kernels, of the water, seepage,
// boundary and sand-water terms and of the water adhesion are written out by
// hand below; the DEM + capillary contact, the wall forces and the drag use
// forward-mode dual numbers (sf_dual.cuh) over their few inputs. Branch
// conditions (contact, friction cap, damping sign, positive voidage, water
// clamp, viscosity switch) are taken from the forward values.
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

// Pair kernels run G consecutive threads (lanes of one warp) per slot: lane
// `part` takes neighbour entries part, part + G, ... and the per-slot sums
// are reduced over the G lanes before lane 0 writes them. Small scenes have
// too few slots to hide the latency of one long neighbour loop per thread;
// G = 1 is the one-thread-per-slot layout of large scenes.
#define SF_ADJ_PROLOGUE_G                                                     \
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;                    \
    const int slot = gid / G, part = gid % G;                                 \
    const int sid = blockScene[(blockIdx.x * (blockDim.x / G)) / kSlotAlign]; \
    const SceneDev& S = scenes[sid];

// ------------------------------------------------------ neighbour cursors
// The neighbours of one label (list, or the stencil when the list
// overflowed) from a single call site, so that the loop body is inlined.
template <bool kSand, int G = 1> struct LabelCursor {
    const SceneDev* S;
    const unsigned* cs;
    const float4* pos4;
    const unsigned* p;
    long long step;
    float3 pi;
    int n, k, x, x1, y, y0, y1, z0, z1, part;
    unsigned j, jEnd, hits;
    bool stencil;

    // part in [0, G): this lane's share, every G-th neighbour from the part-th
    __device__ __forceinline__ LabelCursor(const SceneDev& s, const NbrLists& L, int slot, float3 p_i,
                                           const float4* __restrict__ pos, int part_ = 0)
        : S(&s), cs(L.cs), pos4(pos), pi(p_i), k(part_), part(part_), j(0), jEnd(0), hits(0) {
        const unsigned c = L.cnt[slot];
        stencil = int(c & 0xFFFFu) + int(c >> 16) > L.cap;
        n = kSand ? int(c & 0xFFFFu) : int(c >> 16);
        p = L.nbr + slot + (kSand ? size_t(0) : size_t(L.cap - 1) * size_t(L.M));
        step = kSand ? L.M : -L.M;
        x = x1 = y = y0 = y1 = z0 = z1 = 0;
        if (stencil) {
            const int3 cc = cellOf(s, p_i);
            x = max(cc.x - 1, 0);
            x1 = min(cc.x + 1, s.gx - 1);
            y0 = max(cc.y - 1, 0);
            y1 = min(cc.y + 1, s.gy - 1);
            y = y0 - 1;
            z0 = max(cc.z - 1, 0);
            z1 = min(cc.z + 1, s.gz - 1) + 1;
        }
    }
    __device__ __forceinline__ bool next(int& out) {
        if (!stencil) {
            if (k >= n) return false;
            out = int(p[k * step]);
            k += G;
            return true;
        }
        for (;;) {
            while (j < jEnd) {
                const unsigned c = j++;
                const float4 pj = pos4[c];
                if ((kSand ? pj.w < 0.f : pj.w > 0.f) && inReach(*S, pi - xyz(pj))) {
                    if (G > 1 && int(hits++ % unsigned(G)) != part) continue;
                    out = int(c);
                    return true;
                }
            }
            if (++y > y1) {
                y = y0;
                if (++x > x1) return false;
            }
            const int b = S->cell_off + (x * S->gy + y) * S->gz;
            j = cs[b + z0];
            jEnd = cs[b + z1];
        }
    }
};

// Boundary particles within reach (list, or the boundary stencil on overflow).
template <int G = 1> struct BoundaryCursor {
    const SceneDev* S;
    const unsigned* bcs;
    const float4* bpos4;
    const unsigned* p;
    long long M;
    float3 pi;
    int n, k, x, x1, y, y0, y1, z0, z1, part;
    unsigned j, jEnd, hits;
    bool stencil;

    __device__ __forceinline__ BoundaryCursor(const SceneDev& s, const NbrLists& L, int slot, float3 p_i,
                                              const float4* __restrict__ bpos, int part_ = 0)
        : S(&s), bcs(L.bcs), bpos4(bpos), p(L.bnbr + slot), M(L.M), pi(p_i), k(part_), part(part_), j(0), jEnd(0),
          hits(0) {
        n = L.bcnt[slot];
        stencil = n > kMaxBNbr;
        x = x1 = y = y0 = y1 = z0 = z1 = 0;
        if (stencil) {
            const int3 cc = cellOf(s, p_i);
            x = max(cc.x - 1, 0);
            x1 = min(cc.x + 1, s.gx - 1);
            y0 = max(cc.y - 1, 0);
            y1 = min(cc.y + 1, s.gy - 1);
            y = y0 - 1;
            z0 = max(cc.z - 1, 0);
            z1 = min(cc.z + 1, s.gz - 1) + 1;
        }
    }
    __device__ __forceinline__ bool next(int& out) {
        if (!stencil) {
            if (k >= n) return false;
            out = int(p[size_t(k) * size_t(M)]);
            k += G;
            return true;
        }
        for (;;) {
            while (j < jEnd) {
                const unsigned c = j++;
                if (inReach(*S, pi - xyz(bpos4[c]))) {
                    if (G > 1 && int(hits++ % unsigned(G)) != part) continue;
                    out = int(c);
                    return true;
                }
            }
            if (++y > y1) {
                y = y0;
                if (++x > x1) return false;
            }
            const int b = S->cell_off + (x * S->gy + y) * S->gz;
            j = bcs[b + z0];
            jEnd = bcs[b + z1];
        }
    }
};

// ------------------------------------------------------- small helpers
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
__device__ __forceinline__ void operator-=(float3& a, float3 b) {
    a.x -= b.x;
    a.y -= b.y;
    a.z -= b.z;
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

// ------------------------------------------- SPH kernels and their VJPs
// Spiky gradient G(d) = phi(r) d (SpikyKernelGrad, cuda_sph_kernel.cuh:110-117)
// and its symmetric Jacobian phi I + psi d d^T.
struct SpikyD {
    float3 g;
    float phi, psi;
};
__device__ __forceinline__ SpikyD spikyD(const SceneDev& S, float3 d) {
    SpikyD o;
    const float r = len3(d);
    if (r >= S.h || r < kEps) {
        o.g = mk3(0.f, 0.f, 0.f);
        o.phi = 0.f;
        o.psi = 0.f;
        return o;
    }
    const float hr = S.h - r;
    o.phi = S.spiky * hr * hr / r;
    o.g = o.phi * d;
    o.psi = -S.spiky * hr * (S.h + r) / (r * r * r);
    return o;
}
__device__ __forceinline__ float3 spikyVjp(const SpikyD& s, float3 d, float3 u) {
    return s.phi * u + (s.psi * dot3(u, d)) * d;
}
// Gradient of the Poly6 kernel W(|d|) with respect to d.
__device__ __forceinline__ float3 poly6Grad(const SceneDev& S, float3 d) {
    const float r2 = dot3(d, d);
    if (r2 >= S.h2) return mk3(0.f, 0.f, 0.f);
    const float t = S.h2 - r2;
    return (-6.f * S.poly6 * t * t) * d;
}
// Cotangents of P = p / max(eps, D^2), D = rho / max(eps, e) chained into (rho, p, e).
__device__ __forceinline__ float3 chainPressureTerm(float Pbar, float Dbar, float p, float rho, float e) {
    const float D = rho / fmaxf(kEps, e);
    const float D2 = D * D;
    const float pb = Pbar / fmaxf(kEps, D2);
    if (D2 > kEps) Dbar += Pbar * (-2.f * p * D / (D2 * D2));
    const float rb = Dbar / fmaxf(kEps, e);
    const float eb = e > kEps ? Dbar * (-rho / (e * e)) : 0.f;
    return mk3(rb, pb, eb);
}

// ------------------------------------------ dual-number pair terms
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
// Derivative of QuadraticBezierCoeff (cuda_sf_utils.cuh:57-82) in sr, branch
// by branch: first segment dB/dt = 2 (1 - t)(py1 - py0) with t = sr / px1;
// second segment dB/dt = 2 t (py2 - py1) with t = (b + sqrt(c + d (px1 - sr))) / e.
__device__ __forceinline__ float bezierDeriv(const BezierDev& G, float sr) {
    if (sr < 0.f || sr >= 1.f) return 0.f;
    if (sr <= G.px1) return 2.f * (1.f - sr / G.px1) * (G.py1 - G.py0) / G.px1;
    const float root = sqrtf(G.c + G.d * (G.px1 - sr));
    const float t = (G.b + root) / G.e;
    return 2.f * t * (G.py2 - G.py1) * (-G.d / (2.f * G.e * root));
}

// Vector-Jacobian product of the adhesion on water i from sand j,
// F = B(sat_j) m_i m_j A(l) d / l (d = x_i - x_j, l = |d| in (h/2, h], where
// the Akinci spline A is non-zero): with g = A / l,
//   u^T dF/dd = B m_i m_j (g u + g'(l) (d.u / l) d),  g' = A'(l) / l - A / l^2,
//   u^T dF/dsat_j = B'(sat_j) m_i m_j g (d.u),
// A = c q^(1/4) with q = -4 l^2 / h + 6 l - 2 h, A' = c q^(-3/4) (6 - 8 l / h) / 4.
__device__ __forceinline__ void adhesionVjp(const SceneDev& S, float3 d, float satJ, float mi, float mj, float3 u,
                                            float3& gd, float& gsat) {
    const float l2 = dot3(d, d), l = sqrtf(l2);
    gd = mk3(0.f, 0.f, 0.f);
    gsat = 0.f;
    if (!(2.f * l > S.h && l <= S.h)) return;
    const float q = -4.f * l * l / S.h + 6.f * l - 2.f * S.h;
    const float A = S.adh_coef * powf(q, 0.25f);
    // dA/dl = adh_coef q^(-3/4) (6 - 8l/h) / 4, taken as 0 at q = 0 (l = h)
    const float dAdl = q != 0.f ? 0.25f * S.adh_coef * powf(q, -0.75f) * (6.f - 8.f * l / S.h) : 0.f;
    const float m = mi * mj;
    const float du = dot3(d, u);
    const float g = A / l;
    const float gp = dAdl / l - A / l2;
    gd = (bezier(S.adhG, satJ) * m) * (g * u + (gp * du / l) * d);
    gsat = bezierDeriv(S.adhG, satJ) * m * g * du;
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
            g = (2.f * S.adj_seed_scale) * d;
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

// A2: water momentum (ComputeSFWaterLinearMomentum_CUDA, acc = g + a - F_adh / m).
// Water pair term of particle k from water j, d = x_k - x_j, dv = v_k - v_j:
//   a_k(k,j) = m_j T,  a_j(j,k) = -m_k T,
//   T = -(P_k + P_j) G(d) - [dv.d < 0] Pi G(d),  Pi = kappa dv.d / (d.d + eps),
//   kappa = -nu / (D_k + D_j),  D = rho / max(eps, e),  P = p / max(eps, D^2),
// so both ends are served by the cotangent c = m_j a-bar_k - m_k a-bar_j on T.
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kAdjWater(const SceneDev* __restrict__ scenes,
                                                        const int* __restrict__ blockScene, AdjBuffers A,
                                                        PassBuffers b) {
    SF_ADJ_PROLOGUE_G
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const NbrLists& L = b.lists;
    const float3 xk = xyz(pk4);
    const float4 vk4 = b.vel4[slot];
    const float3 vk = xyz(vk4);
    const float rhoK = vk4.w, pK = b.aux4[slot].x, epsK = b.aux4[slot].w;
    float3 gx = mk3(0.f, 0.f, 0.f), gv = gx;
    if (pk4.w > 0.f) {
        const float mk = pk4.w;
        const float3 ak = xyz(A.acc[slot]);
        if (part == 0) A.adh[slot] = f4(ak / -mk);
        const float2 dpk = b.dp[slot];
        const float Dk = dpk.x;
        const float Pk = dpk.y;
        float Pbar = 0.f, Dbar = 0.f, pbar = 0.f;
        LabelCursor<false, G> wc(S, L, slot, xk, b.pos4, part);
        for (int j; wc.next(j);) {
            if (j == slot) continue;
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            const SpikyD sp = spikyD(S, d);
            if (sp.phi == 0.f && sp.psi == 0.f) continue;
            const float4 vj4 = b.vel4[j];
            const float2 dpj = b.dp[j];
            const float Dj = dpj.x;
            const float Pj = dpj.y;
            const float3 c = pj4.w * ak - mk * xyz(A.acc[j]);
            const float cg = dot3(c, sp.g);
            float coef = -(Pk + Pj);
            Pbar -= cg;
            const float3 dv = vk - xyz(vj4);
            const float dd = dot3(dv, d);
            if (dd < 0.f) {
                const float q = dot3(d, d) + kEps;
                const float sD = Dk + Dj;
                const float kappa = -S.nu / sD;
                coef -= kappa * (dd / q);
                gx += (-cg * kappa) * (dv / q - (2.f * dd / (q * q)) * d);
                gv += (-cg * kappa / q) * d;
                Dbar += cg * (-(dd / q) * S.nu / (sD * sD));
            }
            gx += coef * spikyVjp(sp, d, c);
        }
        // seepage terms of sand j: (-m_j p_k / max(eps, D_k rho_j)) G(d) - W(d) / D_k drag_j
        LabelCursor<true, G> sc(S, L, slot, xk, b.pos4, part);
        for (int j; sc.next(j);) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            const SpikyD sp = spikyD(S, d);
            const float mj = -pj4.w, rhoJ = b.vel4[j].w;
            const float3 dragJ = xyz(b.drag4[j]);
            const float den = Dk * rhoJ;
            const float ug = dot3(ak, sp.g), ud = dot3(ak, dragJ);
            gx += (-mj * pK / fmaxf(kEps, den)) * spikyVjp(sp, d, ak) + (-ud / Dk) * poly6Grad(S, d);
            pbar += ug * (-mj / fmaxf(kEps, den));
            if (den > kEps) Dbar += ug * (mj * pK * rhoJ / (den * den));
            Dbar += ud * poly6(S, len3(d)) / (Dk * Dk);
        }
        // boundary pressure and viscosity (rho0 as the density)
        const float gam0 = -S.rho0 / fmaxf(kEps, S.rho0 * S.rho0);
        const float kb = -S.bnu / (2.f * S.rho0);
        BoundaryCursor<G> bc(S, L, slot, xk, b.bpos4, part);
        for (int bb; bc.next(bb);) {
            const float4 bj = b.bpos4[bb];
            const float vol = fabsf(bj.w);
            const float3 d = xk - xyz(bj);
            const SpikyD sp = spikyD(S, d);
            const float ug = dot3(ak, sp.g);
            const float gam = gam0 * vol;
            pbar += gam * ug;
            float coef = gam * pK;
            const float dd = dot3(vk, d);
            if (dd < 0.f) {
                const float q = dot3(d, d) + kEps;
                const float w = -vol * S.rho0 * kb;
                coef += w * (dd / q);
                gx += (ug * w) * (vk / q - (2.f * dd / (q * q)) * d);
                gv += (ug * w / q) * d;
            }
            gx += coef * spikyVjp(sp, d, ak);
        }
        Pbar = groupSum<G>(Pbar);
        Dbar = groupSum<G>(Dbar);
        pbar = groupSum<G>(pbar);
        if (part == 0) {
            const float3 s3 = chainPressureTerm(Pbar, Dbar, pK, rhoK, epsK);
            float4 s = A.s[slot];
            s.x += s3.x;
            s.y += s3.y + pbar;
            s.z += s3.z;
            A.s[slot] = s;
        }
    } else {
        // sand k in the seepage term of water i: d = x_i - x_k
        const float mk = -pk4.w;
        const float3 dragK = xyz(b.drag4[slot]);
        float3 gdrag = mk3(0.f, 0.f, 0.f);
        LabelCursor<false, G> wc(S, L, slot, xk, b.pos4, part);
        for (int i; wc.next(i);) {
            const float4 pi4 = b.pos4[i];
            const float3 d = xyz(pi4) - xk;
            const SpikyD sp = spikyD(S, d);
            const float Di = b.dp[i].x;
            const float3 ai = xyz(A.acc[i]);
            const float alpha = -mk * b.aux4[i].x / fmaxf(kEps, Di * rhoK);
            gx -= alpha * spikyVjp(sp, d, ai) + (-dot3(ai, dragK) / Di) * poly6Grad(S, d);
            gdrag += (-poly6(S, len3(d)) / Di) * ai;
        }
        gdrag = groupSum3<G>(gdrag);
        if (part == 0) A.drag[slot] = f4(gdrag);
    }
    gx = groupSum3<G>(gx);
    gv = groupSum3<G>(gv);
    if (part != 0) return;
    add3(A.x[slot], gx);
    add3(A.v[slot], gv);
}

// A3a: per sand particle: v_w, drag, walls and shape-boundary DEM; writes
// (f-bar, v_w-bar) and adds the friction / permeability parameter partials.
// paramPartial: 3 floats per block of the lane-split pair kernels (G blocks
// per block of this kernel); this block adds into the first of its G.
__global__ void __launch_bounds__(kSlotAlign) kAdjSandSelf(const SceneDev* __restrict__ scenes,
                                                           const int* __restrict__ blockScene, AdjBuffers A,
                                                           PassBuffers b, float* __restrict__ paramPartial, int G) {
    SF_ADJ_PROLOGUE
    const float4 pk4 = b.pos4[slot];
    float gTan = 0.f, gPerm = 0.f;
    if (pk4.w < 0.f) {
        const float mk = -pk4.w;
        const float3 xk = xyz(pk4), vk = xyz(b.vel4[slot]);
        const float rhoK = b.vel4[slot].w, epsK = b.aux4[slot].w;
        const float tanPhi = sqrtf(S.tan2);
        const float vw = b.dp[slot].y;  // stored by the forward
        const float3 fb = (2.f / mk) * xyz(A.acc[slot]);
        const float3 dragB = xyz(A.drag[slot]);
        // df; seeds eps 0, flow 1-3, v 4-6, permeability scale 7
        const float cd = S.multi ? b.mat4[slot].x : S.cd;
        const auto df = dragT<Dual<8>>(S, dseed<8>(epsK, 0), dvec<8>(xyz(b.flow4[slot]), 1), dvec<8>(vk, 4), mk, rhoK,
                                       cd, dseed<8>(1.f, 7));
        float3 dfb = fb;
        float vwb = 0.f;
        if (vw != 0.f) {  // avg drag = df / v_w: d/dv_w = -avg drag / v_w
            dfb = dfb + dragB / vw;
            vwb = -dot3(dragB, mk3(df.x.v, df.y.v, df.z.v) / vw) / vw;
        }
        A.s[slot].z += vjp(dfb, df, 0);
        A.flow[slot] = f4(vjp3(dfb, df, 1));
        float3 gv = vjp3(dfb, df, 4);
        gPerm = vjp(dfb, df, 7);
        // world walls; seeds x 0-2, v 3-5, tan phi 6
        const auto w = wallsT<Dual<7>>(S, dvec<7>(xk, 0), dvec<7>(vk, 3), dseed<7>(tanPhi, 6));
        float3 gx = vjp3(fb, w, 0);
        gv += vjp3(fb, w, 3);
        gTan = vjp(fb, w, 6);
        if (S.shape_boundary) {
            BoundaryCursor<> bc(S, b.lists, slot, xk, b.bpos4);
            for (int bb; bc.next(bb);) {
                const float4 bj = b.bpos4[bb];
                if (!(bj.w < 0.f)) continue;
                const auto tp = dseed<7>(tanPhi, 6);
                const auto o = demForceT(dvec<7>(xk - xyz(bj), 0), -dvec<7>(vk, 3), S.rij2, S.kn, S.ks, tp * tp);
                gx += vjp3(fb, o, 0);
                gv += vjp3(fb, o, 3);
                gTan += vjp(fb, o, 6);
            }
        }
        add3(A.x[slot], gx);
        add3(A.v[slot], gv);
        A.f[slot] = f4(fb, vwb);
    }
    const float2 t = blockSum2(gTan, gPerm);
    if (threadIdx.x == 0) {
        paramPartial[3 * size_t(blockIdx.x) * G] += t.x;
        paramPartial[3 * size_t(blockIdx.x) * G + 2] += t.y;
    }
}

// A3b: sand pair terms. Contacts (one dual evaluation per pair serves both
// ends: f_j(j,k) = -f_k(k,j)); buoyancy + adhesion and v_w with water, from
// the sand end and from the water end:
//   f_i += [0 < e_j <= 1] (-m_i m_j p_j / max(eps, rho_i D_j)) G(x_i - x_j) + W vol_i avgadh_j,
//   v_w,i += [0 < e_j <= 1] (m_j / D_j) W(x_i - x_j).
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kAdjSandPairs(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene, AdjBuffers A,
                                                            PassBuffers b, float* __restrict__ paramPartial) {
    SF_ADJ_PROLOGUE_G
    const float4 pk4 = b.pos4[slot];
    float gTan = 0.f, gCap = 0.f;
    if (pk4.w != 0.f) {
        const NbrLists& L = b.lists;
        const float3 xk = xyz(pk4);
        const float4 vk4 = b.vel4[slot];
        const float3 vk = xyz(vk4);
        const float4 ak4 = b.aux4[slot];
        const float rhoK = vk4.w, pK = ak4.x, satK = ak4.z, epsK = ak4.w;
        float3 gx = mk3(0.f, 0.f, 0.f), gv = gx;
        if (pk4.w < 0.f) {
            const float mk = -pk4.w;
            const float4 fk4 = A.f[slot];
            const float3 fb = xyz(fk4);
            const float vwb = fk4.w;
            const float tanPhi = sqrtf(S.tan2);
            float gsat = 0.f;
            // contacts: the contact list, or the sand list filtered by the DEM reach
            const int ncon = L.ccnt[slot];
            const bool filtered = ncon > kMaxContact;
            LabelCursor<true, G> sc(S, L, slot, xk, b.pos4, part);
            for (int k = part;; k += G) {
                int j;
                if (!filtered) {
                    if (k >= ncon) break;
                    j = int(L.cnbr[slot + size_t(k) * size_t(L.M)]);
                } else {
                    if (!sc.next(j)) break;
                    if (j == slot) continue;
                    const float3 dd = xyz(b.pos4[j]) - xk;
                    if (!(dot3(dd, dd) < S.dem_reach2)) continue;
                }
                const float3 d = xyz(b.pos4[j]) - xk;
                const float3 c = fb - xyz(A.f[j]);
                // DEM acts while the spheres overlap (dist < 2r), the liquid
                // bridge only at gaps 0 < H < rupture: at most one of the two
                // is non-zero, so each gets its own narrower dual evaluation
                const float dist = len3(d);
                if (S.rij2 - dist > 0.f) {
                    // seeds d 0-2, dv 3-5, tan phi 6
                    const auto tp = dseed<7>(tanPhi, 6);
                    const auto o = demForceT(dvec<7>(d, 0), dvec<7>(xyz(b.vel4[j]) - vk, 3), S.rij2, S.kn, S.ks, tp * tp);
                    gx -= vjp3(c, o, 0);
                    gv -= vjp3(c, o, 3);
                    gTan += vjp(fb, o, 6);
                } else if (dist - (S.dem_radius + S.dem_radius) < S.cap_srupt) {
                    // seeds d 0-2, sat_k 3, capillary scale 4
                    const auto o = capillaryForceT(S, dvec<5>(d, 0), (dseed<5>(satK, 3) + b.aux4[j].z) / 2.f,
                                                   dseed<5>(1.f, 4));
                    gx -= vjp3(c, o, 0);
                    gsat += vjp(c, o, 3);
                    gCap += vjp(fb, o, 4);
                }
            }
            const float volK = mk / fmaxf(kEps, rhoK);
            LabelCursor<false, G> wc(S, L, slot, xk, b.pos4, part);
            for (int j; wc.next(j);) {
                const float4 pj4 = b.pos4[j];
                const float3 d = xk - xyz(pj4);
                const float3 gW = poly6Grad(S, d);
                gx += (volK * dot3(fb, xyz(b.avgadh4[j]))) * gW;
                const float ej = b.aux4[j].w;
                if (ej > 0.f && ej <= 1.f) {
                    const float Dj = b.dp[j].x;
                    const float sigma = -mk * pj4.w * b.aux4[j].x / fmaxf(kEps, rhoK * Dj);
                    gx += sigma * spikyVjp(spikyD(S, d), d, fb) + (vwb * pj4.w / Dj) * gW;
                }
            }
            gsat = groupSum<G>(gsat);
            if (part == 0) A.s[slot].w += gsat;
        } else {
            // water k in the terms of sand i: d = x_i - x_k
            const float mk = pk4.w;
            const float3 avgAdhK = xyz(b.avgadh4[slot]);
            const bool inBand = epsK > 0.f && epsK <= 1.f;
            const float Dk = rhoK / fmaxf(kEps, epsK);
            float3 gadh = mk3(0.f, 0.f, 0.f);
            float pbar = 0.f, Dbar = 0.f;
            LabelCursor<true, G> sc(S, L, slot, xk, b.pos4, part);
            for (int i; sc.next(i);) {
                const float4 pi4 = b.pos4[i];
                const float4 fi4 = A.f[i];
                const float3 fi = xyz(fi4);
                const float3 d = xyz(pi4) - xk;
                const float mi = -pi4.w, rhoI = b.vel4[i].w;
                const float volI = mi / fmaxf(kEps, rhoI);
                const float W = poly6(S, len3(d));
                const float3 gW = poly6Grad(S, d);
                gadh += (W * volI) * fi;
                gx -= (volI * dot3(fi, avgAdhK)) * gW;
                if (inBand) {
                    const float den = rhoI * Dk;
                    const SpikyD sp = spikyD(S, d);
                    const float ug = dot3(fi, sp.g);
                    gx -= (-mi * mk * pK / fmaxf(kEps, den)) * spikyVjp(sp, d, fi) + (fi4.w * mk / Dk) * gW;
                    pbar += ug * (-mi * mk / fmaxf(kEps, den));
                    if (den > kEps) Dbar += ug * (mi * mk * pK * rhoI / (den * den));
                    Dbar += fi4.w * (-mk * W / (Dk * Dk));
                }
            }
            gadh = groupSum3<G>(gadh);
            pbar = groupSum<G>(pbar);
            Dbar = groupSum<G>(Dbar);
            if (part == 0) {
                add3(A.avgadh[slot], gadh);
                float4 s = A.s[slot];
                s.x += Dbar / fmaxf(kEps, epsK);
                s.y += pbar;
                if (epsK > kEps) s.z += Dbar * (-rhoK / (epsK * epsK));
                A.s[slot] = s;
            }
        }
        gx = groupSum3<G>(gx);
        gv = groupSum3<G>(gv);
        if (part == 0) {
            add3(A.x[slot], gx);
            add3(A.v[slot], gv);
        }
    }
    const float2 t = blockSum2(gTan, gCap);
    if (threadIdx.x == 0) {
        paramPartial[3 * blockIdx.x] += t.x;
        paramPartial[3 * blockIdx.x + 1] += t.y;
    }
}

// A4a: sand: voidage = num / den -> (num-bar, den-bar); water: adhesion
// cotangent total (F_adh-bar + avg-bar / v_s) and v_s-bar.
__global__ void __launch_bounds__(kSlotAlign) kAdjVoidSelf(AdjBuffers A, PassBuffers b) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const float3 xk = xyz(pk4);
    if (pk4.w < 0.f) {
        // voidage = num / den, with den and the quotient stored by the forward
        const float den = b.dp[slot].x;
        // quotient rule without squaring den (a small den would underflow)
        const float eb = A.s[slot].z;
        A.r[slot] = den != 0.f ? make_float4(eb / den, -(eb / den) * b.aux4[slot].w, 0.f, 0.f)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        const float vs = b.adh4[slot].w;  // stored by the forward
        const float3 avgB = xyz(A.avgadh[slot]);
        float3 tot = xyz(A.adh[slot]);
        float vsb = 0.f;
        if (vs != 0.f) {  // avg = F / v_s: d/dv_s = -avg / v_s
            tot = tot + avgB / vs;
            vsb = -dot3(avgB, xyz(b.avgadh4[slot])) / vs;
        }
        A.r[slot] = f4(tot, vsb);
    }
}

// A4b: voidage / adhesion pair terms from both ends.
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kAdjVoidPairs(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene, AdjBuffers A,
                                                            PassBuffers b) {
    SF_ADJ_PROLOGUE_G
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const float3 xk = xyz(pk4);
    const float rhoK = b.vel4[slot].w;
    float3 gx = mk3(0.f, 0.f, 0.f);
    if (pk4.w < 0.f) {
        const float mk = -pk4.w;
        const float4 rk = A.r[slot];
        const float satK = b.aux4[slot].z;
        const float vk = mk / rhoK;
        float gsat = 0.f;
        LabelCursor<false, G> wc(S, b.lists, slot, xk, b.pos4, part);
        for (int j; wc.next(j);) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xyz(pj4) - xk;  // x_j - x_k
            const float3 gW = poly6Grad(S, d);
            // own num / den sums over W(x_k - x_j): gradient -gW
            const float vj = pj4.w / b.vel4[j].w;
            gx -= (rk.x * b.aux4[j].y * vj + rk.y * vj) * gW;
            // k in the adhesion and v_s of water j; seeds d 0-2, sat_k 3
            const float4 rj = A.r[j];
            if (2.f * dot3(d, d) > 0.5f * S.h2) {  // the adhesion spline vanishes for |d| <= h / 2
                float3 gd;
                float gs;
                adhesionVjp(S, d, satK, pj4.w, mk, xyz(rj), gd, gs);
                gx -= gd;
                gsat += gs;
            }
            gx -= (rj.w * vk) * gW;
        }
        gsat = groupSum<G>(gsat);
        if (part == 0) A.s[slot].w += gsat;
    } else {
        const float mk = pk4.w;
        const float4 rk = A.r[slot];
        const float epsfK = b.aux4[slot].y;
        float grho = 0.f, geps = 0.f;
        LabelCursor<true, G> sc(S, b.lists, slot, xk, b.pos4, part);
        for (int j; sc.next(j);) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            const float3 gW = poly6Grad(S, d);
            // own adhesion and v_s terms
            if (2.f * dot3(d, d) > 0.5f * S.h2) {
                float3 gd;
                float gs;
                adhesionVjp(S, d, b.aux4[j].z, mk, -pj4.w, xyz(rk), gd, gs);
                gx += gd;
            }
            gx += (rk.w * (-pj4.w / b.vel4[j].w)) * gW;
            // k in num / den of sand j: (e_f,k n + m) V_k W(x_j - x_k), V_k = m_k / rho_k
            const float4 rj = A.r[j];
            const float Vk = mk / rhoK;
            const float W = poly6(S, len3(d));
            const float s = rj.x * epsfK + rj.y;
            gx += (s * Vk) * gW;
            geps += rj.x * Vk * W;
            grho += s * (-mk / (rhoK * rhoK)) * W;
        }
        grho = groupSum<G>(grho);
        geps = groupSum<G>(geps);
        if (part == 0) {
            float4 s = A.s[slot];
            s.x += grho;
            s.z += geps;
            A.s[slot] = s;
        }
    }
    gx = groupSum3<G>(gx);
    if (part == 0) add3(A.x[slot], gx);
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
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kAdjFlowPairs(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene, AdjBuffers A,
                                                            PassBuffers b) {
    SF_ADJ_PROLOGUE_G
    const float4 pk4 = b.pos4[slot];
    if (pk4.w == 0.f) return;
    const float3 xk = xyz(pk4);
    float3 gx = mk3(0.f, 0.f, 0.f), gv = gx;
    if (pk4.w < 0.f) {
        const float4 rk = A.r[slot];
        const float vk = -pk4.w / b.vel4[slot].w;
        LabelCursor<false, G> wc(S, b.lists, slot, xk, b.pos4, part);
        for (int j; wc.next(j);) {
            const float4 pj4 = b.pos4[j];
            const float4 vj4 = b.vel4[j];
            const float3 gW = poly6Grad(S, xk - xyz(pj4));  // d W(x_k - x_j) / d x_k = d W(x_j - x_k) / d x_k
            // own sums v_j V_j W and V_j W; k in the fluid voidage 1 - V_k W of water j
            const float vj = pj4.w / vj4.w;
            gx += (vj * (dot3(xyz(rk), xyz(vj4)) + rk.w) - A.s[j].z * vk) * gW;
        }
    } else {
        const float mk = pk4.w;
        const float ek = A.s[slot].z;
        const float3 vk3 = xyz(b.vel4[slot]);
        const float rhoK = b.vel4[slot].w;
        const float Vk = mk / rhoK;
        float grho = 0.f;
        LabelCursor<true, G> sc(S, b.lists, slot, xk, b.pos4, part);
        for (int j; sc.next(j);) {
            const float4 pj4 = b.pos4[j];
            const float3 d = xk - xyz(pj4);
            const float3 gW = poly6Grad(S, d);
            // own fluid voidage 1 - sum V_j W(x_k - x_j), and k in the flow /
            // saturation sums of sand j: V_k W(x_j - x_k) (v_k, 1)
            const float4 rj = A.r[j];
            const float s = dot3(xyz(rj), vk3) + rj.w;
            gx += (ek * pj4.w / b.vel4[j].w + s * Vk) * gW;
            const float W = poly6(S, len3(d));
            grho += s * (-mk / (rhoK * rhoK)) * W;
            gv += (Vk * W) * xyz(rj);
        }
        grho = groupSum<G>(grho);
        if (part == 0) A.s[slot].x += grho;
    }
    gx = groupSum3<G>(gx);
    gv = groupSum3<G>(gv);
    if (part != 0) return;
    add3(A.x[slot], gx);
    add3(A.v[slot], gv);
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
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kAdjDensityPairs(const SceneDev* __restrict__ scenes,
                                                               const int* __restrict__ blockScene, AdjBuffers A,
                                                               PassBuffers b) {
    SF_ADJ_PROLOGUE_G
    const float4 pk4 = b.pos4[slot];
    if (!(pk4.w > 0.f)) return;
    const float3 xk = xyz(pk4);
    const float mk = pk4.w;
    const float rk = A.r[slot].x;
    float3 gx = mk3(0.f, 0.f, 0.f);
    LabelCursor<false, G> wc(S, b.lists, slot, xk, b.pos4, part);
    for (int j; wc.next(j);) {
        if (j == slot) continue;
        const float4 pj4 = b.pos4[j];
        gx += (rk * pj4.w + A.r[j].x * mk) * poly6Grad(S, xk - xyz(pj4));
    }
    BoundaryCursor<G> bc(S, b.lists, slot, xk, b.bpos4, part);
    for (int bb; bc.next(bb);) {
        const float4 bj = b.bpos4[bb];
        gx += (rk * S.rho0 * fabsf(bj.w)) * poly6Grad(S, xk - xyz(bj));
    }
    gx = groupSum3<G>(gx);
    if (part == 0) add3(A.x[slot], gx);
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

__global__ void kAdjStore(PassBuffers b, const int* __restrict__ pid, AdjSlab s) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    s.pos[slot] = b.pos4[slot];
    s.vel[slot] = b.vel4[slot];
    s.acc[slot] = b.acc4[slot];
    s.adh[slot] = b.adh4[slot];
    s.avgadh[slot] = b.avgadh4[slot];
    s.mat[slot] = b.mat4[slot];
    s.pid[slot] = pid[slot];
}

// ------------------------------------------------------------ launchers
void launchAdjStore(const LaunchCtx& c, const PassBuffers& b, const int* pid, const AdjSlab& s) {
    kAdjStore<<<c.slotBlocks, kSlotAlign, 0, c.stream>>>(b, pid, s);
}

void launchAdjSeed(const LaunchCtx& c, const float4* pos4, const int* pid, const float* target, float4* adjX,
                   float4* adjV, float2* lossPartial) {
    kAdjSeed<<<c.slotBlocks, kSlotAlign, 0, c.stream>>>(c.scenes, c.blockScene, pos4, pid, target, adjX, adjV,
                                                        lossPartial);
}

template <int G>
void launchAdjPairs(const LaunchCtx& c, const AdjBuffers& A, const PassBuffers& b, float* paramPartial, int level) {
    const dim3 g(c.slotBlocks * G), t(kSlotAlign);
    const cudaStream_t s = c.stream;
    switch (level) {
    case 0: kAdjWater<G><<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b); break;
    case 1: kAdjSandPairs<G><<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b, paramPartial); break;
    case 2: kAdjVoidPairs<G><<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b); break;
    case 3: kAdjFlowPairs<G><<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b); break;
    default: kAdjDensityPairs<G><<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b); break;
    }
}

void launchPairs(const LaunchCtx& c, const AdjBuffers& A, const PassBuffers& b, float* paramPartial, int lanes,
                 int level) {
    switch (lanes) {
    case 2: launchAdjPairs<2>(c, A, b, paramPartial, level); break;
    case 4: launchAdjPairs<4>(c, A, b, paramPartial, level); break;
    case 8: launchAdjPairs<8>(c, A, b, paramPartial, level); break;
    default: launchAdjPairs<1>(c, A, b, paramPartial, level); break;
    }
}

int launchAdjSubstep(const LaunchCtx& c, const AdjBuffers& A, const PassBuffers& b, const int* pid, float dt,
                     float* paramPartial, int lanes) {
    const dim3 g(c.slotBlocks), t(kSlotAlign);
    const cudaStream_t s = c.stream;
    kAdjIntegrate<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b, pid, dt);
    launchPairs(c, A, b, paramPartial, lanes, 0);
    kAdjSandSelf<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b, paramPartial, lanes);
    launchPairs(c, A, b, paramPartial, lanes, 1);
    kAdjVoidSelf<<<g, t, 0, s>>>(A, b);
    launchPairs(c, A, b, paramPartial, lanes, 2);
    kAdjFlowSelf<<<g, t, 0, s>>>(A, b);
    launchPairs(c, A, b, paramPartial, lanes, 3);
    kAdjDensitySelf<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b);
    launchPairs(c, A, b, paramPartial, lanes, 4);
    kAdjFinish<<<g, t, 0, s>>>(c.scenes, c.blockScene, A, b.pos4, pid);
    return 11;
}

}  // namespace sfg
