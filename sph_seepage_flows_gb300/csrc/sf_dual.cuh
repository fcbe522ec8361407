// Forward-mode dual numbers for the pair Jacobians of the adjoint.
//
// Dual<K> carries a value and K tangent components. The pair functions of
// the substep are written once below as templates on the scalar type; called
// with T = Dual<K> and the inputs of interest seeded with unit tangents,
// they return the Jacobian columns of their outputs with respect to those
// inputs, which the adjoint kernels contract with the output cotangents
// (a vector-Jacobian product assembled from K Jacobian-vector products).
// Branch conditions are evaluated on the values, as in the forward pass.
#pragma once

#include "sf_device.cuh"

namespace sfg {

template <int K> struct Dual {
    float v;
    float d[K];
};

template <int K> __device__ __forceinline__ Dual<K> dconst(float v) {
    Dual<K> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = 0.f;
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> dseed(float v, int k) {
    Dual<K> r = dconst<K>(v);
    r.d[k] = 1.f;
    return r;
}

#define SF_DUAL_BINOP(OP, DV, DD)                                                          \
    template <int K> __device__ __forceinline__ Dual<K> operator OP(Dual<K> a, Dual<K> b) { \
        Dual<K> r;                                                                         \
        r.v = DV;                                                                          \
        _Pragma("unroll") for (int k = 0; k < K; ++k) r.d[k] = DD;                         \
        return r;                                                                          \
    }
SF_DUAL_BINOP(+, a.v + b.v, a.d[k] + b.d[k])
SF_DUAL_BINOP(-, a.v - b.v, a.d[k] - b.d[k])
SF_DUAL_BINOP(*, a.v * b.v, a.d[k] * b.v + a.v * b.d[k])
#undef SF_DUAL_BINOP

template <int K> __device__ __forceinline__ Dual<K> operator/(Dual<K> a, Dual<K> b) {
    Dual<K> r;
    r.v = a.v / b.v;
    const float ib = 1.f / b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator-(Dual<K> a) {
    Dual<K> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator*(float s, Dual<K> a) {
    Dual<K> r;
    r.v = s * a.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = s * a.d[k];
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator*(Dual<K> a, float s) { return s * a; }
template <int K> __device__ __forceinline__ Dual<K> operator+(Dual<K> a, float s) {
    a.v += s;
    return a;
}
template <int K> __device__ __forceinline__ Dual<K> operator+(float s, Dual<K> a) { return a + s; }
template <int K> __device__ __forceinline__ Dual<K> operator-(Dual<K> a, float s) {
    a.v -= s;
    return a;
}
template <int K> __device__ __forceinline__ Dual<K> operator-(float s, Dual<K> a) { return (-a) + s; }
template <int K> __device__ __forceinline__ Dual<K> operator/(Dual<K> a, float s) { return (1.f / s) * a; }
template <int K> __device__ __forceinline__ Dual<K> operator/(float s, Dual<K> a) { return dconst<K>(s) / a; }

template <int K> __device__ __forceinline__ Dual<K> dsqrt(Dual<K> a) {
    Dual<K> r;
    r.v = sqrtf(a.v);
    const float g = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <int K> __device__ __forceinline__ Dual<K> dpow(Dual<K> a, float e) {
    Dual<K> r;
    r.v = powf(a.v, e);
    const float g = a.v != 0.f ? e * powf(a.v, e - 1.f) : 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = g * a.d[k];
    return r;
}
// max(c, a) with the derivative of the selected branch (fmaxf of the forward pass)
template <int K> __device__ __forceinline__ Dual<K> dmaxc(float c, Dual<K> a) {
    return a.v > c ? a : dconst<K>(c);
}

__device__ __forceinline__ float val(float x) { return x; }
template <int K> __device__ __forceinline__ float val(const Dual<K>& x) { return x.v; }
__device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
template <int K> __device__ __forceinline__ Dual<K> tsqrt(Dual<K> x) { return dsqrt(x); }
__device__ __forceinline__ float tpow(float x, float e) { return powf(x, e); }
template <int K> __device__ __forceinline__ Dual<K> tpow(Dual<K> x, float e) { return dpow(x, e); }
__device__ __forceinline__ float tmaxc(float c, float x) { return fmaxf(c, x); }
template <int K> __device__ __forceinline__ Dual<K> tmaxc(float c, Dual<K> x) { return dmaxc(c, x); }
__device__ __forceinline__ float tabs(float x) { return fabsf(x); }
template <int K> __device__ __forceinline__ Dual<K> tabs(Dual<K> x) { return x.v < 0.f ? -x : x; }

template <typename T> struct V3T {
    T x, y, z;
};
template <typename T> __device__ __forceinline__ V3T<T> v3(T x, T y, T z) { return V3T<T>{x, y, z}; }
template <typename T> __device__ __forceinline__ V3T<T> operator+(V3T<T> a, V3T<T> b) {
    return v3(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename T> __device__ __forceinline__ V3T<T> operator-(V3T<T> a, V3T<T> b) {
    return v3(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <typename T> __device__ __forceinline__ V3T<T> operator-(V3T<T> a) { return v3(-a.x, -a.y, -a.z); }
template <typename T, typename S> __device__ __forceinline__ V3T<T> operator*(V3T<T> a, S s) {
    return v3(a.x * s, a.y * s, a.z * s);
}
template <typename T, typename S> __device__ __forceinline__ V3T<T> operator*(S s, V3T<T> a) {
    return v3(s * a.x, s * a.y, s * a.z);
}
template <typename T, typename S> __device__ __forceinline__ V3T<T> operator/(V3T<T> a, S s) {
    return v3(a.x / s, a.y / s, a.z / s);
}
template <typename T> __device__ __forceinline__ T dotT(V3T<T> a, V3T<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> __device__ __forceinline__ T lenT(V3T<T> a) { return tsqrt(dotT(a, a)); }

// --------------------------------------------------- templated pair physics
// The same formulas as the forward kernels (sf_device.cuh, sf_kernels.cu).
template <typename T> __device__ __forceinline__ T poly6T(const SceneDev& S, T r) {
    T r2 = r * r;
    if (val(r2) >= S.h2) return r2 * 0.f;
    T d = S.h2 - r2;
    return S.poly6 * d * d * d;
}
template <typename T> __device__ __forceinline__ V3T<T> spikyGradT(const SceneDev& S, V3T<T> r) {
    T rl = lenT(r);
    if (val(rl) >= S.h || val(rl) < kEps) return r * 0.f;
    T d = S.h - rl;
    return (S.spiky * d * d / rl) * r;
}
template <typename T> __device__ __forceinline__ T bezierT(const BezierDev& G, T sr, float scale) {
    if (val(sr) < 0.f) return sr * 0.f + scale * G.py0;
    if (val(sr) >= 1.f) return sr * 0.f + scale * G.py2;
    if (val(sr) <= G.px1) {
        const T t = sr / G.px1;
        const T omt = 1.f - t;
        return scale * (omt * omt * G.py0 + 2.f * t * omt * G.py1 + t * t * G.py1);
    }
    const T t = (G.b + tsqrt(G.c + G.d * (G.px1 - sr))) / G.e;
    const T omt = 1.f - t;
    return scale * (omt * omt * G.py1 + 2.f * t * omt * G.py1 + t * t * G.py2);
}
// ComputeDemForces with tan^2(phi) as a (possibly dual) input
template <typename T> __device__ __forceinline__ V3T<T> demForceT(V3T<T> dij, V3T<T> vij, float rij, float kn, float ks,
                                                                  T tan2) {
    T dist = lenT(dij);
    T pen = rij - dist;
    if (!(val(pen) > 0.f)) return dij * 0.f;
    V3T<T> n = dij / dist;
    T de = dotT(vij, n);
    V3T<T> vt = vij - de * n;
    V3T<T> fn = (kn * pen) * n;
    V3T<T> fs = (-ks) * vt;
    T maxFs = dotT(fn, fn) * tan2;
    if (val(dotT(fs, fs)) > val(maxFs)) fs = fs * (tsqrt(maxFs) / lenT(fs));
    return -fn - fs;
}
// ComputeDemCapillaryForces with the Bezier coefficient scaled by capScale
template <typename T> __device__ __forceinline__ V3T<T> capillaryForceT(const SceneDev& S, V3T<T> dij, T sr, T capScale) {
    const float r = S.dem_radius;
    T dist = lenT(dij);
    T H = dist - (r + r);
    if (!(val(H) < S.cap_srupt && val(H) > 0.f)) return dij * 0.f;
    V3T<T> N = dij / dist;
    T coeff = capScale * bezierT(S.capG, sr, 1.f);
    T d = -H + tsqrt(H * H + S.cap_vlb_pir);
    T phi = tsqrt(2.f * H / r * (-1.f + tsqrt(1.f + S.cap_vlb / (S.cap_pir * H * H))));
    T ncp = S.cap_m2pi * coeff * r * S.cap_cos / (1.f + H / (2.f * d));
    T stf = S.cap_m2pi * coeff * r * phi * S.cap_sin;
    return (-N) * (ncp + stf);
}

}  // namespace sfg
