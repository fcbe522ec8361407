// ORACLE -- test infrastructure, not product code.
//
// CPU restatement of the sph_seepage_flows coupled SPH-DEM substep, used only
// as the checker by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline leg. It follows the reference kernels line by line: same loop
// nesting (27-cell stencil in the m = 0..26 order, then the particles of each
// cell in sorted order, one sub-loop per force term), same operand order in
// every expression, same quirks. It is templated on the arithmetic type:
// float reproduces the reference's FP32 arithmetic (IEEE, no fast-math), and
// double is the error yardstick. OpenMP parallelises the per-particle passes
// (every pass is a gather: particle i writes only its own entries).
//
// Every function cites the reference file:line it restates; paths are inside
// the sph_seepage_flows project:
//   SFGPU = seepage_flows_cuda/include/kiri_pbs_cuda/solver/seepageflow/cuda_sph_sf_solver_gpu.cuh
//   DEM   = seepage_flows_cuda/include/kiri_pbs_cuda/solver/dem/cuda_dem_solver_common_gpu.cuh
//   SPHC  = seepage_flows_cuda/include/kiri_pbs_cuda/solver/sph/cuda_sph_solver_common_gpu.cuh
//   KERN  = seepage_flows_cuda/include/kiri_pbs_cuda/kernel/cuda_sph_kernel.cuh
//   UTIL  = seepage_flows_cuda/include/kiri_pbs_cuda/solver/seepageflow/cuda_sf_utils.cuh
//   TAIT  = seepage_flows_cuda/include/kiri_pbs_cuda/solver/seepageflow/cuda_wcsph_sf_solver_gpu.cuh
//   WCSPH = seepage_flows_cuda/src/kiri_pbs_cuda/solver/seepage_flow/cuda_wcsph_sf_solver.{cpp,cu}
//   SOLV  = seepage_flows_cuda/src/kiri_pbs_cuda/solver/seepage_flow/cuda_sph_sf_solver.{cpp,cu}
//   PART  = seepage_flows_cuda/{include,src}/kiri_pbs_cuda/particle/cuda_sf_particles.{cuh,cu}
//   THR   = seepage_flows_cuda/include/kiri_pbs_cuda/thrust_helper/helper_thrust.cuh
//   SRCH  = seepage_flows_cuda/src/kiri_pbs_cuda/searcher/cuda_neighbor_searcher.cu
//   SYSG  = seepage_flows_cuda/include/kiri_pbs_cuda/system/cuda_sph_system_gpu.cuh
//   SYS   = seepage_flows_cuda/src/kiri_pbs_cuda/system/cuda_sf_system.cu

#include "../include/sf_capi.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace sfo {

// Forward-mode dual number: a value and one FP64 tangent. Sim<Dual1> (FP64
// values) runs the FP64 restatement while carrying the derivative of every
// quantity along one direction (initial positions / velocities or one
// parameter), the exact pathwise directional derivative that a reverse-mode
// gradient must reproduce. Sim<DualF> does the same on the FP32 trajectory:
// its values are formed with the FP32 restatement's float operations in the
// same order, so they equal Sim<float>'s bit for bit. Comparisons and
// branches use the value.
template <typename V> struct DualT {
    V v = V(0);
    double d = 0.0;
    DualT() = default;
    DualT(double x) : v(V(x)), d(0.0) {}  // NOLINT: constants convert implicitly
    DualT(double x, double t) : v(V(x)), d(t) {}
    explicit operator double() const { return double(v); }
    explicit operator float() const { return float(v); }
    explicit operator int() const { return int(v); }
    explicit operator long() const { return long(v); }
    explicit operator long long() const { return (long long)(v); }
    DualT& operator+=(DualT b) { v += b.v; d += b.d; return *this; }
    DualT& operator-=(DualT b) { v -= b.v; d -= b.d; return *this; }
    DualT& operator*=(DualT b) { d = d * double(b.v) + double(v) * b.d; v *= b.v; return *this; }
    DualT& operator/=(DualT b) {
        const V q = v / b.v;
        d = (d - double(q) * b.d) / double(b.v);
        v = q;
        return *this;
    }
};
using Dual1 = DualT<double>;
using DualF = DualT<float>;
template <typename V> inline DualT<V> mkDual(V v, double d) {
    DualT<V> r;
    r.v = v;
    r.d = d;
    return r;
}
template <typename V> inline DualT<V> operator+(DualT<V> a, DualT<V> b) { return mkDual(V(a.v + b.v), a.d + b.d); }
template <typename V> inline DualT<V> operator-(DualT<V> a, DualT<V> b) { return mkDual(V(a.v - b.v), a.d - b.d); }
template <typename V> inline DualT<V> operator-(DualT<V> a) { return mkDual(V(-a.v), -a.d); }
template <typename V> inline DualT<V> operator*(DualT<V> a, DualT<V> b) {
    return mkDual(V(a.v * b.v), a.d * double(b.v) + double(a.v) * b.d);
}
template <typename V> inline DualT<V> operator/(DualT<V> a, DualT<V> b) {
    const V q = a.v / b.v;
    return mkDual(q, (a.d - double(q) * b.d) / double(b.v));
}
template <typename V> inline bool operator<(DualT<V> a, DualT<V> b) { return a.v < b.v; }
template <typename V> inline bool operator>(DualT<V> a, DualT<V> b) { return a.v > b.v; }
template <typename V> inline bool operator<=(DualT<V> a, DualT<V> b) { return a.v <= b.v; }
template <typename V> inline bool operator>=(DualT<V> a, DualT<V> b) { return a.v >= b.v; }
template <typename V> inline bool operator==(DualT<V> a, DualT<V> b) { return a.v == b.v; }
template <typename V> inline bool operator!=(DualT<V> a, DualT<V> b) { return a.v != b.v; }
// mixed with plain numbers (the value type's constants)
template <typename V> inline DualT<V> operator+(DualT<V> a, double b) { return a + DualT<V>(b); }
template <typename V> inline DualT<V> operator+(double a, DualT<V> b) { return DualT<V>(a) + b; }
template <typename V> inline DualT<V> operator-(DualT<V> a, double b) { return a - DualT<V>(b); }
template <typename V> inline DualT<V> operator-(double a, DualT<V> b) { return DualT<V>(a) - b; }
template <typename V> inline DualT<V> operator*(DualT<V> a, double b) { return a * DualT<V>(b); }
template <typename V> inline DualT<V> operator*(double a, DualT<V> b) { return DualT<V>(a) * b; }
template <typename V> inline DualT<V> operator/(DualT<V> a, double b) { return a / DualT<V>(b); }
template <typename V> inline DualT<V> operator/(double a, DualT<V> b) { return DualT<V>(a) / b; }
template <typename V> inline bool operator<(DualT<V> a, double b) { return a.v < V(b); }
template <typename V> inline bool operator>(DualT<V> a, double b) { return a.v > V(b); }
template <typename V> inline bool operator<(double a, DualT<V> b) { return V(a) < b.v; }
template <typename V> inline bool operator>(double a, DualT<V> b) { return V(a) > b.v; }

// Math functions of the restatement: the std functions for float / double,
// their derivatives for the dual numbers (values by the value type's std
// function, as the plain restatement of that precision forms them).
inline float tsqrt(float x) { return std::sqrt(x); }
inline double tsqrt(double x) { return std::sqrt(x); }
template <typename V> inline DualT<V> tsqrt(DualT<V> a) {
    const V r = std::sqrt(a.v);
    return mkDual(r, r > V(0) ? a.d / (2.0 * double(r)) : 0.0);
}
inline float tpow(float a, float b) { return std::pow(a, b); }
inline double tpow(double a, double b) { return std::pow(a, b); }
template <typename V> inline DualT<V> tpow(DualT<V> a, DualT<V> b) {
    const V r = std::pow(a.v, b.v);
    const double av = double(a.v), bv = double(b.v);
    double d = av != 0.0 ? bv * std::pow(av, bv - 1.0) * a.d : 0.0;
    if (b.d != 0.0 && av > 0.0) d += std::log(av) * double(r) * b.d;
    return mkDual(r, d);
}
inline float tfmax(float a, float b) { return std::fmax(a, b); }
inline double tfmax(double a, double b) { return std::fmax(a, b); }
template <typename V> inline DualT<V> tfmax(DualT<V> a, DualT<V> b) { return (a.v > b.v || b.v != b.v) ? a : b; }
inline float tfmin(float a, float b) { return std::fmin(a, b); }
inline double tfmin(double a, double b) { return std::fmin(a, b); }
template <typename V> inline DualT<V> tfmin(DualT<V> a, DualT<V> b) { return (a.v < b.v || b.v != b.v) ? a : b; }
inline float tfabs(float x) { return std::fabs(x); }
inline double tfabs(double x) { return std::fabs(x); }
template <typename V> inline DualT<V> tfabs(DualT<V> a) { return a.v < V(0) ? -a : a; }
inline float tcos(float x) { return std::cos(x); }
inline double tcos(double x) { return std::cos(x); }
template <typename V> inline DualT<V> tcos(DualT<V> a) {
    return mkDual(V(std::cos(a.v)), -std::sin(double(a.v)) * a.d);
}
inline float tsin(float x) { return std::sin(x); }
inline double tsin(double x) { return std::sin(x); }
template <typename V> inline DualT<V> tsin(DualT<V> a) {
    return mkDual(V(std::sin(a.v)), std::cos(double(a.v)) * a.d);
}

// A parameter value, carrying the tangent t when T is Dual1.
template <typename T> inline T seeded(float v, double t) {
    (void)t;
    return T(v);
}
template <> inline Dual1 seeded<Dual1>(float v, double t) { return Dual1(double(v), t); }
template <> inline DualF seeded<DualF>(float v, double t) { return DualF(double(v), t); }

// KIRI_EPSILON and KIRI_PI (seepage_flows_cuda/include/kiri_pbs_cuda/kiri_pbs_pch.cuh:52-54).
template <typename T> constexpr T kEps() { return T(1e-6f); }
// Both are float literals in the reference, so the FP64 oracle takes their float values.
template <typename T> constexpr T kPi() { return T(3.141592653589793238462643383279502884197f); }

template <typename T> struct V3 {
    T x, y, z;
};
template <typename T> inline V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename T> inline V3<T> operator+(V3<T> a, V3<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> inline V3<T> operator-(V3<T> a, V3<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> inline V3<T> operator-(V3<T> a) { return mk(-a.x, -a.y, -a.z); }
template <typename T> inline V3<T> operator*(V3<T> a, V3<T> b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> inline V3<T> operator*(V3<T> a, T s) { return mk(a.x * s, a.y * s, a.z * s); }
template <typename T> inline V3<T> operator*(T s, V3<T> a) { return mk(s * a.x, s * a.y, s * a.z); }
template <typename T> inline V3<T> operator/(V3<T> a, T s) { return mk(a.x / s, a.y / s, a.z / s); }
template <typename T> inline void operator+=(V3<T>& a, V3<T> b) { a.x += b.x; a.y += b.y; a.z += b.z; }
// helper_math.h dot / length / lengthSquared (cuda_helper/helper_math.h:1277-1323, math/cuda_math_utils.cuh:74)
template <typename T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> inline T length(V3<T> v) { return tsqrt(dot(v, v)); }
template <typename T> inline T lengthSquared(V3<T> v) { return dot(v, v); }
template <typename T> inline T tmax(T a, T b) { return tfmax(a, b); }
template <typename T> inline T tmin(T a, T b) { return tfmin(a, b); }
// sgn (math/cuda_math_utils.cuh:77-82): int in {-1,0,1}, converted back to T
template <typename T> inline T sgnT(T v) { return T(int(T(0) < v) - int(v < T(0))); }

// Poly6Kernel (KERN:79-98)
template <typename T> struct Poly6 {
    T h, coef, h2;
    explicit Poly6(T radius) : h(radius) {
        h2 = h * h;
        T ih = T(1) / h;
        T ih3 = ih * ih * ih;
        T ih9 = ih3 * ih3 * ih3;
        coef = T(315) * ih9 / (T(64) * kPi<T>());
    }
    T operator()(T r) const {
        T r2 = r * r;
        if (r2 >= h2) return T(0);
        T d = h2 - r2;
        return coef * d * d * d;
    }
};

// SpikyKernelGrad (KERN:100-118)
template <typename T> struct SpikyGrad {
    T h, coef;
    explicit SpikyGrad(T radius) : h(radius) {
        T h2 = h * h;
        T h6 = h2 * h2 * h2;
        coef = T(-45) / (kPi<T>() * h6);
    }
    V3<T> operator()(V3<T> r) const {
        T rlen = length(r);
        if (rlen >= h || rlen < kEps<T>()) return mk(T(0), T(0), T(0));
        T d = h - rlen;
        return coef * d * d / rlen * r;
    }
};

// AdhesionAkinci13 (KERN:189-203)
template <typename T> struct Adhesion {
    T coef, h;
    explicit Adhesion(T radius) : h(radius) { coef = T(0.007f) / tpow(h, T(3.25f)); }
    T operator()(T r) const {
        if (T(2) * r > h && r <= h) return coef * tpow(T(-4) * r * r / h + T(6) * r - T(2) * h, T(0.25f));
        return T(0);
    }
};

// QuadraticBezierCoeff (UTIL:36-83), including the first segment's use of
// py1 for both control ordinates (UTIL:74).
template <typename T> struct Bezier {
    T a, b, c, d, e, py0, py1, px1, py2;
    Bezier(T py0_, T py1_, T px1_, T py2_) : py0(py0_), py1(py1_), px1(px1_), py2(py2_) {
        a = (px1 + T(1)) / T(4);
        b = T(-2) * a;
        c = b * b;
        d = T(-4) * (T(1) + b - px1);
        e = T(2) * (T(1) + b - px1);
    }
    T rx2t(T sr) const { return (b + tsqrt(c + d * (px1 - sr))) / e; }
    T operator()(T sr) const {
        if (sr < T(0)) return py0;
        if (sr >= T(1)) return py2;
        if (sr <= px1) {
            const T t = sr / px1;
            const T omt = T(1) - t;
            return omt * omt * py0 + T(2) * t * omt * py1 + t * t * py1;
        }
        const T t = rx2t(sr);
        const T omt = T(1) - t;
        return omt * omt * py1 + T(2) * t * omt * py1 + t * t * py2;
    }
};

// ComputeDemForces (DEM:20-51)
template <typename T> V3<T> demForce(V3<T> dij, V3<T> vij, T rij, T kn, T ks, T tanFrictionAngle) {
    V3<T> f = mk(T(0), T(0), T(0));
    T dist = length(dij);
    T pen = rij - dist;
    if (pen > T(0)) {
        V3<T> n = dij / dist;
        T dot_e = dot(vij, n);
        V3<T> vt = vij - dot_e * n;
        V3<T> fn = kn * pen * n;
        V3<T> fs = -ks * vt;
        T max_fs = lengthSquared(fn) * tpow(tanFrictionAngle, T(2));
        if (lengthSquared(fs) > max_fs) {
            T ratio = tsqrt(max_fs) / length(fs);
            fs = fs * ratio;
        }
        f = -fn - fs;
    }
    return f;
}

// ComputeDemCapillaryForces (DEM:53-90)
template <typename T> V3<T> capillaryForce(V3<T> dij, T radiusi, T sr, const Bezier<T>& G) {
    V3<T> f = mk(T(0), T(0), T(0));
    T contact_angle = T(30) / T(180) * kPi<T>();
    T vlb = T(4) / T(3) * kPi<T>() * tpow(radiusi, T(3)) * T(0.01f) * T(0.01f);
    T s_rupture = (T(1) + T(0.5f) * contact_angle) *
                  (tpow(vlb, T(1.f / 3.f)) + T(0.1f) * tpow(vlb, T(2.f / 3.f)));
    T dist = length(dij);
    T H = dist - (radiusi + radiusi);
    if (H < s_rupture && H > T(0)) {
        V3<T> N = dij / dist;
        T coeff_c = G(sr);
        T d = -H + tsqrt(H * H + vlb / (kPi<T>() * radiusi));
        T phi = tsqrt(T(2) * H / radiusi * (T(-1) + tsqrt(T(1) + vlb / (kPi<T>() * radiusi * H * H))));
        T ncp = T(-2) * kPi<T>() * coeff_c * radiusi * tcos(contact_angle) / (T(1) + H / (T(2) * d));
        T stf = T(-2) * kPi<T>() * coeff_c * radiusi * phi * tsin(contact_angle);
        f = -N * (ncp + stf);
    }
    return f;
}

// Upper bound of the distances at which any pair term is non-zero; used only
// to skip pairs whose every term is exactly zero (the reference adds +0 there).
template <typename T> T capillaryReach(T radiusi) {
    T contact_angle = T(30) / T(180) * kPi<T>();
    T vlb = T(4) / T(3) * kPi<T>() * tpow(radiusi, T(3)) * T(0.01f) * T(0.01f);
    T s_rupture = (T(1) + T(0.5f) * contact_angle) *
                  (tpow(vlb, T(1.f / 3.f)) + T(0.1f) * tpow(vlb, T(2.f / 3.f)));
    return T(2) * radiusi + s_rupture;
}

struct Int3 {
    int x, y, z;
};

template <typename T> struct Sim {
    // ---- parameters (sf_params, converted from the reference's float values) ----
    sf_params P;
    sf_boundary_params B;
    sf_solver_params S;
    int sort_multi = 1;  // SearcherParticleType::SEEPAGE_MULTI
    V3<T> lp, hp;
    T cell;
    Int3 g;
    int64_t G;  // number of cells
    // ---- particle state (reference layout: one array per field) ----
    int64_t n = 0;
    std::vector<int32_t> label;
    std::vector<int64_t> id, key;
    std::vector<V3<T>> pos, vel, acc, col, avgFlow, avgDrag, adhesion, avgAdhesion, cda0asat;
    std::vector<T> radius, mass, density, pressure, voidage, saturation, maxSat, amc, amcp;
    std::vector<T> accScale, pressureScale;  // FP64 error yardsticks (sum of |terms|)
    // ---- boundary ----
    int64_t nb = 0;
    std::vector<V3<T>> bpos;
    std::vector<int32_t> blabel;
    std::vector<T> bvolume;
    std::vector<int64_t> cellStart, bcellStart;
    // ---- solver state ----
    int64_t numSub = 1;
    T maxAccLen = 0;
    // parameter whose tangent is seeded (Sim<Dual1>): 0 none, 1 tan friction
    // angle, 2 capillary scale (factor on c0, cmc, csat), 3 permeability scale
    // (factor on cd)
    int seedParam = 0;
    T param(float v, int which, bool relative) const {
        return seeded<T>(v, which != 0 && which == seedParam ? (relative ? double(v) : 1.0) : 0.0);
    }

    static T f2t(float v) { return T(v); }
    V3<T> f3(const float* v) const { return mk(T(v[0]), T(v[1]), T(v[2])); }

    // ThrustHelper::ComputeGridXYZByPos3 / Pos2GridXYZ (THR:56-64, 92-114)
    Int3 p2xyz(V3<T> p) const {
        V3<T> rel = p - lp;
        Int3 r;
        r.x = std::min(std::max(toInt(rel.x / cell), 0), g.x - 1);
        r.y = std::min(std::max(toInt(rel.y / cell), 0), g.y - 1);
        r.z = std::min(std::max(toInt(rel.z / cell), 0), g.z - 1);
        return r;
    }
    // (int) truncation toward zero, saturating like the GPU conversion for
    // values a float position can produce.
    static int toInt(T v) {
        if (!(v == v)) return 0;
        if (v >= T(2147483520.0)) return 2147483647;
        if (v <= T(-2147483648.0)) return std::numeric_limits<int>::min();
        return int(v);
    }
    // GridXYZ2GridHash (THR:116-129): out of range -> G
    int64_t xyz2hash(int x, int y, int z) const {
        if (x >= 0 && x < g.x && y >= 0 && y < g.y && z >= 0 && z < g.z)
            return (int64_t(x) * g.y + y) * g.z + z;
        return G;
    }
    // Pos2GridHash (THR:66-89)
    int64_t pos2hash(V3<T> p) const {
        Int3 c = p2xyz(p);
        return int64_t(c.x) * g.y * g.z + int64_t(c.y) * g.z + c.z;
    }
    // Neighbor cell m of the 27-cell stencil (e.g. SFGPU:468-473).
    int64_t stencil(Int3 c, int m) const {
        return xyz2hash(c.x + (m / 9 - 1), c.y + ((m % 9) / 3 - 1), c.z + (m % 3 - 1));
    }

    void init(const sf_params* p, const sf_boundary_params* b, const sf_solver_params* s,
              const sf_scene_init* in, int sortMulti) {
        P = *p;
        B = *b;
        S = *s;
        sort_multi = sortMulti;
        lp = f3(B.lowest_point);
        hp = f3(B.highest_point);
        cell = T(B.kernel_radius);
        g = Int3{B.grid_size[0], B.grid_size[1], B.grid_size[2]};
        G = int64_t(g.x) * g.y * g.z;
        n = in->n;
        label.assign(in->label, in->label + n);
        id.resize(n);
        for (int64_t i = 0; i < n; ++i) id[i] = i;
        key.assign(n, 0);
        auto v3 = [&](const float* a, std::vector<V3<T>>& dst, int64_t cnt) {
            dst.assign(cnt, mk(T(0), T(0), T(0)));
            if (a)
                for (int64_t i = 0; i < cnt; ++i) dst[i] = mk(T(a[3 * i]), T(a[3 * i + 1]), T(a[3 * i + 2]));
        };
        auto v1 = [&](const float* a, std::vector<T>& dst, int64_t cnt) {
            dst.assign(cnt, T(0));
            if (a)
                for (int64_t i = 0; i < cnt; ++i) dst[i] = T(a[i]);
        };
        v3(in->pos, pos, n);
        v3(in->vel, vel, n);
        v3(in->col, col, n);
        v3(in->cda0asat, cda0asat, n);
        v1(in->mass, mass, n);
        v1(in->radius, radius, n);
        amc.assign(n, T(0));
        amcp.assign(n, T(0));
        if (in->amcamcp)
            for (int64_t i = 0; i < n; ++i) {
                amc[i] = T(in->amcamcp[2 * i]);
                amcp[i] = T(in->amcamcp[2 * i + 1]);
            }
        acc.assign(n, mk(T(0), T(0), T(0)));
        avgFlow = avgDrag = adhesion = avgAdhesion = acc;
        density.assign(n, T(0));
        pressure = voidage = saturation = maxSat = accScale = pressureScale = density;
        nb = in->nb;
        v3(in->bpos, bpos, nb);
        blabel.assign(nb, 0);
        if (in->blabel) blabel.assign(in->blabel, in->blabel + nb);
        bvolume.assign(nb, T(0));
        cellStart.assign(G + 1, 0);
        bcellStart.assign(G + 1, 0);
        buildBoundary();
        numSub = 1;
    }

    // CudaSFParticles::AddSphParticles (cuda_sf_particles.cu:50-68): num water
    // particles appended after the live ones with the given position, colour,
    // velocity, mass and radius; refused when Size() + num >= MaxSize() (the
    // caller passes the capacity). The reference leaves the new entries of the
    // other arrays as they were; here they start at zero, which is what the
    // next substep's passes overwrite or never read for water.
    bool addSphParticles(const float* pos3, int64_t num, const float* c, const float* v, float m, float r,
                         int64_t capacity) {
        if (n + num >= capacity) return false;
        const V3<T> zero = mk(T(0), T(0), T(0));
        for (int64_t k = 0; k < num; ++k) {
            label.push_back(0);
            id.push_back(n + k);
            key.push_back(0);
            pos.push_back(f3(pos3 + 3 * k));
            vel.push_back(f3(v));
            col.push_back(f3(c));
            mass.push_back(T(m));
            radius.push_back(T(r));
            for (auto* a : {&acc, &avgFlow, &avgDrag, &adhesion, &avgAdhesion, &cda0asat}) a->push_back(zero);
            for (auto* a : {&density, &pressure, &voidage, &saturation, &maxSat, &amc, &amcp, &accScale,
                            &pressureScale})
                a->push_back(T(0));
        }
        n += num;
        return true;
    }

    // Stable counting sort by key: the permutation thrust::sort_by_key gives
    // for integer keys (SRCH:64-116).
    std::vector<int64_t> stableOrder(const std::vector<int64_t>& k, std::vector<int64_t>& start) const {
        const int64_t cnt = int64_t(k.size());
        start.assign(G + 1, 0);
        for (int64_t i = 0; i < cnt; ++i) start[k[i]]++;  // CountingInCell_CUDA (searcher_gpu.cuh:18-25)
        int64_t run = 0;                                  // thrust::exclusive_scan (SRCH:47)
        for (int64_t c = 0; c <= G; ++c) {
            int64_t v = start[c];
            start[c] = run;
            run += v;
        }
        std::vector<int64_t> next(start.begin(), start.end() - 1), order(cnt);
        for (int64_t i = 0; i < cnt; ++i) order[next[k[i]]++] = i;
        return order;
    }
    template <typename V> static void permute(std::vector<V>& a, const std::vector<int64_t>& order) {
        std::vector<V> t(a.size());
        for (size_t i = 0; i < order.size(); ++i) t[i] = a[order[i]];
        a.swap(t);
    }

    // Boundary searcher build + Akinci boundary volume at system construction
    // (cuda_base_system.cu:26 -> SRCH:36-51,125-139; SYS:121-136; SYSG:19-67).
    void buildBoundary() {
        std::vector<int64_t> bk(nb);
        for (int64_t i = 0; i < nb; ++i) bk[i] = pos2hash(bpos[i]);
        std::vector<int64_t> order = stableOrder(bk, bcellStart);
        permute(bpos, order);
        permute(blabel, order);
        Poly6<T> W(cell);
        std::vector<T> vol(nb, T(0));
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < nb; ++i) {
            Int3 c = p2xyz(bpos[i]);
            T v = T(0);
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                for (int64_t j = bcellStart[hsh]; j < bcellStart[hsh + 1]; ++j)
                    if (i != j) v += W(length(bpos[i] - bpos[j]));
            }
            vol[i] = T(1) / tmax(v, kEps<T>());
        }
        bvolume.swap(vol);
    }

    // CudaGNBaseSearcher::BuildGNSearcher (SRCH:36-51) with the SEEPAGE_MULTI
    // SortData (SRCH:85-112): every persistent array is permuted; acc,
    // density, ... are recomputed every substep and are not.
    void sortStage() {
        for (int64_t i = 0; i < n; ++i) key[i] = pos2hash(pos[i]);
        std::vector<int64_t> order = stableOrder(key, cellStart);
        permute(label, order);
        permute(pos, order);
        permute(vel, order);
        permute(col, order);
        permute(radius, order);
        permute(mass, order);
        permute(maxSat, order);
        permute(id, order);
        permute(key, order);
        if (sort_multi) {
            permute(cda0asat, order);
            permute(amc, order);
            permute(amcp, order);
        }
    }

    // CudaSphSFSolver::ExtraForces (SOLV.cu:390-402) for one label (-1 = all)
    void extraForces(int which) {
        V3<T> gv = f3(P.gravity);
        for (int64_t i = 0; i < n; ++i)
            if (which < 0 || label[i] == which) {
                acc[i] = mk(T(0), T(0), T(0)) + gv;
                accScale[i] = length(gv);
            }
    }

    // ComputeSFDensity_CUDA + ComputeSFFluidDensity + ComputeBoundaryDensity
    // (SFGPU:408-480; SPHC:70-87). The self term enters twice: once as m_i W(0)
    // and once inside the j loop.
    void densityPass() {
        Poly6<T> W(cell);
        const T rho0 = T(P.sph_density), rho1 = T(P.dem_density);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] == 1) {
                density[i] = rho1;
                continue;
            }
            Int3 c = p2xyz(pos[i]);
            T d = mass[i] * W(T(0));
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                for (int64_t j = cellStart[hsh]; j < cellStart[hsh + 1]; ++j)
                    if (label[i] == label[j]) d += mass[j] * W(length(pos[i] - pos[j]));
                for (int64_t j = bcellStart[hsh]; j < bcellStart[hsh + 1]; ++j)
                    d += rho0 * bvolume[j] * W(length(pos[i] - bpos[j]));
            }
            density[i] = d;
        }
    }

    // ComputeSFPressureByTait_CUDA (TAIT:19-44) for WCSPH, ComputeSFPressure_CUDA
    // (SFGPU:482-508, negativeScale 1 per SOLV.cu:51-66) for plain SPH.
    void pressurePass() {
        const T rho0 = T(P.sph_density), stiff = T(P.sph_stiff);
        const bool tait = P.solver_type == SF_SOLVER_WCSPH;
        const T neg = tait ? T(S.negative_scale) : T(1);
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] == 0) {
                T p;
                if (tait) {
                    T x7 = tpow(density[i] / rho0, T(7));
                    p = stiff * (x7 - T(1));
                    pressureScale[i] = stiff * x7;
                } else {
                    p = stiff * (density[i] - rho0);
                    pressureScale[i] = stiff * density[i];
                }
                if (p < T(0)) p *= neg;
                pressure[i] = p;
            } else if (label[i] == 1) {
                pressure[i] = T(0);
                pressureScale[i] = T(0);
            }
        }
    }

    // ComputeSFAvgFlow_CUDA with ComputeSFSandVolume / ComputeSFAvgFlow
    // (SFGPU:111-173, 510-572).
    void avgFlowPass() {
        Poly6<T> W(cell);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            Int3 c = p2xyz(pos[i]);
            T v_s = 0, v_w = 0, sand_volume = 0;
            V3<T> avg_s = mk(T(0), T(0), T(0)), avg_w = avg_s;
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                const int64_t j0 = cellStart[hsh], j1 = cellStart[hsh + 1];
                for (int64_t j = j0; j < j1; ++j)
                    if (label[j] == 1 && density[j] != T(0)) {
                        T vj = mass[j] / density[j];
                        T wij = W(length(pos[i] - pos[j]));
                        sand_volume += vj * wij;
                    }
                for (int64_t j = j0; j < j1; ++j) {
                    T vj = mass[j] / density[j];
                    T wij = W(length(pos[i] - pos[j]));
                    if (label[i] == 1 && label[j] == 0) {
                        avg_s += vel[j] * vj * wij;
                        v_s += vj * wij;
                    } else if (label[i] == 0 && label[j] == 1) {
                        avg_w += vel[j] * vj * wij;
                        v_w += vj * wij;
                    }
                }
            }
            if (label[i] == 0 && v_w != T(0))
                avgFlow[i] = avg_w / v_w;
            else if (label[i] == 1 && v_s != T(0))
                avgFlow[i] = avg_s / v_s;
            else
                avgFlow[i] = mk(T(0), T(0), T(0));
            voidage[i] = T(1) - sand_volume;
            saturation[i] = v_s;
        }
    }

    // ComputeSFSandVoidage_CUDA + ComputeSFSandVoidage (SFGPU:209-238, 680-721).
    void sandVoidagePass() {
        Poly6<T> W(cell);
        std::vector<T> out(voidage);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] != 1) continue;
            Int3 c = p2xyz(pos[i]);
            T num = 0, den = 0;
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                for (int64_t j = cellStart[hsh]; j < cellStart[hsh + 1]; ++j)
                    if (label[i] == 1 && label[j] == 0) {
                        T vj = mass[j] / density[j];
                        T wij = W(length(pos[i] - pos[j]));
                        num += voidage[j] * vj * wij;
                        den += vj * wij;
                    }
            }
            out[i] = den != T(0) ? num / den : T(0);
        }
        voidage.swap(out);
    }

    // Compute[Multi]SFWaterAdhesionForces_CUDA + ComputeSFWaterAdhesionForces
    // (SFGPU:175-207, 574-678). MULTI_SF hard-codes QuadraticBezierCoeff(0, 1.5, 0.5, 0.8)
    // (SFGPU:667); SF uses (a0, amc, amcp, asat) (SOLV.cu:119).
    void adhesionPass() {
        Poly6<T> W(cell);
        Adhesion<T> A(cell);
        Bezier<T> G_ = P.sf_type == SF_TYPE_MULTI_SF
                           ? Bezier<T>(T(0.f), T(1.5f), T(0.5f), T(0.8f))
                           : Bezier<T>(T(P.sf_a0), T(P.sf_amc), T(P.sf_amc_p), T(P.sf_asat));
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] != 0) continue;
            Int3 c = p2xyz(pos[i]);
            T v_s = 0;
            V3<T> ad = mk(T(0), T(0), T(0));
            T sc = 0;
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                for (int64_t j = cellStart[hsh]; j < cellStart[hsh + 1]; ++j)
                    if (label[i] == 0 && label[j] == 1) {
                        V3<T> dpij = pos[i] - pos[j];
                        T ldp = length(dpij);
                        T wij = W(ldp);
                        T adij = A(ldp);
                        V3<T> t = G_(saturation[j]) * mass[i] * mass[j] * adij * dpij / tmax(kEps<T>(), ldp);
                        ad += t;
                        sc += length(t);
                        T vj = mass[j] / density[j];
                        v_s += vj * wij;
                    }
            }
            adhesion[i] = ad;
            if (v_s != T(0)) avgAdhesion[i] = ad / v_s;
            (void)sc;
        }
    }

    // ComputeSFWetSandColor_CUDA (SFGPU:952-977)
    void wetColorPass() {
        V3<T> dry = f3(P.sf_dry_sand_color), wet = f3(P.sf_wet_sand_color);
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] != 1) continue;
            V3<T> blend = col[i];
            if (maxSat[i] < saturation[i]) blend = dry + (wet - dry) * saturation[i];
            col[i] = blend;
            if (maxSat[i] < saturation[i]) maxSat[i] = saturation[i];
        }
    }

    // Compute[Multi]SFSandLinearMomentum_CUDA (SFGPU:723-897) with
    // ComputeSFUniRadiusDemForces (21-50), ComputeSFUniRadiusDemCapillaryForces
    // (83-109), ComputeSFSandBuoyancyForces (240-273), ComputeSFSandAdhesionTerm
    // (314-341), ComputeSFUniRadiusDemBoundaryForces (52-81) and
    // ComputeDemWorldBoundaryForces (DEM:132-199). acc += 2 (f + df) / m.
    void sandMomentumPass() {
        Poly6<T> W(cell);
        SpikyGrad<T> nablaW(cell);
        Bezier<T> Gc(param(P.sf_c0, 2, true), param(P.sf_cmc, 2, true), T(P.sf_cmc_p),
                     param(P.sf_csat, 2, true));  // SOLV.cu:249,308
        const T radius_ = T(P.dem_particle_radius), waterRadius = T(P.sph_particle_radius);
        const T young = T(P.dem_young), poisson = T(P.dem_poisson), tanF = param(P.dem_tan_friction_angle, 1, false);
        const T gravity = T(tfabs(P.gravity[1]));  // abs(params.gravity.y), cuda_wcsph_sf_solver.cpp:106,136
        const T rho0 = T(P.sph_density);
        const bool multi = P.sf_type == SF_TYPE_MULTI_SF;
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] != 1) continue;
            T v_w = 0, sc = 0;
            V3<T> f = mk(T(0), T(0), T(0)), df = f;
            Int3 c = p2xyz(pos[i]);
            auto addf = [&](V3<T> t) {
                f += t;
                sc += length(t);
            };
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                const int64_t j0 = cellStart[hsh], j1 = cellStart[hsh + 1];
                for (int64_t j = j0; j < j1; ++j)
                    if (i != j && label[i] == label[j]) {
                        V3<T> dij = pos[j] - pos[i];
                        T rij = T(2) * radius_;
                        V3<T> vij = vel[j] - vel[i];
                        T kn = young * radius_;
                        T ks = kn * poisson;
                        addf(demForce(dij, vij, rij, kn, ks, tanF));
                    }
                for (int64_t j = j0; j < j1; ++j)
                    if (i != j && label[i] == label[j]) {
                        V3<T> dij = pos[j] - pos[i];
                        T avg_sr = (saturation[i] + saturation[j]) / T(2);
                        addf(capillaryForce(dij, radius_, avg_sr, Gc));
                    }
                for (int64_t j = j0; j < j1; ++j)
                    if (i != j && label[i] == 1 && label[j] == 0 && voidage[j] > T(0) && voidage[j] <= T(1)) {
                        T di = density[i];
                        T dj = density[j] / tmax(kEps<T>(), voidage[j]);
                        V3<T> dij = pos[i] - pos[j];
                        T wij = W(length(dij));
                        V3<T> nab = nablaW(dij);
                        v_w += mass[j] / dj * wij;
                        addf(-mass[i] * mass[j] * pressure[j] / tmax(kEps<T>(), di * dj) * nab);
                    }
                for (int64_t j = j0; j < j1; ++j)
                    if (label[i] == 1 && label[j] == 0) {
                        V3<T> dij = pos[i] - pos[j];
                        T wij = W(length(dij));
                        T v = mass[i] / tmax(kEps<T>(), density[i]);
                        addf(wij * v * avgAdhesion[j]);
                    }
                for (int64_t j = bcellStart[hsh]; j < bcellStart[hsh + 1]; ++j)
                    if (blabel[j] == 1) {
                        V3<T> dij = pos[i] - bpos[j];
                        T rij = T(2) * radius_;
                        T kn = young * radius_;
                        T ks = kn * poisson;
                        V3<T> vij = mk(-vel[i].x, -vel[i].y, -vel[i].z);
                        addf(demForce(dij, vij, rij, kn, ks, tanF));
                    }
            }
            // ComputeDemWorldBoundaryForces (DEM:132-199); the z-min wall tests 2*rij (DEM:191).
            {
                const V3<T> pi = pos[i], vi = vel[i];
                T rij = waterRadius + radius_;
                T kn = young * radius_;
                T ks = kn * poisson;
                auto wall = [&](V3<T> N, T diff) { addf(demForce(N * diff, -vi, rij, kn, ks, tanF)); };
                if (pi.x > hp.x - rij) wall(mk(T(1), T(0), T(0)), tfabs(pi.x - hp.x));
                if (pi.x < lp.x + rij) wall(mk(T(-1), T(0), T(0)), tfabs(pi.x - lp.x));
                if (pi.y > hp.y - rij) wall(mk(T(0), T(1), T(0)), tfabs(pi.y - hp.y));
                if (pi.y < lp.y + rij) wall(mk(T(0), T(-1), T(0)), tfabs(pi.y - lp.y));
                if (pi.z > hp.z - rij) wall(mk(T(0), T(0), T(1)), tfabs(pi.z - hp.z));
                if (pi.z < lp.z + T(2) * rij) wall(mk(T(0), T(0), T(-1)), tfabs(pi.z - lp.z));
            }
            if (voidage[i] < T(1) && voidage[i] > T(0)) {
                T cd = multi ? cda0asat[i].x : param(P.sf_cd, 3, true);
                T dragCoeff = cd * tpow(voidage[i], T(3)) / tpow(T(1) - voidage[i], T(2));
                if (dragCoeff != T(0))
                    df = gravity * rho0 * tpow(voidage[i], T(2)) / dragCoeff * (avgFlow[i] - vel[i]) * mass[i] /
                         density[i];
            }
            avgDrag[i] = v_w != T(0) ? df / v_w : mk(T(0), T(0), T(0));
            acc[i] += T(2) * (f + df) / mass[i];
            accScale[i] += T(2) * (sc + length(df)) / mass[i];
        }
    }

    // ComputeSFWaterLinearMomentum_CUDA (SFGPU:899-950) with
    // ComputeSFWaterPressureTerm (343-369), ComputeSFWaterArtificialViscosity
    // (371-406), ComputeSFWaterSeepageTerm (275-312), ComputeBoundaryPressure and
    // ComputeBoundaryViscosity (SPHC:89-139), both called with rho0 in place of
    // the particle density (SFGPU:944-945). acc += a - F_adh / m.
    void waterMomentumPass() {
        Poly6<T> W(cell);
        SpikyGrad<T> nablaW(cell);
        const T rho0 = T(P.sph_density), nu = T(P.sph_nu), bnu = T(P.sph_bnu);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] != 0) continue;
            V3<T> a = mk(T(0), T(0), T(0));
            T sc = 0;
            auto adda = [&](V3<T> t) {
                a += t;
                sc += length(t);
            };
            Int3 c = p2xyz(pos[i]);
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                const int64_t j0 = cellStart[hsh], j1 = cellStart[hsh + 1];
                for (int64_t j = j0; j < j1; ++j)
                    if (i != j && label[i] == label[j]) {
                        T di = density[i] / tmax(kEps<T>(), voidage[i]);
                        T dj = density[j] / tmax(kEps<T>(), voidage[j]);
                        adda(-mass[j] *
                             (pressure[i] / tmax(kEps<T>(), di * di) + pressure[j] / tmax(kEps<T>(), dj * dj)) *
                             nablaW(pos[i] - pos[j]));
                    }
                for (int64_t j = j0; j < j1; ++j)
                    if (i != j && label[i] == label[j]) {
                        V3<T> dpij = pos[i] - pos[j];
                        V3<T> dv = vel[i] - vel[j];
                        T dd = dot(dv, dpij);
                        if (dd < T(0)) {
                            T di = density[i] / tmax(kEps<T>(), voidage[i]);
                            T dj = density[j] / tmax(kEps<T>(), voidage[j]);
                            T pij = -nu / (di + dj) * (dd / (lengthSquared(dpij) + kEps<T>()));
                            adda(-mass[j] * pij * nablaW(dpij));
                        }
                    }
                for (int64_t j = j0; j < j1; ++j)
                    if (i != j && label[i] == 0 && label[j] == 1) {
                        T di = density[i] / tmax(kEps<T>(), voidage[i]);
                        T dj = density[j];
                        V3<T> dij = pos[i] - pos[j];
                        T wij = W(length(dij));
                        V3<T> nab = nablaW(dij);
                        V3<T> buoy = -mass[j] * pressure[i] / tmax(kEps<T>(), di * dj) * nab;
                        V3<T> drag = -wij / di * avgDrag[j];
                        adda(buoy + drag);
                        sc += length(buoy) + length(drag) - length(buoy + drag);
                    }
                const int64_t b0 = bcellStart[hsh], b1 = bcellStart[hsh + 1];
                for (int64_t j = b0; j < b1; ++j)
                    adda(-rho0 * bvolume[j] * (pressure[i] / tmax(kEps<T>(), rho0 * rho0)) * nablaW(pos[i] - bpos[j]));
                for (int64_t j = b0; j < b1; ++j) {
                    V3<T> dpij = pos[i] - bpos[j];
                    T dd = dot(vel[i], dpij);
                    if (dd < T(0)) {
                        T pij = -bnu / (T(2) * rho0) * (dd / (lengthSquared(dpij) + kEps<T>()));
                        adda(-bvolume[j] * rho0 * pij * nablaW(dpij));
                    }
                }
            }
            acc[i] += a - adhesion[i] / mass[i];
            accScale[i] += sc + length(adhesion[i]) / mass[i];
        }
    }

    // ComputeSubTimeStepsByCFL (WCSPH.cu:35-58): the first maximum of |acc|
    // over all particles; N_sub = (size_t)(T / dt*). Plain SPH uses
    // renderInterval / params.dt (SOLV.cpp:23).
    void cflPass(T renderInterval) {
        int64_t best = 0;
        T bestLen = n > 0 ? length(acc[0]) : T(0);
        for (int64_t i = 1; i < n; ++i) {
            T l = length(acc[i]);
            if (bestLen < l) {
                bestLen = l;
                best = i;
            }
        }
        (void)best;
        maxAccLen = bestLen;
        const T m = T(P.sph_mass), h = T(B.kernel_radius);
        if (P.solver_type == SF_SOLVER_WCSPH) {
            T maxForce = bestLen * m;
            T bySpeed = T(0.4f) * h / T(S.speed_of_sound);
            T byForce = T(0.25f) * tsqrt(h * m / maxForce);
            T desired = tmin(T(S.time_step_limit_scale) * tmin(bySpeed, byForce), T(P.dt));
            numSub = int64_t(renderInterval / desired);
        } else {
            numSub = int64_t(renderInterval / T(P.dt));
        }
    }

    // dt of the adaptive substep's Advect: WCSPH advects by renderInterval /
    // N_sub (WCSPH.cpp:168-172), plain SPH by params.dt whatever N_sub rounds
    // to (SOLV.cpp:23, 141-146).
    T advectDt(T renderInterval) const {
        return P.solver_type == SF_SOLVER_WCSPH ? renderInterval / T(numSub) : T(P.dt);
    }

    // CudaSphSFSolver::Advect (SOLV.cu:355-388) = CudaSFParticles::Advect
    // (PART.cu:18-48, AccDampingForSand PART.cuh:19-40) + SFWaterBoundaryConstrain_CUDA
    // (SFGPU:979-1074) + the two adhesion clears.
    void advectPass(T dt) {
        const T damping = T(P.dem_damping);
        const T radius_ = T(P.sph_particle_radius);
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] == 1) {
                V3<T> a = acc[i];
                V3<T> q = a * (vel[i] + T(0.5f) * dt * a);
                V3<T> s = mk(sgnT(q.x), sgnT(q.y), sgnT(q.z));
                acc[i] = a * (mk(T(1), T(1), T(1)) - damping * s);
            }
        }
        for (int64_t i = 0; i < n; ++i) vel[i] = vel[i] + dt * acc[i];
        for (int64_t i = 0; i < n; ++i) pos[i] = pos[i] + dt * vel[i];
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (label[i] != 0) continue;
            V3<T> tp = pos[i], tv = vel[i];
            if (tp.x > hp.x - T(2) * radius_) { tp.x = hp.x - T(2) * radius_; tv.x = tmin(tv.x, T(0)); }
            if (tp.x < lp.x + T(2) * radius_) { tp.x = lp.x + T(2) * radius_; tv.x = tmax(tv.x, T(0)); }
            if (tp.y > hp.y - T(2) * radius_) { tp.y = hp.y - T(2) * radius_; tv.y = tmin(tv.y, T(0)); }
            if (tp.y < lp.y + T(2) * radius_) { tp.y = lp.y + T(2) * radius_; tv.y = tmax(tv.y, T(0)); }
            if (tp.z > hp.z - T(2) * radius_) { tp.z = hp.z - T(2) * radius_; tv.z = tmin(tv.z, T(0)); }
            if (tp.z < lp.z + T(2) * radius_) { tp.z = lp.z + T(2) * radius_; tv.z = tmax(tv.z, T(0)); }
            Int3 c = p2xyz(pos[i]);
            for (int m = 0; m < 27; ++m) {
                int64_t hsh = stencil(c, m);
                if (hsh == G) continue;
                for (int64_t j = bcellStart[hsh]; j < bcellStart[hsh + 1]; ++j)
                    if (blabel[j] == 1) {
                        T dpij = length(pos[i] - bpos[j]);
                        T overlap = dpij - T(2) * radius_;
                        if (overlap < T(0)) {
                            V3<T> nn = (pos[i] - bpos[j]) / dpij;
                            tv = tv * T(0);
                            tp += nn * -overlap;
                        }
                    }
            }
            pos[i] = tp;
            vel[i] = tv;
        }
        for (int64_t i = 0; i < n; ++i) {
            adhesion[i] = mk(T(0), T(0), T(0));
            avgAdhesion[i] = adhesion[i];
        }
    }

    void runStage(int stage, T timeArg, bool adaptive) {
        switch (stage) {
        case SF_STAGE_SORT: sortStage(); break;
        case SF_STAGE_DENSITY: densityPass(); pressurePass(); break;
        case SF_STAGE_AVGFLOW: avgFlowPass(); break;
        case SF_STAGE_VOIDAGE_ADHESION: sandVoidagePass(); adhesionPass(); wetColorPass(); break;
        case SF_STAGE_SAND_MOMENTUM: extraForces(1); sandMomentumPass(); break;
        case SF_STAGE_WATER_MOMENTUM: extraForces(0); waterMomentumPass(); break;
        case SF_STAGE_INTEGRATE: {
            T dt = timeArg;
            if (adaptive) {
                cflPass(timeArg);
                dt = advectDt(timeArg);
            }
            advectPass(dt);
            break;
        }
        default: break;
        }
    }

    // One reference substep in the order of CudaWCSphSFSolver::UpdateSolver
    // (WCSPH.cpp:34-178) preceded by BuildGNSearcher (SYS:68).
    void substep(T timeArg, bool adaptive) {
        sortStage();
        extraForces(-1);
        densityPass();
        pressurePass();
        avgFlowPass();
        sandVoidagePass();
        adhesionPass();
        sandMomentumPass();
        waterMomentumPass();
        wetColorPass();
        T dt = timeArg;
        if (adaptive) {
            cflPass(timeArg);
            dt = advectDt(timeArg);
        }
        advectPass(dt);
    }
};

struct Handle {
    // 32, 64, 65 = FP64 with one forward-mode tangent, 66 = the FP32
    // trajectory with one FP64 forward-mode tangent
    int precision;
    Sim<float> f;
    Sim<double> d;
    Sim<Dual1> j;
    Sim<DualF> jf;
    template <typename F> auto visit(F&& fn) {
        if (precision == 66) return fn(jf);
        if (precision == 65) return fn(j);
        if (precision == 64) return fn(d);
        return fn(f);
    }
    // the forward-mode handles only
    template <typename F> int visitDual(F&& fn) {
        if (precision == 66) return fn(jf);
        if (precision == 65) return fn(j);
        return SF_ERR_INVALID;
    }
};

// Tangents (Sim<Dual1> / Sim<DualF>) of positions or velocities, in the current internal order.
template <typename D> inline int tangentField(Sim<D>& s, int field, double* get, const double* set, int64_t count) {
    if (count != s.n || (field != SF_FIELD_POS && field != SF_FIELD_VEL)) return SF_ERR_INVALID;
    std::vector<V3<D>>& a = field == SF_FIELD_POS ? s.pos : s.vel;
    for (int64_t i = 0; i < s.n; ++i) {
        if (set) {
            a[i].x.d = set[3 * i];
            a[i].y.d = set[3 * i + 1];
            a[i].z.d = set[3 * i + 2];
        } else {
            get[3 * i] = a[i].x.d;
            get[3 * i + 1] = a[i].y.d;
            get[3 * i + 2] = a[i].z.d;
        }
    }
    return SF_OK;
}

template <typename T> int getField(Sim<T>& s, int field, double* dst, int64_t count) {
    const int64_t n = (field >= SF_BFIELD_POS && field < 100) ? s.nb : s.n;
    if (count != n) return SF_ERR_INVALID;
    auto put3 = [&](const std::vector<V3<T>>& a) {
        for (int64_t i = 0; i < n; ++i) {
            dst[3 * i] = double(a[i].x);
            dst[3 * i + 1] = double(a[i].y);
            dst[3 * i + 2] = double(a[i].z);
        }
    };
    auto put1 = [&](const auto& a) {
        for (int64_t i = 0; i < n; ++i) dst[i] = double(a[i]);
    };
    switch (field) {
    case SF_FIELD_POS: put3(s.pos); break;
    case SF_FIELD_VEL: put3(s.vel); break;
    case SF_FIELD_ACC: put3(s.acc); break;
    case SF_FIELD_COL: put3(s.col); break;
    case SF_FIELD_LABEL: put1(s.label); break;
    case SF_FIELD_RADIUS: put1(s.radius); break;
    case SF_FIELD_MASS: put1(s.mass); break;
    case SF_FIELD_DENSITY: put1(s.density); break;
    case SF_FIELD_PRESSURE: put1(s.pressure); break;
    case SF_FIELD_VOIDAGE: put1(s.voidage); break;
    case SF_FIELD_SATURATION: put1(s.saturation); break;
    case SF_FIELD_MAX_SATURATION: put1(s.maxSat); break;
    case SF_FIELD_AVG_FLOW: put3(s.avgFlow); break;
    case SF_FIELD_AVG_DRAG: put3(s.avgDrag); break;
    case SF_FIELD_ADHESION: put3(s.adhesion); break;
    case SF_FIELD_AVG_ADHESION: put3(s.avgAdhesion); break;
    case SF_FIELD_CDA0ASAT: put3(s.cda0asat); break;
    case SF_FIELD_AMCAMCP:
        for (int64_t i = 0; i < n; ++i) {
            dst[2 * i] = double(s.amc[i]);
            dst[2 * i + 1] = double(s.amcp[i]);
        }
        break;
    case SF_FIELD_ID: put1(s.id); break;
    case SF_FIELD_KEY: put1(s.key); break;
    case SF_BFIELD_POS: put3(s.bpos); break;
    case SF_BFIELD_LABEL: put1(s.blabel); break;
    case SF_BFIELD_VOLUME: put1(s.bvolume); break;
    case 100: put1(s.accScale); break;       // |acc| yardstick: sum of |terms|
    case 101: put1(s.pressureScale); break;  // pressure yardstick: stiff * (rho/rho0)^7
    default: return SF_ERR_INVALID;
    }
    return SF_OK;
}

template <typename T> int setField(Sim<T>& s, int field, const double* src, int64_t count) {
    const int64_t n = (field >= SF_BFIELD_POS) ? s.nb : s.n;
    if (count != n) return SF_ERR_INVALID;
    auto get3 = [&](std::vector<V3<T>>& a) {
        for (int64_t i = 0; i < n; ++i) a[i] = mk(T(src[3 * i]), T(src[3 * i + 1]), T(src[3 * i + 2]));
    };
    auto get1 = [&](auto& a) {
        using E = typename std::decay<decltype(a[0])>::type;
        for (int64_t i = 0; i < n; ++i) a[i] = E(src[i]);
    };
    switch (field) {
    case SF_FIELD_POS: get3(s.pos); break;
    case SF_FIELD_VEL: get3(s.vel); break;
    case SF_FIELD_ACC: get3(s.acc); break;
    case SF_FIELD_COL: get3(s.col); break;
    case SF_FIELD_LABEL: get1(s.label); break;
    case SF_FIELD_RADIUS: get1(s.radius); break;
    case SF_FIELD_MASS: get1(s.mass); break;
    case SF_FIELD_DENSITY: get1(s.density); break;
    case SF_FIELD_PRESSURE: get1(s.pressure); break;
    case SF_FIELD_VOIDAGE: get1(s.voidage); break;
    case SF_FIELD_SATURATION: get1(s.saturation); break;
    case SF_FIELD_MAX_SATURATION: get1(s.maxSat); break;
    case SF_FIELD_AVG_FLOW: get3(s.avgFlow); break;
    case SF_FIELD_AVG_DRAG: get3(s.avgDrag); break;
    case SF_FIELD_ADHESION: get3(s.adhesion); break;
    case SF_FIELD_AVG_ADHESION: get3(s.avgAdhesion); break;
    case SF_FIELD_CDA0ASAT: get3(s.cda0asat); break;
    case SF_FIELD_AMCAMCP:
        for (int64_t i = 0; i < n; ++i) {
            s.amc[i] = T(src[2 * i]);
            s.amcp[i] = T(src[2 * i + 1]);
        }
        break;
    case SF_FIELD_ID: get1(s.id); break;
    case SF_FIELD_KEY: get1(s.key); break;
    default: return SF_ERR_INVALID;
    }
    return SF_OK;
}

}  // namespace sfo

extern "C" {

// Create an oracle over one scene. precision: 32 or 64. sort_multi: 1 =
// SearcherParticleType::SEEPAGE_MULTI (all arrays permuted), 0 = SEEPAGE.
void* sfo_create(int precision, const sf_params* p, const sf_boundary_params* b, const sf_solver_params* s,
                 const sf_scene_init* in, int sort_multi) {
    auto* h = new sfo::Handle();
    h->precision = (precision == 64 || precision == 65 || precision == 66) ? precision : 32;
    h->visit([&](auto& sim) {
        sim.init(p, b, s, in, sort_multi);
        return 0;
    });
    return h;
}

void sfo_destroy(void* hv) { delete static_cast<sfo::Handle*>(hv); }

int sfo_size(void* hv, int64_t* n, int64_t* nb) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) {
        *n = sim.n;
        *nb = sim.nb;
        return int(SF_OK);
    });
}

int sfo_get_field(void* hv, int field, double* dst, int64_t count) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) { return sfo::getField(sim, field, dst, count); });
}

int sfo_set_field(void* hv, int field, const double* src, int64_t count) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) { return sfo::setField(sim, field, src, count); });
}

// which: 0 = particle cell table, 1 = boundary cell table (G+1 entries)
int sfo_get_cell_table(void* hv, int which, int64_t* dst, int64_t count) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) {
        const std::vector<int64_t>& t = which ? sim.bcellStart : sim.cellStart;
        if (count != int64_t(t.size())) return int(SF_ERR_INVALID);
        std::memcpy(dst, t.data(), sizeof(int64_t) * t.size());
        return int(SF_OK);
    });
}

int sfo_run_stage(void* hv, int stage, double time_arg, int adaptive) {
    if (stage < 0 || stage >= SF_STAGE_COUNT) return SF_ERR_INVALID;
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) {
        using T = typename std::decay<decltype(sim.maxAccLen)>::type;
        sim.runStage(stage, T(time_arg), adaptive != 0);
        return int(SF_OK);
    });
}

// n substeps; adaptive != 0: each is UpdateSystem(time_arg), else dt = time_arg.
int sfo_substeps(void* hv, double time_arg, int adaptive, int64_t n) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) {
        using T = typename std::decay<decltype(sim.maxAccLen)>::type;
        for (int64_t k = 0; k < n; ++k) sim.substep(T(time_arg), adaptive != 0);
        return int(SF_OK);
    });
}

// The adaptive frame loop of seepage_flows/src/seepageflow/main.cpp:235-247.
int sfo_frame_adaptive(void* hv, double render_interval, int64_t* n_calls) {
    int64_t calls = 0;
    static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) {
        using T = typename std::decay<decltype(sim.maxAccLen)>::type;
        T remaining = T(render_interval);
        while (remaining > T(1e-6f)) {
            sim.substep(remaining, true);
            remaining -= remaining / T(sim.numSub);
            ++calls;
        }
        return 0;
    });
    if (n_calls) *n_calls = calls;
    return SF_OK;
}

// AddSphParticles of num points (label 0); capacity plays MaxSize().
// Returns SF_ERR_CAPACITY (nothing added) when Size() + num >= capacity.
int sfo_add_sph_particles(void* hv, const float* pos3, int64_t num, const float* col, const float* vel, float mass,
                          float radius, int64_t capacity) {
    if (num < 0 || (num > 0 && !pos3) || !col || !vel) return SF_ERR_INVALID;
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) {
        return sim.addSphParticles(pos3, num, col, vel, mass, radius, capacity) ? int(SF_OK) : int(SF_ERR_CAPACITY);
    });
}

int64_t sfo_num_substeps(void* hv) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) { return sim.numSub; });
}

double sfo_max_acc(void* hv) {
    return static_cast<sfo::Handle*>(hv)->visit([&](auto& sim) { return double(sim.maxAccLen); });
}

// Forward-mode handles (precision 65): tangents of positions / velocities
// (3 doubles per particle, current internal order; before the first sort
// that is the creation order) and the parameter to differentiate by.
int sfo_set_tangent(void* hv, int field, const double* src, int64_t count) {
    return static_cast<sfo::Handle*>(hv)->visitDual(
        [&](auto& s) { return sfo::tangentField(s, field, nullptr, src, count); });
}

int sfo_get_tangent(void* hv, int field, double* dst, int64_t count) {
    return static_cast<sfo::Handle*>(hv)->visitDual(
        [&](auto& s) { return sfo::tangentField(s, field, dst, nullptr, count); });
}

// which: 0 none, 1 tan friction angle, 2 capillary scale, 3 permeability scale.
// The permeability tangent also seeds the per-particle cd of sand (MULTI scenes).
int sfo_seed_param(void* hv, int which) {
    if (which < 0 || which > 3) return SF_ERR_INVALID;
    return static_cast<sfo::Handle*>(hv)->visitDual([&](auto& s) {
        s.seedParam = which;
        for (int64_t i = 0; i < s.n; ++i)
            s.cda0asat[i].x.d = (which == 3 && s.label[i] == 1) ? double(s.cda0asat[i].x.v) : 0.0;
        return int(SF_OK);
    });
}

// Largest distance at which a pair term can be non-zero for these params.
double sfo_interaction_reach(const sf_params* p, const sf_boundary_params* b) {
    double c = sfo::capillaryReach<double>(double(p->dem_particle_radius));
    return std::max(double(b->kernel_radius), c);
}

int sfo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"
