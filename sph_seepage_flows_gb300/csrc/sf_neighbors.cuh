// Neighbour iteration shared by the substep passes (sf_kernels.cu) and their
// adjoint (sf_adjoint.cu): the 27-cell stencil walk and the per-label and
// boundary neighbour lists built by the density pass.
#pragma once

#include "sf_device.cuh"
#include "sf_kernels.h"

namespace sfg {

// The lane-split passes run G consecutive threads per slot (G = 1, 2, 4 or 8,
// chosen per handle by the slot count): lane `part` takes every G-th
// neighbour and lane 0 adds up the lanes' sums and writes the slot. Their
// sums are already in a different order from the reference's, so the split
// only moves FP32 rounding; small scenes get G times the threads in flight.
#define SF_SLOT_PROLOGUE_G                                                      \
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;                      \
    const int slot = gid / G, part = gid % G;                                   \
    const int sid = blockScene[(blockIdx.x * (blockDim.x / G)) / kSlotAlign];   \
    const SceneDev& S = scenes[sid];

// 27-cell stencil of the reference, with the global cell index of cell m.
template <typename F>
__device__ __forceinline__ void forEachCell(const SceneDev& S, int3 c, F&& f) {
#pragma unroll 1
    for (int dx = -1; dx <= 1; ++dx) {
        const int x = c.x + dx;
        if (x < 0 || x >= S.gx) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = c.y + dy;
            if (y < 0 || y >= S.gy) continue;
            const int base = S.cell_off + (x * S.gy + y) * S.gz;
#pragma unroll 1
            for (int dz = -1; dz <= 1; ++dz) {
                const int z = c.z + dz;
                if (z < 0 || z >= S.gz) continue;
                f(base + z);
            }
        }
    }
}

__device__ __forceinline__ bool inReach(const SceneDev& S, float3 d) { return dot3(d, d) < S.reach2; }

// A list entry; kLast marks the substep's last pass over this list, whose
// entry loads are evict-first so that they do not push the gathered
// per-particle arrays out of L2.
template <bool kLast> __device__ __forceinline__ unsigned listEntry(const unsigned* __restrict__ p) {
    return kLast ? __ldcs(p) : *p;
}

// Neighbours of one label within reach of slot, in stencil order: the sand
// part (kSand) or the water part of the list, or the stencil when the list
// overflowed. With G lanes per slot, lane `part` gets every G-th of them
// starting at the part-th (G = 1: all, in order).
template <bool kSand, int G = 1, bool kLast = false, typename F>
__device__ __forceinline__ void forLabelNeighbors(const SceneDev& S, const NbrLists& L, int slot, float3 pi,
                                                  const float4* __restrict__ pos4, F&& f, int part = 0) {
    const unsigned c = L.cnt[slot];
    if (int(c & 0xFFFFu) + int(c >> 16) <= L.cap) {
        const int n = kSand ? int(c & 0xFFFFu) : int(c >> 16);
        const unsigned* __restrict__ p = L.nbr + slot + (kSand ? 0 : size_t(L.cap - 1) * L.M);
        const long long step = kSand ? L.M : -L.M;
        // indices are loaded a group ahead so the neighbour gathers of
        // consecutive entries overlap
        int k = part;
        for (; k + 3 * G < n; k += 4 * G) {
            const int j0 = int(listEntry<kLast>(p + k * step)), j1 = int(listEntry<kLast>(p + (k + G) * step));
            const int j2 = int(listEntry<kLast>(p + (k + 2 * G) * step));
            const int j3 = int(listEntry<kLast>(p + (k + 3 * G) * step));
            f(j0);
            f(j1);
            f(j2);
            f(j3);
        }
        for (; k < n; k += G) f(int(listEntry<kLast>(p + k * step)));
    } else {
        // stencil walk in the same order: 9 (dx, dy) columns, 3 contiguous z-cells each
        const int3 c = cellOf(S, pi);
        const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, S.gz - 1) + 1;
        unsigned hits = 0;
        for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
            for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y) {
                const int base = S.cell_off + (x * S.gy + y) * S.gz;
                for (unsigned j = L.cs[base + z0]; j < L.cs[base + z1]; ++j) {
                    const float4 pj = pos4[j];
                    if ((kSand ? pj.w < 0.f : pj.w > 0.f) && inReach(S, pi - xyz(pj)))
                        if (G == 1 || int(hits++ % unsigned(G)) == part) f(int(j));
                }
            }
    }
}
template <int G = 1, bool kLast = false, typename F>
__device__ __forceinline__ void forSandNeighbors(const SceneDev& S, const NbrLists& L, int slot, float3 pi,
                                                 const float4* __restrict__ pos4, F&& f, int part = 0) {
    forLabelNeighbors<true, G, kLast>(S, L, slot, pi, pos4, f, part);
}
template <int G = 1, bool kLast = false, typename F>
__device__ __forceinline__ void forWaterNeighbors(const SceneDev& S, const NbrLists& L, int slot, float3 pi,
                                                  const float4* __restrict__ pos4, F&& f, int part = 0) {
    forLabelNeighbors<false, G, kLast>(S, L, slot, pi, pos4, f, part);
}

// Boundary particles within reach of slot, in stencil order (lane-strided
// like forLabelNeighbors).
template <int G = 1, typename F>
__device__ __forceinline__ void forBoundaryNeighbors(const SceneDev& S, const NbrLists& L, int slot, float3 pi,
                                                     const float4* __restrict__ bpos4, F&& f, int part = 0) {
    const int c = L.bcnt[slot];
    if (c <= kMaxBNbr) {
        const unsigned* __restrict__ p = L.bnbr + slot;
#pragma unroll 1
        for (int k = part; k < c; k += G) f(int(p[size_t(k) * L.M]));
    } else {
        const int3 c = cellOf(S, pi);
        const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, S.gz - 1) + 1;
        unsigned hits = 0;
        for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
            for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y) {
                const int base = S.cell_off + (x * S.gy + y) * S.gz;
                for (unsigned j = L.bcs[base + z0]; j < L.bcs[base + z1]; ++j)
                    if (inReach(S, pi - xyz(bpos4[j])))
                        if (G == 1 || int(hits++ % unsigned(G)) == part) f(int(j));
            }
    }
}

// N floats of one neighbour's terms.
template <int N> struct Terms {
    float v[N];
};

// The neighbours of one label, with sums that must keep the single-thread
// order: in rounds of G list entries, lane `part` evaluates term(j) of entry
// round * G + part, then every lane folds the round's G terms in entry order
// (fold(t) adds t's floats to the accumulators). Every lane ends with the
// same sums, formed with the same operations in the same order as one
// thread walking the list, so G only changes how many threads share the
// term evaluations. An overflowed list is walked in full by every lane.
template <bool kSand, int G, int N, typename Term, typename Fold>
__device__ __forceinline__ void forLabelNeighborsOrdered(const SceneDev& S, const NbrLists& L, int slot, float3 pi,
                                                         const float4* __restrict__ pos4, int part, Term&& term,
                                                         Fold&& fold) {
    const unsigned c = L.cnt[slot];
    if (G == 1 || int(c & 0xFFFFu) + int(c >> 16) > L.cap) {
        forLabelNeighbors<kSand>(S, L, slot, pi, pos4, [&](int j) { fold(term(j)); });
        return;
    }
    const int n = kSand ? int(c & 0xFFFFu) : int(c >> 16);
    const unsigned* __restrict__ p = L.nbr + slot + (kSand ? 0 : size_t(L.cap - 1) * L.M);
    const long long step = kSand ? L.M : -L.M;
    const unsigned lane = threadIdx.x & 31u, base = lane & ~unsigned(G - 1);
    const unsigned mask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << base;
    for (int k0 = 0; k0 < n; k0 += G) {
        Terms<N> t;
        if (k0 + part < n) {
            t = term(int(p[(k0 + part) * step]));
        } else {
#pragma unroll
            for (int q = 0; q < N; ++q) t.v[q] = 0.f;
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            Terms<N> u;
#pragma unroll
            for (int q = 0; q < N; ++q) u.v[q] = __shfl_sync(mask, t.v[q], int(base) + g);
            if (k0 + g < n) fold(u);
        }
    }
}

// Sum over the G lanes of a slot (G consecutive lanes of one warp, G divides
// 32; all G lanes call it).
template <int G> __device__ __forceinline__ float groupSum(float v) {
    if (G > 1) {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned mask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (lane & ~unsigned(G - 1));
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    }
    return v;
}
template <int G> __device__ __forceinline__ float3 groupSum3(float3 v) {
    return make_float3(groupSum<G>(v.x), groupSum<G>(v.y), groupSum<G>(v.z));
}

}  // namespace sfg
