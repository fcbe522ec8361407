// Neighbor passes, integrator and boundary-volume kernels of the GB300
// seepage-flow substep. One thread per slot; each block of kSlotAlign slots
// belongs to one scene (blockScene). Every pass is a gather: a thread writes
// only its own slot, so no pass needs atomics except the per-scene max |acc|.
//
// Neighbour lists. The density pass walks the reference's 27-cell stencil
// (m = 0..26, dx-major, e.g. cuda_sph_sf_solver_gpu.cuh:468-477) once per
// particle and records every particle (and every boundary particle) within
// the interaction reach into a column-major list (entry k of slot i at
// k * M + i, so a warp reads 128 contiguous bytes per entry): sand
// neighbours from the front, water neighbours from the back, each in stencil
// order. Pairs beyond the reach have all terms exactly +0 in the reference,
// so the later passes iterate only the list (~35 entries instead of ~216
// stencil candidates), one label class at a time (no label divergence). A
// particle whose list overflows falls back to the stencil walk.
//
// Each thread walks its own stencil as 9 contiguous ranges (the 3 z-cells
// of one (dx, dy) column are adjacent in the sorted order); a branch-free
// pass over each chunk of 32 candidates marks those in reach, and only the
// marked ones are processed, in stencil order.
//
// Summation order. Every accumulator of the density, average-flow, voidage,
// saturation and adhesion passes receives one label class of neighbours, in
// stencil order, exactly as in the reference kernel, so those fields are
// bit-identical to the reference's FP32 arithmetic (near walls the water
// density merges its water and boundary lists cell by cell, the reference's
// interleaving of fluid and boundary terms). The
// two momentum passes evaluate all terms of a neighbour together, sand
// neighbours before water neighbours, instead of one sub-loop per term and
// cell, which reorders their FP32 sums (differences ~1e-7 of the sum of term
// magnitudes).
#include <algorithm>

#include "sf_device.cuh"
#include "sf_kernels.h"
#include "sf_neighbors.cuh"

namespace sfg {

#define SF_SLOT_PROLOGUE                                                   \
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;                \
    const int sid = blockScene[(blockIdx.x * blockDim.x) / kSlotAlign];    \
    const SceneDev& S = scenes[sid];

// ----------------------------------------------------------- boundary volume
// ComputeBoundaryVolume_CUDA (cuda_sph_system_gpu.cuh:19-67): V_b = 1 / max(sum_{j != i} W, eps).
__global__ void kBoundaryVolume(const SceneDev* __restrict__ scenes, int sid, float4* __restrict__ bpos4,
                                const int* __restrict__ blabel, const unsigned int* __restrict__ bcs) {
    const SceneDev& S = scenes[sid];
    const int i = S.b_off + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.b_off + S.nb) return;
    const float3 pi = xyz(bpos4[i]);
    float v = 0.f;
    forEachCell(S, cellOf(S, pi), [&](int cell) {
        for (unsigned j = bcs[cell]; j < bcs[cell + 1]; ++j)
            if (int(j) != i) v += poly6(S, len3(pi - xyz(bpos4[j])));
    });
    const float vol = 1.f / fmaxf(v, kEps);
    bpos4[i].w = blabel[i] == 1 ? -vol : vol;
}

// ------------------------------------------------------------ density stage
// Water density of ComputeSFDensity_CUDA + ComputeSFFluidDensity +
// ComputeBoundaryDensity (cuda_sph_sf_solver_gpu.cuh:408-480,
// cuda_sph_solver_common_gpu.cuh:70-87): m_i W(0) plus, cell by cell of the
// stencil, the water particles of the cell then the boundary particles of
// the cell.
__device__ __forceinline__ float exactDensity(const SceneDev& S, const NbrListsW& L, float3 pi, float mi,
                                              const float4* __restrict__ pos4, const float4* __restrict__ bpos4) {
    float d = mi * S.W0;
    const int3 c = cellOf(S, pi);
    for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
        for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y)
            for (int z = max(c.z - 1, 0); z <= min(c.z + 1, S.gz - 1); ++z) {
                const int cell = S.cell_off + (x * S.gy + y) * S.gz + z;
                for (unsigned j = L.cs[cell]; j < L.cs[cell + 1]; ++j) {
                    const float4 pj = pos4[j];
                    if (pj.w > 0.f) {
                        const float3 dij = pi - xyz(pj);
                        if (inReach(S, dij)) d += pj.w * poly6(S, len3(dij));
                    }
                }
                for (unsigned j = L.bcs[cell]; j < L.bcs[cell + 1]; ++j) {
                    const float4 bj = bpos4[j];
                    const float3 dij = pi - xyz(bj);
                    if (inReach(S, dij)) d += S.rho0 * fabsf(bj.w) * poly6(S, len3(dij));
                }
            }
    return d;
}

// Conservative reach test for building the lists, as a sign: negative when
// the pair is in reach. Evaluated with fused multiply-adds (cheaper); any
// pair it admits or rejects differently from the exact test lies within 1e-5
// of the reach, where every term is exactly zero.
__device__ __forceinline__ float reachSign(const SceneDev& S, float3 d) {
    return __fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, __fmaf_rn(d.z, d.z, -S.reach2)));
}
__device__ __forceinline__ bool inReachFast(const SceneDev& S, float3 d) { return reachSign(S, d) < 0.f; }

// Water density from the lists: m_i W(0), then cell by cell of the stencil
// the water neighbours of the cell and the boundary neighbours of the cell
// (both lists are in stencil order, i.e. in increasing cell index, so the
// walk merges them by the cell tables). Terms of listed pairs beyond the
// exact reach are +0, which leaves every partial sum unchanged.
__device__ __forceinline__ float listDensity(const SceneDev& S, const NbrListsW& L, int slot, int cW, int bc,
                                             float3 pi, float mi, const float4* __restrict__ pos4,
                                             const float4* __restrict__ bpos4) {
    float d = mi * S.W0;
    const long long M = L.M;
    const unsigned* __restrict__ wp = L.nbr + slot + size_t(L.cap - 1) * M;
    if (bc == 0) {
        int k = 0;
        for (; k + 4 <= cW; k += 4) {
            const unsigned j0 = wp[-k * M], j1 = wp[-(k + 1) * M], j2 = wp[-(k + 2) * M], j3 = wp[-(k + 3) * M];
            const float4 p0 = pos4[j0], p1 = pos4[j1], p2 = pos4[j2], p3 = pos4[j3];
            d += p0.w * poly6(S, len3(pi - xyz(p0)));
            d += p1.w * poly6(S, len3(pi - xyz(p1)));
            d += p2.w * poly6(S, len3(pi - xyz(p2)));
            d += p3.w * poly6(S, len3(pi - xyz(p3)));
        }
        for (; k < cW; ++k) {
            const float4 pj = pos4[wp[-k * M]];
            d += pj.w * poly6(S, len3(pi - xyz(pj)));
        }
        return d;
    }
    const unsigned* __restrict__ bp = L.bnbr + slot;
    const int3 c = cellOf(S, pi);
    const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, S.gz - 1) + 1;
    int kw = 0, kb = 0;
    for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
        for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y) {
            const int base = S.cell_off + (x * S.gy + y) * S.gz;
            for (int z = z0; z < z1; ++z) {
                const unsigned wEnd = L.cs[base + z + 1];
                for (; kw < cW; ++kw) {
                    const unsigned j = wp[-kw * M];
                    if (j >= wEnd) break;
                    const float4 pj = pos4[j];
                    d += pj.w * poly6(S, len3(pi - xyz(pj)));
                }
                const unsigned bEnd = L.bcs[base + z + 1];
                for (; kb < bc; ++kb) {
                    const unsigned j = bp[kb * M];
                    if (j >= bEnd) break;
                    const float4 bj = bpos4[j];
                    d += S.rho0 * fabsf(bj.w) * poly6(S, len3(pi - xyz(bj)));
                }
            }
        }
    return d;
}

// Records a neighbour count above 7/8 of the list capacity in the scene's
// list_need (the largest such count of the warp, one atomic per warp); the
// host reads it after the call and grows the lists to hold it with headroom,
// so that a slowly compressing state grows its lists before any overflows.
__device__ __forceinline__ void recordListNeed(const NbrListsW& L, unsigned int& need, int count) {
    if (count <= L.cap - L.cap / 8) return;
    const unsigned active = __activemask();
    const unsigned m = __reduce_max_sync(active, unsigned(count));
    if ((threadIdx.x & 31u) == unsigned(__ffs(active) - 1)) atomicMax(&need, m);
}

// Shared-memory staging of a block's stencil candidates (kDensity<true>).
// The slots of a block are consecutive in the cell order, so their particles
// lie in one or two (x, y) cell columns for nearly every block; for each such
// source column the block copies the 9 stencil columns over the z-cells its
// particles reach into shared memory (coalesced, one warp per column) and the
// walk reads every candidate from there. sG[k] / sO[k]: first slot and shared
// offset of staged column k = 9 * source column + stencil column. A block with
// more source columns, or with more candidates than its shared capacity,
// walks global memory. Lists and results are identical either way; the tuner
// times both forms.
constexpr int kStageSources = 2;
constexpr int kStageCols = 9 * kStageSources;
constexpr int kBigInt = 0x7fffffff;
struct StageTable {
    unsigned g[kStageCols];      // first global slot of each staged column
    unsigned o[kStageCols + 1];  // shared offset of each staged column (+ total)
    int red[8];                  // block reductions (see stageBlock)
};

// Fills the table and the shared positions of the block's candidates;
// returns the number of staged source columns (0: walk global memory). Every
// thread of the block calls it.
__device__ __forceinline__ int stageBlock(const SceneDev& S, const NbrListsW& L, const float4* __restrict__ pos4,
                                          bool live, int3 c, StageTable& T, float4* sPos, int stageCap) {
    const int lane = threadIdx.x & 31;
    const int col = c.x * S.gy + c.y;
    if (threadIdx.x < 8) T.red[threadIdx.x] = kBigInt;
    __syncthreads();
    {  // first and last source column (maxima as minima of negations)
        const int a = __reduce_min_sync(~0u, live ? col : kBigInt);
        const int b = __reduce_min_sync(~0u, live ? -col : kBigInt);
        if (lane == 0) {
            atomicMin(&T.red[0], a);
            atomicMin(&T.red[1], b);
        }
    }
    __syncthreads();
    const int colA = T.red[0], colB = -T.red[1];
    {  // any column between them, and the z-range of each
        const bool inA = live && col == colA, inB = live && col == colB;
        const int m = __reduce_min_sync(~0u, live && col > colA ? col : kBigInt);
        const int za = __reduce_min_sync(~0u, inA ? c.z : kBigInt);
        const int zA = __reduce_min_sync(~0u, inA ? -c.z : kBigInt);
        const int zb = __reduce_min_sync(~0u, inB ? c.z : kBigInt);
        const int zB = __reduce_min_sync(~0u, inB ? -c.z : kBigInt);
        if (lane == 0) {
            atomicMin(&T.red[2], m);
            atomicMin(&T.red[3], za);
            atomicMin(&T.red[4], zA);
            atomicMin(&T.red[5], zb);
            atomicMin(&T.red[6], zB);
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // lane k < 9 * sources: staged column k, its range from the cell table
        const int nsrc = colA == kBigInt ? 0 : (colB == colA ? 1 : (T.red[2] == colB ? 2 : 3));
        unsigned g = 0u, cnt = 0u;
        const int src = lane / 9, m = lane % 9;
        if (nsrc <= kStageSources && src < nsrc) {
            const int cl = src ? colB : colA;
            const int x = cl / S.gy + m / 3 - 1, y = cl % S.gy + m % 3 - 1;
            const int zlo = max((src ? T.red[5] : T.red[3]) - 1, 0);
            const int zhi = min(-(src ? T.red[6] : T.red[4]) + 1, S.gz - 1) + 1;
            if (x >= 0 && x < S.gx && y >= 0 && y < S.gy) {
                const int base = S.cell_off + (x * S.gy + y) * S.gz;
                g = L.cs[base + zlo];
                cnt = L.cs[base + zhi] - g;
            }
        }
        unsigned inc = cnt;  // inclusive prefix of the column lengths
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(~0u, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane < kStageCols) {
            T.g[lane] = g;
            T.o[lane] = inc - cnt;
        }
        const unsigned total = __shfl_sync(~0u, inc, 31);
        if (lane == 0) {
            T.o[kStageCols] = total;
            T.red[7] = (nsrc >= 1 && nsrc <= kStageSources && total <= unsigned(stageCap)) ? nsrc : 0;
        }
    }
    __syncthreads();
    const int staged = T.red[7];
    if (staged) {
        const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int k = warp; k < 9 * staged; k += nw) {
            const unsigned g = T.g[k], o = T.o[k], cnt = T.o[k + 1] - o;
            for (unsigned i = lane; i < cnt; i += 32u) sPos[o + i] = pos4[g + i];
        }
        __syncthreads();
    }
    return staged;
}

// Builds the neighbour lists (sand / water / boundary, each in stencil
// order, plus the sand-sand contact list) and computes the density, fused
// with ComputeSFPressureByTait_CUDA (cuda_wcsph_sf_solver_gpu.cuh:19-44) or
// ComputeSFPressure_CUDA (cuda_sph_sf_solver_gpu.cuh:482-508). The stencil is
// walked as 9 contiguous ranges (the 3 z-cells of one (dx, dy) column are
// adjacent in the sorted order), which visits the same particles in the same
// order as the 27-cell loop with far fewer divergent loop exits. The walk
// only appends list entries; the contact filter and the density sum then run
// over the finished lists, where the lanes of a warp stay together.
// The walk is bound by load latency: a register budget of 40 (6 blocks of
// kSlotAlign threads per SM) buys occupancy that outweighs the few values it
// moves to the stack. kStaged reads the candidates from the block's staged
// copy (stageBlock, stageCap positions of dynamic shared memory; 48
// registers, since its shared memory already bounds the resident blocks).
template <bool kStaged>
__global__ void __launch_bounds__(kSlotAlign, kStaged ? 5 : 6) kDensity(const SceneDev* __restrict__ scenes,
                                                                     const int* __restrict__ blockScene,
                                                                     SceneState* __restrict__ state, NbrListsW L,
                                                                     const float4* __restrict__ pos4,
                                                                     const float4* __restrict__ bpos4,
                                                                     float4* __restrict__ vel4,
                                                                     float4* __restrict__ aux4, int stageCap) {
    SF_SLOT_PROLOGUE
    extern __shared__ float4 sPos[];
    __shared__ StageTable T;
    if (slot == S.slot_off) state[sid].amax_bits = 0u;
    const float4 pi4 = pos4[slot];
    int staged = 0;
    if constexpr (kStaged) staged = stageBlock(S, L, pos4, pi4.w != 0.f, cellOf(S, xyz(pi4)), T, sPos, stageCap);
    if (pi4.w == 0.f) return;
    const float3 pi = xyz(pi4);
    const int3 c = cellOf(S, pi);
    const bool water = pi4.w > 0.f;
    const long long M = L.M;
    unsigned* __restrict__ nb = L.nbr + slot;
    unsigned* __restrict__ bnb = L.bnbr + slot;
    int cS = 0, cW = 0, bc = 0;
    const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, S.gz - 1) + 1;
    // staged columns of this particle's source column
    int src9 = 0;
    if constexpr (kStaged) src9 = (staged == 2 && c.x * S.gy + c.y != T.red[0]) ? 9 : 0;
    // no boundary particle within the 27 cells: the boundary ranges are empty
    const bool nearB = !L.bnear || L.bnear[S.cell_off + localHash(S, c)] != 0;
#pragma unroll 1
    for (int dx = -1; dx <= 1; ++dx) {
        const int x = c.x + dx;
        if (x < 0 || x >= S.gx) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = c.y + dy;
            if (y < 0 || y >= S.gy) continue;
            const int base = S.cell_off + (x * S.gy + y) * S.gz;
            const unsigned jEnd = L.cs[base + z1];
            // chunks of up to 32 candidates: a branch-free pass shifts the
            // sign of each candidate's reach test and its sand bit (the sign
            // of w) into two masks (candidate t ends at bit n-1-t), then the
            // marked ones are appended in order
#pragma unroll 1
            for (unsigned j0 = L.cs[base + z0]; j0 < jEnd; j0 += 32u) {
                const int n = int(min(32u, jEnd - j0));
                unsigned rev = 0u, srev = 0u;
                if (kStaged && staged) {
                    const int k = src9 + (dx + 1) * 3 + (dy + 1);
                    const float4* sp = sPos + (int(j0) + int(T.o[k]) - int(T.g[k]));
#pragma unroll 4
                    for (int t = 0; t < n; ++t) {
                        const float4 q = sp[t];
                        rev = __funnelshift_l(__float_as_uint(reachSign(S, pi - xyz(q))), rev, 1);
                        srev = __funnelshift_l(__float_as_uint(q.w), srev, 1);
                    }
                } else {
#pragma unroll 4
                    for (int t = 0; t < n; ++t) {
                        const float4 q = pos4[j0 + unsigned(t)];
                        rev = __funnelshift_l(__float_as_uint(reachSign(S, pi - xyz(q))), rev, 1);
                        srev = __funnelshift_l(__float_as_uint(q.w), srev, 1);
                    }
                }
                const unsigned hit = __brev(rev) >> (32 - n), sand = __brev(srev) >> (32 - n);
                // the list overflows when the two parts meet: from then on
                // nothing reads it, so the order of the two appends is free
                for (unsigned m = hit & sand; m; m &= m - 1u) {
                    if (cS + cW < L.cap) nb[cS * M] = j0 + unsigned(__ffs(m) - 1);
                    ++cS;
                }
                for (unsigned m = hit & ~sand; m; m &= m - 1u) {
                    if (cS + cW < L.cap) nb[(L.cap - 1 - cW) * M] = j0 + unsigned(__ffs(m) - 1);
                    ++cW;
                }
            }
            if (!nearB) continue;
            const unsigned bEnd = L.bcs[base + z1];
            for (unsigned j = L.bcs[base + z0]; j < bEnd; ++j) {
                if (!inReachFast(S, pi - xyz(bpos4[j]))) continue;
                if (bc < kMaxBNbr) bnb[bc * M] = j;
                ++bc;
            }
        }
    }
    const bool listed = cS + cW <= L.cap;
    int cc = 0;
    if (!water) {
        // sand-sand pairs within the DEM + liquid-bridge reach, in stencil order
        unsigned* __restrict__ cnb = L.cnbr + slot;
        auto contact = [&](unsigned j, float3 pj) {
            if (j == unsigned(slot)) return;
            const float3 dij = pi - pj;
            if (dot3(dij, dij) < S.dem_reach2) {
                if (cc < kMaxContact) cnb[cc * M] = j;
                ++cc;
            }
        };
        if (listed) {
            // indices and positions are loaded a group ahead (the entries
            // were just written and come back from L2)
            for (int k0 = 0; k0 < cS; k0 += 4) {
                unsigned jj[4];
                float3 pp[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) jj[u] = k0 + u < cS ? nb[(k0 + u) * M] : unsigned(slot);
#pragma unroll
                for (int u = 0; u < 4; ++u) pp[u] = xyz(pos4[jj[u]]);
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (k0 + u < cS) contact(jj[u], pp[u]);
            }
        } else {
            for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
                for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y) {
                    const int base = S.cell_off + (x * S.gy + y) * S.gz;
                    for (unsigned j = L.cs[base + z0]; j < L.cs[base + z1]; ++j) {
                        const float4 pj = pos4[j];
                        if (pj.w < 0.f && inReachFast(S, pi - xyz(pj))) contact(j, xyz(pj));
                    }
                }
        }
    }
    L.cnt[slot] = unsigned(min(cS, 0xFFFF)) | (unsigned(min(cW, 0xFFFF)) << 16);
    L.bcnt[slot] = bc;
    L.ccnt[slot] = cc;
    // a list more than 7/8 full asks the host to grow the capacity before it
    // overflows; a full one walks the stencil until then (same results,
    // slower)
    recordListNeed(L, state[sid].list_need, cS + cW);
    float density, pressure = 0.f;
    if (!water) {
        density = S.rho1;
    } else {
        // the reference interleaves boundary terms cell by cell; without
        // complete lists the stencil is walked again
        density = listed && bc <= kMaxBNbr ? listDensity(S, L, slot, cW, bc, pi, pi4.w, pos4, bpos4)
                                           : exactDensity(S, L, pi, pi4.w, pos4, bpos4);
        if (S.tait) {
            pressure = S.stiff * (powf(density / S.rho0, 7.f) - 1.f);
            if (pressure < 0.f) pressure *= S.neg_scale;
        } else {
            pressure = S.stiff * (density - S.rho0);
            if (pressure < 0.f) pressure *= 1.f;
        }
    }
    vel4[slot].w = density;
    aux4[slot].x = pressure;
}

// The density pass with G lanes per slot (small scenes), with lists, counts,
// density and pressure identical to kDensity's. The 32-candidate chunks of
// the stencil walk, in stencil order, are dealt round-robin to the lanes; in
// each round every lane tests its chunk at the same time, and the round's
// hits are appended at the positions a single thread would have given them
// (prefix counts over the lanes in chunk order, then the rank within the
// chunk). Boundary candidates and the entries of the contact filter are
// dealt one per lane and ranked by a ballot; the water density folds the
// round's terms in list order. The rare paths (water with boundary
// neighbours, overflowed lists) run in lane 0.
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kDensityLanes(const SceneDev* __restrict__ scenes,
                                                            const int* __restrict__ blockScene,
                                                            SceneState* __restrict__ state, NbrListsW L,
                                                            const float4* __restrict__ pos4,
                                                            const float4* __restrict__ bpos4,
                                                            float4* __restrict__ vel4, float4* __restrict__ aux4) {
    SF_SLOT_PROLOGUE_G
    if (part == 0 && slot == S.slot_off) state[sid].amax_bits = 0u;
    const float4 pi4 = pos4[slot];
    if (pi4.w == 0.f) return;
    const float3 pi = xyz(pi4);
    const int3 c = cellOf(S, pi);
    const bool water = pi4.w > 0.f;
    const long long M = L.M;
    unsigned* __restrict__ nb = L.nbr + slot;
    const unsigned lane = threadIdx.x & 31u, gbase = lane & ~unsigned(G - 1);
    const unsigned gmask = ((1u << G) - 1u) << gbase;
    int cS = 0, cW = 0;
    const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, S.gz - 1) + 1;
    unsigned myJ0 = 0u, myHit = 0u, mySand = 0u;
    // appends the round's hits at their single-thread positions
    auto flush = [&]() {
        const int ns = __popc(myHit & mySand), nw = __popc(myHit & ~mySand);
        int ps = ns, pw = nw;  // inclusive prefix over the lanes, in chunk order
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const int ts = __shfl_up_sync(gmask, ps, o, G), tw = __shfl_up_sync(gmask, pw, o, G);
            if (part >= o) {
                ps += ts;
                pw += tw;
            }
        }
        ps -= ns;
        pw -= nw;
        for (unsigned m = myHit; m; m &= m - 1u) {
            const int t = __ffs(m) - 1;
            const unsigned low = myHit & ((1u << t) - 1u);
            if (cS + cW + ps + pw + __popc(low) < L.cap) {  // the single thread's overflow test
                if ((mySand >> t) & 1u)
                    nb[(cS + ps + __popc(low & mySand)) * M] = myJ0 + unsigned(t);
                else
                    nb[(L.cap - 1 - (cW + pw + __popc(low & ~mySand))) * M] = myJ0 + unsigned(t);
            }
        }
        // round totals: the last lane's inclusive prefix
        cS += __shfl_sync(gmask, ps + ns, int(gbase) + G - 1);
        cW += __shfl_sync(gmask, pw + nw, int(gbase) + G - 1);
        myHit = mySand = 0u;
    };
    // the 9 column ranges of the stencil (particles and boundary), loaded
    // together up front: on a small scene the walk is a latency chain
    // (the boundary ranges only where a boundary particle is within the 27
    // cells; elsewhere they are empty)
    const bool nearB = !L.bnear || L.bnear[S.cell_off + localHash(S, c)] != 0;
    unsigned cb[9], ce[9], bb[9], be[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) {
        const int x = c.x + m / 3 - 1, y = c.y + m % 3 - 1;
        cb[m] = ce[m] = bb[m] = be[m] = 0u;
        if (x >= 0 && x < S.gx && y >= 0 && y < S.gy) {
            const int base = S.cell_off + (x * S.gy + y) * S.gz;
            cb[m] = L.cs[base + z0];
            ce[m] = L.cs[base + z1];
            if (nearB) {
                bb[m] = L.bcs[base + z0];
                be[m] = L.bcs[base + z1];
            }
        }
    }
    // chunk q of the stencil order: column m with pre[m] <= q < pre[m + 1]
    int pre[10];
    pre[0] = 0;
#pragma unroll
    for (int m = 0; m < 9; ++m) pre[m + 1] = pre[m] + int((ce[m] - cb[m] + 31u) / 32u);
    const int nq = pre[9];
    // round r: lane part tests chunk r * G + part (all lanes at once)
#pragma unroll 1
    for (int r0 = 0; r0 < nq; r0 += G) {
        const int qq = r0 + part;
        if (qq < nq) {
            unsigned j0 = 0u, jEnd = 0u;
#pragma unroll
            for (int m = 0; m < 9; ++m)
                if (qq >= pre[m] && qq < pre[m + 1]) {
                    j0 = cb[m] + 32u * unsigned(qq - pre[m]);
                    jEnd = ce[m];
                }
            const int n = int(min(32u, jEnd - j0));
            unsigned rev = 0u, srev = 0u;
#pragma unroll 8
            for (int t = 0; t < n; ++t) {
                const float4 qv = pos4[j0 + unsigned(t)];
                rev = __funnelshift_l(__float_as_uint(reachSign(S, pi - xyz(qv))), rev, 1);
                srev = __funnelshift_l(__float_as_uint(qv.w), srev, 1);
            }
            if (n > 0) {  // always, as every chunk index maps to a non-empty column
                myJ0 = j0;
                myHit = __brev(rev) >> (32 - n);
                mySand = __brev(srev) >> (32 - n);
            }
        }
        flush();
    }
    __syncwarp(gmask);  // the group's list entries are visible to every lane
    const bool listed = cS + cW <= L.cap;
    int bc = 0;
    {
        // boundary candidates dealt to the lanes one at a time, in stencil
        // order; a ballot ranks the hits
        unsigned* __restrict__ bnb = L.bnbr + slot;
#pragma unroll
        for (int m = 0; m < 9; ++m) {
#pragma unroll 1
            for (unsigned j0 = bb[m]; j0 < be[m]; j0 += unsigned(G)) {
                const unsigned j = j0 + unsigned(part);
                const bool in = j < be[m] && inReachFast(S, pi - xyz(bpos4[j]));
                const unsigned ball = __ballot_sync(gmask, in) >> gbase;
                if (in) {
                    const int r = bc + __popc(ball & ((1u << part) - 1u));
                    if (r < kMaxBNbr) bnb[r * M] = j;
                }
                bc += __popc(ball);
            }
        }
    }
    int cc = 0;
    if (!water) {
        unsigned* __restrict__ cnb = L.cnbr + slot;
        if (listed) {
            for (int k0 = 0; k0 < cS; k0 += G) {
                const int k = k0 + part;
                bool in = false;
                unsigned j = 0u;
                if (k < cS) {
                    j = nb[k * M];
                    if (j != unsigned(slot)) {
                        const float3 dij = pi - xyz(pos4[j]);
                        in = dot3(dij, dij) < S.dem_reach2;
                    }
                }
                const unsigned ball = __ballot_sync(gmask, in) >> gbase;
                if (in) {
                    const int r = cc + __popc(ball & ((1u << part) - 1u));
                    if (r < kMaxContact) cnb[r * M] = j;
                }
                cc += __popc(ball);
            }
        } else if (part == 0) {
            for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
                for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y) {
                    const int base = S.cell_off + (x * S.gy + y) * S.gz;
                    for (unsigned j = L.cs[base + z0]; j < L.cs[base + z1]; ++j) {
                        const float4 pj = pos4[j];
                        if (!(pj.w < 0.f) || !inReachFast(S, pi - xyz(pj)) || j == unsigned(slot)) continue;
                        const float3 dij = pi - xyz(pj);
                        if (dot3(dij, dij) < S.dem_reach2) {
                            if (cc < kMaxContact) cnb[cc * M] = j;
                            ++cc;
                        }
                    }
                }
        }
    }
    float density = S.rho1;
    if (water) {
        if (listed && bc == 0) {
            // m_i W(0), then the water list in order, G entries per round
            float d = pi4.w * S.W0;
            const unsigned* __restrict__ wp = L.nbr + slot + size_t(L.cap - 1) * M;
            for (int k0 = 0; k0 < cW; k0 += G) {
                float t = 0.f;
                if (k0 + part < cW) {
                    const float4 pj = pos4[wp[-(k0 + part) * M]];
                    t = pj.w * poly6(S, len3(pi - xyz(pj)));
                }
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const float u = __shfl_sync(gmask, t, int(gbase) + g);
                    if (k0 + g < cW) d += u;
                }
            }
            density = d;
        } else if (part == 0) {
            density = listed && bc <= kMaxBNbr ? listDensity(S, L, slot, cW, bc, pi, pi4.w, pos4, bpos4)
                                               : exactDensity(S, L, pi, pi4.w, pos4, bpos4);
        }
    }
    if (part != 0) return;
    L.cnt[slot] = unsigned(min(cS, 0xFFFF)) | (unsigned(min(cW, 0xFFFF)) << 16);
    L.bcnt[slot] = bc;
    L.ccnt[slot] = cc;
    // a list more than 7/8 full asks the host to grow the capacity before it
    // overflows; a full one walks the stencil until then (same results,
    // slower)
    recordListNeed(L, state[sid].list_need, cS + cW);
    float pressure = 0.f;
    if (water) {
        if (S.tait) {
            pressure = S.stiff * (powf(density / S.rho0, 7.f) - 1.f);
            if (pressure < 0.f) pressure *= S.neg_scale;
        } else {
            pressure = S.stiff * (density - S.rho0);
            if (pressure < 0.f) pressure *= 1.f;
        }
    }
    vel4[slot].w = density;
    aux4[slot].x = pressure;
}

// ------------------------------------------------------------ avg-flow stage
// ComputeSFAvgFlow_CUDA with ComputeSFSandVolume and ComputeSFAvgFlow
// (cuda_sph_sf_solver_gpu.cuh:111-173, 510-572). The two sub-loops feed
// disjoint accumulators, so one sweep keeps every sum's reference order.
// Small scenes run G lanes per slot: the lanes share the term evaluations
// and fold the terms in list order (forLabelNeighborsOrdered), so the sums
// stay bit-identical.
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kAvgFlow(const SceneDev* __restrict__ scenes,
                                                       const int* __restrict__ blockScene, NbrLists L,
                                                       const float4* __restrict__ pos4,
                                                       const float4* __restrict__ vel4, float4* __restrict__ aux4,
                                                       float4* __restrict__ flow4, float2* __restrict__ vrec2,
                                                       float4* __restrict__ grec4) {
    SF_SLOT_PROLOGUE_G
    const float4 pi4 = pos4[slot];
    if (pi4.w == 0.f) return;
    const float3 pi = xyz(pi4);
    const bool sandI = pi4.w < 0.f;
    float v_s = 0.f, v_w = 0.f, sand_volume = 0.f;
    float3 avg_s = mk3(0.f, 0.f, 0.f), avg_w = avg_s;
    // sand neighbours: sand volume (every i) and, for water i, the sand average flow
    forLabelNeighborsOrdered<true, G, 6>(
        S, L, slot, pi, pos4, part,
        [&](int j) {
            const float4 pj = pos4[j];
            const float4 vj4 = vel4[j];
            const float mj = -pj.w;
            const float wij = poly6(S, len3(pi - xyz(pj)));
            Terms<6> t;
            t.v[0] = vj4.w != 0.f ? mj / vj4.w * wij : 0.f;
            t.v[1] = vj4.w != 0.f ? 1.f : 0.f;
            t.v[2] = t.v[3] = t.v[4] = t.v[5] = 0.f;
            if (!sandI) {
                const float vj = mj / vj4.w;
                const float3 a = xyz(vj4) * vj * wij;
                t.v[2] = a.x;
                t.v[3] = a.y;
                t.v[4] = a.z;
                t.v[5] = vj * wij;
            }
            return t;
        },
        [&](const Terms<6>& t) {
            if (t.v[1] != 0.f) sand_volume += t.v[0];
            if (!sandI) {
                avg_w += mk3(t.v[2], t.v[3], t.v[4]);
                v_w += t.v[5];
            }
        });
    // water neighbours of sand i: the water average flow and the saturation
    if (sandI) {
        forLabelNeighborsOrdered<false, G, 4>(
            S, L, slot, pi, pos4, part,
            [&](int j) {
                const float4 pj = pos4[j];
                const float4 vj4 = vel4[j];
                const float vj = pj.w / vj4.w;
                const float wij = poly6(S, len3(pi - xyz(pj)));
                const float3 a = xyz(vj4) * vj * wij;
                Terms<4> t;
                t.v[0] = a.x;
                t.v[1] = a.y;
                t.v[2] = a.z;
                t.v[3] = vj * wij;
                return t;
            },
            [&](const Terms<4>& t) {
                avg_s += mk3(t.v[0], t.v[1], t.v[2]);
                v_s += t.v[3];
            });
    }
    if (part != 0) return;
    float3 avg;
    if (!sandI && v_w != 0.f)
        avg = avg_w / v_w;
    else if (sandI && v_s != 0.f)
        avg = avg_s / v_s;
    else
        avg = mk3(0.f, 0.f, 0.f);
    // w: the adhesion Bezier factor of a sand particle's saturation, which
    // every water neighbour's adhesion term uses (computed once here)
    const float bz = sandI ? bezier(S.adhG, v_s) : 0.f;
    flow4[slot] = make_float4(avg.x, avg.y, avg.z, bz);
    float4 a = aux4[slot];
    a.y = 1.f - sand_volume;
    a.z = v_s;
    a.w = a.y;  // the reference's voidage array holds the fluid voidage until the sand pass
    aux4[slot] = a;
    // the records the later passes gather (the same products their terms form)
    const float4 vi4 = vel4[slot];
    if (sandI) {
        vrec2[slot] = make_float2(bz, -pi4.w / vi4.w);
        grec4[slot] = make_float4(vi4.x, vi4.y, vi4.z, v_s);
    } else {
        const float vol = pi4.w / vi4.w;
        vrec2[slot] = make_float2(a.y * vol, vol);
    }
}

// ------------------------------------------------ voidage / adhesion stage
// Sand: ComputeSFSandVoidage_CUDA (cuda_sph_sf_solver_gpu.cuh:209-238,
// 680-721) and ComputeSFWetSandColor_CUDA (952-977). Water: the SF or MULTI
// water adhesion kernel (175-207, 574-678). Reads the fluid voidage (aux.y)
// of water neighbours and writes the final voidage (aux.w) of sand slots.
// Lane-split like kAvgFlow (order-preserving sums).
template <int G>
__global__ void __launch_bounds__(kSlotAlign) kVoidageAdhesion(
    const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene, NbrLists L,
    const float4* __restrict__ pos4, const float4* __restrict__ vel4, float4* __restrict__ aux4,
    const float4* __restrict__ flow4, float4* __restrict__ adh4, float4* __restrict__ avgadh4,
    float4* __restrict__ col4, float2* __restrict__ dp, const float2* __restrict__ vrec2,
    float4* __restrict__ grec4) {
    SF_SLOT_PROLOGUE_G
    const float4 pi4 = pos4[slot];
    if (pi4.w == 0.f) return;
    const float3 pi = xyz(pi4);
    if (pi4.w < 0.f) {
        const float sat = aux4[slot].z;
        float num = 0.f, den = 0.f;
        forLabelNeighborsOrdered<false, G, 2>(
            S, L, slot, pi, pos4, part,
            [&](int j) {
                const float4 pj = pos4[j];
                const float2 r = vrec2[j];  // (fluid voidage x volume, volume)
                const float3 dij = pi - xyz(pj);
                const float wij = poly6(S, len3(dij));
                Terms<2> t;
                t.v[0] = r.x * wij;
                t.v[1] = r.y * wij;
                return t;
            },
            [&](const Terms<2>& t) {
                num += t.v[0];
                den += t.v[1];
            });
        if (part != 0) return;
        aux4[slot].w = den != 0.f ? num / den : 0.f;
        dp[slot] = make_float2(den, 0.f);  // the quotient's denominator, for the adjoint
        // wet-sand colour ratchet
        float4 c = col4[slot];
        if (c.w < sat) {
            c.x = S.dry[0] + (S.wet[0] - S.dry[0]) * sat;
            c.y = S.dry[1] + (S.wet[1] - S.dry[1]) * sat;
            c.z = S.dry[2] + (S.wet[2] - S.dry[2]) * sat;
            c.w = sat;
            col4[slot] = c;
        }
        adh4[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        avgadh4[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        const float mi = pi4.w;
        float v_s = 0.f;
        float3 ad = mk3(0.f, 0.f, 0.f);
        forLabelNeighborsOrdered<true, G, 4>(
            S, L, slot, pi, pos4, part,
            [&](int j) {
                const float4 pj = pos4[j];
                const float2 r = vrec2[j];  // (adhesion Bezier factor of sat_j, volume)
                const float3 dpij = pi - xyz(pj);
                const float ldp = len3(dpij);
                const float wij = poly6(S, ldp);
                const float adij = adhesionSpline(S, ldp);
                const float mj = -pj.w;
                const float3 a = r.x * mi * mj * adij * dpij / fmaxf(kEps, ldp);
                const float vj = r.y;
                Terms<4> t;
                t.v[0] = a.x;
                t.v[1] = a.y;
                t.v[2] = a.z;
                t.v[3] = vj * wij;
                return t;
            },
            [&](const Terms<4>& t) {
                ad += mk3(t.v[0], t.v[1], t.v[2]);
                v_s += t.v[3];
            });
        if (part != 0) return;
        adh4[slot] = make_float4(ad.x, ad.y, ad.z, v_s);  // w: the average's denominator, for the adjoint
        const float3 avg = v_s != 0.f ? ad / v_s : mk3(0.f, 0.f, 0.f);
        // the effective density and pressure term, with the operations every
        // momentum pair term of this particle uses
        const float4 ai = aux4[slot];
        const float4 vi4 = vel4[slot];
        const float D = vi4.w / fmaxf(kEps, ai.w);
        const float P = ai.x / fmaxf(kEps, D * D);
        dp[slot] = make_float2(D, P);
        avgadh4[slot] = make_float4(avg.x, avg.y, avg.z, D);  // w: D, for the sand momentum pass
        grec4[slot] = make_float4(vi4.x, vi4.y, vi4.z, P);
    }
}

// -------------------------------------------------------------- integrate
// ComputeSubTimeStepsByCFL (cuda_wcsph_sf_solver.cu:35-58) on the device,
// then CudaSFParticles::Advect with AccDampingForSand (cuda_sf_particles.cu:
// 18-48, cuda_sf_particles.cuh:19-40) and SFWaterBoundaryConstrain_CUDA
// (cuda_sph_sf_solver_gpu.cuh:979-1074). adaptive: timeArg is the render
// interval and dt = timeArg / N_sub; otherwise dt = timeArg.
__device__ __forceinline__ long long cflSubsteps(const SceneDev& S, float amax, float T) {
    if (!S.wcsph) {
        const float q = T / S.params_dt;
        return q >= 9.2e18f ? (long long)9.2e18f : (long long)q;
    }
    const float maxForce = amax * S.cfl_mass;
    const float byForce = 0.25f * sqrtf(S.cfl_hm / maxForce);
    const float inner = byForce < S.cfl_by_speed ? byForce : S.cfl_by_speed;  // std::min
    const float scaled = S.cfl_scale * inner;
    const float desired = S.params_dt < scaled ? S.params_dt : scaled;
    const float q = T / desired;
    return q >= 9.2e18f ? (long long)9.2e18f : (long long)q;
}

__global__ void kIntegrate(const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene,
                           SceneState* __restrict__ state, float timeArg, const float* __restrict__ timeArgDev,
                           int adaptive,
                           const unsigned int* __restrict__ bcs, const float4* __restrict__ bpos4,
                           float4* __restrict__ pos4, float4* __restrict__ vel4, float4* __restrict__ acc4,
                           float4* __restrict__ adh4, float4* __restrict__ avgadh4) {
    SF_SLOT_PROLOGUE
    if (timeArgDev) timeArg = *timeArgDev;  // a graph-replayed step reads the time from the device
    float dt = timeArg;
    if (adaptive) {
        // WCSPH advects by renderInterval / N_sub (cuda_wcsph_sf_solver.cpp:168-172); plain
        // SPH by params.dt, whatever N_sub = renderInterval / params.dt rounds to
        // (cuda_sph_sf_solver.cpp:23, 141-146)
        const long long ns = cflSubsteps(S, __uint_as_float(state[sid].amax_bits), timeArg);
        dt = S.wcsph ? timeArg / float(ns) : S.params_dt;
        if (slot == S.slot_off) {
            state[sid].n_sub = ns;
            state[sid].dt = dt;
        }
    } else if (slot == S.slot_off) {
        state[sid].dt = dt;
    }
    float4 p4 = pos4[slot];
    if (p4.w == 0.f) return;
    float4 v4 = vel4[slot];
    float3 a = xyz(acc4[slot]);
    float3 v = xyz(v4);
    if (p4.w < 0.f) {
        const float3 q = a * (v + 0.5f * dt * a);
        const float3 s = mk3(float(sgn1(q.x)), float(sgn1(q.y)), float(sgn1(q.z)));
        a = a * (mk3(1.f, 1.f, 1.f) - S.damping * s);
        acc4[slot] = make_float4(a.x, a.y, a.z, 0.f);
    }
    v = v + dt * a;
    float3 p = xyz(p4) + dt * v;
    if (p4.w > 0.f) {
        const float r2 = 2.f * S.sph_radius;
        float3 tp = p, tv = v;
        if (tp.x > S.hpx - r2) { tp.x = S.hpx - r2; tv.x = fminf(tv.x, 0.f); }
        if (tp.x < S.lpx + r2) { tp.x = S.lpx + r2; tv.x = fmaxf(tv.x, 0.f); }
        if (tp.y > S.hpy - r2) { tp.y = S.hpy - r2; tv.y = fminf(tv.y, 0.f); }
        if (tp.y < S.lpy + r2) { tp.y = S.lpy + r2; tv.y = fmaxf(tv.y, 0.f); }
        if (tp.z > S.hpz - r2) { tp.z = S.hpz - r2; tv.z = fminf(tv.z, 0.f); }
        if (tp.z < S.lpz + r2) { tp.z = S.lpz + r2; tv.z = fmaxf(tv.z, 0.f); }
        if (S.shape_boundary) {  // only boundary particles with label 1 push water out
            forEachCell(S, cellOf(S, p), [&](int cell) {
                for (unsigned j = bcs[cell]; j < bcs[cell + 1]; ++j) {
                    const float4 bj = bpos4[j];
                    if (!(bj.w < 0.f)) continue;
                    const float dpij = len3(p - xyz(bj));
                    const float overlap = dpij - r2;
                    if (overlap < 0.f) {
                        const float3 nn = (p - xyz(bj)) / dpij;
                        tv = tv * 0.f;
                        tp += nn * -overlap;
                    }
                }
            });
        }
        p = tp;
        v = tv;
    }
    pos4[slot] = make_float4(p.x, p.y, p.z, p4.w);
    vel4[slot] = make_float4(v.x, v.y, v.z, v4.w);
    // the two thrust::fill clears of cuda_sph_sf_solver.cu:384-385
    adh4[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    avgadh4[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------------- neighbour-count probe
// The list capacity probe: particles within the interaction reach of each
// particle, walked like the density pass, maxed over all particles.
__global__ void kNeighborCountMax(const SceneDev* __restrict__ scenes, const int* __restrict__ blockScene,
                                  const float4* __restrict__ pos4, const unsigned int* __restrict__ cs,
                                  unsigned int* maxCount) {
    SF_SLOT_PROLOGUE
    const float4 pi4 = pos4[slot];
    unsigned n = 0;
    if (pi4.w != 0.f) {
        const float3 pi = xyz(pi4);
        const int3 c = cellOf(S, pi);
        const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, S.gz - 1) + 1;
        for (int x = max(c.x - 1, 0); x <= min(c.x + 1, S.gx - 1); ++x)
            for (int y = max(c.y - 1, 0); y <= min(c.y + 1, S.gy - 1); ++y) {
                const int base = S.cell_off + (x * S.gy + y) * S.gz;
                for (unsigned j = cs[base + z0]; j < cs[base + z1]; ++j) n += inReachFast(S, pi - xyz(pos4[j])) ? 1u : 0u;
            }
    }
    for (int o = 16; o > 0; o >>= 1) n = max(n, __shfl_xor_sync(0xffffffffu, n, o));
    if ((threadIdx.x & 31) == 0 && n > 0) atomicMax(maxCount, n);
}

// ------------------------------------------------------------ launchers
int lanesForSlots(long long totalSlots, int smCount) {
    int g = 1;
    while (g < 8 && totalSlots * g < 2048LL * smCount) g *= 2;
    return g;
}

// Blocks of a tuned pass over all slots.
static inline int grid(const LaunchCtx& c, int pass) { return c.slotBlocks * (kSlotAlign / c.block[pass]); }

void launchNeighborCountMax(const LaunchCtx& c, const float4* pos4, const unsigned int* cs, unsigned int* maxCount) {
    kNeighborCountMax<<<c.slotBlocks, kSlotAlign, 0, c.stream>>>(c.scenes, c.blockScene, pos4, cs, maxCount);
}

void launchBoundaryVolume(const LaunchCtx& c, int sid, int nb, float4* bpos4, const int* blabel,
                          const unsigned int* bcs) {
    if (nb <= 0) return;
    kBoundaryVolume<<<(nb + 255) / 256, 256, 0, c.stream>>>(c.scenes, sid, bpos4, blabel, bcs);
}

template <int G> void launchDensityLanes(const LaunchCtx& c, const PassBuffers& b) {
    kDensityLanes<G><<<grid(c, kPassDensity) * G, c.block[kPassDensity], 0, c.stream>>>(
        c.scenes, c.blockScene, c.state, b.listsW, b.pos4, b.bpos4, b.vel4, b.aux4);
}
void launchDensity(const LaunchCtx& c, const PassBuffers& b) {
    switch (c.lanes) {
    case 2: launchDensityLanes<2>(c, b); break;
    case 4: launchDensityLanes<4>(c, b); break;
    case 8: launchDensityLanes<8>(c, b); break;
    default:
        if (c.densityStaged) {
            // 14 positions per thread (a block of 128 consecutive slots
            // needs ~10.4 on the 1M embankment), within 48 KB per block
            const int cap = std::min(14 * c.block[kPassDensity], kDensityStageMax);
            kDensity<true><<<grid(c, kPassDensity), c.block[kPassDensity], size_t(cap) * sizeof(float4), c.stream>>>(
                c.scenes, c.blockScene, c.state, b.listsW, b.pos4, b.bpos4, b.vel4, b.aux4, cap);
        } else {
            kDensity<false><<<grid(c, kPassDensity), c.block[kPassDensity], 0, c.stream>>>(
                c.scenes, c.blockScene, c.state, b.listsW, b.pos4, b.bpos4, b.vel4, b.aux4, 0);
        }
        break;
    }
}

template <int G> void launchAvgFlowG(const LaunchCtx& c, const PassBuffers& b) {
    kAvgFlow<G><<<grid(c, kPassAvgFlow) * G, c.block[kPassAvgFlow], 0, c.stream>>>(
        c.scenes, c.blockScene, b.lists, b.pos4, b.vel4, b.aux4, b.flow4, b.vrec2, b.grec4);
}
void launchAvgFlow(const LaunchCtx& c, const PassBuffers& b) {
    switch (c.lanes) {
    case 2: launchAvgFlowG<2>(c, b); break;
    case 4: launchAvgFlowG<4>(c, b); break;
    case 8: launchAvgFlowG<8>(c, b); break;
    default: launchAvgFlowG<1>(c, b); break;
    }
}

template <int G> void launchVoidageAdhesionG(const LaunchCtx& c, const PassBuffers& b) {
    kVoidageAdhesion<G><<<grid(c, kPassVoidage) * G, c.block[kPassVoidage], 0, c.stream>>>(
        c.scenes, c.blockScene, b.lists, b.pos4, b.vel4, b.aux4, b.flow4, b.adh4, b.avgadh4, b.col4, b.dp, b.vrec2,
        b.grec4);
}
void launchVoidageAdhesion(const LaunchCtx& c, const PassBuffers& b) {
    switch (c.lanes) {
    case 2: launchVoidageAdhesionG<2>(c, b); break;
    case 4: launchVoidageAdhesionG<4>(c, b); break;
    case 8: launchVoidageAdhesionG<8>(c, b); break;
    default: launchVoidageAdhesionG<1>(c, b); break;
    }
}

void launchIntegrate(const LaunchCtx& c, const PassBuffers& b, float timeArg, int adaptive, const float* timeArgDev) {
    kIntegrate<<<grid(c, kPassIntegrate), c.block[kPassIntegrate], 0, c.stream>>>(c.scenes, c.blockScene, c.state,
                                                          timeArg, timeArgDev, adaptive,
                                                          b.lists.bcs, b.bpos4, b.pos4, b.vel4, b.acc4, b.adh4,
                                                          b.avgadh4);
}

}  // namespace sfg
