// Stable LSD radix sort of 32-bit cell keys, cell-start table and reorder.
//
// Replaces the reference's neighbor-grid build (cuda_neighbor_searcher.cu:
// 36-51, 64-116): thrust::sort_by_key on the cell keys with the particle
// arrays as values (a stable sort, so particles of one cell keep their
// previous relative order), then an atomic histogram + exclusive scan for
// cellStart. Here one stable sort of (key, slot) pairs yields the
// permutation, one gather applies it to every persistent array, and
// cellStart[c] is the lower bound of c in the sorted keys. The result is the
// same permutation and the same table as the reference's.
//
// Per digit pass (8-bit digits, or 9-11 bits when that saves a pass): kHist
// (per-tile digit counts), kScanTiles (per digit, exclusive scan over tiles)
// and kScatter (digit offsets, in-tile stable rank: rounds of 256 keys in
// index order, warp match for the rank inside a warp, shared per-warp digit
// counts for the rank across warps, moved into the running digit offsets by
// the warp leaders of each round). The first pass takes its tile histograms
// from the key kernel (kKeysHist), and the reorder writes the cell table
// (cellStart[c] = lower bound of c) as it gathers, so a sort stage of two
// digit passes is six launches.
#include "sf_device.cuh"
#include "sf_kernels.h"

namespace sfg {

constexpr int kSortThreads = 256;

int sortTiles(int n, int items) { return (n + kSortThreads * items - 1) / (kSortThreads * items); }

int sortItemsFor(int n, int smCount) {
    for (int items = 8; items > 1; items >>= 1)
        if (sortTiles(n, items) >= 2 * smCount) return items;
    return 1;
}

template <int kSortItems, int kBits>
__global__ void __launch_bounds__(kSortThreads) kHist(const unsigned int* __restrict__ keys, int n, int shift,
                                                      unsigned int* __restrict__ hist, int tiles) {
    constexpr int kTile = kSortThreads * kSortItems;
    constexpr int R = 1 << kBits, kPer = R / kSortThreads;
    __shared__ unsigned int h[R];
#pragma unroll
    for (int q = 0; q < kPer; ++q) h[threadIdx.x * kPer + q] = 0;
    __syncthreads();
    const int base = blockIdx.x * kTile;
    // all of the thread's keys are loaded before the first shared-memory add
    unsigned int k[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * kSortThreads + threadIdx.x;
        k[r] = idx < n ? keys[idx] : 0u;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r)
        if (base + r * kSortThreads + int(threadIdx.x) < n) atomicAdd(&h[(k[r] >> shift) & unsigned(R - 1)], 1u);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int d = threadIdx.x * kPer + q;
        hist[size_t(d) * tiles + blockIdx.x] = h[d];
    }
}

// The cell keys (slotKey) of one tile of slots and the tile's histogram of
// their first digit: kHist of the first pass fused into the key computation.
// Rounds of 256 slots are 256-slot blocks of one scene each.
template <int kSortItems, int kBits>
__global__ void __launch_bounds__(kSortThreads) kKeysHist(const SceneDev* __restrict__ scenes,
                                                          const int* __restrict__ blockScene,
                                                          const float4* __restrict__ pos4,
                                                          unsigned int* __restrict__ keys, unsigned int* errWord,
                                                          int n, unsigned int* __restrict__ hist, int tiles) {
    constexpr int kTile = kSortThreads * kSortItems;
    constexpr int R = 1 << kBits, kPer = R / kSortThreads;
    __shared__ unsigned int h[R];
#pragma unroll
    for (int q = 0; q < kPer; ++q) h[threadIdx.x * kPer + q] = 0;
    __syncthreads();
    const int base = blockIdx.x * kTile;
    // positions are loaded in groups of (up to) four before their keys
    constexpr int kGroup = kSortItems < 4 ? kSortItems : 4;
#pragma unroll 1
    for (int r0 = 0; r0 < kSortItems; r0 += kGroup) {
        float4 p[kGroup];
        int sid[kGroup];
#pragma unroll
        for (int u = 0; u < kGroup; ++u) {
            const int slot = base + (r0 + u) * kSortThreads + threadIdx.x;
            sid[u] = slot < n ? blockScene[slot / kSlotAlign] : 0;
            p[u] = slot < n ? pos4[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kGroup; ++u) {
            const int slot = base + (r0 + u) * kSortThreads + threadIdx.x;
            if (slot < n) {
                const unsigned int k = slotKey(scenes[sid[u]], p[u], errWord);
                keys[slot] = k;
                atomicAdd(&h[k & unsigned(R - 1)], 1u);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int d = threadIdx.x * kPer + q;
        hist[size_t(d) * tiles + blockIdx.x] = h[d];
    }
}

template <int kSortItems>
static void launchKeysHistI(const LaunchCtx& c, int n, const float4* pos4, unsigned int* keys,
                            const SortScratch& sc) {
    switch (sc.digitBits) {
    case 9:
        kKeysHist<kSortItems, 9><<<sc.tiles, kSortThreads, 0, c.stream>>>(c.scenes, c.blockScene, pos4, keys,
                                                                          c.errWord, n, sc.hist, sc.tiles);
        break;
    case 10:
        kKeysHist<kSortItems, 10><<<sc.tiles, kSortThreads, 0, c.stream>>>(c.scenes, c.blockScene, pos4, keys,
                                                                           c.errWord, n, sc.hist, sc.tiles);
        break;
    case 11:
        kKeysHist<kSortItems, 11><<<sc.tiles, kSortThreads, 0, c.stream>>>(c.scenes, c.blockScene, pos4, keys,
                                                                           c.errWord, n, sc.hist, sc.tiles);
        break;
    default:
        kKeysHist<kSortItems, 8><<<sc.tiles, kSortThreads, 0, c.stream>>>(c.scenes, c.blockScene, pos4, keys,
                                                                          c.errWord, n, sc.hist, sc.tiles);
        break;
    }
}

void launchKeysHist(const LaunchCtx& c, int n, const float4* pos4, unsigned int* keys, const SortScratch& sc) {
    switch (sc.items) {
    case 1: launchKeysHistI<1>(c, n, pos4, keys, sc); break;
    case 2: launchKeysHistI<2>(c, n, pos4, keys, sc); break;
    case 4: launchKeysHistI<4>(c, n, pos4, keys, sc); break;
    default: launchKeysHistI<8>(c, n, pos4, keys, sc); break;
    }
}

// Per-digit exclusive scan over tiles: block d scans hist[d * tiles ..
// d * tiles + tiles) in place and writes the digit's total.
__global__ void __launch_bounds__(kSortThreads) kScanTiles(unsigned int* __restrict__ hist, int tiles,
                                                           unsigned int* __restrict__ digitTotal) {
    __shared__ unsigned int part[kSortThreads];
    unsigned int* h = hist + size_t(blockIdx.x) * tiles;
    unsigned int carry = 0;
    for (int base = 0; base < tiles; base += kSortThreads) {
        const int t = base + threadIdx.x;
        const unsigned int v = t < tiles ? h[t] : 0u;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kSortThreads; o <<= 1) {
            const unsigned int u = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
            __syncthreads();
            part[threadIdx.x] += u;
            __syncthreads();
        }
        if (t < tiles) h[t] = carry + part[threadIdx.x] - v;
        carry += part[kSortThreads - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) digitTotal[blockIdx.x] = carry;
}

template <int kSortItems, int kBits>
__global__ void __launch_bounds__(kSortThreads) kScatter(const unsigned int* __restrict__ keysIn,
                                                         const unsigned int* __restrict__ valsIn,
                                                         unsigned int* __restrict__ keysOut,
                                                         unsigned int* __restrict__ valsOut, int n, int shift,
                                                         const unsigned int* __restrict__ hist, int tiles,
                                                         const unsigned int* __restrict__ digitTotal) {
    constexpr int kWarps = kSortThreads / 32;
    constexpr int kTile = kSortThreads * kSortItems;
    constexpr int R = 1 << kBits, kPer = R / kSortThreads;
    __shared__ unsigned int base[R];
    __shared__ unsigned int running[R];
    __shared__ unsigned char cnt[kWarps][R];  // keys of a digit per warp in one round (<= 32)
    __shared__ unsigned int warpSum[kWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // digit offsets: exclusive scan of the digit totals (kPer consecutive
    // digits per thread, then a block scan of the threads' sums)
    unsigned int tot[kPer], sum = 0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        tot[q] = digitTotal[tid * kPer + q];
        sum += tot[q];
    }
    unsigned int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warpSum[warp] = incl;
    __syncthreads();
    unsigned int acc = incl - sum;
    for (int w = 0; w < warp; ++w) acc += warpSum[w];
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int d = tid * kPer + q;
        base[d] = acc + hist[size_t(d) * tiles + blockIdx.x];
        acc += tot[q];
        running[d] = 0;
    }
    unsigned int* cnt32 = reinterpret_cast<unsigned int*>(&cnt[0][0]);
    for (int q = tid; q < kWarps * R / 4; q += kSortThreads) cnt32[q] = 0u;
    __syncthreads();
    const unsigned int ltMask = (1u << lane) - 1u;
    const int tileBase = blockIdx.x * kTile;
    // the thread's keys and values of every round are loaded up front, so the
    // rounds (three barriers each) do not wait for global loads
    unsigned int kr[kSortItems], vr[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = tileBase + r * kSortThreads + tid;
        kr[r] = idx < n ? keysIn[idx] : 0u;
        vr[r] = idx < n ? (valsIn ? valsIn[idx] : unsigned(idx)) : 0u;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = tileBase + r * kSortThreads + tid;
        const bool valid = idx < n;
        const unsigned int k = kr[r], v = vr[r];
        const unsigned int d = valid ? (k >> shift) & unsigned(R - 1) : unsigned(R);
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const unsigned int rank = __popc(peers & ltMask);
        const bool leader = valid && rank == 0;
        if (leader) cnt[warp][d] = (unsigned char)__popc(peers);
        __syncthreads();
        if (valid) {
            unsigned int pre = 0;
            for (int w = 0; w < warp; ++w) pre += cnt[w][d];
            const unsigned int pos = base[d] + running[d] + pre + rank;
            keysOut[pos] = k;
            valsOut[pos] = v;
        }
        __syncthreads();
        // only the digits of this round: the warp leaders move their counts
        if (leader) {
            atomicAdd(&running[d], unsigned(__popc(peers)));
            cnt[warp][d] = 0;
        }
        __syncthreads();
    }
}

template <int kSortItems, int kBits>
static void launchPassT(cudaStream_t s, int n, int shift, const unsigned int* kIn, const unsigned int* vIn,
                        unsigned int* kOut, unsigned int* vOut, const SortScratch& sc, bool histDone) {
    const int tiles = sc.tiles;
    if (!histDone) kHist<kSortItems, kBits><<<tiles, kSortThreads, 0, s>>>(kIn, n, shift, sc.hist, tiles);
    kScanTiles<<<1 << kBits, kSortThreads, 0, s>>>(sc.hist, tiles, sc.digitTotal);
    kScatter<kSortItems, kBits><<<tiles, kSortThreads, 0, s>>>(kIn, vIn, kOut, vOut, n, shift, sc.hist, tiles,
                                                               sc.digitTotal);
}

template <int kSortItems>
static void launchPass(cudaStream_t s, int n, int shift, int bits, const unsigned int* kIn,
                       const unsigned int* vIn, unsigned int* kOut, unsigned int* vOut, const SortScratch& sc,
                       bool histDone) {
    switch (bits) {
    case 9: launchPassT<kSortItems, 9>(s, n, shift, kIn, vIn, kOut, vOut, sc, histDone); break;
    case 10: launchPassT<kSortItems, 10>(s, n, shift, kIn, vIn, kOut, vOut, sc, histDone); break;
    case 11: launchPassT<kSortItems, 11>(s, n, shift, kIn, vIn, kOut, vOut, sc, histDone); break;
    default: launchPassT<kSortItems, 8>(s, n, shift, kIn, vIn, kOut, vOut, sc, histDone); break;
    }
}

int sortDigitBits(int keyBits) {
    const int passes8 = (keyBits + 7) / 8, passes11 = (keyBits + 10) / 11;
    if (passes11 >= passes8) return 8;
    return (keyBits + passes11 - 1) / passes11;  // the narrowest digits for that many passes
}

int radixSort(cudaStream_t s, int n, int bits, unsigned int* keys, SortScratch& sc, unsigned int** keysOut,
              unsigned int** permOut, bool firstHistDone) {
    const int digit = sc.digitBits ? sc.digitBits : 8;
    const int passes = (bits + digit - 1) / digit;
    unsigned int* kIn = keys;
    unsigned int* kOut = sc.keysAlt;
    unsigned int* vIn = nullptr;
    unsigned int* vOut = sc.vals;
    int launches = 0;
    for (int p = 0; p < passes; ++p) {
        const int shift = digit * p;
        const bool histDone = p == 0 && firstHistDone;
        switch (sc.items) {
        case 1: launchPass<1>(s, n, shift, digit, kIn, vIn, kOut, vOut, sc, histDone); break;
        case 2: launchPass<2>(s, n, shift, digit, kIn, vIn, kOut, vOut, sc, histDone); break;
        case 4: launchPass<4>(s, n, shift, digit, kIn, vIn, kOut, vOut, sc, histDone); break;
        default: launchPass<8>(s, n, shift, digit, kIn, vIn, kOut, vOut, sc, histDone); break;
        }
        launches += histDone ? 2 : 3;
        // next pass reads what this one wrote
        unsigned int* t = kIn;
        kIn = kOut;
        kOut = t;
        vIn = vOut;
        vOut = (vOut == sc.vals) ? sc.valsAlt : sc.vals;
    }
    *keysOut = kIn;
    *permOut = vIn;
    return launches;
}

__global__ void kCellStart(int n, int nCells, const unsigned int* __restrict__ sk, unsigned int* __restrict__ cs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > nCells) return;
    int lo = 0, hi = n;  // first index with sk[i] >= c
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sk[mid] < unsigned(c))
            lo = mid + 1;
        else
            hi = mid;
    }
    cs[c] = unsigned(lo);
}

void launchCellStart(cudaStream_t s, int n, int nCells, const unsigned int* sortedKeys, unsigned int* cellStart) {
    kCellStart<<<(nCells + 1 + 255) / 256, 256, 0, s>>>(n, nCells, sortedKeys, cellStart);
}

// cellStart[c] = v for c in [lo, hi), written by the lanes of one warp
// (all 32 call it): short runs by their own lane, long runs (the empty cells
// before a sparse region, up to whole empty slabs of the grid) by the whole
// warp, one run after the other, in 16-byte stores (the table is 16-byte
// aligned).
__device__ __forceinline__ void fillCellRuns(unsigned int* __restrict__ cs, unsigned int lo, unsigned int hi,
                                             unsigned int v) {
    constexpr unsigned int kShort = 8;
    if (hi - lo <= kShort)
        for (unsigned int c = lo; c < hi; ++c) cs[c] = v;
    const unsigned int lane = threadIdx.x & 31u;
    for (unsigned int longRuns = __ballot_sync(0xffffffffu, hi - lo > kShort); longRuns; longRuns &= longRuns - 1u) {
        const int src = __ffs(longRuns) - 1;
        const unsigned int l = __shfl_sync(0xffffffffu, lo, src), h = __shfl_sync(0xffffffffu, hi, src);
        const unsigned int w = __shfl_sync(0xffffffffu, v, src);
        const unsigned int a = min(h, (l + 3u) & ~3u), b = a + ((h - a) & ~3u);  // [a, b): whole 16-byte words
        if (lane < a - l) cs[l + lane] = w;
        if (lane < h - b) cs[b + lane] = w;
        const uint4 w4 = make_uint4(w, w, w, w);
        for (unsigned int q = a / 4u + lane; q < b / 4u; q += 32u) reinterpret_cast<uint4*>(cs)[q] = w4;
    }
}

__global__ void kReorder(int n, const unsigned int* __restrict__ perm, const float4* __restrict__ pos,
                         const float4* __restrict__ vel, const float4* __restrict__ col,
                         const float4* __restrict__ mat, const float2* __restrict__ amc, const int* __restrict__ pid,
                         float4* __restrict__ posOut, float4* __restrict__ velOut, float4* __restrict__ colOut,
                         float4* __restrict__ matOut, float2* __restrict__ amcOut, int* __restrict__ pidOut,
                         const unsigned int* __restrict__ sk, int nCells, unsigned int* __restrict__ cs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;  // n is a multiple of 32: whole warps stay
    // cell table (the lower bound of every cell in the sorted keys): index i
    // starts the cells after its predecessor's key up to its own key; the
    // last index also ends the table
    // (keys above nCells, which only a corrupt position could give, are
    // clamped: that leaves every lower bound in [0, nCells] unchanged)
    const unsigned int top = unsigned(nCells);
    const unsigned int k = min(sk[i], top);
    fillCellRuns(cs, i == 0 ? 0u : min(sk[i - 1], top) + 1u, k + 1u, unsigned(i));
    fillCellRuns(cs, k + 1u, i == n - 1 ? unsigned(nCells) + 1u : k + 1u, unsigned(n));
    const unsigned int o = perm[i];
    posOut[i] = pos[o];
    velOut[i] = vel[o];
    colOut[i] = col[o];
    matOut[i] = mat[o];
    amcOut[i] = amc[o];
    pidOut[i] = pid[o];
}

void launchReorder(cudaStream_t s, int n, const unsigned int* perm, const float4* pos, const float4* vel,
                   const float4* col, const float4* mat, const float2* amc, const int* pid, float4* posOut,
                   float4* velOut, float4* colOut, float4* matOut, float2* amcOut, int* pidOut,
                   const unsigned int* sortedKeys, int nCells, unsigned int* cellStart) {
    kReorder<<<(n + 255) / 256, 256, 0, s>>>(n, perm, pos, vel, col, mat, amc, pid, posOut, velOut, colOut, matOut,
                                            amcOut, pidOut, sortedKeys, nCells, cellStart);
}

}  // namespace sfg
