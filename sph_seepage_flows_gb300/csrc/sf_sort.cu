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
// Per 8-bit digit pass: kHist (per-tile digit counts), kScan (one block,
// digit-major exclusive scan over tiles) and kScatter (in-tile stable rank:
// rounds of 256 keys in index order, warp match for the rank inside a warp,
// shared per-warp digit counts for the rank across warps).
#include "sf_kernels.h"

namespace sfg {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int kScanThreads = 1024;

int sortTiles(int n) { return (n + kTile - 1) / kTile; }

__global__ void __launch_bounds__(kSortThreads) kHist(const unsigned int* __restrict__ keys, int n, int shift,
                                                      unsigned int* __restrict__ hist, int tiles) {
    __shared__ unsigned int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kTile;
#pragma unroll 4
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// In-place exclusive scan of hist[0..len) by one block.
__global__ void __launch_bounds__(kScanThreads) kScan(unsigned int* __restrict__ hist, int len) {
    __shared__ unsigned int part[kScanThreads];
    const int chunk = (len + kScanThreads - 1) / kScanThreads;
    const int b = threadIdx.x * chunk;
    const int e = min(b + chunk, len);
    unsigned int s = 0;
    for (int i = b; i < e; ++i) s += hist[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {
        unsigned int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned int run = part[threadIdx.x] - s;
    for (int i = b; i < e; ++i) {
        const unsigned int v = hist[i];
        hist[i] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kSortThreads) kScatter(const unsigned int* __restrict__ keysIn,
                                                         const unsigned int* __restrict__ valsIn,
                                                         unsigned int* __restrict__ keysOut,
                                                         unsigned int* __restrict__ valsOut, int n, int shift,
                                                         const unsigned int* __restrict__ hist, int tiles) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ unsigned int base[256];
    __shared__ unsigned int running[256];
    __shared__ unsigned int cnt[kWarps][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = hist[tid * tiles + blockIdx.x];
    running[tid] = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) cnt[w][tid] = 0;
    __syncthreads();
    const unsigned int ltMask = (1u << lane) - 1u;
    const int tileBase = blockIdx.x * kTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = tileBase + r * kSortThreads + tid;
        const bool valid = idx < n;
        unsigned int k = 0, v = 0, d = 256u;
        if (valid) {
            k = keysIn[idx];
            v = valsIn ? valsIn[idx] : unsigned(idx);
            d = (k >> shift) & 255u;
        }
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const unsigned int rank = __popc(peers & ltMask);
        if (valid && rank == 0) cnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned int pre = 0;
            for (int w = 0; w < warp; ++w) pre += cnt[w][d];
            const unsigned int pos = base[d] + running[d] + pre + rank;
            keysOut[pos] = k;
            valsOut[pos] = v;
        }
        __syncthreads();
        unsigned int tot = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            tot += cnt[w][tid];
            cnt[w][tid] = 0;
        }
        running[tid] += tot;
        __syncthreads();
    }
}

int radixSort(cudaStream_t s, int n, int bits, unsigned int* keys, SortScratch& sc, unsigned int** keysOut,
              unsigned int** permOut) {
    const int tiles = sortTiles(n);
    const int passes = (bits + 7) / 8;
    unsigned int* kIn = keys;
    unsigned int* kOut = sc.keysAlt;
    unsigned int* vIn = nullptr;
    unsigned int* vOut = sc.vals;
    int launches = 0;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        kHist<<<tiles, kSortThreads, 0, s>>>(kIn, n, shift, sc.hist, tiles);
        kScan<<<1, kScanThreads, 0, s>>>(sc.hist, 256 * tiles);
        kScatter<<<tiles, kSortThreads, 0, s>>>(kIn, vIn, kOut, vOut, n, shift, sc.hist, tiles);
        launches += 3;
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

__global__ void kReorder(int n, const unsigned int* __restrict__ perm, const float4* __restrict__ pos,
                         const float4* __restrict__ vel, const float4* __restrict__ col,
                         const float4* __restrict__ mat, const float2* __restrict__ amc, const int* __restrict__ pid,
                         float4* __restrict__ posOut, float4* __restrict__ velOut, float4* __restrict__ colOut,
                         float4* __restrict__ matOut, float2* __restrict__ amcOut, int* __restrict__ pidOut) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
                   float4* velOut, float4* colOut, float4* matOut, float2* amcOut, int* pidOut) {
    kReorder<<<(n + 255) / 256, 256, 0, s>>>(n, perm, pos, vel, col, mat, amc, pid, posOut, velOut, colOut, matOut,
                                            amcOut, pidOut);
}

}  // namespace sfg
