// Host-side launch interface of the substep kernels (sf_kernels.cu, sf_sort.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sfg {

struct SceneDev;
struct SceneState;

// Passes whose block size the tuner picks (threads per block, a divisor of
// kSlotAlign so that a block never spans two scenes).
enum TunedPass { kPassDensity = 0, kPassAvgFlow, kPassVoidage, kPassSand, kPassWater, kPassIntegrate, kTunedPasses };

// Launch context shared by all passes of one handle.
struct LaunchCtx {
    cudaStream_t stream;
    const SceneDev* scenes;   // device array [n_scenes]
    const int* blockScene;    // device array [slotBlocks]: scene of each kSlotAlign block
    SceneState* state;        // device array [n_scenes]
    unsigned int* errWord;    // device error word
    int slotBlocks;           // total slots / kSlotAlign
    int block[kTunedPasses];  // threads per block of each tuned pass
    int lanes;                // threads per slot of the momentum passes (1, 2, 4 or 8)
    int densityStaged;        // 1: the one-lane density pass stages its candidates in shared memory
};

// Largest shared staging of the density pass, in positions (16 B each): with
// the pass's own shared table it stays within the 48 KB a block gets without
// an opt-in.
constexpr int kDensityStageMax = 3008;

// Neighbour lists of the current substep (column-major: entry k of slot i at
// k * M + i). Particle lists hold sand neighbours from entry 0 upwards and
// water neighbours from entry cap - 1 downwards; cnt packs the two counts
// (sand in the low 16 bits, each saturating at 0xFFFF). Counts summing above
// cap mean the list overflowed: walk the stencil instead. A boundary count
// above kMaxBNbr means the same for the boundary list. The capacity cap is
// chosen per handle from the neighbour counts of its scenes (a multiple of
// 32 between kMinNbr and kMaxNbr).
constexpr int kMinNbr = 64;
constexpr int kMaxNbr = 256;
constexpr int kMaxBNbr = 48;
// Sand-sand pairs within DEM contact + liquid-bridge reach of a sand particle
// (the only pairs with DEM or capillary forces); more means "filter the sand list".
constexpr int kMaxContact = 16;
struct NbrLists {
    const unsigned int* cnt;
    const unsigned int* nbr;
    const int* bcnt;
    const unsigned int* bnbr;
    const int* ccnt;
    const unsigned int* cnbr;
    const unsigned int* cs;   // particle cell table (total_cells + 1)
    const unsigned int* bcs;  // boundary cell table (total_cells + 1)
    // per cell: 1 if a boundary particle lies in the cell or one of its 26
    // neighbours (the boundary is static, so this is set once at creation);
    // null means every cell walks its boundary ranges
    const unsigned char* bnear;
    long long M;              // total slots
    int cap;                  // particle list capacity
};
struct NbrListsW {
    unsigned int* cnt;
    unsigned int* nbr;
    int* bcnt;
    unsigned int* bnbr;
    int* ccnt;
    unsigned int* cnbr;
    const unsigned int* cs;
    const unsigned int* bcs;
    const unsigned char* bnear;
    long long M;
    int cap;
};

// Device buffers the neighbor passes read and write (current sort order).
struct PassBuffers {
    NbrLists lists;
    NbrListsW listsW;
    float4* pos4;
    float4* vel4;
    float4* aux4;
    float4* flow4;
    float4* adh4;
    float4* avgadh4;
    float4* drag4;
    float4* acc4;
    float4* col4;
    float4* mat4;
    const float4* bpos4;
    // water: (D, P) = (rho / max(eps, voidage), p / max(eps, D^2)), the
    // effective density and pressure term every momentum pair term of the
    // particle uses (written by the voidage / adhesion pass); sand: the
    // denominators of its voidage quotient and of its average drag (written
    // by the voidage and sand momentum passes), which the adjoint reads
    // instead of summing them again. adh4.w of water holds the denominator
    // of its average adhesion for the same reason.
    float2* dp;
    // Gather records, rewritten every substep so that a neighbour term loads
    // one record besides the neighbour's position (values bit-identical to
    // the ones the terms used to gather from several arrays):
    //   vrec2, average-flow pass -> voidage / adhesion pass: water (fluid
    //     voidage x volume m / rho, volume), sand (adhesion Bezier factor of
    //     its saturation, volume);
    //   grec4: sand (velocity, saturation) from the average-flow pass, for the
    //     DEM contacts; water (velocity, pressure term P) from the voidage /
    //     adhesion pass, for the water momentum pairs.
    // avgadh4.w of water holds its effective density D for the sand momentum pass.
    float2* vrec2;
    float4* grec4;
};

// Threads per slot of the lane-split passes (momentum passes and the adjoint
// pair kernels) for totalSlots slots on a GPU with smCount SMs: doubled, up
// to 8, while fewer than 2048 threads per SM would run.
int lanesForSlots(long long totalSlots, int smCount);

void launchBoundaryVolume(const LaunchCtx& c, int sid, int nb, float4* bpos4, const int* blabel,
                          const unsigned int* bcs);
void launchDensity(const LaunchCtx& c, const PassBuffers& b);
void launchAvgFlow(const LaunchCtx& c, const PassBuffers& b);
void launchVoidageAdhesion(const LaunchCtx& c, const PassBuffers& b);
void launchSandMomentum(const LaunchCtx& c, const PassBuffers& b);
void launchWaterMomentum(const LaunchCtx& c, const PassBuffers& b);
// timeArgDev: when not null, the kernel reads timeArg from this device scalar
// (graph-replayed steps whose render interval changes from call to call).
void launchIntegrate(const LaunchCtx& c, const PassBuffers& b, float timeArg, int adaptive,
                     const float* timeArgDev = nullptr);
// Largest number of particles within the interaction reach of any particle
// (itself included), atomically maxed into *maxCount; needs the cell table.
void launchNeighborCountMax(const LaunchCtx& c, const float4* pos4, const unsigned int* cs, unsigned int* maxCount);

// ---- stable LSD radix sort of 32-bit cell keys (sf_sort.cu) ----
// Scratch sizes for sorting n keys.
struct SortScratch {
    unsigned int* keysAlt;   // n
    unsigned int* vals;      // n
    unsigned int* valsAlt;   // n
    unsigned int* hist;      // 256 * tiles
    unsigned int* digitTotal;  // 256
    int tiles;               // sortTiles(n, items)
    int items;               // keys per thread of a tile: 1, 2, 4 or 8 (0 means 8)
    int digitBits;           // 8-11 (0 means 8); hist holds 2^digitBits * tiles, digitTotal 2^digitBits
};
// Digit width for keys of keyBits bits: 8, or the narrowest of 9-11 that
// needs fewer passes than 8-bit digits.
int sortDigitBits(int keyBits);
// Tiles of 256 threads x items keys over n keys.
int sortTiles(int n, int items = 8);
// Keys per thread for n keys: the largest of 8, 4, 2 that still gives every
// SM two tiles, else 1 (small sorts are a chain of short launches; smaller
// tiles spread them over more SMs).
int sortItemsFor(int n, int smCount);
// Sorts keys[0..n) (only the low `bits` bits are examined) and writes the
// stable permutation to *permOut (new index -> old index) and the sorted keys
// to *keysOut; both point into keys/scratch buffers. firstHistDone: sc.hist
// already holds the first digit's tile histograms (launchKeysHist). Returns
// kernels launched.
int radixSort(cudaStream_t s, int n, int bits, unsigned int* keys, SortScratch& sc, unsigned int** keysOut,
              unsigned int** permOut, bool firstHistDone = false);
// The cell key of every slot of the handle (n slots, a multiple of 256) and
// the first radix pass's tile histograms into sc.hist, in one launch.
void launchKeysHist(const LaunchCtx& c, int n, const float4* pos4, unsigned int* keys, const SortScratch& sc);
// cellStart[c] = first index i with sortedKeys[i] >= c, for c in [0, nCells]
void launchCellStart(cudaStream_t s, int n, int nCells, const unsigned int* sortedKeys, unsigned int* cellStart);
// Gather the persistent per-slot arrays into sorted order (n a multiple of
// 32) and write the cell table cellStart of the sorted keys (as
// launchCellStart) in the same launch.
void launchReorder(cudaStream_t s, int n, const unsigned int* perm, const float4* pos, const float4* vel,
                   const float4* col, const float4* mat, const float2* amc, const int* pid, float4* posOut,
                   float4* velOut, float4* colOut, float4* matOut, float2* amcOut, int* pidOut,
                   const unsigned int* sortedKeys, int nCells, unsigned int* cellStart);

}  // namespace sfg
