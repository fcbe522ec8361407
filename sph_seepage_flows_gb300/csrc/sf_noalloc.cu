// Allocation-free cell sort (sf_cell_sort_noalloc): the key computation,
// stable radix sort and cell-start table of the sort stage, with every
// scratch word in one static device array instead of handle memory.
//
// The scratch (g_noallocScratch) holds the keys, the ping-pong key and
// permutation buffers, the digit histograms and totals of the radix sort and
// a non-finite-position flag. Its device address is looked up once per
// device with cudaGetSymbolAddress (the first call on a device does it, and
// the first call after that device's context was reset, which is detected
// by asking the runtime whether the cached address is still a device
// address), so the call itself issues only kernels, one memset,
// device-to-device copies and one small device-to-host read. Every
// histogram and total is written before it is read; the flag is the only
// word that must start at zero and is cleared by every call. Calls that
// overlap on the GPU share the scratch and race.
#include "../../include/sf_capi.h"
#include "sf_device.cuh"
#include "sf_kernels.h"

#include <mutex>
#include <string>

namespace sfg {
void setGlobalError(const std::string& msg);  // sf_capi.cu: text for sf_last_error_string(NULL)
}

namespace {

using namespace sfg;

constexpr int kMaxN = SF_NOALLOC_MAX_PARTICLES;
constexpr size_t kFlagWords = 64;               // keeps the arrays behind it 256-byte aligned
constexpr size_t kHistWords = 256 * size_t(kMaxN / 1024);  // >= 256 digit counts per sort tile
constexpr size_t kWords = kFlagWords + 4 * size_t(kMaxN) + 256 + kHistWords;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned int g_noallocScratch[kWords];

// Pos2GridHash of every position (the key of the sort stage for a
// single-scene handle); non-finite positions set the flag.
__global__ void kNoAllocKeys(SceneDev S, const float* __restrict__ pos, int n, unsigned int* __restrict__ keys,
                             unsigned int* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 q = mk3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    if (!(isfinite(q.x) && isfinite(q.y) && isfinite(q.z))) atomicOr(flag, 1u);
    keys[i] = unsigned(localHash(S, cellOf(S, q)));
}

sf_status failWith(sf_status st, const std::string& msg) {
    setGlobalError(msg);
    return st;
}

// Is p still a device address of `device`? After cudaDeviceReset (or any
// teardown of the primary context) the module is loaded again and a cached
// address may be stale; the runtime then no longer knows it as device memory.
bool stillDeviceAddress(const void* p, int device) {
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();  // not sticky: clear it so later checks see only their own errors
        return false;
    }
    return a.type == cudaMemoryTypeDevice && a.device == device;
}

// Device address of the scratch on the current device: looked up on the first
// call on a device and again whenever the cached address went stale.
unsigned int* scratchAddress(int device, std::string& why) {
    static std::mutex mu;
    static unsigned int* addr[kMaxDevices] = {};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= kMaxDevices) {
        why = "device index out of range";
        return nullptr;
    }
    if (addr[device] && !stillDeviceAddress(addr[device], device)) addr[device] = nullptr;
    if (!addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) {
            why = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return nullptr;
        }
        addr[device] = static_cast<unsigned int*>(p);
    }
    return addr[device];
}

}  // namespace

extern "C" sf_status sf_cell_sort_noalloc(const sf_boundary_params* grid, const float* pos_dev, int64_t n,
                                          int32_t* perm_out_dev, int32_t* cell_start_out_dev, void* stream) {
    if (!grid || !cell_start_out_dev || n < 0 || (n > 0 && (!pos_dev || !perm_out_dev)))
        return failWith(SF_ERR_INVALID, "sf_cell_sort_noalloc: null pointer or negative count");
    if (n > kMaxN)
        return failWith(SF_ERR_INVALID, "sf_cell_sort_noalloc: n = " + std::to_string(n) +
                                            " exceeds SF_NOALLOC_MAX_PARTICLES (" + std::to_string(kMaxN) + ")");
    if (!(grid->kernel_radius > 0.f)) return failWith(SF_ERR_INVALID, "sf_cell_sort_noalloc: kernel_radius must be > 0");
    for (int k = 0; k < 3; ++k)
        if (grid->grid_size[k] <= 0) return failWith(SF_ERR_INVALID, "sf_cell_sort_noalloc: grid_size must be positive");
    const int64_t cells = int64_t(grid->grid_size[0]) * grid->grid_size[1] * grid->grid_size[2];
    if (cells > (int64_t(1) << 30)) return failWith(SF_ERR_INVALID, "sf_cell_sort_noalloc: grid above 2^30 cells");
    if (size_t(sortTiles(kMaxN)) * 256 > kHistWords)
        return failWith(SF_ERR_UNSUPPORTED, "sf_cell_sort_noalloc: histogram scratch too small for the sort tiles");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return failWith(SF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    std::string why;
    unsigned int* base = scratchAddress(device, why);
    if (!base) return failWith(SF_ERR_CUDA, "sf_cell_sort_noalloc: " + why);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int ncell = int(cells);
    if (n == 0) {
        e = cudaMemsetAsync(cell_start_out_dev, 0, sizeof(int32_t) * (size_t(ncell) + 1), s);
        return e == cudaSuccess ? SF_OK : failWith(SF_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    }
    unsigned int* flag = base;
    unsigned int* keys = base + kFlagWords;
    SortScratch sc{};
    sc.keysAlt = keys + kMaxN;
    sc.vals = keys + 2 * size_t(kMaxN);
    sc.valsAlt = keys + 3 * size_t(kMaxN);
    sc.digitTotal = keys + 4 * size_t(kMaxN);
    sc.hist = sc.digitTotal + 256;
    sc.tiles = sortTiles(int(n));
    // grid of the sort stage (the cell fields of the scene description)
    SceneDev S{};
    S.lpx = grid->lowest_point[0];
    S.lpy = grid->lowest_point[1];
    S.lpz = grid->lowest_point[2];
    S.cell = grid->kernel_radius;
    S.gx = grid->grid_size[0];
    S.gy = grid->grid_size[1];
    S.gz = grid->grid_size[2];
    S.ncell = ncell;
    int bits = 1;
    while ((int64_t(1) << bits) <= int64_t(ncell)) ++bits;
    if ((e = cudaMemsetAsync(flag, 0, sizeof(unsigned int), s)) != cudaSuccess)
        return failWith(SF_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    kNoAllocKeys<<<int((n + 255) / 256), 256, 0, s>>>(S, pos_dev, int(n), keys, flag);
    unsigned int *sortedKeys = nullptr, *perm = nullptr;
    radixSort(s, int(n), bits, keys, sc, &sortedKeys, &perm);
    launchCellStart(s, int(n), ncell, sortedKeys, reinterpret_cast<unsigned int*>(cell_start_out_dev));
    if ((e = cudaGetLastError()) != cudaSuccess)
        return failWith(SF_ERR_CUDA, std::string("sf_cell_sort_noalloc launch: ") + cudaGetErrorString(e));
    if ((e = cudaMemcpyAsync(perm_out_dev, perm, sizeof(int32_t) * size_t(n), cudaMemcpyDeviceToDevice, s)) !=
        cudaSuccess)
        return failWith(SF_ERR_CUDA, std::string("permutation copy: ") + cudaGetErrorString(e));
    unsigned int flagHost = 0;
    if ((e = cudaMemcpyAsync(&flagHost, flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return failWith(SF_ERR_CUDA, std::string("sf_cell_sort_noalloc sync: ") + cudaGetErrorString(e));
    if (flagHost) return failWith(SF_ERR_DEVICE, "sf_cell_sort_noalloc: non-finite particle position");
    return SF_OK;
}
