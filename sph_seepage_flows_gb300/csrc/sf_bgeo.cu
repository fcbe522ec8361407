// Houdini classic .bgeo point files: the reference's per-frame export
// (ExportBgeoFileCUDA, seepage_flows/include/kiri_utils.h:364-448, through
// the partio library) and its shape import (ReadBgeoFileForGPU /
// ReadMultiBgeoFilesForGPU, kiri_utils.h:252-362).
//
// Layout (version-5 classic bgeo, all words big-endian): int32 magic 'Bgeo',
// char 'V', int32 version 5, eight int32 counts (points, primitives, point
// groups, primitive groups, point attributes but position, vertex, primitive
// and detail attributes); per point attribute: uint16 name length, name,
// uint16 components, int32 type (0 float, 1 int, 4 indexed string, 5 vector)
// and one int32 default per component (an indexed string has its string
// table instead); per point: x, y, z, w = 1 and the attributes' components;
// then the bytes 0x00 0xff. The export writes position, Cd (float 3), pscale
// (float 1) and label (int 1), as the reference does.
//
// The export packs the big-endian point records on the GPU (one 36-byte
// record per particle, staged per block in shared memory and stored as
// 16-byte words), copies them to pinned host memory and writes the file
// with the header in front; the host only adds the header and the two
// trailing bytes.
#include "../../include/sf_capi.h"
#include "sf_kernels.h"

#include <sys/stat.h>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace sfg {

void setGlobalError(const std::string& msg);  // sf_capi.cu: text for sf_last_error_string(NULL)

namespace {

constexpr int kBgeoWords = 9;          // x, y, z, w, Cd r, g, b, pscale, label
constexpr int kPackParticles = 256;    // records per block (9216 bytes, a multiple of 16)

__device__ __forceinline__ unsigned int bigEndian(unsigned int v) { return __byte_perm(v, 0u, 0x0123u); }
__device__ __forceinline__ unsigned int bigEndian(float v) { return bigEndian(__float_as_uint(v)); }

// Writes the block's staged records (cnt particles) to out as 16-byte words.
__device__ __forceinline__ void storeRecords(const uint4* buf4, int p0, int cnt, uint4* __restrict__ out) {
    const int t = threadIdx.x;
    const int words = kBgeoWords * cnt, vec = words / 4, rem = words - 4 * vec;
    uint4* o = out + size_t(p0) * kBgeoWords / 4;  // p0 is a multiple of 256
    for (int q = t; q < vec; q += kPackParticles) o[q] = buf4[q];
    if (t < rem) reinterpret_cast<unsigned int*>(o + vec)[t] = reinterpret_cast<const unsigned int*>(buf4)[4 * vec + t];
}

__device__ __forceinline__ void stageRecord(unsigned int* w, float3 p, float3 c, float r, unsigned int label) {
    w[0] = bigEndian(p.x);
    w[1] = bigEndian(p.y);
    w[2] = bigEndian(p.z);
    w[3] = bigEndian(1.f);
    w[4] = bigEndian(c.x);
    w[5] = bigEndian(c.y);
    w[6] = bigEndian(c.z);
    w[7] = bigEndian(r);
    w[8] = bigEndian(label);
}

// Records of the handle's slots in sorted order: pos4 = (x, y, z, -m for
// sand / m for water), col4 = (colour, max saturation), mat4.w = radius.
__global__ void __launch_bounds__(kPackParticles) kPackBgeo(int n, const float4* __restrict__ pos4,
                                                            const float4* __restrict__ col4,
                                                            const float4* __restrict__ mat4,
                                                            uint4* __restrict__ out) {
    __shared__ uint4 buf4[kPackParticles * kBgeoWords / 4];
    const int t = threadIdx.x, p0 = blockIdx.x * kPackParticles, cnt = min(kPackParticles, n - p0);
    if (t < cnt) {
        const float4 p = pos4[p0 + t], c = col4[p0 + t];
        stageRecord(reinterpret_cast<unsigned int*>(buf4) + kBgeoWords * t, make_float3(p.x, p.y, p.z),
                    make_float3(c.x, c.y, c.z), mat4[p0 + t].w, p.w < 0.f ? unsigned(SF_LABEL_SAND) : 0u);
    }
    __syncthreads();
    storeRecords(buf4, p0, cnt, out);
}

// Records of the reference's export arrays: float3 positions and colours,
// float radii, size_t labels (written as int, as the reference does).
__global__ void __launch_bounds__(kPackParticles) kPackBgeoArrays(int n, const float* __restrict__ pos3,
                                                                  const float* __restrict__ col3,
                                                                  const float* __restrict__ radius,
                                                                  const unsigned long long* __restrict__ label,
                                                                  uint4* __restrict__ out) {
    __shared__ uint4 buf4[kPackParticles * kBgeoWords / 4];
    const int t = threadIdx.x, p0 = blockIdx.x * kPackParticles, cnt = min(kPackParticles, n - p0);
    if (t < cnt) {
        const size_t i = size_t(p0 + t);
        stageRecord(reinterpret_cast<unsigned int*>(buf4) + kBgeoWords * t,
                    make_float3(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]),
                    make_float3(col3[3 * i], col3[3 * i + 1], col3[3 * i + 2]), radius[i],
                    unsigned(label[i]));
    }
    __syncthreads();
    storeRecords(buf4, p0, cnt, out);
}

void putBE32(std::string& s, uint32_t v) {
    for (int k = 3; k >= 0; --k) s.push_back(char((v >> (8 * k)) & 0xffu));
}
void putBE16(std::string& s, uint16_t v) {
    s.push_back(char(v >> 8));
    s.push_back(char(v & 0xffu));
}
uint32_t getBE32(const unsigned char* p) {
    return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | uint32_t(p[3]);
}
uint16_t getBE16(const unsigned char* p) { return uint16_t((uint16_t(p[0]) << 8) | uint16_t(p[1])); }
float beFloat(const unsigned char* p) {
    const uint32_t u = getBE32(p);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

constexpr uint32_t kMagic = (uint32_t('B') << 24) | (uint32_t('g') << 16) | (uint32_t('e') << 8) | uint32_t('o');

// Header of an export of n points (position, Cd, pscale, label).
std::string bgeoHeader(int64_t n) {
    std::string h;
    putBE32(h, kMagic);
    h.push_back('V');
    putBE32(h, 5u);
    const uint32_t counts[8] = {uint32_t(n), 0, 0, 0, 3, 0, 0, 0};
    for (uint32_t c : counts) putBE32(h, c);
    struct Attr {
        const char* name;
        uint16_t count;
        uint32_t type;
    };
    for (const Attr& a : {Attr{"Cd", 3, 0}, Attr{"pscale", 1, 0}, Attr{"label", 1, 1}}) {
        putBE16(h, uint16_t(std::strlen(a.name)));
        h += a.name;
        putBE16(h, a.count);
        putBE32(h, a.type);
        for (int k = 0; k < a.count; ++k) putBE32(h, 0u);
    }
    return h;
}

// mkdir -p (the reference creates a missing export folder).
bool makeDirs(const std::string& path, std::string& err) {
    if (path.empty()) return true;
    std::string cur;
    for (size_t i = 0; i <= path.size(); ++i) {
        if (i < path.size() && path[i] != '/') continue;
        cur = path.substr(0, i);
        if (cur.empty()) continue;
        struct stat st;
        if (stat(cur.c_str(), &st) == 0) {
            if (!S_ISDIR(st.st_mode)) return err = cur + " is not a folder", false;
            continue;
        }
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return err = "mkdir " + cur + ": " + std::strerror(errno), false;
    }
    return true;
}

bool writeBgeo(const std::string& folder, const std::string& name, int64_t n, const void* records,
               std::string& err) {
    if (!makeDirs(folder, err)) return false;
    const std::string path = (folder.empty() ? std::string(".") : folder) + "/" + name + ".bgeo";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return err = "open " + path + ": " + std::strerror(errno), false;
    const std::string head = bgeoHeader(n);
    const char trailer[2] = {0x00, char(0xff)};
    const size_t bytes = size_t(n) * kBgeoWords * 4;
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size() &&
              (bytes == 0 || std::fwrite(records, 1, bytes, f) == bytes) && std::fwrite(trailer, 1, 2, f) == 2;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) err = "write " + path + " failed";
    return ok;
}

}  // namespace

// Pinned host buffer of at least `bytes` (grown by reallocation).
sf_status ensurePinned(void*& p, size_t& have, size_t bytes, std::string& err) {
    if (have >= bytes) return SF_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    have = 0;
    const cudaError_t e = cudaMallocHost(&p, bytes);
    if (e != cudaSuccess) {
        err = std::string("cudaMallocHost export buffer: ") + cudaGetErrorString(e);
        return SF_ERR_CUDA;
    }
    have = bytes;
    return SF_OK;
}

// Packs the records of n slots (handle layout) into dev (device, 36 n bytes,
// 16-byte aligned), copies them into host (pinned) and writes the file.
sf_status exportBgeoSlots(cudaStream_t s, int64_t n, const float4* pos4, const float4* col4, const float4* mat4,
                          void* dev, void* host, const char* folder, const char* name, std::string& err) {
    const size_t bytes = size_t(n) * kBgeoWords * 4;
    if (n > 0) {
        kPackBgeo<<<int((n + kPackParticles - 1) / kPackParticles), kPackParticles, 0, s>>>(
            int(n), pos4, col4, mat4, static_cast<uint4*>(dev));
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            err = std::string("bgeo export: ") + cudaGetErrorString(e);
            return SF_ERR_CUDA;
        }
    }
    return writeBgeo(folder ? folder : "", name, n, host, err) ? SF_OK : SF_ERR_INVALID;
}

}  // namespace sfg

using namespace sfg;

sf_status sf_export_bgeo_device(const char* folder_path, const char* file_name, const float* pos3, const float* col3,
                                const float* radius, const uint64_t* labels, int64_t n, void* stream) {
    if (!file_name || n < 0 || (n > 0 && (!pos3 || !col3 || !radius || !labels)) || n > (int64_t(1) << 30)) {
        setGlobalError("sf_export_bgeo_device: invalid arguments");
        return SF_ERR_INVALID;
    }
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t bytes = size_t(n) * kBgeoWords * 4;
    void* dev = nullptr;
    void* host = nullptr;
    std::string err;
    sf_status st = SF_OK;
    if (n > 0) {
        cudaError_t e = cudaMalloc(&dev, bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&host, bytes);
        if (e == cudaSuccess) {
            kPackBgeoArrays<<<int((n + kPackParticles - 1) / kPackParticles), kPackParticles, 0, s>>>(
                int(n), pos3, col3, radius, reinterpret_cast<const unsigned long long*>(labels),
                static_cast<uint4*>(dev));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            err = std::string("sf_export_bgeo_device: ") + cudaGetErrorString(e);
            st = SF_ERR_CUDA;
        }
    }
    if (st == SF_OK && !writeBgeo(folder_path ? folder_path : "", file_name, n, host, err)) st = SF_ERR_INVALID;
    if (dev) cudaFree(dev);
    if (host) cudaFreeHost(host);
    if (st != SF_OK) setGlobalError(err);
    return st;
}

sf_status sf_read_bgeo(const char* path, int32_t flip_yz, float* xyzs_out, int64_t capacity, int64_t* n_out) {
    auto fail = [](const std::string& msg) {
        setGlobalError("sf_read_bgeo: " + msg);
        return SF_ERR_INVALID;
    };
    if (!path || !n_out) return fail("path and n_out are required");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(std::string("open ") + path + ": " + std::strerror(errno));
    std::vector<unsigned char> d;
    unsigned char chunk[1 << 16];
    for (size_t got; (got = std::fread(chunk, 1, sizeof(chunk), f)) > 0;) d.insert(d.end(), chunk, chunk + got);
    std::fclose(f);
    size_t o = 0;
    auto need = [&](size_t k) { return o + k <= d.size(); };
    if (!need(41) || getBE32(&d[0]) != kMagic || d[4] != 'V' || getBE32(&d[5]) != 5u)
        return fail("not a version-5 classic bgeo file");
    const int64_t n = int32_t(getBE32(&d[9]));
    const int32_t nAttr = int32_t(getBE32(&d[25]));
    if (n < 0 || nAttr < 0) return fail("negative counts");
    o = 41;  // magic, 'V', version and the eight counts
    int width = 4, pscaleAt = -1;
    for (int a = 0; a < nAttr; ++a) {
        if (!need(2)) return fail("truncated attribute table");
        const uint16_t len = getBE16(&d[o]);
        o += 2;
        if (!need(size_t(len) + 6)) return fail("truncated attribute table");
        const std::string name(reinterpret_cast<const char*>(&d[o]), len);
        o += len;
        const uint16_t count = getBE16(&d[o]);
        const uint32_t type = getBE32(&d[o + 2]);
        o += 6;
        if (type == 4) {  // indexed string: its string table follows
            if (!need(4)) return fail("truncated string table");
            const int32_t ns = int32_t(getBE32(&d[o]));
            o += 4;
            for (int32_t k = 0; k < ns; ++k) {
                if (!need(2)) return fail("truncated string table");
                const uint16_t sl = getBE16(&d[o]);
                o += 2;
                if (!need(sl)) return fail("truncated string table");
                o += sl;
            }
        } else if (type == 0 || type == 1 || type == 5) {
            if (!need(size_t(count) * 4)) return fail("truncated attribute defaults");
            o += size_t(count) * 4;
        } else {
            return fail("attribute " + name + " has an unsupported type " + std::to_string(type));
        }
        if (name == "pscale" && type == 0 && count >= 1 && pscaleAt < 0) pscaleAt = width;
        width += count;
    }
    *n_out = n;
    if (!xyzs_out) return SF_OK;
    if (capacity < n) return fail("capacity smaller than the point count");
    if (d.size() - o < size_t(n) * size_t(width) * 4) return fail("truncated point data");
    for (int64_t i = 0; i < n; ++i) {
        const unsigned char* r = &d[o + size_t(i) * size_t(width) * 4];
        const float x = beFloat(r), y = beFloat(r + 4), z = beFloat(r + 8);
        xyzs_out[4 * i] = x;
        xyzs_out[4 * i + 1] = flip_yz ? z : y;
        xyzs_out[4 * i + 2] = flip_yz ? y : z;
        xyzs_out[4 * i + 3] = pscaleAt >= 0 ? beFloat(r + 4 * pscaleAt) : 0.01f;
    }
    return SF_OK;
}
