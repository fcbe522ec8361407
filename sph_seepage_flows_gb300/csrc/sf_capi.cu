// C ABI of the GB300 seepage-flow substep (include/sf_capi.h).
//
// A handle owns all device memory of its scenes (plain cudaMalloc; no
// framework allocator), one CUDA stream and, for fixed-dt runs, captured
// CUDA graphs of two substeps (the persistent arrays ping-pong between two
// buffer sets at every sort, so two substeps return to the same buffers).
#include "../../include/sf_capi.h"
#include "sf_adjoint.h"
#include "sf_device.cuh"
#include "sf_kernels.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

using namespace sfg;

namespace {

constexpr float kPiF = 3.141592653589793238462643383279502884197f;  // KIRI_PI (kiri_pbs_pch.cuh:53)

thread_local std::string g_createError;

struct Bez {
    float py0, py1, px1, py2;
};

// QuadraticBezierCoeff constructor (cuda_sf_utils.cuh:40-55), host float arithmetic.
BezierDev makeBezier(float py0, float py1, float px1, float py2) {
    BezierDev g;
    float a = (px1 + 1.f) / 4.f;
    g.b = -2.f * a;
    g.c = g.b * g.b;
    g.d = -4.f * (1.f + g.b - px1);
    g.e = 2.f * (1.f + g.b - px1);
    g.py0 = py0;
    g.py1 = py1;
    g.px1 = px1;
    g.py2 = py2;
    return g;
}

// Host-side part of the scene description: every constant the reference
// derives from the parameters alone, in the reference's float operations.
SceneDev makeSceneDev(const sf_params& P, const sf_boundary_params& B, const sf_solver_params& Sp) {
    SceneDev S;
    std::memset(&S, 0, sizeof(S));
    S.lpx = B.lowest_point[0];
    S.lpy = B.lowest_point[1];
    S.lpz = B.lowest_point[2];
    S.hpx = B.highest_point[0];
    S.hpy = B.highest_point[1];
    S.hpz = B.highest_point[2];
    S.cell = B.kernel_radius;
    S.gx = B.grid_size[0];
    S.gy = B.grid_size[1];
    S.gz = B.grid_size[2];
    S.ncell = S.gx * S.gy * S.gz;
    const float h = B.kernel_radius;
    // Poly6Kernel / SpikyKernelGrad / AdhesionAkinci13 ctors (cuda_sph_kernel.cuh:82-89,103-108,192-195)
    S.h = h;
    S.h2 = h * h;
    {
        float ih = 1.f / h;
        float ih3 = ih * ih * ih;
        float ih9 = ih3 * ih3 * ih3;
        S.poly6 = 315.f * ih9 / (64.f * kPiF);
        float h2 = h * h;
        float h6 = h2 * h2 * h2;
        S.spiky = -45.f / (kPiF * h6);
        S.adh_coef = 0.007f / powf(h, 3.25f);
        float d = S.h2 - 0.f * 0.f;
        S.W0 = S.poly6 * d * d * d;
    }
    S.rho0 = P.sph_density;
    S.rho1 = P.dem_density;
    S.stiff = P.sph_stiff;
    S.tait = P.solver_type == SF_SOLVER_WCSPH ? 1 : 0;
    S.neg_scale = S.tait ? Sp.negative_scale : 1.f;
    S.nu = P.sph_nu;
    S.bnu = P.sph_bnu;
    S.sph_radius = P.sph_particle_radius;
    S.sph_mass = P.sph_mass;
    const float r = P.dem_particle_radius;
    S.dem_radius = r;
    S.kn = P.dem_young * r;
    S.ks = S.kn * P.dem_poisson;
    S.tan2 = powf(P.dem_tan_friction_angle, 2.f);
    S.damping = P.dem_damping;
    S.rij2 = 2.f * r;
    S.wall_rij = P.sph_particle_radius + r;
    // ComputeDemCapillaryForces constants (cuda_dem_solver_common_gpu.cuh:63-65)
    {
        float contact_angle = 30.f / 180.f * kPiF;
        float vlb = 4.f / 3.f * kPiF * powf(r, 3.f) * 0.01f * 0.01f;
        float s_rupture = (1.f + 0.5f * contact_angle) * (powf(vlb, 1.f / 3.f) + 0.1f * powf(vlb, 2.f / 3.f));
        S.cap_vlb = vlb;
        S.cap_srupt = s_rupture;
        S.cap_vlb_pir = vlb / (kPiF * r);
        S.cap_pir = kPiF * r;
        S.cap_cos = cosf(contact_angle);
        S.cap_sin = sinf(contact_angle);
        S.cap_m2pi = -2.f * kPiF;
        double demReach = double(2.f * r) + double(s_rupture);
        double reach = std::max(double(h), demReach);
        S.reach2 = float(reach * reach * (1.0 + 1e-5));
        S.dem_reach2 = float(demReach * demReach * (1.0 + 1e-5));
    }
    S.capG = makeBezier(P.sf_c0, P.sf_cmc, P.sf_cmc_p, P.sf_csat);
    S.multi = P.sf_type == SF_TYPE_MULTI_SF ? 1 : 0;
    S.adhG = S.multi ? makeBezier(0.f, 1.5f, 0.5f, 0.8f) : makeBezier(P.sf_a0, P.sf_amc, P.sf_amc_p, P.sf_asat);
    S.cd = P.sf_cd;
    S.grav_abs = std::fabs(P.gravity[1]);
    S.gvx = P.gravity[0];
    S.gvy = P.gravity[1];
    S.gvz = P.gravity[2];
    for (int k = 0; k < 3; ++k) {
        S.dry[k] = P.sf_dry_sand_color[k];
        S.wet[k] = P.sf_wet_sand_color[k];
    }
    // ComputeSubTimeStepsByCFL (cuda_wcsph_sf_solver.cu:43-56)
    S.cfl_by_speed = 0.4f * h / Sp.speed_of_sound;
    S.cfl_hm = h * P.sph_mass;
    S.cfl_mass = P.sph_mass;
    S.cfl_scale = Sp.time_step_limit_scale;
    S.adj_seed_scale = 1.f;
    S.params_dt = P.dt;
    S.wcsph = S.tait;
    return S;
}

// Pos2GridHash on the host (helper_thrust.cuh:66-89), same float arithmetic.
int hostHash(const SceneDev& S, float x, float y, float z) {
    auto axis = [](float rel, float cell, int g) {
        float q = rel / cell;
        int v;
        if (!(q == q)) v = 0;
        else if (q >= 2147483520.f) v = 2147483647;
        else if (q <= -2147483648.f) v = INT32_MIN;
        else v = int(q);
        return std::min(std::max(v, 0), g - 1);
    };
    int cx = axis(x - S.lpx, S.cell, S.gx), cy = axis(y - S.lpy, S.cell, S.gy), cz = axis(z - S.lpz, S.cell, S.gz);
    return cx * S.gy * S.gz + cy * S.gz + cz;
}

template <typename T> void devFree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    float dt = 0.f;
    int nodes = 0;
};

}  // namespace

namespace sfg {
// Error text of handle-less entry points (sf_last_error_string(NULL)).
void setGlobalError(const std::string& msg) { g_createError = msg; }

// sf_bgeo.cu: pinned host buffers and the .bgeo export of slots in the handle layout
sf_status ensurePinned(void*& p, size_t& have, size_t bytes, std::string& err);
sf_status exportBgeoSlots(cudaStream_t s, int64_t n, const float4* pos4, const float4* col4, const float4* mat4,
                          void* dev, void* host, const char* folder, const char* name, std::string& err);
}  // namespace sfg

struct sf_handle {
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    int device = 0;
    int nScenes = 0;
    std::vector<sf_params> P;
    std::vector<sf_boundary_params> B;
    std::vector<sf_solver_params> Sp;
    std::vector<SceneDev> hScenes;
    std::vector<int64_t> n, capUser, nextId;
    int totalSlots = 0, totalCells = 0, totalB = 0, sortBits = 1, slotBlocks = 0;
    SceneDev* dScenes = nullptr;
    int* dBlockScene = nullptr;
    SceneState* dState = nullptr;
    unsigned int* dErr = nullptr;
    // persistent per-slot arrays, two buffer sets
    float4* pos[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    float4* col[2] = {nullptr, nullptr};
    float4* mat[2] = {nullptr, nullptr};
    float2* amc[2] = {nullptr, nullptr};
    int* pid[2] = {nullptr, nullptr};
    int cur = 0;
    // per-substep arrays
    float4 *aux = nullptr, *flow = nullptr, *adh = nullptr, *avgadh = nullptr, *drag = nullptr, *acc = nullptr;
    float2* dp = nullptr;
    float2* vrec2 = nullptr;  // gather records, rewritten every substep
    float4* grec4 = nullptr;
    unsigned int *keys = nullptr, *cs = nullptr, *bcs = nullptr;
    unsigned char* bnear = nullptr;  // per cell: a boundary particle within the 27 cells
    unsigned int* nbrCnt = nullptr;
    int* bnbrCnt = nullptr;
    int* cnbrCnt = nullptr;
    unsigned int* cnbr = nullptr;
    unsigned int *nbr = nullptr, *bnbr = nullptr;
    unsigned int* sortedKeys = nullptr;  // points into keys/scratch after a sort
    SortScratch sc{};
    float4* bpos = nullptr;
    int* blabel = nullptr;
    // staging for field access
    void* stage = nullptr;
    size_t stageBytes = 0;
    // pinned host buffer of the .bgeo export
    void* exportHost = nullptr;
    size_t exportHostBytes = 0;
    bool sorted = false;
    int64_t launches = 0;
    GraphCache graph[2];   // two-substep graphs, by starting buffer set
    GraphCache graph1[2];  // one-substep graphs, by starting buffer set
    // sf_step's adaptive substep, by starting buffer set: the integrator reads
    // the render interval from dTimeArg, written before each replay
    GraphCache graphStep[2];
    float* dTimeArg = nullptr;
    bool captureStep = false;  // runStage passes dTimeArg to the integrator while capturing graphStep
    int nbrCap = kMinNbr;                 // particle neighbour list capacity (per slot)
    // list growth: copies of the scene states queued behind the substeps and
    // read once they have landed (pinned, n_scenes each; two in flight at most)
    SceneState* stateHost[2] = {nullptr, nullptr};
    cudaEvent_t stateEvent[2] = {nullptr, nullptr};
    bool statePending[2] = {false, false};
    int64_t listGrowths = 0;
    int block[kTunedPasses] = {kSlotAlign, kSlotAlign, kSlotAlign, kSlotAlign, kSlotAlign, kSlotAlign};
    int lanes = 1;  // threads per slot of the momentum passes and the adjoint pair kernels
    int densityStaged = 0;  // the one-lane density pass stages its candidates in shared memory (tuned)
    unsigned int* dProbe = nullptr;       // neighbour-count probe word
    // reverse-mode buffers, allocated by the first sf_adjoint_run
    AdjBuffers adj{};
    float* adjTarget = nullptr;   // 3 floats per slot, indexed by slot_off + id
    float* adjParam = nullptr;    // 3 per block of the adjoint pair kernels (lanes per slot block)
    // captured store-mode substeps of the adjoint, per buffer set and stored
    // substep slot, for the slab buffer they were captured with
    std::vector<GraphCache> storeGraph[2];
    // captured reverse substeps, per stored substep slot
    std::vector<GraphCache> adjGraph;
    char* storeGraphSlab = nullptr;
    float2* adjLoss = nullptr;    // 1 per slot block
    char* snap = nullptr;         // state snapshots for checkpointing
    size_t snapBytes = 0;
    char* slab = nullptr;         // stored substeps of one checkpoint segment
    size_t slabBytes = 0;
    std::string err;

    sf_status fail(sf_status st, const std::string& msg) {
        err = msg;
        return st;
    }
    sf_status cuda(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return SF_OK;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return SF_ERR_CUDA;
    }
    int adjBlocks() const { return slotBlocks * lanes; }
    static constexpr int kMaxLanes = 8;
    LaunchCtx ctx() const {
        LaunchCtx c;
        c.stream = stream;
        c.scenes = dScenes;
        c.blockScene = dBlockScene;
        c.state = dState;
        c.errWord = dErr;
        c.slotBlocks = slotBlocks;
        for (int k = 0; k < kTunedPasses; ++k) c.block[k] = block[k];
        c.lanes = lanes;
        c.densityStaged = densityStaged;
        return c;
    }
    PassBuffers buffers() const {
        PassBuffers b;
        b.listsW.cnt = nbrCnt;
        b.listsW.nbr = nbr;
        b.listsW.bcnt = bnbrCnt;
        b.listsW.bnbr = bnbr;
        b.listsW.ccnt = cnbrCnt;
        b.listsW.cnbr = cnbr;
        b.listsW.cs = cs;
        b.listsW.bcs = bcs;
        b.listsW.bnear = bnear;
        b.listsW.M = totalSlots;
        b.listsW.cap = nbrCap;
        b.lists.cnt = nbrCnt;
        b.lists.nbr = nbr;
        b.lists.bcnt = bnbrCnt;
        b.lists.bnbr = bnbr;
        b.lists.ccnt = cnbrCnt;
        b.lists.cnbr = cnbr;
        b.lists.cs = cs;
        b.lists.bcs = bcs;
        b.lists.bnear = bnear;
        b.lists.M = totalSlots;
        b.lists.cap = nbrCap;
        b.pos4 = pos[cur];
        b.vel4 = vel[cur];
        b.aux4 = aux;
        b.flow4 = flow;
        b.adh4 = adh;
        b.avgadh4 = avgadh;
        b.drag4 = drag;
        b.acc4 = acc;
        b.col4 = col[cur];
        b.mat4 = mat[cur];
        b.bpos4 = bpos;
        b.dp = dp;
        b.vrec2 = vrec2;
        b.grec4 = grec4;
        return b;
    }
    // Drop the captured substep graphs (after a change of buffers or launch shapes).
    void dropGraphs() {
        for (auto& g : graphStep) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            g.dt = 0.f;
            g.nodes = 0;
        }
        for (auto& g : graph1) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            g.dt = 0.f;
            g.nodes = 0;
        }
        for (auto& g : graph) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            g.dt = 0.f;
            g.nodes = 0;
        }
        for (auto& v : storeGraph) {
            for (auto& g : v)
                if (g.exec) cudaGraphExecDestroy(g.exec);
            v.clear();
        }
        for (auto& g : adjGraph)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        adjGraph.clear();
        storeGraphSlab = nullptr;
    }
    ~sf_handle() {
        for (auto& g : graph)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (auto& g : graph1)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (auto& g : graphStep)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        devFree(dTimeArg);
        devFree(dProbe);
        for (int k = 0; k < 2; ++k) {
            if (stateHost[k]) cudaFreeHost(stateHost[k]);
            if (stateEvent[k]) cudaEventDestroy(stateEvent[k]);
        }
        for (int k = 0; k < 2; ++k) {
            devFree(pos[k]);
            devFree(vel[k]);
            devFree(col[k]);
            devFree(mat[k]);
            devFree(amc[k]);
            devFree(pid[k]);
        }
        devFree(aux);
        devFree(flow);
        devFree(adh);
        devFree(avgadh);
        devFree(drag);
        devFree(acc);
        devFree(dp);
        devFree(vrec2);
        devFree(grec4);
        devFree(keys);
        devFree(nbrCnt);
        devFree(bnbrCnt);
        devFree(nbr);
        devFree(bnbr);
        devFree(cnbrCnt);
        devFree(cnbr);
        devFree(cs);
        devFree(bcs);
        devFree(bnear);
        devFree(sc.keysAlt);
        devFree(sc.vals);
        devFree(sc.valsAlt);
        devFree(sc.hist);
        devFree(sc.digitTotal);
        devFree(bpos);
        devFree(blabel);
        devFree(dScenes);
        devFree(dBlockScene);
        devFree(dState);
        devFree(dErr);
        for (float4** p : {&adj.adjX, &adj.adjV, &adj.x, &adj.v, &adj.acc, &adj.flow, &adj.adh, &adj.avgadh,
                           &adj.drag, &adj.f, &adj.r, &adj.s})
            devFree(*p);
        devFree(adjTarget);
        devFree(adjParam);
        devFree(adjLoss);
        devFree(snap);
        devFree(slab);
        if (stage) cudaFree(stage);
        if (exportHost) cudaFreeHost(exportHost);
        if (ownStream && stream) cudaStreamDestroy(stream);
    }
};

namespace {

// The sort stage: keys (with the first radix pass's tile histograms), stable
// radix sort, reorder into the other buffer set (with the cell table).
sf_status runSort(sf_handle* h) {
    LaunchCtx c = h->ctx();
    launchKeysHist(c, h->totalSlots, h->pos[h->cur], h->keys, h->sc);
    unsigned int* perm = nullptr;
    int l = radixSort(h->stream, h->totalSlots, h->sortBits, h->keys, h->sc, &h->sortedKeys, &perm, true);
    const int o = h->cur, t = 1 - h->cur;
    launchReorder(h->stream, h->totalSlots, perm, h->pos[o], h->vel[o], h->col[o], h->mat[o], h->amc[o], h->pid[o],
                  h->pos[t], h->vel[t], h->col[t], h->mat[t], h->amc[t], h->pid[t], h->sortedKeys, h->totalCells,
                  h->cs);
    h->cur = t;
    h->sorted = true;
    h->launches += 2 + l;
    return h->cuda(cudaGetLastError(), "sort stage launch");
}

sf_status runStage(sf_handle* h, int stage, float timeArg, int adaptive) {
    LaunchCtx c = h->ctx();
    PassBuffers b = h->buffers();
    switch (stage) {
    case SF_STAGE_SORT: return runSort(h);
    case SF_STAGE_DENSITY: launchDensity(c, b); break;
    case SF_STAGE_AVGFLOW: launchAvgFlow(c, b); break;
    case SF_STAGE_VOIDAGE_ADHESION: launchVoidageAdhesion(c, b); break;
    case SF_STAGE_SAND_MOMENTUM: launchSandMomentum(c, b); break;
    case SF_STAGE_WATER_MOMENTUM: launchWaterMomentum(c, b); break;
    case SF_STAGE_INTEGRATE: launchIntegrate(c, b, timeArg, adaptive, h->captureStep ? h->dTimeArg : nullptr); break;
    default: return h->fail(SF_ERR_INVALID, "unknown stage");
    }
    h->launches += 1;
    return h->cuda(cudaGetLastError(), "stage launch");
}

sf_status runSubstep(sf_handle* h, float timeArg, int adaptive) {
    for (int s = 0; s < SF_STAGE_COUNT; ++s) {
        sf_status st = runStage(h, s, timeArg, adaptive);
        if (st != SF_OK) return st;
    }
    return SF_OK;
}

// List capacity for a largest neighbour count: 25% + 8 headroom, a multiple
// of 32 in [kMinNbr, kMaxNbr].
int capacityFor(unsigned maxCount) {
    const int want = int(maxCount + maxCount / 4u + 8u);
    return std::min(kMaxNbr, std::max(kMinNbr, (want + 31) / 32 * 32));
}

// Largest neighbour count of the current state: a sort into the other buffer
// set, the count kernel, then the buffer set and the "not sorted" flag are
// put back (the state itself is unchanged).
sf_status countNeighborsMax(sf_handle* h, unsigned* maxCount) {
    const int cur = h->cur;
    const bool sorted = h->sorted;
    sf_status st = runSort(h);
    if (st) return st;
    if (h->cuda(cudaMemsetAsync(h->dProbe, 0, sizeof(unsigned), h->stream), "probe clear")) return SF_ERR_CUDA;
    launchNeighborCountMax(h->ctx(), h->pos[h->cur], h->cs, h->dProbe);
    h->launches += 1;
    if (h->cuda(cudaMemcpyAsync(maxCount, h->dProbe, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream),
                "probe read") ||
        h->cuda(cudaStreamSynchronize(h->stream), "probe sync"))
        return SF_ERR_CUDA;
    if (!sorted) {
        h->cur = cur;
        h->sorted = false;
    }
    return SF_OK;
}

// Re-allocates the particle lists with `cap` entries per slot. The captured
// graphs hold the old lists and are dropped; the scenes' overflow records
// and the state copies in flight describe the old capacity and are cleared.
sf_status resizeLists(sf_handle* h, int cap) {
    if (h->nbr && h->cuda(cudaStreamSynchronize(h->stream), "sync before list realloc")) return SF_ERR_CUDA;
    devFree(h->nbr);
    if (h->cuda(cudaMalloc(reinterpret_cast<void**>(&h->nbr), sizeof(unsigned) * size_t(h->totalSlots) * cap),
                "cudaMalloc neighbour lists") ||
        h->cuda(cudaMemsetAsync(h->nbr, 0, sizeof(unsigned) * size_t(h->totalSlots) * cap, h->stream),
                "cudaMemset neighbour lists"))
        return SF_ERR_CUDA;
    for (int s = 0; s < h->nScenes; ++s)
        if (h->cuda(cudaMemsetAsync(&h->dState[s].list_need, 0, sizeof(unsigned), h->stream), "clear list_need"))
            return SF_ERR_CUDA;
    h->statePending[0] = h->statePending[1] = false;
    h->nbrCap = cap;
    h->dropGraphs();
    return SF_OK;
}

// (Re)allocates the particle lists for the capacity the current state needs.
sf_status probeListCapacity(sf_handle* h) {
    unsigned mx = 0;
    sf_status st = countNeighborsMax(h, &mx);
    if (st) return st;
    const int cap = capacityFor(mx);
    if (h->nbr && cap == h->nbrCap) return SF_OK;
    return resizeLists(h, cap);
}

// Queues a copy of the scene states behind the work queued so far, into a
// free copy slot; returns the slot, or -1 when both copies are still in flight.
int queueStateCopy(sf_handle* h) {
    for (int k = 0; k < 2; ++k) {
        if (h->statePending[k]) continue;
        if (cudaMemcpyAsync(h->stateHost[k], h->dState, sizeof(SceneState) * size_t(h->nScenes),
                            cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaEventRecord(h->stateEvent[k], h->stream) != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        h->statePending[k] = true;
        return k;
    }
    return -1;
}

// Reads the state copies that have landed (waiting for copy slot `waitSlot`,
// if >= 0) and grows the particle lists when a density pass found a list
// more than 7/8 full: the new capacity holds the largest count reported plus
// the usual headroom (at most kMaxNbr). Particles whose list overflowed in
// the substeps in between walked the stencil, which gives the same results
// more slowly.
sf_status growListsIfFull(sf_handle* h, int waitSlot) {
    unsigned need = 0;
    for (int k = 0; k < 2; ++k) {
        if (!h->statePending[k]) continue;
        const cudaError_t e = k == waitSlot ? cudaEventSynchronize(h->stateEvent[k]) : cudaEventQuery(h->stateEvent[k]);
        if (e == cudaErrorNotReady) continue;
        if (h->cuda(e, "state copy")) return SF_ERR_CUDA;
        h->statePending[k] = false;
        for (int s = 0; s < h->nScenes; ++s) need = std::max(need, h->stateHost[k][s].list_need);
    }
    if (need == 0 || capacityFor(need) <= h->nbrCap) return SF_OK;
    ++h->listGrowths;
    return resizeLists(h, capacityFor(need));
}

bool validScene(const sf_params* p, const sf_boundary_params* b, const sf_scene_init* in, int64_t cap,
                std::string& why) {
    if (!p || !b || !in) return why = "null params or init", false;
    if (in->n < 0 || in->nb < 0) return why = "negative particle count", false;
    if (cap < in->n) return why = "capacity smaller than the particle count", false;
    if (cap > (int64_t(1) << 30)) return why = "capacity above 2^30 slots", false;
    if (in->n > 0 && (!in->pos || !in->col || !in->label || !in->mass || !in->radius))
        return why = "missing per-particle input array", false;
    if (in->nb > 0 && !in->bpos) return why = "missing boundary positions", false;
    if (!(b->kernel_radius > 0.f)) return why = "kernel_radius must be > 0", false;
    for (int k = 0; k < 3; ++k)
        if (b->grid_size[k] <= 0) return why = "grid_size must be positive", false;
    if (int64_t(b->grid_size[0]) * b->grid_size[1] * b->grid_size[2] > (int64_t(1) << 30))
        return why = "grid above 2^30 cells", false;
    if (p->solver_type != SF_SOLVER_SPH && p->solver_type != SF_SOLVER_WCSPH) return why = "bad solver_type", false;
    if (p->sf_type != SF_TYPE_SF && p->sf_type != SF_TYPE_MULTI_SF) return why = "bad sf_type", false;
    for (int64_t i = 0; i < in->n; ++i) {
        if (in->label[i] != SF_LABEL_WATER && in->label[i] != SF_LABEL_SAND)
            return why = "labels must be 0 (water) or 1 (sand)", false;
        if (!(in->mass[i] > 0.f) || !std::isfinite(in->mass[i])) return why = "masses must be finite and > 0", false;
    }
    return true;
}

}  // namespace

extern "C" {

const char* sf_version(void) { return "sph_seepage_flows_gb300 0.1.0 (sm_103a)"; }
int32_t sf_capi_version(void) { return SF_CAPI_VERSION; }

int32_t sf_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

sf_status sf_create(const sf_params* params, const sf_boundary_params* bparams, const sf_solver_params* sparams,
                    const sf_scene_init* init, int64_t capacity, void* stream, sf_handle** out) {
    return sf_create_batched(1, params, bparams, sparams, init, &capacity, stream, out);
}

sf_status sf_create_batched(int32_t n_scenes, const sf_params* params, const sf_boundary_params* bparams,
                            const sf_solver_params* sparams, const sf_scene_init* inits, const int64_t* capacities,
                            void* stream, sf_handle** out) {
    if (!out) return SF_ERR_INVALID;
    *out = nullptr;
    if (n_scenes <= 0 || !params || !bparams || !sparams || !inits || !capacities) {
        g_createError = "invalid arguments";
        return SF_ERR_INVALID;
    }
    for (int s = 0; s < n_scenes; ++s) {
        std::string why;
        if (!validScene(&params[s], &bparams[s], &inits[s], capacities[s], why)) {
            g_createError = "scene " + std::to_string(s) + ": " + why;
            return SF_ERR_INVALID;
        }
    }
    if (sf_device_count() <= 0) {
        g_createError = "no CUDA device visible";
        return SF_ERR_NO_DEVICE;
    }
    sf_handle* h = new (std::nothrow) sf_handle();
    if (!h) return SF_ERR_INVALID;
    auto bail = [&](sf_status st) {
        g_createError = h->err;
        delete h;
        return st;
    };
    cudaGetDevice(&h->device);
    if (stream) {
        h->stream = static_cast<cudaStream_t>(stream);
    } else {
        if (h->cuda(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate"))
            return bail(SF_ERR_CUDA);
        h->ownStream = true;
    }
    h->nScenes = n_scenes;
    h->P.assign(params, params + n_scenes);
    h->B.assign(bparams, bparams + n_scenes);
    h->Sp.assign(sparams, sparams + n_scenes);
    h->n.resize(n_scenes);
    h->capUser.resize(n_scenes);
    h->nextId.resize(n_scenes);
    std::vector<int> blockScene;
    int slotOff = 0, cellOff = 0, bOff = 0;
    for (int s = 0; s < n_scenes; ++s) {
        SceneDev S = makeSceneDev(params[s], bparams[s], sparams[s]);
        const int64_t cap = std::max<int64_t>(capacities[s], 1);
        const int slots = int((cap + kSlotAlign - 1) / kSlotAlign) * kSlotAlign;
        S.slot_off = slotOff;
        S.slot_cap = slots;
        S.cell_off = cellOff;
        S.b_off = bOff;
        S.nb = int(inits[s].nb);
        h->hScenes.push_back(S);
        for (int k = 0; k < slots / kSlotAlign; ++k) blockScene.push_back(s);
        slotOff += slots;
        cellOff += S.ncell + 1;
        bOff += S.nb;
        h->n[s] = inits[s].n;
        h->capUser[s] = capacities[s];
        h->nextId[s] = inits[s].n;
    }
    h->totalSlots = slotOff;
    h->totalCells = cellOff;
    h->totalB = bOff;
    h->slotBlocks = slotOff / kSlotAlign;
    h->sortBits = 1;
    while ((int64_t(1) << h->sortBits) <= int64_t(h->totalCells)) ++h->sortBits;
    const size_t M = size_t(h->totalSlots);
    const size_t F4 = sizeof(float4) * M;
#define SF_ALLOC(ptr, bytes)                                                             \
    if (h->cuda(cudaMalloc(reinterpret_cast<void**>(&(ptr)), (bytes)), "cudaMalloc " #ptr)) \
        return bail(SF_ERR_CUDA);                                                        \
    if (h->cuda(cudaMemsetAsync((ptr), 0, (bytes), h->stream), "cudaMemset " #ptr)) return bail(SF_ERR_CUDA);
    for (int k = 0; k < 2; ++k) {
        SF_ALLOC(h->pos[k], F4);
        SF_ALLOC(h->vel[k], F4);
        SF_ALLOC(h->col[k], F4);
        SF_ALLOC(h->mat[k], F4);
        SF_ALLOC(h->amc[k], sizeof(float2) * M);
        SF_ALLOC(h->pid[k], sizeof(int) * M);
    }
    SF_ALLOC(h->aux, F4);
    SF_ALLOC(h->flow, F4);
    SF_ALLOC(h->adh, F4);
    SF_ALLOC(h->avgadh, F4);
    SF_ALLOC(h->drag, F4);
    SF_ALLOC(h->acc, F4);
    SF_ALLOC(h->dp, sizeof(float2) * M);
    SF_ALLOC(h->vrec2, sizeof(float2) * M);
    SF_ALLOC(h->grec4, sizeof(float4) * M);
    SF_ALLOC(h->keys, sizeof(unsigned) * M);
    SF_ALLOC(h->nbrCnt, sizeof(unsigned) * M);
    SF_ALLOC(h->bnbrCnt, sizeof(int) * M);
    SF_ALLOC(h->bnbr, sizeof(unsigned) * M * kMaxBNbr);
    SF_ALLOC(h->cnbrCnt, sizeof(int) * M);
    SF_ALLOC(h->cnbr, sizeof(unsigned) * M * kMaxContact);
    SF_ALLOC(h->sc.keysAlt, sizeof(unsigned) * M);
    SF_ALLOC(h->sc.vals, sizeof(unsigned) * M);
    SF_ALLOC(h->sc.valsAlt, sizeof(unsigned) * M);
    {
        int dev = 0, sms = 0;
        if (h->cuda(cudaGetDevice(&dev), "cudaGetDevice") ||
            h->cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))
            return bail(SF_ERR_CUDA);
        h->sc.items = sortItemsFor(h->totalSlots, sms);
        h->lanes = lanesForSlots(h->totalSlots, sms);
    }
    h->sc.tiles = sortTiles(h->totalSlots, h->sc.items);
    // digits of 8 bits, or 9-11 when that saves a pass; room for the widest
    // digits and the smallest tiles, so that the tuner can change both
    h->sc.digitBits = sortDigitBits(h->sortBits);
    const int maxRadix = 1 << std::max(8, h->sc.digitBits);
    SF_ALLOC(h->sc.hist, sizeof(unsigned) * size_t(maxRadix) * size_t(sortTiles(h->totalSlots, 1)));
    SF_ALLOC(h->sc.digitTotal, sizeof(unsigned) * size_t(maxRadix));
    SF_ALLOC(h->cs, sizeof(unsigned) * (size_t(h->totalCells) + 1));
    SF_ALLOC(h->bcs, sizeof(unsigned) * (size_t(h->totalCells) + 1));
    SF_ALLOC(h->bnear, std::max<size_t>(1, size_t(h->totalCells)));
    SF_ALLOC(h->bpos, sizeof(float4) * std::max<size_t>(1, size_t(h->totalB)));
    SF_ALLOC(h->blabel, sizeof(int) * std::max<size_t>(1, size_t(h->totalB)));
    SF_ALLOC(h->dScenes, sizeof(SceneDev) * n_scenes);
    SF_ALLOC(h->dBlockScene, sizeof(int) * blockScene.size());
    SF_ALLOC(h->dState, sizeof(SceneState) * n_scenes);
    SF_ALLOC(h->dErr, sizeof(unsigned));
    SF_ALLOC(h->dProbe, sizeof(unsigned));
    SF_ALLOC(h->dTimeArg, sizeof(float));
#undef SF_ALLOC
    for (int k = 0; k < 2; ++k)
        if (h->cuda(cudaMallocHost(reinterpret_cast<void**>(&h->stateHost[k]), sizeof(SceneState) * n_scenes),
                    "cudaMallocHost state copy") ||
            h->cuda(cudaEventCreateWithFlags(&h->stateEvent[k], cudaEventDisableTiming), "state copy event"))
            return bail(SF_ERR_CUDA);
    // host staging of the initial state
    std::vector<float4> hpos(M, make_float4(0, 0, 0, 0)), hvel(M, make_float4(0, 0, 0, 0)),
        hcol(M, make_float4(0, 0, 0, 0)), hmat(M, make_float4(0, 0, 0, 0));
    std::vector<float2> hamc(M, make_float2(0, 0));
    std::vector<int> hpid(M, -1);
    std::vector<float4> hbpos(std::max(1, h->totalB), make_float4(0, 0, 0, 0));
    std::vector<int> hblabel(std::max(1, h->totalB), 0);
    std::vector<unsigned> hbcs(size_t(h->totalCells) + 1, 0);
    std::vector<unsigned char> hbnear(std::max<size_t>(1, size_t(h->totalCells)), 0);
    std::vector<SceneState> hstate(n_scenes);
    for (int s = 0; s < n_scenes; ++s) {
        const sf_scene_init& in = inits[s];
        const SceneDev& S = h->hScenes[s];
        for (int64_t i = 0; i < in.n; ++i) {
            const size_t k = size_t(S.slot_off + i);
            const float m = in.mass[i];
            hpos[k] = make_float4(in.pos[3 * i], in.pos[3 * i + 1], in.pos[3 * i + 2],
                                  in.label[i] == SF_LABEL_SAND ? -m : m);
            if (in.vel) hvel[k] = make_float4(in.vel[3 * i], in.vel[3 * i + 1], in.vel[3 * i + 2], 0.f);
            hcol[k] = make_float4(in.col[3 * i], in.col[3 * i + 1], in.col[3 * i + 2], 0.f);
            float4 mt = make_float4(0.f, 0.f, 0.f, in.radius[i]);
            if (in.cda0asat) {
                mt.x = in.cda0asat[3 * i];
                mt.y = in.cda0asat[3 * i + 1];
                mt.z = in.cda0asat[3 * i + 2];
            }
            hmat[k] = mt;
            if (in.amcamcp) hamc[k] = make_float2(in.amcamcp[2 * i], in.amcamcp[2 * i + 1]);
            hpid[k] = int(i);
        }
        // boundary searcher: stable sort by cell + cell table (cuda_neighbor_searcher.cu:36-51,125-139)
        std::vector<int> bk(static_cast<size_t>(in.nb));
        for (int64_t i = 0; i < in.nb; ++i) bk[i] = hostHash(S, in.bpos[3 * i], in.bpos[3 * i + 1], in.bpos[3 * i + 2]);
        std::vector<int64_t> order(static_cast<size_t>(in.nb));
        for (int64_t i = 0; i < in.nb; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return bk[a] < bk[b]; });
        std::vector<unsigned> cnt(static_cast<size_t>(S.ncell) + 1, 0u);
        for (int64_t i = 0; i < in.nb; ++i) cnt[bk[i]]++;
        unsigned run = unsigned(S.b_off);
        for (int c = 0; c <= S.ncell; ++c) {
            hbcs[size_t(S.cell_off + c)] = run;
            run += cnt[c];
        }
        // cells with a boundary particle in their 27-cell stencil: the density
        // pass walks the boundary ranges only there
        for (int c = 0; c < S.ncell; ++c) {
            if (!cnt[c]) continue;
            const int cx = c / (S.gy * S.gz), cy = (c / S.gz) % S.gy, cz = c % S.gz;
            for (int x = std::max(cx - 1, 0); x <= std::min(cx + 1, S.gx - 1); ++x)
                for (int y = std::max(cy - 1, 0); y <= std::min(cy + 1, S.gy - 1); ++y)
                    for (int z = std::max(cz - 1, 0); z <= std::min(cz + 1, S.gz - 1); ++z)
                        hbnear[size_t(S.cell_off + (x * S.gy + y) * S.gz + z)] = 1;
        }
        for (int64_t i = 0; i < in.nb; ++i) {
            const int64_t o = order[i];
            hbpos[size_t(S.b_off + i)] = make_float4(in.bpos[3 * o], in.bpos[3 * o + 1], in.bpos[3 * o + 2], 0.f);
            hblabel[size_t(S.b_off + i)] = in.blabel ? in.blabel[o] : 0;
        }
        hstate[s].n = int(in.n);
        hstate[s].n_sub = 1;
        for (int64_t i = 0; i < in.nb; ++i)
            if (in.blabel && in.blabel[i] == 1) h->hScenes[s].shape_boundary = 1;
    }
    hbcs[size_t(h->totalCells)] = unsigned(h->totalB);
    auto up = [&](void* d, const void* src, size_t bytes, const char* what) {
        return h->cuda(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, h->stream), what);
    };
    if (up(h->pos[0], hpos.data(), F4, "upload pos") || up(h->vel[0], hvel.data(), F4, "upload vel") ||
        up(h->col[0], hcol.data(), F4, "upload col") || up(h->mat[0], hmat.data(), F4, "upload mat") ||
        up(h->amc[0], hamc.data(), sizeof(float2) * M, "upload amc") ||
        up(h->pid[0], hpid.data(), sizeof(int) * M, "upload pid") ||
        up(h->bpos, hbpos.data(), sizeof(float4) * hbpos.size(), "upload bpos") ||
        up(h->blabel, hblabel.data(), sizeof(int) * hblabel.size(), "upload blabel") ||
        up(h->bcs, hbcs.data(), sizeof(unsigned) * hbcs.size(), "upload bcs") ||
        up(h->bnear, hbnear.data(), hbnear.size(), "upload bnear") ||
        up(h->dScenes, h->hScenes.data(), sizeof(SceneDev) * n_scenes, "upload scenes") ||
        up(h->dBlockScene, blockScene.data(), sizeof(int) * blockScene.size(), "upload blockScene") ||
        up(h->dState, hstate.data(), sizeof(SceneState) * n_scenes, "upload state"))
        return bail(SF_ERR_CUDA);
    // Akinci boundary volume (cuda_sf_system.cu:121-136)
    LaunchCtx c = h->ctx();
    for (int s = 0; s < n_scenes; ++s) {
        launchBoundaryVolume(c, s, h->hScenes[s].nb, h->bpos, h->blabel, h->bcs);
        h->launches += h->hScenes[s].nb > 0 ? 1 : 0;
    }
    if (h->cuda(cudaGetLastError(), "boundary volume") || h->cuda(cudaStreamSynchronize(h->stream), "create sync"))
        return bail(SF_ERR_CUDA);
    // neighbour list capacity from the initial neighbour counts
    if (probeListCapacity(h) != SF_OK) return bail(SF_ERR_CUDA);
    *out = h;
    return SF_OK;
}

sf_status sf_destroy(sf_handle* h) {
    if (!h) return SF_ERR_INVALID;
    cudaStreamSynchronize(h->stream);
    delete h;
    return SF_OK;
}

sf_status sf_set_params(sf_handle* h, int32_t scene, const sf_params* p) {
    if (!h || !p || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    if (p->solver_type != SF_SOLVER_SPH && p->solver_type != SF_SOLVER_WCSPH)
        return h->fail(SF_ERR_INVALID, "bad solver_type");
    if (p->sf_type != SF_TYPE_SF && p->sf_type != SF_TYPE_MULTI_SF) return h->fail(SF_ERR_INVALID, "bad sf_type");
    h->P[scene] = *p;
    SceneDev S = makeSceneDev(*p, h->B[scene], h->Sp[scene]);
    const SceneDev& old = h->hScenes[scene];
    S.slot_off = old.slot_off;
    S.slot_cap = old.slot_cap;
    S.cell_off = old.cell_off;
    S.b_off = old.b_off;
    S.nb = old.nb;
    S.shape_boundary = old.shape_boundary;
    S.adj_seed_scale = old.adj_seed_scale;
    h->hScenes[scene] = S;
    return h->cuda(cudaMemcpyAsync(h->dScenes + scene, &S, sizeof(SceneDev), cudaMemcpyHostToDevice, h->stream),
                   "upload params");
}

sf_status sf_set_adjoint_seed_scale(sf_handle* h, int32_t scene, float scale) {
    if (!h || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    if (!(scale > 0.f) || !std::isfinite(scale)) return h->fail(SF_ERR_INVALID, "seed scale must be finite and > 0");
    SceneDev& S = h->hScenes[scene];
    S.adj_seed_scale = scale;
    return h->cuda(cudaMemcpyAsync(&h->dScenes[scene].adj_seed_scale, &S.adj_seed_scale, sizeof(float),
                                   cudaMemcpyHostToDevice, h->stream),
                   "upload seed scale");
}

sf_status sf_get_params(const sf_handle* h, int32_t scene, sf_params* p) {
    if (!h || !p || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    *p = h->P[scene];
    return SF_OK;
}

sf_status sf_run_stage(sf_handle* h, int32_t stage, float time_arg, int32_t adaptive) {
    if (!h) return SF_ERR_INVALID;
    if (stage < 0 || stage >= SF_STAGE_COUNT) return h->fail(SF_ERR_INVALID, "unknown stage");
    if (stage != SF_STAGE_SORT && !h->sorted) return h->fail(SF_ERR_INVALID, "run the sort stage first");
    return runStage(h, stage, time_arg, adaptive);
}

// sf_step's adaptive substep as a graph starting from buffer set h->cur,
// captured on first use: the integrator reads the render interval from
// h->dTimeArg, which sf_step writes before each replay.
static sf_status ensureStepGraph(sf_handle* h, GraphCache& g) {
    if (g.exec) return SF_OK;
    const int curBefore = h->cur;
    const int64_t launchesBefore = h->launches;
    cudaGraph_t graph = nullptr;
    sf_status st = h->cuda(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (st) return st;
    h->captureStep = true;
    st = runSubstep(h, 0.f, 1);
    h->captureStep = false;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    h->cur = curBefore;
    g.nodes = int(h->launches - launchesBefore);
    h->launches = launchesBefore;
    if (st != SF_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (h->cuda(ce, "end capture")) return SF_ERR_CUDA;
    st = h->cuda(cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
    cudaGraphDestroy(graph);
    return st;
}

sf_status sf_step(sf_handle* h, float render_interval, int64_t* n_substeps_out, float* ms_out) {
    if (!h) return SF_ERR_INVALID;
    if (sf_status gs = growListsIfFull(h, -1)) return gs;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms_out) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, h->stream);
    }
    // the substep is replayed from a captured graph; its render interval goes
    // to the device first (a pageable source: the copy is staged before the
    // call returns)
    const float t = render_interval;
    if (h->cuda(cudaMemcpyAsync(h->dTimeArg, &t, sizeof(float), cudaMemcpyHostToDevice, h->stream), "step time"))
        return SF_ERR_CUDA;
    GraphCache& g = h->graphStep[h->cur];
    sf_status st = ensureStepGraph(h, g);
    if (st != SF_OK) return st;
    if (h->cuda(cudaGraphLaunch(g.exec, h->stream), "graph launch")) return SF_ERR_CUDA;
    h->launches += g.nodes;
    h->cur = 1 - h->cur;
    h->sorted = true;
    queueStateCopy(h);
    if (ms_out) {
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(ms_out, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    if (n_substeps_out) {
        SceneState s0;
        st = h->cuda(cudaMemcpyAsync(&s0, h->dState, sizeof(SceneState), cudaMemcpyDeviceToHost, h->stream),
                     "read n_sub");
        if (st) return st;
        st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
        if (st) return st;
        *n_substeps_out = s0.n_sub;
    }
    return h->cuda(cudaGetLastError(), "sf_step");
}

sf_status sf_frame_adaptive(sf_handle* h, float render_interval, int64_t* n_calls_out) {
    if (!h) return SF_ERR_INVALID;
    if (h->nScenes != 1) return h->fail(SF_ERR_UNSUPPORTED, "sf_frame_adaptive needs a single-scene handle");
    float remaining = render_interval;
    int64_t calls = 0;
    while (remaining > kEps) {  // main.cpp:240-247
        int64_t nsub = 0;
        sf_status st = sf_step(h, remaining, &nsub, nullptr);
        if (st != SF_OK) return st;
        if (nsub <= 0) return h->fail(SF_ERR_INVALID, "CFL gave zero sub-steps for the remaining time");
        remaining -= remaining / float(nsub);
        ++calls;
    }
    if (n_calls_out) *n_calls_out = calls;
    return SF_OK;
}

// The captured graph of `nsub` fixed-dt substeps starting from buffer set
// h->cur (captured on first use and whenever dt changes).
static sf_status ensureGraph(sf_handle* h, GraphCache& g, int nsub, float dt) {
    if (g.exec && g.dt == dt) return SF_OK;
    if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    const int curBefore = h->cur;
    const int64_t launchesBefore = h->launches;
    cudaGraph_t graph = nullptr;
    sf_status st = h->cuda(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (st) return st;
    for (int k = 0; k < nsub && st == SF_OK; ++k) st = runSubstep(h, dt, 0);
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    h->cur = curBefore;
    g.nodes = int(h->launches - launchesBefore);
    h->launches = launchesBefore;
    if (st != SF_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (h->cuda(ce, "end capture")) return SF_ERR_CUDA;
    st = h->cuda(cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
    cudaGraphDestroy(graph);
    if (st) return st;
    g.dt = dt;
    return SF_OK;
}

namespace {

// n fixed-dt substeps replayed from the captured graphs.
sf_status queueSubstepsFixed(sf_handle* h, float dt, int64_t n) {
    sf_status st = SF_OK;
    if (n % 2 == 1) {  // the odd substep from a one-substep graph of this buffer set
        GraphCache& g1 = h->graph1[h->cur];
        if ((st = ensureGraph(h, g1, 1, dt))) return st;
        if (h->cuda(cudaGraphLaunch(g1.exec, h->stream), "graph launch")) return SF_ERR_CUDA;
        h->launches += g1.nodes;
        h->cur = 1 - h->cur;
    }
    if (n >= 2) {
        GraphCache& g = h->graph[h->cur];
        if ((st = ensureGraph(h, g, 2, dt))) return st;
        for (int64_t k = n % 2; k + 2 <= n; k += 2) {
            if (h->cuda(cudaGraphLaunch(g.exec, h->stream), "graph launch")) return SF_ERR_CUDA;
            h->launches += g.nodes;
        }
    }
    h->sorted = true;
    return SF_OK;
}

// Substeps between list checks in a long call.
constexpr int64_t kListCheckEvery = 64;

}  // namespace

// A call queues its substeps without waiting for them, except in long calls:
// there, after each block of kListCheckEvery substeps, the host waits until
// the block before it has run (the GPU keeps the newer block queued) and
// grows the lists if one was found full.
sf_status sf_substeps_fixed(sf_handle* h, float dt, int64_t n) {
    if (!h || n < 0) return SF_ERR_INVALID;
    if (n == 0) return SF_OK;
    sf_status st = growListsIfFull(h, n > kListCheckEvery ? 0 : -1);
    if (st == SF_OK && n > kListCheckEvery) st = growListsIfFull(h, 1);
    if (st) return st;
    int prevSlot = -1;
    for (int64_t done = 0; done < n;) {
        const int64_t m = std::min(kListCheckEvery, n - done);
        if ((st = queueSubstepsFixed(h, dt, m))) return st;
        done += m;
        const int slot = queueStateCopy(h);
        if (done < n && prevSlot >= 0 && (st = growListsIfFull(h, prevSlot))) return st;
        prevSlot = slot;
    }
    return SF_OK;
}

// ---------------------------------------------------------------- fields
namespace {

__global__ void kGetField(int field, int n, int slotOff, int cellOff, int order, const float4* __restrict__ pos,
                          const float4* __restrict__ vel, const float4* __restrict__ col,
                          const float4* __restrict__ mat, const float2* __restrict__ amc,
                          const int* __restrict__ pid, const float4* __restrict__ aux, const float4* __restrict__ flow,
                          const float4* __restrict__ adh, const float4* __restrict__ avgadh,
                          const float4* __restrict__ drag, const float4* __restrict__ acc,
                          const unsigned int* __restrict__ keys, const unsigned int* __restrict__ cnt, void* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = slotOff + i;
    const int o = order == SF_ORDER_ID ? pid[s] : i;
    float* f = static_cast<float*>(out);
    int* iv = static_cast<int*>(out);
    auto put3 = [&](float4 v) {
        f[3 * o] = v.x;
        f[3 * o + 1] = v.y;
        f[3 * o + 2] = v.z;
    };
    switch (field) {
    case SF_FIELD_POS: put3(pos[s]); break;
    case SF_FIELD_VEL: put3(vel[s]); break;
    case SF_FIELD_ACC: put3(acc[s]); break;
    case SF_FIELD_COL: put3(col[s]); break;
    case SF_FIELD_LABEL: iv[o] = pos[s].w < 0.f ? SF_LABEL_SAND : SF_LABEL_WATER; break;
    case SF_FIELD_RADIUS: f[o] = mat[s].w; break;
    case SF_FIELD_MASS: f[o] = fabsf(pos[s].w); break;
    case SF_FIELD_DENSITY: f[o] = vel[s].w; break;
    case SF_FIELD_PRESSURE: f[o] = aux[s].x; break;
    case SF_FIELD_VOIDAGE: f[o] = aux[s].w; break;
    case SF_FIELD_SATURATION: f[o] = aux[s].z; break;
    case SF_FIELD_MAX_SATURATION: f[o] = col[s].w; break;
    case SF_FIELD_AVG_FLOW: put3(flow[s]); break;
    case SF_FIELD_AVG_DRAG: put3(drag[s]); break;
    case SF_FIELD_ADHESION: put3(adh[s]); break;
    case SF_FIELD_AVG_ADHESION: put3(avgadh[s]); break;
    case SF_FIELD_CDA0ASAT: put3(mat[s]); break;
    case SF_FIELD_AMCAMCP:
        f[2 * o] = amc[s].x;
        f[2 * o + 1] = amc[s].y;
        break;
    case SF_FIELD_ID: iv[o] = pid[s]; break;
    case SF_FIELD_KEY: iv[o] = keys ? int(keys[s]) - cellOff : -1; break;
    case SF_FIELD_NEIGHBORS: iv[o] = cnt ? int(cnt[s] & 0xFFFFu) + int(cnt[s] >> 16) : 0; break;
    default: break;
    }
}

// The values the passes derive from a slot's fields for later passes (the
// w components, the water (D, P) pair and the gather records), recomputed
// with the passes' operations after a field was set, so that running the
// later stages gives the same results as after the passes themselves.
__device__ void refreshDerived(int s, const float4* pos, const float4* vel, const float4* aux, float4* flow,
                               float4* avgadh, float4* drag, float2* dp, float2* vrec2, float4* grec4,
                               const SceneDev& S) {
    const float4 p = pos[s], v = vel[s], a = aux[s];
    if (p.w < 0.f) {
        const float bz = bezier(S.adhG, a.z);
        flow[s].w = bz;
        drag[s].w = v.w;
        vrec2[s] = make_float2(bz, -p.w / v.w);
        grec4[s] = make_float4(v.x, v.y, v.z, a.z);
    } else if (p.w > 0.f) {
        const float vol = p.w / v.w;
        vrec2[s] = make_float2(a.y * vol, vol);
        const float D = v.w / fmaxf(kEps, a.w);
        const float P = a.x / fmaxf(kEps, D * D);
        dp[s] = make_float2(D, P);
        avgadh[s].w = D;
        grec4[s] = make_float4(v.x, v.y, v.z, P);
    }
}

__global__ void kSetField(int field, int n, int slotOff, int order, float4* pos, float4* vel, float4* col,
                          float4* mat, float2* amc, const int* __restrict__ pid, float4* aux, float4* flow,
                          float4* adh, float4* avgadh, float4* drag, float4* acc, float2* dp, float2* vrec2,
                          float4* grec4, const void* in, const SceneDev* __restrict__ scene) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = slotOff + i;
    const int o = order == SF_ORDER_ID ? pid[s] : i;
    const float* f = static_cast<const float*>(in);
    const int* iv = static_cast<const int*>(in);
    auto set3 = [&](float4* a) {
        float4 v = a[s];
        v.x = f[3 * o];
        v.y = f[3 * o + 1];
        v.z = f[3 * o + 2];
        a[s] = v;
    };
    switch (field) {
    case SF_FIELD_POS: set3(pos); break;
    case SF_FIELD_VEL: set3(vel); break;
    case SF_FIELD_ACC: set3(acc); break;
    case SF_FIELD_COL: set3(col); break;
    case SF_FIELD_LABEL: {
        const float m = fabsf(pos[s].w);
        pos[s].w = iv[o] == SF_LABEL_SAND ? -m : m;
        break;
    }
    case SF_FIELD_RADIUS: mat[s].w = f[o]; break;
    case SF_FIELD_MASS: pos[s].w = pos[s].w < 0.f ? -f[o] : f[o]; break;
    case SF_FIELD_DENSITY: vel[s].w = f[o]; break;
    case SF_FIELD_PRESSURE: aux[s].x = f[o]; break;
    case SF_FIELD_VOIDAGE: aux[s].w = f[o]; aux[s].y = f[o]; break;
    case SF_FIELD_SATURATION: aux[s].z = f[o]; break;
    case SF_FIELD_MAX_SATURATION: col[s].w = f[o]; break;
    case SF_FIELD_AVG_FLOW: set3(flow); break;
    case SF_FIELD_AVG_DRAG: set3(drag); break;
    case SF_FIELD_ADHESION: set3(adh); break;
    case SF_FIELD_AVG_ADHESION: set3(avgadh); break;
    case SF_FIELD_CDA0ASAT: set3(mat); break;
    case SF_FIELD_AMCAMCP: amc[s] = make_float2(f[2 * o], f[2 * o + 1]); break;
    default: break;
    }
    switch (field) {
    case SF_FIELD_VEL: case SF_FIELD_LABEL: case SF_FIELD_MASS: case SF_FIELD_DENSITY: case SF_FIELD_PRESSURE:
    case SF_FIELD_VOIDAGE: case SF_FIELD_SATURATION:
        refreshDerived(s, pos, vel, aux, flow, avgadh, drag, dp, vrec2, grec4, *scene);
        break;
    default: break;
    }
}

int fieldWidth(int field) {
    switch (field) {
    case SF_FIELD_POS: case SF_FIELD_VEL: case SF_FIELD_ACC: case SF_FIELD_COL: case SF_FIELD_AVG_FLOW:
    case SF_FIELD_AVG_DRAG: case SF_FIELD_ADHESION: case SF_FIELD_AVG_ADHESION: case SF_FIELD_CDA0ASAT:
    case SF_BFIELD_POS:
        return 3;
    case SF_FIELD_AMCAMCP: return 2;
    case SF_FIELD_LABEL: case SF_FIELD_RADIUS: case SF_FIELD_MASS: case SF_FIELD_DENSITY: case SF_FIELD_PRESSURE:
    case SF_FIELD_VOIDAGE: case SF_FIELD_SATURATION: case SF_FIELD_MAX_SATURATION: case SF_FIELD_ID:
    case SF_FIELD_KEY: case SF_FIELD_NEIGHBORS: case SF_BFIELD_LABEL: case SF_BFIELD_VOLUME:
        return 1;
    default: return 0;
    }
}

// The xyz of one float4 slot array in sorted order <-> a packed n x 3 float
// buffer (16-byte aligned), moved as whole 16-byte words through shared
// memory: a block of 256 particles covers 192 words of the buffer, so pinned
// host memory read or written over the host link sees full-line accesses
// instead of three 4-byte accesses per particle.
constexpr int kVecParticles = 256;
__global__ void __launch_bounds__(kVecParticles) kGetVec3(int n, int slotOff, const float4* __restrict__ src,
                                                          float4* __restrict__ out) {
    __shared__ float4 buf4[kVecParticles * 3 / 4];
    float* buf = reinterpret_cast<float*>(buf4);
    const int t = threadIdx.x, p0 = blockIdx.x * kVecParticles, cnt = min(kVecParticles, n - p0);
    if (t < cnt) {
        const float4 v = src[slotOff + p0 + t];
        buf[3 * t] = v.x;
        buf[3 * t + 1] = v.y;
        buf[3 * t + 2] = v.z;
    }
    __syncthreads();
    float4* o = out + size_t(p0) * 3 / 4;  // p0 is a multiple of 4
    const int words = 3 * cnt / 4, rem = 3 * cnt - 4 * words;
    if (t < words) o[t] = buf4[t];
    if (t < rem) reinterpret_cast<float*>(o + words)[t] = buf[4 * words + t];
}
__global__ void __launch_bounds__(kVecParticles) kSetVec3(int n, int slotOff, float4* __restrict__ dst,
                                                          const float4* __restrict__ in, float4* __restrict__ rec) {
    __shared__ float4 buf4[kVecParticles * 3 / 4];
    float* buf = reinterpret_cast<float*>(buf4);
    const int t = threadIdx.x, p0 = blockIdx.x * kVecParticles, cnt = min(kVecParticles, n - p0);
    const float4* src = in + size_t(p0) * 3 / 4;
    const int words = 3 * cnt / 4, rem = 3 * cnt - 4 * words;
    if (t < words) buf4[t] = src[t];
    if (t < rem) buf[4 * words + t] = reinterpret_cast<const float*>(src + words)[t];
    __syncthreads();
    if (t < cnt) {
        float4 v = dst[slotOff + p0 + t];
        v.x = buf[3 * t];
        v.y = buf[3 * t + 1];
        v.z = buf[3 * t + 2];
        dst[slotOff + p0 + t] = v;
        if (rec) {  // velocities: the copy in the gather records
            float4 r = rec[slotOff + p0 + t];
            r.x = v.x;
            r.y = v.y;
            r.z = v.z;
            rec[slotOff + p0 + t] = r;
        }
    }
}

// The float4 slot array whose xyz is field (3-wide float fields), else null.
float4* vec3Array(sf_handle* h, int field) {
    const int c = h->cur;
    switch (field) {
    case SF_FIELD_POS: return h->pos[c];
    case SF_FIELD_VEL: return h->vel[c];
    case SF_FIELD_ACC: return h->acc;
    case SF_FIELD_COL: return h->col[c];
    case SF_FIELD_AVG_FLOW: return h->flow;
    case SF_FIELD_AVG_DRAG: return h->drag;
    case SF_FIELD_ADHESION: return h->adh;
    case SF_FIELD_AVG_ADHESION: return h->avgadh;
    case SF_FIELD_CDA0ASAT: return h->mat[c];
    default: return nullptr;
    }
}

// Device address of page-locked (pinned) host memory, which kernels can
// read and write directly over the host link; nullptr for other memory.
void* mappedHostPointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

sf_status ensureStage(sf_handle* h, size_t bytes) {
    if (h->stageBytes >= bytes) return SF_OK;
    if (h->stage) cudaFree(h->stage);
    h->stage = nullptr;
    h->stageBytes = 0;
    if (h->cuda(cudaMalloc(&h->stage, bytes), "cudaMalloc staging")) return SF_ERR_CUDA;
    h->stageBytes = bytes;
    return SF_OK;
}

__global__ void kGetBoundary(int field, int n, int bOff, const float4* __restrict__ bpos, const int* __restrict__ bl,
                             void* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 b = bpos[bOff + i];
    float* f = static_cast<float*>(out);
    if (field == SF_BFIELD_POS) {
        f[3 * i] = b.x;
        f[3 * i + 1] = b.y;
        f[3 * i + 2] = b.z;
    } else if (field == SF_BFIELD_LABEL) {
        static_cast<int*>(out)[i] = bl[bOff + i];
    } else {
        f[i] = fabsf(b.w);
    }
}

}  // namespace

namespace {

// sf_get_field without its final host synchronisation (the copy is queued on
// the handle's stream).
sf_status getFieldQueued(sf_handle* h, int32_t scene, int32_t field, int32_t order, void* dst, int64_t count,
                         int32_t dst_on_device) {
    if (!h || !dst || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    const int w = fieldWidth(field);
    if (w == 0) return h->fail(SF_ERR_INVALID, "unknown field");
    if (order != SF_ORDER_SORTED && order != SF_ORDER_ID) return h->fail(SF_ERR_INVALID, "unknown order");
    const SceneDev& S = h->hScenes[scene];
    const bool bfield = field >= SF_BFIELD_POS;
    const int64_t n = bfield ? S.nb : h->n[scene];
    if (count != n) return h->fail(SF_ERR_INVALID, "count must equal the scene's particle count");
    const size_t bytes = size_t(n) * size_t(w) * 4;
    if (n == 0) return SF_OK;
    void* target = dst;
    // pinned host memory in sorted order is written by the gather kernel
    // directly (coalesced); anything else goes through the device stage
    void* mapped = (!dst_on_device && order == SF_ORDER_SORTED) ? mappedHostPointer(dst) : nullptr;
    if (!dst_on_device) {
        if (mapped) {
            target = mapped;
        } else {
            if (ensureStage(h, bytes)) return SF_ERR_CUDA;
            target = h->stage;
        }
    }
    const int blocks = int((n + 255) / 256);
    float4* vec = bfield || order != SF_ORDER_SORTED ? nullptr : vec3Array(h, field);
    if (vec && (reinterpret_cast<uintptr_t>(target) & 15u) == 0) {
        kGetVec3<<<int((n + kVecParticles - 1) / kVecParticles), kVecParticles, 0, h->stream>>>(
            int(n), S.slot_off, vec, static_cast<float4*>(target));
    } else if (bfield) {
        kGetBoundary<<<blocks, 256, 0, h->stream>>>(field, int(n), S.b_off, h->bpos, h->blabel, target);
    } else {
        const int c = h->cur;
        kGetField<<<blocks, 256, 0, h->stream>>>(field, int(n), S.slot_off, S.cell_off, order, h->pos[c], h->vel[c],
                                                 h->col[c], h->mat[c], h->amc[c], h->pid[c], h->aux, h->flow,
                                                 h->adh, h->avgadh, h->drag, h->acc, h->sorted ? h->sortedKeys : nullptr,
                                                 h->sorted ? h->nbrCnt : nullptr, target);
    }
    if (h->cuda(cudaGetLastError(), "get_field launch")) return SF_ERR_CUDA;
    if (!dst_on_device && !mapped &&
        h->cuda(cudaMemcpyAsync(dst, h->stage, bytes, cudaMemcpyDeviceToHost, h->stream), "get_field D2H"))
        return SF_ERR_CUDA;
    return SF_OK;
}

}  // namespace

sf_status sf_get_field(sf_handle* h, int32_t scene, int32_t field, int32_t order, void* dst, int64_t count,
                       int32_t dst_on_device) {
    sf_status st = getFieldQueued(h, scene, field, order, dst, count, dst_on_device);
    if (st || dst_on_device) return st;
    return h->cuda(cudaStreamSynchronize(h->stream), "get_field sync");
}

sf_status sf_get_fields(sf_handle* h, int32_t scene, int32_t n_fields, const int32_t* fields, int32_t order,
                        void* const* dsts, int64_t count, int32_t dst_on_device) {
    if (!h || n_fields < 0 || (n_fields > 0 && (!fields || !dsts))) return SF_ERR_INVALID;
    for (int32_t k = 0; k < n_fields; ++k)
        if (sf_status st = getFieldQueued(h, scene, fields[k], order, dsts[k], count, dst_on_device)) return st;
    if (dst_on_device || n_fields == 0) return SF_OK;
    return h->cuda(cudaStreamSynchronize(h->stream), "get_fields sync");
}

namespace {

// sf_set_field without its final host synchronisation.
sf_status setFieldQueued(sf_handle* h, int32_t scene, int32_t field, int32_t order, const void* src, int64_t count,
                         int32_t src_on_device) {
    if (!h || !src || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    const int w = fieldWidth(field);
    if (w == 0 || field >= SF_BFIELD_POS || field == SF_FIELD_ID || field == SF_FIELD_KEY ||
        field == SF_FIELD_NEIGHBORS)
        return h->fail(SF_ERR_INVALID, "field cannot be set");
    if (order != SF_ORDER_SORTED && order != SF_ORDER_ID) return h->fail(SF_ERR_INVALID, "unknown order");
    const SceneDev& S = h->hScenes[scene];
    const int64_t n = h->n[scene];
    if (count != n) return h->fail(SF_ERR_INVALID, "count must equal the scene's particle count");
    if (n == 0) return SF_OK;
    const size_t bytes = size_t(n) * size_t(w) * 4;
    const void* from = src;
    // pinned host memory in sorted order is read by the scatter kernel directly
    void* mapped = (!src_on_device && order == SF_ORDER_SORTED) ? mappedHostPointer(src) : nullptr;
    if (!src_on_device) {
        if (mapped) {
            from = mapped;
        } else {
            if (ensureStage(h, bytes)) return SF_ERR_CUDA;
            if (h->cuda(cudaMemcpyAsync(h->stage, src, bytes, cudaMemcpyHostToDevice, h->stream), "set_field H2D"))
                return SF_ERR_CUDA;
            from = h->stage;
        }
    }
    const int c = h->cur;
    float4* vec = order == SF_ORDER_SORTED ? vec3Array(h, field) : nullptr;
    if (vec && (reinterpret_cast<uintptr_t>(from) & 15u) == 0)
        kSetVec3<<<int((n + kVecParticles - 1) / kVecParticles), kVecParticles, 0, h->stream>>>(
            int(n), S.slot_off, vec, static_cast<const float4*>(from), field == SF_FIELD_VEL ? h->grec4 : nullptr);
    else
        kSetField<<<int((n + 255) / 256), 256, 0, h->stream>>>(field, int(n), S.slot_off, order, h->pos[c],
                                                               h->vel[c], h->col[c], h->mat[c], h->amc[c], h->pid[c],
                                                               h->aux, h->flow, h->adh, h->avgadh, h->drag, h->acc,
                                                               h->dp, h->vrec2, h->grec4, from, h->dScenes + scene);
    return h->cuda(cudaGetLastError(), "set_field launch");
}

}  // namespace

sf_status sf_set_field(sf_handle* h, int32_t scene, int32_t field, int32_t order, const void* src, int64_t count,
                       int32_t src_on_device) {
    sf_status st = setFieldQueued(h, scene, field, order, src, count, src_on_device);
    if (st || src_on_device) return st;
    return h->cuda(cudaStreamSynchronize(h->stream), "set_field sync");
}

sf_status sf_set_fields(sf_handle* h, int32_t scene, int32_t n_fields, const int32_t* fields, int32_t order,
                        const void* const* srcs, int64_t count, int32_t src_on_device) {
    if (!h || n_fields < 0 || (n_fields > 0 && (!fields || !srcs))) return SF_ERR_INVALID;
    for (int32_t k = 0; k < n_fields; ++k)
        if (sf_status st = setFieldQueued(h, scene, fields[k], order, srcs[k], count, src_on_device)) return st;
    if (src_on_device || n_fields == 0) return SF_OK;
    return h->cuda(cudaStreamSynchronize(h->stream), "set_fields sync");
}

sf_status sf_export_bgeo(sf_handle* h, int32_t scene, const char* folder_path, const char* file_name) {
    if (!h) return SF_ERR_INVALID;
    if (scene < 0 || scene >= h->nScenes || !file_name) return h->fail(SF_ERR_INVALID, "bad scene or file name");
    const SceneDev& S = h->hScenes[scene];
    const int64_t n = h->n[scene];
    const size_t bytes = std::max<size_t>(16, size_t(n) * 36);
    if (ensureStage(h, bytes) || ensurePinned(h->exportHost, h->exportHostBytes, bytes, h->err)) return SF_ERR_CUDA;
    const int c = h->cur;
    return exportBgeoSlots(h->stream, n, h->pos[c] + S.slot_off, h->col[c] + S.slot_off, h->mat[c] + S.slot_off,
                           h->stage, h->exportHost, folder_path, file_name, h->err);
}

sf_status sf_get_cell_table(sf_handle* h, int32_t scene, int32_t which, int64_t* dst, int64_t count) {
    if (!h || !dst || scene < 0 || scene >= h->nScenes || (which != 0 && which != 1)) return SF_ERR_INVALID;
    const SceneDev& S = h->hScenes[scene];
    if (count != int64_t(S.ncell) + 1) return h->fail(SF_ERR_INVALID, "count must be G + 1");
    if (which == 0 && !h->sorted) return h->fail(SF_ERR_INVALID, "no cell table before the first sort");
    std::vector<unsigned> t(static_cast<size_t>(count));
    if (h->cuda(cudaMemcpyAsync(t.data(), (which ? h->bcs : h->cs) + S.cell_off, sizeof(unsigned) * t.size(),
                                cudaMemcpyDeviceToHost, h->stream),
                "cell table D2H") ||
        h->cuda(cudaStreamSynchronize(h->stream), "cell table sync"))
        return SF_ERR_CUDA;
    const int64_t base = which ? S.b_off : S.slot_off;
    for (size_t c = 0; c < t.size(); ++c) dst[c] = int64_t(t[c]) - base;
    return SF_OK;
}

sf_status sf_get_grid(const sf_handle* h, int32_t scene, int32_t grid_size[3], int64_t* n_cells) {
    if (!h || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    const SceneDev& S = h->hScenes[scene];
    if (grid_size) {
        grid_size[0] = S.gx;
        grid_size[1] = S.gy;
        grid_size[2] = S.gz;
    }
    if (n_cells) *n_cells = S.ncell;
    return SF_OK;
}

sf_status sf_size(const sf_handle* h, int32_t scene, int64_t* n, int64_t* capacity) {
    if (!h || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    if (n) *n = h->n[scene];
    if (capacity) *capacity = h->capUser[scene];
    return SF_OK;
}

sf_status sf_num_scenes(const sf_handle* h, int32_t* n_scenes) {
    if (!h || !n_scenes) return SF_ERR_INVALID;
    *n_scenes = h->nScenes;
    return SF_OK;
}

sf_status sf_num_substeps(sf_handle* h, int32_t scene, int64_t* n_sub) {
    if (!h || !n_sub || scene < 0 || scene >= h->nScenes) return SF_ERR_INVALID;
    SceneState s;
    if (h->cuda(cudaMemcpyAsync(&s, h->dState + scene, sizeof(SceneState), cudaMemcpyDeviceToHost, h->stream),
                "read state") ||
        h->cuda(cudaStreamSynchronize(h->stream), "sync"))
        return SF_ERR_CUDA;
    *n_sub = s.n_sub;
    return SF_OK;
}

sf_status sf_add_sph_particles(sf_handle* h, int32_t scene, const float* pos3, int64_t n, const float col[3],
                               const float vel[3], float mass, float radius) {
    if (!h || scene < 0 || scene >= h->nScenes || n < 0 || (n > 0 && !pos3) || !col || !vel)
        return SF_ERR_INVALID;
    if (!(mass > 0.f)) return h->fail(SF_ERR_INVALID, "mass must be > 0");
    // cuda_sf_particles.cu:54-58: refuse when Size() + num >= MaxSize()
    if (h->n[scene] + n >= h->capUser[scene])
        return h->fail(SF_ERR_CAPACITY, "Current SPH particles numbers exceed maximum particles.");
    if (n == 0) return SF_OK;
    const SceneDev& S = h->hScenes[scene];
    std::vector<float4> p(static_cast<size_t>(n)), v(static_cast<size_t>(n)), c(static_cast<size_t>(n)), m(static_cast<size_t>(n));
    std::vector<float2> a(static_cast<size_t>(n), make_float2(0.f, 0.f));
    std::vector<int> id(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        p[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], mass);
        v[i] = make_float4(vel[0], vel[1], vel[2], 0.f);
        c[i] = make_float4(col[0], col[1], col[2], 0.f);
        m[i] = make_float4(0.f, 0.f, 0.f, radius);
        id[i] = int(h->nextId[scene] + i);
    }
    const size_t off = size_t(S.slot_off + h->n[scene]);
    const int k = h->cur;
    auto up = [&](void* d, const void* s, size_t b) {
        return h->cuda(cudaMemcpyAsync(d, s, b, cudaMemcpyHostToDevice, h->stream), "add particles H2D");
    };
    if (up(h->pos[k] + off, p.data(), sizeof(float4) * n) || up(h->vel[k] + off, v.data(), sizeof(float4) * n) ||
        up(h->col[k] + off, c.data(), sizeof(float4) * n) || up(h->mat[k] + off, m.data(), sizeof(float4) * n) ||
        up(h->amc[k] + off, a.data(), sizeof(float2) * n) || up(h->pid[k] + off, id.data(), sizeof(int) * n) ||
        h->cuda(cudaStreamSynchronize(h->stream), "add particles sync"))
        return SF_ERR_CUDA;
    h->n[scene] += n;
    h->nextId[scene] += n;
    return SF_OK;
}

namespace {

// Scatters one scene's persistent arrays from buffer set o to t by particle
// id: live slot s goes to slotOff + pid[s]; parked slots keep their place.
__global__ void kResetOrder(int slots, int n, int slotOff, const float4* __restrict__ pos, const float4* __restrict__ vel,
                            const float4* __restrict__ col, const float4* __restrict__ mat,
                            const float2* __restrict__ amc, const int* __restrict__ pid, float4* __restrict__ pos2,
                            float4* __restrict__ vel2, float4* __restrict__ col2, float4* __restrict__ mat2,
                            float2* __restrict__ amc2, int* __restrict__ pid2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots) return;
    const int s = slotOff + i;
    const int id = pid[s];
    const int d = (i < n && id >= 0 && id < n) ? slotOff + id : s;
    pos2[d] = pos[s];
    vel2[d] = vel[s];
    col2[d] = col[s];
    mat2[d] = mat[s];
    amc2[d] = amc[s];
    pid2[d] = id;
}

}  // namespace

sf_status sf_reset_order(sf_handle* h) {
    if (!h) return SF_ERR_INVALID;
    const int o = h->cur, t = 1 - h->cur;
    for (int sc = 0; sc < h->nScenes; ++sc) {
        const SceneDev& S = h->hScenes[sc];
        const int slots = S.slot_cap;
        if (slots <= 0) continue;
        kResetOrder<<<(slots + 255) / 256, 256, 0, h->stream>>>(
            slots, int(h->n[sc]), S.slot_off, h->pos[o], h->vel[o], h->col[o], h->mat[o], h->amc[o], h->pid[o],
            h->pos[t], h->vel[t], h->col[t], h->mat[t], h->amc[t], h->pid[t]);
        h->launches += 1;
    }
    h->cur = t;
    h->sorted = false;
    return h->cuda(cudaGetLastError(), "reset order launch");
}

sf_status sf_check_error(sf_handle* h, uint32_t* flags) {
    if (!h || !flags) return SF_ERR_INVALID;
    unsigned v = 0;
    if (h->cuda(cudaMemcpyAsync(&v, h->dErr, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream), "read error") ||
        h->cuda(cudaMemsetAsync(h->dErr, 0, sizeof(unsigned), h->stream), "clear error") ||
        h->cuda(cudaStreamSynchronize(h->stream), "sync"))
        return SF_ERR_CUDA;
    *flags = v;
    return v ? SF_ERR_DEVICE : SF_OK;
}

sf_status sf_synchronize(sf_handle* h) {
    if (!h) return SF_ERR_INVALID;
    return h->cuda(cudaStreamSynchronize(h->stream), "sf_synchronize");
}

sf_status sf_get_list_capacity(const sf_handle* h, int32_t* capacity, int64_t* growths) {
    if (!h) return SF_ERR_INVALID;
    if (capacity) *capacity = h->nbrCap;
    if (growths) *growths = h->listGrowths;
    return SF_OK;
}

sf_status sf_launch_count(const sf_handle* h, int64_t* launches) {
    if (!h || !launches) return SF_ERR_INVALID;
    *launches = h->launches;
    return SF_OK;
}

sf_status sf_set_tuning(sf_handle* h, int32_t block_size, int32_t items_per_thread) {
    if (!h) return SF_ERR_INVALID;
    if (items_per_thread != 0 && items_per_thread != 1)
        return h->fail(SF_ERR_UNSUPPORTED, "the passes handle one particle slot per thread");
    if (block_size == 0) return SF_OK;
    if (block_size != 32 && block_size != 64 && block_size != 128 && block_size != 256)
        return h->fail(SF_ERR_INVALID, "block_size must be 32, 64, 128 or 256");
    for (int k = 0; k < kTunedPasses; ++k) h->block[k] = block_size;
    h->dropGraphs();
    return SF_OK;
}

sf_status sf_set_density_staging(sf_handle* h, int32_t staged) {
    if (!h) return SF_ERR_INVALID;
    if (staged != 0 && staged != 1) return h->fail(SF_ERR_INVALID, "staged must be 0 or 1");
    h->densityStaged = staged;
    h->dropGraphs();
    return SF_OK;
}

sf_status sf_get_density_staging(const sf_handle* h, int32_t* staged) {
    if (!h || !staged) return SF_ERR_INVALID;
    *staged = h->densityStaged;
    return SF_OK;
}

sf_status sf_set_lanes(sf_handle* h, int32_t lanes) {
    if (!h) return SF_ERR_INVALID;
    if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8)
        return h->fail(SF_ERR_INVALID, "lanes must be 0 (automatic), 1, 2, 4 or 8");
    if (lanes == 0) {
        int dev = 0, sms = 0;
        if (h->cuda(cudaGetDevice(&dev), "cudaGetDevice") ||
            h->cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))
            return SF_ERR_CUDA;
        lanes = lanesForSlots(h->totalSlots, sms);
    }
    h->lanes = lanes;
    h->dropGraphs();
    return SF_OK;
}

sf_status sf_autotune(sf_handle* h, float dt, int32_t* block_sizes_out, int32_t* list_capacity_out) {
    if (!h) return SF_ERR_INVALID;
    if (!(dt > 0.f) || !std::isfinite(dt)) return h->fail(SF_ERR_INVALID, "dt must be finite and > 0");
    sf_status st = SF_OK;
    if (!h->sorted && (st = runSort(h))) return st;
    if ((st = probeListCapacity(h))) return st;
    if (h->slab) {  // stored-substep slabs depend on the list capacity
        if (h->cuda(cudaStreamSynchronize(h->stream), "sync before slab release")) return SF_ERR_CUDA;
        devFree(h->slab);
        h->slabBytes = 0;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (h->cuda(cudaEventCreate(&e0), "event") || h->cuda(cudaEventCreate(&e1), "event")) return SF_ERR_CUDA;
    // device time of five launches of fn (after one untimed)
    auto timed = [&](auto&& fn, float& ms) -> sf_status {
        sf_status r = fn();
        if (r) return r;
        cudaEventRecord(e0, h->stream);
        for (int k = 0; k < 5 && r == SF_OK; ++k) r = fn();
        cudaEventRecord(e1, h->stream);
        if (r) return r;
        if (h->cuda(cudaEventSynchronize(e1), "tune sync") || h->cuda(cudaEventElapsedTime(&ms, e0, e1), "tune time"))
            return SF_ERR_CUDA;
        return SF_OK;
    };
    // sort tile size and digit width: sorting the sorted state again is the identity
    {
        float best = 0.f;
        int bestItems = h->sc.items, bestDigit = h->sc.digitBits;
        const int wide = sortDigitBits(h->sortBits);
        for (int digit : {8, wide}) {
            for (int items : {8, 4, 2, 1}) {
                if (st) break;
                h->sc.items = items;
                h->sc.digitBits = digit;
                h->sc.tiles = sortTiles(h->totalSlots, items);
                float ms = 0.f;
                if ((st = timed([&] { return runSort(h); }, ms))) break;
                if (best == 0.f || ms < best) {
                    best = ms;
                    bestItems = items;
                    bestDigit = digit;
                }
            }
            if (wide == 8) break;
        }
        h->sc.items = bestItems;
        h->sc.digitBits = bestDigit;
        h->sc.tiles = sortTiles(h->totalSlots, bestItems);
    }
    // lanes per particle and the block size of every neighbour pass: every
    // pass recomputes its outputs from inputs it does not write, so repeating
    // it on the current state is harmless; the integrator is not repeated (it
    // advances the state) and keeps its block size
    const int candidates[3] = {64, 128, 256};
    const int stages[kTunedPasses - 1] = {SF_STAGE_DENSITY, SF_STAGE_AVGFLOW, SF_STAGE_VOIDAGE_ADHESION,
                                          SF_STAGE_SAND_MOMENTUM, SF_STAGE_WATER_MOMENTUM};
    for (int s = SF_STAGE_DENSITY; s <= SF_STAGE_WATER_MOMENTUM && st == SF_OK; ++s) st = runStage(h, s, dt, 0);
    // (with one lane the density pass is timed with and without its
    // shared-memory staging as well)
    float bestTotal = 0.f;
    int bestLanes = h->lanes, bestBlock[kTunedPasses - 1], bestStaged = 0;
    for (int p = 0; p < kTunedPasses - 1; ++p) bestBlock[p] = h->block[p];
    for (int lanes : {1, 2, 4, 8}) {
        if (st) break;
        h->lanes = lanes;
        float total = 0.f;
        int block[kTunedPasses - 1], staged = 0;
        for (int p = 0; p < kTunedPasses - 1 && st == SF_OK; ++p) {
            float best = 0.f;
            block[p] = h->block[p];
            const int forms = (p == kPassDensity && lanes == 1) ? 2 : 1;
            for (int f = 0; f < forms && st == SF_OK; ++f) {
                h->densityStaged = f;
                for (int bs : candidates) {
                    h->block[p] = bs;
                    float ms = 0.f;
                    if ((st = timed([&] { return runStage(h, stages[p], dt, 0); }, ms))) break;
                    if (best == 0.f || ms < best) {
                        best = ms;
                        block[p] = bs;
                        if (p == kPassDensity) staged = f;
                    }
                }
            }
            h->densityStaged = 0;
            h->block[p] = block[p];
            total += best;
        }
        if (st == SF_OK && (bestTotal == 0.f || total < bestTotal)) {
            bestTotal = total;
            bestLanes = lanes;
            bestStaged = staged;
            for (int p = 0; p < kTunedPasses - 1; ++p) bestBlock[p] = block[p];
        }
    }
    h->lanes = bestLanes;
    h->densityStaged = bestStaged;
    for (int p = 0; p < kTunedPasses - 1; ++p) h->block[p] = bestBlock[p];
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    h->dropGraphs();
    if (block_sizes_out)
        for (int k = 0; k < kTunedPasses; ++k) block_sizes_out[k] = h->block[k];
    if (list_capacity_out) *list_capacity_out = h->nbrCap;
    return SF_OK;
}

sf_status sf_get_tuning(const sf_handle* h, int32_t* block_sizes_out, int32_t* lanes_out, int32_t* sort_items_out,
                        int32_t* sort_digit_bits_out) {
    if (!h) return SF_ERR_INVALID;
    if (block_sizes_out)
        for (int k = 0; k < kTunedPasses; ++k) block_sizes_out[k] = h->block[k];
    if (lanes_out) *lanes_out = h->lanes;
    if (sort_items_out) *sort_items_out = h->sc.items ? h->sc.items : 8;
    if (sort_digit_bits_out) *sort_digit_bits_out = h->sc.digitBits ? h->sc.digitBits : 8;
    return SF_OK;
}

const char* sf_last_error_string(const sf_handle* h) { return h ? h->err.c_str() : g_createError.c_str(); }

// ---------------------------------------------------------------- adjoint
namespace {

// One snapshot = the persistent per-slot arrays of the current buffer set
// (pos, vel, col, mat, amc, pid), which fully determine the next substeps
// including the summation order of the stable sort.
size_t snapStride(const sf_handle* h) {
    return size_t(h->totalSlots) * (4 * sizeof(float4) + sizeof(float2) + sizeof(int));
}

sf_status snapCopy(sf_handle* h, char* snap, bool save) {
    const size_t M = size_t(h->totalSlots);
    const int c = h->cur;
    void* arrays[6] = {h->pos[c], h->vel[c], h->col[c], h->mat[c], h->amc[c], h->pid[c]};
    const size_t bytes[6] = {sizeof(float4) * M, sizeof(float4) * M, sizeof(float4) * M,
                             sizeof(float4) * M, sizeof(float2) * M, sizeof(int) * M};
    size_t off = 0;
    for (int k = 0; k < 6; ++k) {
        void* dst = save ? static_cast<void*>(snap + off) : arrays[k];
        const void* src = save ? arrays[k] : static_cast<const void*>(snap + off);
        if (h->cuda(cudaMemcpyAsync(dst, src, bytes[k], cudaMemcpyDeviceToDevice, h->stream), "snapshot copy"))
            return SF_ERR_CUDA;
        off += bytes[k];
    }
    return SF_OK;
}

// One slab = what the adjoint of one substep reads (AdjSlab), 256-byte aligned.
size_t slabStride(const sf_handle* h) {
    const size_t M = size_t(h->totalSlots);
    const size_t b = M * (sizeof(unsigned) * (1 + size_t(h->nbrCap) + kMaxContact) + sizeof(int) * 2 + sizeof(unsigned) * kMaxBNbr +
                          9 * sizeof(float4) + sizeof(float2) + sizeof(int)) +
                     sizeof(unsigned) * (size_t(h->totalCells) + 1);
    return (b + 255) / 256 * 256;
}

AdjSlab slabAt(const sf_handle* h, char* base) {
    const size_t M = size_t(h->totalSlots);
    AdjSlab s;
    char* p = base;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += bytes;
        return r;
    };
    s.pos = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.vel = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.aux = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.flow = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.drag = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.acc = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.adh = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.avgadh = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.mat = reinterpret_cast<float4*>(take(sizeof(float4) * M));
    s.dp = reinterpret_cast<float2*>(take(sizeof(float2) * M));
    s.nbr = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * M * size_t(h->nbrCap)));
    s.bnbr = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * M * kMaxBNbr));
    s.cnbr = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * M * kMaxContact));
    s.cnt = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * M));
    s.bcnt = reinterpret_cast<int*>(take(sizeof(int) * M));
    s.ccnt = reinterpret_cast<int*>(take(sizeof(int) * M));
    s.pid = reinterpret_cast<int*>(take(sizeof(int) * M));
    s.cs = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * (size_t(h->totalCells) + 1)));
    return s;
}

// The pass buffers of a stored substep.
PassBuffers slabBuffers(const sf_handle* h, const AdjSlab& s) {
    PassBuffers b = h->buffers();
    b.lists.cnt = s.cnt;
    b.lists.nbr = s.nbr;
    b.lists.bcnt = s.bcnt;
    b.lists.bnbr = s.bnbr;
    b.lists.ccnt = s.ccnt;
    b.lists.cnbr = s.cnbr;
    b.lists.cs = s.cs;
    b.listsW = NbrListsW{s.cnt, s.nbr, s.bcnt, s.bnbr, s.ccnt, s.cnbr, s.cs, h->bcs, h->bnear, b.lists.M,
                         h->nbrCap};
    b.pos4 = s.pos;
    b.vel4 = s.vel;
    b.aux4 = s.aux;
    b.flow4 = s.flow;
    b.drag4 = s.drag;
    b.acc4 = s.acc;
    b.adh4 = s.adh;
    b.avgadh4 = s.avgadh;
    b.mat4 = s.mat;
    b.dp = s.dp;
    b.col4 = nullptr;
    return b;
}

// One fixed-dt substep whose lists, cell table and per-substep fields are
// written straight into the slab (the handle's own buffers are swapped out
// for the passes that produce them), with the fields the integrator
// overwrites copied in before it runs.
sf_status runSubstepStore(sf_handle* h, float dt, const AdjSlab& s) {
    unsigned *cnt = h->nbrCnt, *nbr = h->nbr, *bnbr = h->bnbr, *cnbr = h->cnbr, *cs = h->cs;
    int *bcnt = h->bnbrCnt, *ccnt = h->cnbrCnt;
    float4 *aux = h->aux, *flow = h->flow, *drag = h->drag;
    float2* dp = h->dp;
    h->dp = s.dp;
    h->nbrCnt = s.cnt;
    h->nbr = s.nbr;
    h->bnbr = s.bnbr;
    h->cnbr = s.cnbr;
    h->cs = s.cs;
    h->bnbrCnt = s.bcnt;
    h->cnbrCnt = s.ccnt;
    h->aux = s.aux;
    h->flow = s.flow;
    h->drag = s.drag;
    sf_status st = SF_OK;
    for (int k = SF_STAGE_SORT; k <= SF_STAGE_WATER_MOMENTUM && st == SF_OK; ++k) st = runStage(h, k, dt, 0);
    if (st == SF_OK) {
        launchAdjStore(h->ctx(), h->buffers(), h->pid[h->cur], s);
        h->launches += 1;
    }
    h->nbrCnt = cnt;
    h->nbr = nbr;
    h->bnbr = bnbr;
    h->cnbr = cnbr;
    h->cs = cs;
    h->bnbrCnt = bcnt;
    h->cnbrCnt = ccnt;
    h->aux = aux;
    h->flow = flow;
    h->drag = drag;
    h->dp = dp;
    if (st != SF_OK) return st;
    return runStage(h, SF_STAGE_INTEGRATE, dt, 0);
}

// One store-mode substep into stored-substep slot t, replayed from a graph
// captured per buffer set and slot on first use (and again when dt or the
// slab buffer changes): the ~20 launches of a substep cost more than the
// kernels themselves on small scenes.
sf_status runSubstepStoreGraphed(sf_handle* h, float dt, int64_t t) {
    if (h->storeGraphSlab != h->slab) {
        h->dropGraphs();
        h->storeGraphSlab = h->slab;
    }
    std::vector<GraphCache>& v = h->storeGraph[h->cur];
    if (int64_t(v.size()) <= t) v.resize(size_t(t) + 1);
    GraphCache& g = v[size_t(t)];
    if (!g.exec || g.dt != dt) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        const int curBefore = h->cur;
        const int64_t launchesBefore = h->launches;
        cudaGraph_t graph = nullptr;
        sf_status st = h->cuda(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (st) return st;
        st = runSubstepStore(h, dt, slabAt(h, h->slab + size_t(t) * slabStride(h)));
        cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
        h->cur = curBefore;
        g.nodes = int(h->launches - launchesBefore);
        h->launches = launchesBefore;
        if (st != SF_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (h->cuda(ce, "end capture")) return SF_ERR_CUDA;
        st = h->cuda(cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
        cudaGraphDestroy(graph);
        if (st) return st;
        g.dt = dt;
    }
    if (h->cuda(cudaGraphLaunch(g.exec, h->stream), "graph launch")) return SF_ERR_CUDA;
    h->launches += g.nodes;
    h->cur = 1 - h->cur;
    h->sorted = true;
    return SF_OK;
}

// The reverse substep of stored-substep slot t, replayed from a graph
// captured per slot (the adjoint buffers, partials and slabs are fixed).
sf_status runAdjSubstepGraphed(sf_handle* h, float dt, int64_t t) {
    if (h->storeGraphSlab != h->slab) {
        h->dropGraphs();
        h->storeGraphSlab = h->slab;
    }
    if (int64_t(h->adjGraph.size()) <= t) h->adjGraph.resize(size_t(t) + 1);
    GraphCache& g = h->adjGraph[size_t(t)];
    if (!g.exec || g.dt != dt) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        sf_status st = h->cuda(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (st) return st;
        const AdjSlab sl = slabAt(h, h->slab + size_t(t) * slabStride(h));
        g.nodes = launchAdjSubstep(h->ctx(), h->adj, slabBuffers(h, sl), sl.pid, dt, h->adjParam, h->lanes);
        const cudaError_t le = cudaGetLastError();
        const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
        if (h->cuda(le, "adjoint launch") || h->cuda(ce, "end capture")) {
            if (graph) cudaGraphDestroy(graph);
            return SF_ERR_CUDA;
        }
        st = h->cuda(cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
        cudaGraphDestroy(graph);
        if (st) return st;
        g.dt = dt;
    }
    if (h->cuda(cudaGraphLaunch(g.exec, h->stream), "graph launch")) return SF_ERR_CUDA;
    h->launches += g.nodes;
    return SF_OK;
}

sf_status growBuffer(sf_handle* h, char*& p, size_t& have, size_t need, const char* what) {
    if (have >= need) return SF_OK;
    if (p && h->cuda(cudaStreamSynchronize(h->stream), "sync before realloc")) return SF_ERR_CUDA;
    devFree(p);
    have = 0;
    if (h->cuda(cudaMalloc(reinterpret_cast<void**>(&p), need), what)) return SF_ERR_CUDA;
    have = need;
    return SF_OK;
}

sf_status ensureAdjoint(sf_handle* h, size_t snapshots, size_t slabs) {
    const size_t M = size_t(h->totalSlots);
    if (!h->adj.adjX) {
        for (float4** p : {&h->adj.adjX, &h->adj.adjV, &h->adj.x, &h->adj.v, &h->adj.acc, &h->adj.flow, &h->adj.adh,
                           &h->adj.avgadh, &h->adj.drag, &h->adj.f, &h->adj.r, &h->adj.s}) {
            if (h->cuda(cudaMalloc(reinterpret_cast<void**>(p), sizeof(float4) * M), "cudaMalloc adjoint") ||
                h->cuda(cudaMemsetAsync(*p, 0, sizeof(float4) * M, h->stream), "cudaMemset adjoint"))
                return SF_ERR_CUDA;
        }
        if (h->cuda(cudaMalloc(reinterpret_cast<void**>(&h->adjTarget), sizeof(float) * 3 * M), "cudaMalloc target") ||
            h->cuda(cudaMalloc(reinterpret_cast<void**>(&h->adjParam),
                               sizeof(float) * 3 * size_t(h->slotBlocks) * sf_handle::kMaxLanes),
                    "cudaMalloc param partials") ||
            h->cuda(cudaMalloc(reinterpret_cast<void**>(&h->adjLoss), sizeof(float2) * size_t(h->slotBlocks)),
                    "cudaMalloc loss partials") ||
            h->cuda(cudaMemsetAsync(h->adjTarget, 0, sizeof(float) * 3 * M, h->stream), "cudaMemset target"))
            return SF_ERR_CUDA;
    }
    if (growBuffer(h, h->snap, h->snapBytes, snapshots * snapStride(h), "cudaMalloc snapshots")) return SF_ERR_CUDA;
    if (growBuffer(h, h->slab, h->slabBytes, slabs * slabStride(h),
                   "cudaMalloc stored substeps (lower checkpoint_every to use less memory)"))
        return SF_ERR_CUDA;
    return SF_OK;
}

}  // namespace

sf_status sf_adjoint_run(sf_handle* h, float dt, int64_t n_substeps, int64_t checkpoint_every,
                         const float* target_pos, float* loss_out, float* grad_params_out, float* grad_pos0_out,
                         float* grad_vel0_out, float* ms_out) {
    if (!h) return SF_ERR_INVALID;
    if (!target_pos || !loss_out) return h->fail(SF_ERR_INVALID, "target_pos and loss_out are required");
    if (!(dt > 0.f) || !std::isfinite(dt)) return h->fail(SF_ERR_INVALID, "dt must be finite and > 0");
    if (n_substeps < 1) return h->fail(SF_ERR_INVALID, "n_substeps must be >= 1");
    if (checkpoint_every < 1) return h->fail(SF_ERR_INVALID, "checkpoint_every must be >= 1");
    const int64_t T = n_substeps, K = std::min(checkpoint_every, n_substeps);
    const int64_t nSeg = (T + K - 1) / K;
    const int64_t lastLen = T - (nSeg - 1) * K;
    // lists found full by earlier calls grow first (the stored substeps are sized by the capacity)
    if (sf_status gs = growListsIfFull(h, -1)) return gs;
    // snapshots: segment starts [0, nSeg - 1) and the final state; slabs: one segment
    if (ensureAdjoint(h, size_t(nSeg), size_t(K))) return SF_ERR_CUDA;
    const size_t sStride = snapStride(h);
    auto snapAt = [&](int64_t k) { return h->snap + size_t(k) * sStride; };
    char* finalSnap = snapAt(nSeg - 1);

    // targets into the slot_off + id layout
    int64_t off = 0;
    for (int s = 0; s < h->nScenes; ++s) {
        const int64_t n = h->n[s];
        if (n > 0 && h->cuda(cudaMemcpyAsync(h->adjTarget + 3 * size_t(h->hScenes[s].slot_off), target_pos + 3 * off,
                                             sizeof(float) * 3 * size_t(n), cudaMemcpyHostToDevice, h->stream),
                             "target H2D"))
            return SF_ERR_CUDA;
        off += n;
    }
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    for (auto& e : ev)
        if (h->cuda(cudaEventCreate(&e), "event create")) return SF_ERR_CUDA;
    struct EventGuard {
        cudaEvent_t* e;
        ~EventGuard() {
            for (int k = 0; k < 3; ++k)
                if (e[k]) cudaEventDestroy(e[k]);
        }
    } guard{ev};
    cudaEventRecord(ev[0], h->stream);

    // forward: a checkpoint at the start of every segment but the last, whose
    // substeps are stored as they run
    sf_status st = SF_OK;
    for (int64_t seg = 0; seg + 1 < nSeg; ++seg) {
        if ((st = snapCopy(h, snapAt(seg), true))) return st;
        if ((st = sf_substeps_fixed(h, dt, K))) return st;
    }
    for (int64_t t = 0; t < lastLen; ++t)
        if ((st = runSubstepStoreGraphed(h, dt, t))) return st;
    launchAdjSeed(h->ctx(), h->pos[h->cur], h->pid[h->cur], h->adjTarget, h->adj.adjX, h->adj.adjV, h->adjLoss);
    h->launches += 1;
    if ((st = snapCopy(h, finalSnap, true))) return st;
    if (h->cuda(cudaMemsetAsync(h->adjParam, 0, sizeof(float) * 3 * size_t(h->adjBlocks()), h->stream),
                "clear parameter partials"))
        return SF_ERR_CUDA;
    cudaEventRecord(ev[1], h->stream);

    // reverse, segment by segment: recompute and store a segment, then run
    // its substeps' adjoints backwards
    for (int64_t seg = nSeg - 1; seg >= 0; --seg) {
        const int64_t len = seg == nSeg - 1 ? lastLen : K;
        if (seg != nSeg - 1) {
            if ((st = snapCopy(h, snapAt(seg), false))) return st;
            for (int64_t t = 0; t < len; ++t)
                if ((st = runSubstepStoreGraphed(h, dt, t))) return st;
        }
        for (int64_t t = len - 1; t >= 0; --t)
            if ((st = runAdjSubstepGraphed(h, dt, t))) return st;
    }
    cudaEventRecord(ev[2], h->stream);
    if ((st = snapCopy(h, finalSnap, false))) return st;

    // per-scene reductions in block order, and the id-ordered gradients
    std::vector<float2> lossPart(size_t(h->slotBlocks));
    std::vector<float> paramPart(3 * size_t(h->adjBlocks()));
    std::vector<float4> gx, gv;
    if (h->cuda(cudaMemcpyAsync(lossPart.data(), h->adjLoss, sizeof(float2) * lossPart.size(), cudaMemcpyDeviceToHost,
                                h->stream),
                "loss D2H") ||
        h->cuda(cudaMemcpyAsync(paramPart.data(), h->adjParam, sizeof(float) * paramPart.size(),
                                cudaMemcpyDeviceToHost, h->stream),
                "parameter gradient D2H") ||
        h->cuda(cudaStreamSynchronize(h->stream), "adjoint sync"))
        return SF_ERR_CUDA;
    off = 0;
    for (int s = 0; s < h->nScenes; ++s) {
        const SceneDev& S = h->hScenes[s];
        double l = 0.0, ns = 0.0, g[3] = {0.0, 0.0, 0.0};
        for (int b = S.slot_off / kSlotAlign; b < (S.slot_off + S.slot_cap) / kSlotAlign; ++b) {
            l += lossPart[size_t(b)].x;
            ns += lossPart[size_t(b)].y;
        }
        for (int b = S.slot_off / kSlotAlign * h->lanes; b < (S.slot_off + S.slot_cap) / kSlotAlign * h->lanes; ++b)
            for (int k = 0; k < 3; ++k) g[k] += paramPart[3 * size_t(b) + size_t(k)];
        const double inv = ns > 0.0 ? 1.0 / ns : 0.0;
        loss_out[s] = float(l * inv);
        // the cotangents were seeded with adj_seed_scale x dL/dx: take it out
        const double ginv = inv / double(S.adj_seed_scale);
        if (grad_params_out)
            for (int k = 0; k < 3; ++k) grad_params_out[3 * s + k] = float(g[k] * ginv);
        const int64_t n = h->n[s];
        for (int which = 0; which < 2; ++which) {
            float* out = which ? grad_vel0_out : grad_pos0_out;
            if (!out || n == 0) continue;
            std::vector<float4>& buf = which ? gv : gx;
            buf.resize(size_t(n));
            if (h->cuda(cudaMemcpyAsync(buf.data(), (which ? h->adj.adjV : h->adj.adjX) + S.slot_off,
                                        sizeof(float4) * size_t(n), cudaMemcpyDeviceToHost, h->stream),
                        "gradient D2H") ||
                h->cuda(cudaStreamSynchronize(h->stream), "gradient sync"))
                return SF_ERR_CUDA;
            for (int64_t i = 0; i < n; ++i) {
                out[3 * (off + i)] = float(double(buf[size_t(i)].x) * ginv);
                out[3 * (off + i) + 1] = float(double(buf[size_t(i)].y) * ginv);
                out[3 * (off + i) + 2] = float(double(buf[size_t(i)].z) * ginv);
            }
        }
        off += n;
    }
    if (ms_out) {
        cudaEventElapsedTime(&ms_out[0], ev[0], ev[1]);
        cudaEventElapsedTime(&ms_out[1], ev[1], ev[2]);
    }
    queueStateCopy(h);
    return h->cuda(cudaGetLastError(), "sf_adjoint_run");
}

}  // extern "C"
