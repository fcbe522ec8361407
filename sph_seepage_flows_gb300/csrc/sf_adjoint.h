// Host-side launch interface of the reverse-mode adjoint of the fixed-dt
// substep (sf_adjoint.cu).
#pragma once

#include "sf_kernels.h"

namespace sfg {

// Cotangent buffers. adjX / adjV are indexed by scene slot_off + particle id
// (they survive the sort); the rest are per slot of the current substep.
struct AdjBuffers {
    float4* adjX;    // d loss / d position: of the substep's output on entry, of its input on exit
    float4* adjV;    // d loss / d velocity, same convention
    float4* x;       // per slot: cotangent of the substep's input position
    float4* v;       // per slot: cotangent of the substep's input velocity
    float4* acc;     // cotangent of the momentum passes' acceleration
    float4* flow;    // sand: cotangent of the average flow velocity
    float4* adh;     // water: cotangent of the adhesion force
    float4* avgadh;  // water: cotangent of the average adhesion force
    float4* drag;    // sand: cotangent of the average drag force
    float4* f;       // sand: (cotangent of the force sum f, cotangent of v_w)
    float4* r;       // per-level scratch (ratios of the quotient fields)
    float4* s;       // (density, pressure, voidage, saturation) cotangents
};

// Everything the adjoint of one substep reads, stored by its forward pass:
// the neighbour lists, the cell table and the per-slot fields in sorted
// order as they stand after the water-momentum pass (before integration).
struct AdjSlab {
    unsigned int* cnt;
    unsigned int* nbr;
    int* bcnt;
    unsigned int* bnbr;
    int* ccnt;
    unsigned int* cnbr;
    unsigned int* cs;
    float4 *aux, *flow, *drag, *acc, *adh, *avgadh, *pos, *vel, *mat;
    float2* dp;
    int* pid;
};
// Copies the fields the integrator overwrites (pos, vel, acc, adhesion,
// average adhesion) and the sorted mat / pid into the slab.
void launchAdjStore(const LaunchCtx& c, const PassBuffers& b, const int* pid, const AdjSlab& s);

// Seeds adjX / adjV from L = mean over sand of |x - target|^2 (target indexed
// like adjX), written unnormalised (2 (x - target)); lossPartial[block] =
// (sum of |x - target|^2 over the block's sand, sand count).
void launchAdjSeed(const LaunchCtx& c, const float4* pos4, const int* pid, const float* target, float4* adjX,
                   float4* adjV, float2* lossPartial);
// One substep's adjoint, run after the forward stages sort .. water momentum
// of that substep were recomputed into b. Adds the block partials of the
// parameter cotangents (tan friction angle, capillary scale, permeability
// scale) into paramPartial[3 * block + k]. Returns kernels launched.
// lanes: threads per slot of the pair kernels (1, 2, 4 or 8; lanesForSlots);
// paramPartial holds 3 floats per block of the pair kernels, i.e. lanes
// blocks per kSlotAlign slots.
int launchAdjSubstep(const LaunchCtx& c, const AdjBuffers& A, const PassBuffers& b, const int* pid, float dt,
                     float* paramPartial, int lanes);

}  // namespace sfg
