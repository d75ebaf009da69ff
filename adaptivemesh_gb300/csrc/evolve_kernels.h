// evolve_kernels.h -- launch interfaces of the evolution kernels (kernels_evolve.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "evolve.h"

namespace amr {

// Analytic initial data on every cell of the first `used` slots, into three buffer sets (the root's
// ghost layer, the outer boundary, is never refilled, so every state buffer holds it).
struct EvoInitArgs {
    float* out1[kMaxFields];
    float* out2[kMaxFields];
    float* out3[kMaxFields];
    const uint32_t* positions;
    uint32_t used, n, t;
    int nf, physics;
    float outer_size;
    InitData id;
};

// Ghost fill of X (the state being filled) for the faces normal to `axis` of the listed slots.
struct EvoGhostArgs {
    float* X[kMaxFields];
    const float* old_f[kMaxFields];
    const float* new_f[kMaxFields];
    const uint64_t* boundaries;
    const uint8_t* evolved;       // per slot: 1 if the slot is evolved (not covered by eight children)
    const uint32_t* items;
    uint32_t n_items;
    uint32_t n, p, t;
    uint32_t substep, max_depth;
    int axis;
    int nf;
    float c_stage;                // time of the state being filled, as a fraction of the target's step
    uint32_t interp_floats;       // shared memory of the interpolating faces (set by the launcher)
    int* err;                     // raised when a face needs more than that
};

// Device addresses of the four constraint buffers (H, M_x, M_y, M_z; inner layout).
struct ConsPtrs {
    float* c[4];
};

// Restriction of the listed slots: old <- new, child-covered cells from the child (fourth order).
struct EvoRestrictArgs {
    float* old_f[kMaxFields];
    const float* new_f[kMaxFields];
    const int32_t* children;
    const uint32_t* items;
    uint32_t n_items;
    uint32_t n, p, t;
    int nf;
    int fgroup;   // fields per CTA: the grid's y extent is ceil(nf / fgroup)
};
// Fields per CTA when restricting domains with children: each covered cell costs 64 loads per field,
// so those CTAs take few fields and many run side by side (the leaves' straight copies take all).
constexpr int kEvoRestrictGroup = 4;

// Tile features of the learned estimator and the plain criterion's indicator, per listed slot
// (kernels_evolve.cu, k_evo_features): features [slot][3][8^3], indicator [slot].
struct EvoFeatureArgs {
    const float* state[kMaxFields];
    const uint32_t* positions;
    const uint32_t* items;
    uint32_t n_items;
    uint32_t n, p, t;
    float outer_size;
    float* features;
    float* indicator;
};
cudaError_t launch_evo_features(const EvoFeatureArgs& g, cudaStream_t st);

// Prolongation of new domains: every padded cell of each listed child, in every buffer, by tricubic
// interpolation of its parent's padded cells.  The items of one launch share a depth.
struct EvoProlongArgs {
    float* bufs[2 * kMaxFields];
    const int32_t* items;   // (node, parent, offset) triples
    uint32_t n_items, nbuf;
    uint32_t n, p, t;
    int floor_buf[2];       // buffers whose values are kept at or above floor_val (-1: none)
    float floor_val;
    // per buffer: 0 interpolates the stored values; 2 and 4 interpolate the square and the fourth
    // root of (stored + 1) and raise the result back (the lapse and the conformal factor, stored
    // less 1, which fall to zero at a puncture as r^2 and r^4 while their roots stay smooth)
    signed char root[2 * kMaxFields];
};
cudaError_t launch_evo_prolong(const EvoProlongArgs& g, cudaStream_t st);

bool evo_config_supported(uint32_t n, uint32_t p);
cudaError_t launch_evo_restrict(const EvoRestrictArgs& g, cudaStream_t st);
cudaError_t launch_evo_init(const EvoInitArgs& a, cudaStream_t st);
cudaError_t launch_evo_derivs(const EvoArgs& a, cudaStream_t st);
// The derivative pass's compiled slab depths for size_domain n (written to out, at most 4); their count.
uint32_t evo_deriv_zs_candidates(uint32_t n, uint32_t* out);
cudaError_t launch_evo_rhs(const EvoArgs& a, cudaStream_t st);
cudaError_t launch_evo_ghost(const EvoGhostArgs& g, cudaStream_t st);
cudaError_t launch_evo_constraints(const EvoArgs& a, const ConsPtrs& cons, cudaStream_t st);
// FP64 norms of the constraints over the composite grid of the listed slots (interior cells no child
// covers), leaving out cells within the excision radius of a puncture: out[0] rms H, [1] max |H|,
// [2] rms |M|, [3] max |M|, [4] cells.  `part` holds 5 doubles per slot.
struct EvoNormArgs {
    ConsPtrs cons;
    const uint32_t* items;
    uint32_t n_items, n;
    const uint32_t* positions;
    const int32_t* children;
    float outer_size;
    float excision2;
    int n_punctures;
    float pos[4][3];
};
cudaError_t launch_evo_norms(const EvoNormArgs& g, double* part, double* out, cudaStream_t st);

}  // namespace amr
