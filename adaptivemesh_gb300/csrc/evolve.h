// evolve.h -- full BSSN evolution (moving-puncture form) and the scalar wave u_tt = Δu on the
// octree of domains, the physics the reference's BSSN plugin stops short of: its BSSN_AMR_data
// only recomputes metric derivatives and Christoffel symbols (BSSN.h:143-159) and its one time
// integrator is SimpleWave's two-stage update (SimpleWave.h:7-46).  Everything here keeps the
// reference's data layout (padded domains slot*T^3, face boundary words, the 0..2^max_depth-1
// substep counter with 2:1 subcycling, AMR.h:634-644) and is checked against the FP64 oracle
// oracle/bssn_evolve.c.
//
// Scheme, per substep (the reference's counter; the domains active at it advance one step of
// their own dt = cfl * dx):
//   restriction   old <- new of every active domain; a cell covered by a child <- the child's state
//                 at the cell's centre by the 4-point midpoint rule along each axis (fourth order;
//                 the reference's 2x2x2 mean, AMR.h:961-996, is second order)
//   RK4           four stages over every active domain (covered parents included: a same-depth
//                 neighbour of a covered parent takes its ghost values from it at every stage):
//                 derivative pass, then pointwise right-hand side and stage update; the ghost cells
//                 of each stage's state and of the final state are filled from the neighbours
//                 (three passes, x then y then z, so that edges and corners are filled too)
//   ghost values  same-depth neighbour: its state at the same stage; coarser neighbour active at
//                 this substep: old + (its stage state - old) * 2^-Δdepth; coarser neighbour in the
//                 middle of its step: old + (new - old) * (k' + c_stage) / 2^Δdepth.  Space
//                 interpolation from a coarser neighbour is tricubic (the reference's 10-point
//                 quadratic rule, AMR.h:672-699, leaves O(h^3) ghost errors that second-derivative
//                 stencils turn into O(h)); same-depth values are copied.  The root's ghost layer
//                 keeps the initial data (the outer boundary) unless the root is periodic.
// Finite differences: 4th-order centred first and second derivatives (mixed ones as the product of
// first-derivative stencils), 6th-derivative Kreiss-Oliger dissipation (3 ghost cells needed).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "amr_types.h"

namespace amr {

// BSSN fields, one padded buffer each.
enum BssnField : int {
    F_CHI = 0,                    // conformal factor chi = det(gamma)^(-1/3)
    F_GXX = 1, F_GXY, F_GXZ, F_GYY, F_GYZ, F_GZZ,   // conformal metric (det 1)
    F_K = 7,                      // trace of the extrinsic curvature
    F_AXX = 8, F_AXY, F_AXZ, F_AYY, F_AYZ, F_AZZ,   // trace-free conformal extrinsic curvature
    F_GAMX = 14, F_GAMY, F_GAMZ,  // conformal connection functions
    F_ALPHA = 17,                 // lapse
    F_BETAX = 18, F_BETAY, F_BETAZ,   // shift
    F_BX = 21, F_BY, F_BZ,        // Gamma-driver auxiliary
    BSSN_NF = 24
};
// The BSSN fields are stored as their deviation from flat space: chi, the conformal metric's
// diagonal and the lapse less 1.  Derivatives, interpolation, restriction and the RK update are the
// same for both forms (the offsets are constants), but single-precision rounding then acts on the
// deviation (for a weak field ~1e-2 of the value), which lowers the rounding noise that second
// derivatives amplify by 1/dx^2 by the same factor.
__host__ __device__ constexpr float bssn_offset(int f) {
    return (f == 0 || f == 1 || f == 4 || f == 6 || f == 17) ? 1.f : 0.f;
}

// Wave equation fields: u and v = u_t.
enum WaveField : int { W_U = 0, W_V = 1, WAVE_NF = 2 };

constexpr int kMaxFields = 24;

// Derivative scratch written by the derivative pass, one float per inner cell each (slot * N^3 +
// cell).  Symmetric second derivatives in the order xx, yy, zz, xy, xz, yz; first derivatives
// x, y, z.  Where the right-hand side only uses a contraction with the inverse conformal metric,
// the pass stores the contraction: GLAP[ij] = gt^lm d_l d_m gt_ij, BELAP[i] = gt^jk d_j d_k beta^i,
// and DDIVB[j] = d_j d_k beta^k.  EXTRA[f] is the advection term beta^k d_k u_f plus the
// Kreiss-Oliger term of field f.
enum BssnDeriv : int {
    D_CHI1 = 0,                   // 3
    D_CHI2 = 3,                   // 6
    D_G1 = 9,                     // 6 components x 3
    D_GLAP = 27,                  // 6
    D_K1 = 33,                    // 3
    D_GAM1 = 36,                  // 3 components x 3: d_j Gamma^i at D_GAM1 + 3 i + j
    D_AL1 = 45,                   // 3
    D_AL2 = 48,                   // 6
    D_BE1 = 54,                   // 3 components x 3: d_j beta^i at D_BE1 + 3 i + j
    D_BELAP = 63,                 // 3
    D_DDIVB = 66,                 // 3
    D_EXTRA = 69,                 // 24
    BSSN_ND = 93,
    D_AT1 = 93,                   // constraint mode only: d_k A_ij at D_AT1 + 3 c + k (6 components)
    BSSN_ND_CONSTRAINTS = 111
};
enum WaveDeriv : int { WD_LAP = 0, WD_EXTRA = 1, WAVE_ND = 3 };

// Physics and gauge choices (the C ABI's amr_evolution, resolved).
struct EvoParams {
    int physics;          // 0 BSSN, 1 scalar wave
    int slicing;          // AMR_SLICING_*: 1+log (d_t alpha = -2 alpha K) or harmonic (-alpha^2 K)
    int shift;            // 0: frozen shift, 1: Gamma-driver
    float eta;            // Gamma-driver damping
    float ko_sigma;       // Kreiss-Oliger strength
    float cfl;            // dt = cfl * dx at every depth
    float chi_floor;      // chi is floored at this value where it divides
    float outer_size;     // edge of the root domain
};

// Analytic initial data (the C ABI's amr_initial_data, resolved).
struct InitData {
    int kind;             // AMR_ID_*
    float amplitude;      // gauge wave A
    float wavelength;     // gauge wave d (the root edge for a periodic box)
    int n_punctures;      // Brill-Lindquist punctures (<= 4)
    float mass[4];
    float pos[4][3];
    float width;          // Gaussian pulse width (wave equation)
};

// Per-call device arguments of the evolution kernels.
struct EvoArgs {
    float* fields[kMaxFields];    // stage input S (padded)
    float* out[kMaxFields];       // stage output (padded interior written)
    float* old_f[kMaxFields];     // state at the start of the step (padded)
    float* acc[kMaxFields];       // RK accumulator (inner layout)
    float* deriv;                 // derivative scratch: nd planes of slots * N^3 floats
    uint64_t deriv_stride;        // floats per derivative plane (slots * N^3)
    const uint32_t* positions;
    const uint32_t* items;        // active evolved slots
    uint32_t n_items;
    uint32_t n, p, t;             // size_domain, padding_domain, n + 2p
    float dt0;                    // dt at depth 0
    int stage;                    // 1..4
    int constraints;              // derivative pass: also store d_k A_ij
    uint32_t deriv_zs;            // derivative pass: interior z-planes per slab (0: the default)
    EvoParams prm;
    int* err;
};

}  // namespace amr
