/* amr_oracle.h -- CPU restatement of AdaptiveMesh's per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA kernels are compared with this restatement:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs
 * load it (through oracle/oracle.py).  The product never links or calls it.
 *
 * Every function restates one piece of the reference (file:line given beside it) in
 * plain C over the reference's own data layout:
 *   padded field  : slot*t^3 + (z*t + y)*t + x            (t = n + 2p), float
 *   inner field   : slot*n^3 + (z*n + y)*n + x            float or compressed_float3 (uint32)
 *   positions     : octree_abs_pos words (AMR.h:22-55)
 *   boundaries    : domain_boundary 8-byte words, 6 per slot (AMR.h:56-100)
 * Single-precision arithmetic follows the operation order of the reference's device
 * build (--use_fast_math: fused multiply-adds, flush-to-zero); see the ORC_* flags.
 * Build: gcc -O2 -ffp-contract=off -fopenmp (oracle/build_oracle.py).
 */
#ifndef AMR_ORACLE_H
#define AMR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint32_t n;          /* size_domain (interior edge)            AMR.h:11 */
    uint32_t p;          /* padding_domain (ghost width)           AMR.h:12 */
    float outer_size;    /* root edge length                       AMR.h:10 */
    float inv_dx[9];     /* 2^depth / outer_dx for depth 0..8      AMR.h:1176 */
    float outer_dt;      /* outer_dx * 0.4                         AMR.h:17 */
    float outer_dx;      /* outer_size / size_domain               AMR.h:16 */
    uint32_t flags;      /* ORC_* below */
} orc_cfg;

/* ORC_FUSED_NOISE: the stochastic codec adds its noise with one fused multiply-add instead of
 *                  a rounded product then a sum.  The reference's host build and its device
 *                  build's standalone encoder round the product (pinned on the device by
 *                  tests/golden/codec_fused_probe_inputs.npz); the encodes its device build
 *                  inlines into the stencil and Christoffel kernels fuse it (pinned against its
 *                  BSSN plugin on the 585-domain tree), so the kernel restatements run with it.
 * ORC_FTZ:         flush subnormal inputs/results of the codec to zero (device build). */
#define ORC_FUSED_NOISE 1u
#define ORC_FTZ 2u

void orc_cfg_init(orc_cfg* c, uint32_t n, uint32_t p, float outer_size, uint32_t flags);

/* ---- fast_prng (tensors.h:276-304) and compressed_float3 (tensors.h:305-394) ---- */
int32_t orc_prng_int(int32_t* state);
float orc_prng_float(int32_t* state);
int32_t orc_prng_ranged(int32_t* state, int32_t lo, int32_t hi);
uint32_t orc_cf3_encode(float x, float y, float z, int32_t* rng /* NULL: deterministic */, uint32_t flags);
void orc_cf3_decode(uint32_t w, float* xyz);
void orc_cf3_encode_seeded(const float* xyz, const int32_t* seeds, int64_t n, uint32_t* out, uint32_t flags);
int32_t orc_cf3_encode_stream(const float* xyz, int64_t n, int32_t seed, uint32_t* out, uint32_t flags);
void orc_cf3_encode_det(const float* xyz, int64_t n, uint32_t* out, uint32_t flags);
void orc_cf3_decode_n(const uint32_t* in, int64_t n, float* xyz);

/* ---- tensor algebra (tensors.h:133-244) ---- */
void orc_sym_inverse(const float* m6, float* out6);
float orc_sym_determinant(const float* m6);
float orc_trace_contra_sym(const float* c6, const float* m6);
void orc_sym_times_vec(const float* m6, const float* v3, float* out3);

/* ---- octree helpers (AMR.h:22-116) ---- */
uint32_t orc_reverse_bits(uint32_t a);
uint32_t orc_sum_coordinates(uint32_t a, uint32_t b, int overflow);
uint32_t orc_diff_coordinates(uint32_t a, uint32_t b, int overflow);
uint64_t orc_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx);

/* ---- kernels (all slots < used; inactive / unused slots are skipped) ---- */
/* __differentiate, AMR.h:1152-1219; d2if may be NULL (gradient-only variant) */
void orc_differentiate(const orc_cfg* c, const float* field, uint32_t* dif, uint32_t* d2if,
                       const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed);
/* __mixed_partials, AMR.h:1221-1266 */
void orc_mixed_partials(const orc_cfg* c, const float* field, uint32_t* off,
                        const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed);
/* __deriv_trace, BSSN.h:7-22; metric6 = six padded component buffers */
void orc_deriv_trace(const orc_cfg* c, const uint32_t* hess_diag, const uint32_t* hess_off, const float* const* metric6,
                     float* out, const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth);
/* __compute_raised_christoffel_symbols, BSSN.h:55-91.  mode 0 = as the reference (multiplies by the
 * metric), mode 1 = multiplies by the inverse metric. */
void orc_christoffel(const orc_cfg* c, const float* const* metric6, const uint32_t* const* derivs6, int32_t seed,
                     uint32_t* const* out6, const uint32_t* positions, uint32_t used, uint32_t substep,
                     uint32_t max_depth, int mode);
/* __copy_boundaries (Lagrange variant), AMR.h:634-762 */
void orc_copy_boundaries(const orc_cfg* c, float* old_f, float* new_f, const uint64_t* boundaries, uint32_t used,
                         uint32_t substep, uint32_t max_depth, int copy_only_new);
/* __copy_new_to_old, AMR.h:961-996 */
void orc_copy_new_to_old(const orc_cfg* c, float* old_f, const float* new_f, const uint32_t* positions,
                         const int32_t* children, uint32_t used, uint32_t substep, uint32_t max_depth);
/* __copy_to_child, AMR.h:1053-1073 */
void orc_copy_to_child(const orc_cfg* c, float* buf, uint32_t offset, int32_t child, int32_t parent);
/* __predictor_step / __corrector_step, SimpleWave.h:7-46 */
/* rasterise_to_image, AMR.h:1313-1365: width x height RGBA floats of the z = z_slice plane */
void orc_rasterise(const orc_cfg* c, const float* data, const int32_t* children, uint32_t width, uint32_t height,
                   float z_slice, int boxes, float* rgba);
void orc_wave_step(const orc_cfg* c, int corrector, const float* old_f, const uint32_t* derivs, const uint32_t* hess,
                   float* new_f, const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth);
/* __amr_criterion_1 and __amr_criterion_2, SimpleWave.h:91-139 */
void orc_criterion(const orc_cfg* c, const uint32_t* derivs, const uint32_t* hess, float* crit,
                   const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth);

/* ---- FP64 restatements (no quantisation), for error reports ---- */
void orc_differentiate_f64(const orc_cfg* c, const float* field, double* grad3, double* hdiag3, double* hoff3,
                           const uint32_t* positions, uint32_t used);

/* ---- one BSSN_AMR_data::timestep (BSSN.h:104-170) over a fixed octree ----
 * state: cyij_old[6], cyij_new[6] (padded), outputs cyij_k[6], cGijk[6] (cf3), cRij[6] (inner float).
 * *timer is the octree's timer_helper (AMR.h:178), *rng the plugin's fast_prng state (BSSN.h:106).
 * The substep loop runs until the timer wraps to 0, as BSSN.h:160-168.  `slot_begin/slot_end`
 * restrict the per-node work to a slot range (for bounded CPU samples); pass 0, used for all. */
void orc_bssn_timestep(const orc_cfg* c, float* const* old6, float* const* new6, uint32_t* const* dmet6,
                       uint32_t* const* chr6, float* const* ricci6, const uint32_t* positions, const int32_t* children,
                       const uint64_t* boundaries, uint32_t used, uint32_t max_depth, uint32_t* timer, int32_t* rng,
                       uint32_t slot_begin, uint32_t slot_end);

/* ---- the same timestep in double precision with no quantisation (oracle/fp64_path.c): the FP64
 * host oracle for error reports and the FP64 CPU stencil path.  old6/new6 padded doubles;
 * grad6[k], chr6[k]: 3 doubles per inner cell; ric6[k]: 1 double per inner cell.  Every slot. */
void orc_bssn_timestep_f64(const orc_cfg* c, double* const* old6, double* const* new6, double* const* grad6,
                           double* const* chr6, double* const* ric6, const uint32_t* positions,
                           const int32_t* children, const uint64_t* boundaries, uint32_t used, uint32_t max_depth,
                           uint32_t* timer);

/* ---- the evolution (oracle/bssn_evolve.c): the full BSSN system and the scalar wave, RK4 on the octree
 * with 2:1 subcycling, in double precision -- the FP64 host oracle of the GPU evolutions.  No
 * counterpart in the reference ("parity unpinned by the reference"). */
typedef struct {
    uint32_t n, p;          /* size_domain, padding_domain (3) */
    float outer_size;       /* root edge */
    int physics;            /* 0 BSSN, 1 scalar wave */
    int slicing;            /* 0: 1+log, 1: harmonic */
    int shift;              /* 0: frozen, 1: Gamma-driver */
    float eta, ko_sigma, cfl, chi_floor;
    int id_kind;            /* 0 flat, 1 gauge wave, 2 Brill-Lindquist, 3 Gaussian pulse */
    float amplitude, wavelength;
    int n_punctures;
    float mass[4];
    float pos[4][3];
    float width;
} orc_evo;
void orc_evo_initial_data(const orc_evo* e, double* const* fields, const uint32_t* positions, uint32_t used);
void orc_evo_timestep(const orc_evo* e, double* const* oldf, double* const* newf, double* const* stagef,
                      double* const* acc, const uint32_t* positions, const int32_t* children,
                      const uint64_t* boundaries, uint32_t used, uint32_t max_depth, uint32_t* timer);
void orc_evo_constraints(const orc_evo* e, double* const* fields, const uint32_t* positions, const int32_t* children,
                         uint32_t used, double excision, double* const* cons4, double* out5);
void orc_periodic_boundaries(const uint32_t* positions, const int32_t* children, uint32_t used, uint64_t* out);

/* parallel.h:10-82, 215-251, 385-421 -- the reference's scan and reductions over `n` elements of
 * `ncomp` values; dtype 0 uint32, 1 int32, 2 float32 (flushing subnormals as the device build).
 * The array ends as the reference leaves it; orc_extreme writes the result to `result`. */
void orc_scan(int dtype, int ncomp, void* data, uint32_t n);
void orc_extreme(int dtype, int ncomp, int is_max, void* data, uint32_t n, void* result);
int orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
