// kernels.h -- launch interfaces of the GB300 kernels (host-callable, no device code).
#pragma once

#include <cstddef>
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "amr_types.h"

// Compiled (size_domain, padding_domain) pairs.  (28, 2) is the reference as shipped; (16, 3) and
// (32, 3) are the benchmark sizes; (8, 2) keeps small test cases cheap.
#define AMR_FOR_EACH_CONFIG(X) X(16, 3) X(28, 2) X(32, 3) X(8, 2)
// Pairs with the six-component fused kernel (six rings of 2p+2 padded planes, or of half-plane
// tiles for 32^3 domains).
#define AMR_FOR_EACH_BSSN_CONFIG(X) X(16, 3) X(28, 2) X(32, 3) X(8, 2)

namespace amr {

// cudaFuncSetAttribute(kernel, MaxDynamicSharedMemorySize) once per device: the attribute belongs
// to a device's context, so `mask` keeps one bit per device ordinal (< 64) where it is set.
// Concurrent first calls set it twice, which is harmless.
template <class K>
cudaError_t ensure_smem_limit(K* kernel, size_t bytes, std::atomic<uint64_t>& mask) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
    if (bit && (mask.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) mask.fetch_or(bit, std::memory_order_release);
    return e;
}

enum StencilKind { SK_GRAD = 0, SK_GRAD_HESS = 1, SK_MIXED = 2, SK_BSSN = 3 };

struct StencilArgs {
    const float* field[6];        // padded input components
    uint32_t* grad[6];            // compressed gradients (SK_GRAD, SK_GRAD_HESS: [0]; SK_BSSN: all six)
    uint32_t* hdiag;              // SK_GRAD_HESS: compressed diagonal Hessian
    uint32_t* hoff;               // SK_MIXED: compressed off-diagonal Hessian
    float* lap[6];                // SK_BSSN: g^kl d_k d_l g_ij per component (inner layout)
    uint32_t* chr[6];             // SK_BSSN: compressed Christoffel symbols
    int32_t seed_d[6];            // launch seeds of the derivative launches, per component
    int32_t seed_m[6];            // launch seeds of the mixed-partial launches, per component
    int32_t seed_c;               // launch seed of the Christoffel launch
    const int32_t* seed_ptr;      // if set, the seeds are read from device memory instead:
                                  // seed_d[k] = seed_ptr[2k], seed_m[k] = seed_ptr[2k+1], seed_c = seed_ptr[12]
    int christoffel_mode;         // AMR_CHRISTOFFEL_*
    const uint32_t* positions;    // octree_abs_pos per slot
    const uint32_t* items;        // domains to process (nullptr: item i is slot i)
    uint32_t n_items;
    // single-operator kinds: with zsplit > 1 (a divisor of N), every item is cut into zsplit
    // z-ranges, one work unit each (few items: spread over the grid); 0 or 1: whole items
    uint32_t zsplit;
    uint32_t substep, max_depth;
    Geo geo;
    int* err;                     // set to 1 if a bounded wait gave up
    // Restriction of leaves fused into the pass (SK_BSSN): with children set, a domain without
    // children reads its planes from leaf_src[k] and writes them to field[k] (old <- new,
    // AMR.h:961-996), while a domain with children reads field[k] (restricted beforehand).
    const float* leaf_src[6];
    const int32_t* children;
    // Failure-path test hooks of the fused pass (SK_BSSN), host-set, off when 0: spin_limit
    // replaces the polls a data wait may take before it gives up (kMaxSpins); with withhold = q + 1
    // the producer of every CTA skips its q-th plane request, so the waits on that plane run out.
    // Waits for copies already issued (the drain before a CTA leaves) always use kMaxSpins.
    uint32_t spin_limit;
    uint32_t withhold;
};

template <int N, int P, int KIND>
cudaError_t launch_stencil_t(const StencilArgs& a, uint32_t grid, cudaStream_t st);
template <int N, int P, int KIND>
size_t stencil_smem_bytes();

// Pointwise kernels (kernels_point.cu).  Sizes are run-time values; nothing is templated.
struct Dims {
    uint32_t n, p, t;             // size_domain, padding_domain, n + 2p
};
inline Dims make_dims(const amr_config& c) { return Dims{c.size_domain, c.padding_domain, c.size_domain + 2 * c.padding_domain}; }

cudaError_t launch_cf3_encode(const float* xyz, const int32_t* seeds, uint64_t n, uint32_t* out, cudaStream_t st);
cudaError_t launch_cf3_decode(const uint32_t* w, uint64_t n, float* xyz, cudaStream_t st);
cudaError_t launch_deriv_trace(Dims d, const uint32_t* hd, const uint32_t* ho, float* const* metric6, float* out,
                               const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth,
                               cudaStream_t st);
cudaError_t launch_christoffel(Dims d, float* const* metric6, uint32_t* const* der6, int32_t seed, uint32_t* const* out6,
                               const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, int mode,
                               cudaStream_t st);
cudaError_t launch_wave_step(Dims d, const Geo& g, int corrector, const float* old_f, const uint32_t* der,
                             const uint32_t* hess, float* new_f, const uint32_t* positions, uint32_t used,
                             uint32_t substep, uint32_t max_depth, cudaStream_t st);
cudaError_t launch_rasterise(Dims d, const float* data, const int32_t* children, uint32_t used, uint32_t width,
                             uint32_t height, float z_slice, int boxes, float* raster, cudaStream_t st);
// Write n words into device memory with kernels that carry them as launch parameters (1 000 per
// launch; *launched counts the launches): a small upload that never queues on a copy engine
// behind bulk transfers.
cudaError_t launch_store_words(int32_t* dst, const int32_t* words, uint32_t n, cudaStream_t st, uint32_t* launched);
// Device-to-device copy of n 4-byte words (128-bit accesses where both addresses allow), one launch.
cudaError_t launch_copy_words(void* dst, const void* src, uint64_t n, cudaStream_t st);
// Up to kMax device-to-device copies of n 4-byte words in one launch (16-byte aligned buffers).
struct CopyList {
    static constexpr uint32_t kMax = 36;
    struct Item {
        void* dst;
        const void* src;
        uint64_t n;
    } item[kMax];
    uint32_t n = 0;
};
cudaError_t launch_copy_many(const CopyList& l, cudaStream_t st);
cudaError_t launch_criterion(Dims d, const Geo& g, const uint32_t* der, const uint32_t* hess, float* crit,
                             const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth,
                             cudaStream_t st);

// Restriction / prolongation / ghost fill (kernels_amr.cu).  `ncomp` components are processed in
// one launch (component k at fields_old[k], fields_new[k]).
struct FieldSet {
    float* old_f[6];
    float* new_f[6];
    int ncomp;
};
cudaError_t launch_copy_new_to_old(Dims d, const FieldSet& f, const uint32_t* positions, const int32_t* children,
                                   const uint32_t* items, uint32_t n_items, uint32_t substep, uint32_t max_depth,
                                   cudaStream_t st, bool parents_only = false);
cudaError_t launch_copy_to_child(Dims d, float* buf, uint32_t offset, int32_t child, int32_t parent, cudaStream_t st);
// Prolongation of n_items new nodes at once into each of nbuf (<= 12) buffers; items holds
// (child, parent, offset) triples in device memory, none a parent of another.
// FP64 norms of a padded field over the leaf domains' interior cells (reduce.cu): out4 = sum, sum
// of squares, largest magnitude, cell count; synchronises the stream; returns an AMR_* status.
int field_norms(uint32_t n, uint32_t p, const float* field, const uint32_t* positions, const int32_t* children,
                uint32_t used, double* out4, cudaStream_t st);
cudaError_t launch_copy_to_children(Dims d, float* const* bufs, int nbuf, const int32_t* items, uint32_t n_items,
                                    cudaStream_t st);
// Staging for the ghost fill (the innermost layer of the three lower faces, old and new):
// 2 * ncomp * 3 * n^2 floats per slot.
size_t ghost_scratch_floats(Dims d, uint32_t used, int ncomp);
// sources_restricted: the caller guarantees that every domain active at `substep` has had old <- new
// (restriction) since its new field last changed -- as inside a plugin's timestep, whose phase
// order is restriction, predictor, ghost fill.  A copy_only_new fill then reads the innermost lower
// layer of an active source's new field from old (equal before the fill) and writes every ghost
// value in place, in one launch without staging.
cudaError_t launch_copy_boundaries(Dims d, const FieldSet& f, const uint64_t* boundaries, uint32_t used,
                                   uint32_t substep, uint32_t max_depth, int copy_only_new, float* scratch,
                                   cudaStream_t st, bool sources_restricted = false);

}  // namespace amr
