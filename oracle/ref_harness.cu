// ref_harness.cu -- extern "C" access to the reference's own code for parity checks.
//
// TEST INFRASTRUCTURE ONLY: this builds the reference-build library oracle/_ref/libamr_ref_<cfg>.so
// from the reference's unmodified headers (staged by oracle/build_ref.py).  Only the
// tests, the smoke check and the benchmark's reference leg load it; the product never does.
//
// Host entry points (refh_*) run the reference's __host__ __device__ code on the CPU:
// fast_prng (AdaptiveMesh/tensors.h:276-304), compressed_float3 (tensors.h:305-394),
// float3x3_sym algebra (tensors.h:133-244) and the octree AMR<T> (AMR.h:118-294).
// Device entry points (refd_*) launch the reference's __global__ kernels with the
// launch shapes of the reference's own wrappers (AMR.h:880-1310, BSSN.h:24-102,
// SimpleWave.h:48-150), and drive whole BSSN_AMR_data / wave_AMR_data plugins.
// Build flags follow the reference's Release configuration (--use_fast_math,
// AdaptiveMesh.vcxproj:79-84).
#include "ref_shim.h"
#include "AMR.h"
#include "BSSN.h"
#include "SimpleWave.h"
#include "parallel.h"

#include <cstdint>

#define REF_API extern "C" __attribute__((visibility("default")))

static_assert(sizeof(compressed_float3) == 4, "cf3 size");
static_assert(sizeof(domain_boundary) == 8, "domain_boundary size");
static_assert(sizeof(octree_abs_pos) == 4, "octree_abs_pos size");

// ------------------------------------------------------------------ constants
REF_API void refh_constants(uint32_t* u4, float* f3) {
    u4[0] = size_domain; u4[1] = padding_domain; u4[2] = total_size_domain; u4[3] = depth_limit;
    f3[0] = outer_size; f3[1] = outer_dx; f3[2] = outer_dt;
}

// ------------------------------------------------------------------ host PRNG / codec
REF_API void refh_prng_ints(int32_t seed, int n, int32_t* out) {
    fast_prng r(seed);
    for (int i = 0; i < n; i++) out[i] = r.generate_int();
}
REF_API void refh_prng_floats(int32_t seed, int n, float* out) {
    fast_prng r(seed);
    for (int i = 0; i < n; i++) out[i] = r.generate_float();
}
REF_API void refh_prng_ranged(int32_t seed, int n, int32_t lo, int32_t hi, int32_t* out) {
    fast_prng r(seed);
    for (int i = 0; i < n; i++) out[i] = r.generate_int(lo, hi);
}
// One generator shared by consecutive encodes (as inside a kernel thread).
REF_API int32_t refh_cf3_encode_stream(const float* xyz, int n, int32_t seed, uint32_t* out) {
    fast_prng r(seed);
    for (int i = 0; i < n; i++)
        out[i] = compressed_float3(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), r).data;
    return r.seed;
}
// A fresh generator per element, seeded by seeds[i].
REF_API void refh_cf3_encode_seeded(const float* xyz, const int32_t* seeds, int n, uint32_t* out) {
    for (int i = 0; i < n; i++) {
        fast_prng r(seeds[i]);
        out[i] = compressed_float3(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), r).data;
    }
}
REF_API void refh_cf3_encode_det(const float* xyz, int n, uint32_t* out) {
    for (int i = 0; i < n; i++)
        out[i] = compressed_float3(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2])).data;
}
REF_API void refh_cf3_decode(const uint32_t* in, int n, float* xyz) {
    for (int i = 0; i < n; i++) {
        compressed_float3 c; c.data = in[i];
        float3 v = (float3)c;
        xyz[3 * i] = v.x; xyz[3 * i + 1] = v.y; xyz[3 * i + 2] = v.z;
    }
}

// ------------------------------------------------------------------ octree (host)
REF_API uint32_t refh_sum_coordinates(uint32_t a, uint32_t b, int overflow) { return yield_sum_coordinates(a, b, overflow != 0); }
REF_API uint32_t refh_diff_coordinates(uint32_t a, uint32_t b, int overflow) { return yield_diff_coordinates(a, b, overflow != 0); }
REF_API uint32_t refh_reverse_bits(uint32_t a) { return reverse_bits(a); }
REF_API void refh_abs_position(uint32_t pos, float* out3) {
    octree_abs_pos p; p.data = pos;
    float3 v = p.absolute_central_position();
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}
REF_API uint64_t refh_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx) {
    octree_abs_pos a, b; a.data = this_pos; b.data = other_pos;
    domain_boundary d(a, b, other_idx);
    uint64_t raw; memcpy(&raw, &d, 8);
    return raw;
}
REF_API void refh_boundary_decode(uint64_t raw, int32_t* target, uint32_t* depth_diff, int32_t* curr_depth,
                                  float* rel_scale, float* rel_pos3) {
    domain_boundary d; memcpy(&d, &raw, 8);
    *target = d.target_idx(); *depth_diff = d.depth_diff(); *curr_depth = d.curr_depth();
    *rel_scale = d.rel_scale();
    float3 r = d.rel_pos_t(); rel_pos3[0] = r.x; rel_pos3[1] = r.y; rel_pos3[2] = r.z;
}

// AMR<T> never initialises timer_helper (AMR.h:178, constructor AMR.h:189-191); this harness
// starts it at 0, the value a fresh timestep loop assumes.
struct RefOctree { AMR<blank_AMR_data> amr; explicit RefOctree(uint32_t s) : amr(s) { amr.timer_helper = 0u; } };
REF_API void* refh_octree_create(uint32_t slots) { return new RefOctree(slots); }
REF_API void refh_octree_destroy(void* h) { delete (RefOctree*)h; }
REF_API void refh_octree_add_node(void* h, int32_t parent, int32_t offset) { ((RefOctree*)h)->amr.add_node(parent, offset); }
REF_API void refh_octree_remove_node(void* h, int32_t idx) { ((RefOctree*)h)->amr.remove_node(idx); }
REF_API void refh_octree_increment_timer(void* h) { ((RefOctree*)h)->amr.increment_timer(); }
REF_API uint32_t refh_octree_find_node_idx(void* h, uint32_t packed, uint32_t maxd) {
    return ((RefOctree*)h)->amr.find_node_idx(packed, maxd);
}
template <class A>
static void dump_octree(A& amr, uint32_t* positions, int32_t* parent, int32_t* children, uint64_t* boundaries,
                        uint32_t* lifetime, uint32_t* scalars) {
    const uint32_t s = amr.max_slots;
    if (positions) memcpy(positions, amr.positions.cpu_buffer_ptr, s * 4);
    if (parent) memcpy(parent, amr.parent_idx_b.cpu_buffer_ptr, s * 4);
    if (children) memcpy(children, amr.children_idx_b.cpu_buffer_ptr, s * 32);
    if (boundaries) memcpy(boundaries, amr.boundaries.cpu_buffer_ptr, s * 48);
    if (lifetime) memcpy(lifetime, amr.lifetime.cpu_buffer_ptr, s * 4);
    if (scalars) {
        scalars[0] = amr.timer_helper; scalars[1] = (uint32_t)amr.read_max_depth();
        scalars[2] = amr.read_first_free_slot(); scalars[3] = amr.curr_used_slots(); scalars[4] = amr.max_slots;
    }
}
REF_API void refh_octree_state(void* h, uint32_t* positions, int32_t* parent, int32_t* children, uint64_t* boundaries,
                               uint32_t* lifetime, uint32_t* scalars) {
    dump_octree(((RefOctree*)h)->amr, positions, parent, children, boundaries, lifetime, scalars);
}

// ------------------------------------------------------------------ host tensor algebra
REF_API void refh_sym_inverse(const float* m6, int n, float* out6) {
    for (int i = 0; i < n; i++) {
        const float* a = m6 + 6 * i;
        float3x3_sym s(a[0], a[1], a[2], a[3], a[4], a[5]);
        float3x3_sym r = s.inverse();
        float* o = out6 + 6 * i;
        o[0] = r.xx; o[1] = r.xy; o[2] = r.xz; o[3] = r.yy; o[4] = r.yz; o[5] = r.zz;
    }
}

// ------------------------------------------------------------------ device: codec
__global__ void k_ref_cf3_encode_seeded(const float* xyz, const int32_t* seeds, int n, uint32_t* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fast_prng r(seeds[i]);
    out[i] = compressed_float3(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), r).data;
}
__global__ void k_ref_cf3_encode_det(const float* xyz, int n, uint32_t* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = compressed_float3(make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2])).data;
}
__global__ void k_ref_cf3_decode(const uint32_t* in, int n, float* xyz) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    compressed_float3 c; c.data = in[i];
    float3 v = (float3)c;
    xyz[3 * i] = v.x; xyz[3 * i + 1] = v.y; xyz[3 * i + 2] = v.z;
}
__global__ void k_ref_prng_floats(const int32_t* seeds, int n, int draws, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fast_prng r(seeds[i]);
    for (int k = 0; k < draws; k++) out[(size_t)i * draws + k] = r.generate_float();
}
__global__ void k_ref_sym_inverse(const float* m6, int n, float* out6) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* a = m6 + 6 * i;
    float3x3_sym r = float3x3_sym(a[0], a[1], a[2], a[3], a[4], a[5]).inverse();
    float* o = out6 + 6 * i;
    o[0] = r.xx; o[1] = r.xy; o[2] = r.xz; o[3] = r.yy; o[4] = r.yz; o[5] = r.zz;
}
// Probes of the reference's __device__ helpers on arbitrary inputs, compiled with the
// same flags as its kernels; used to pin the operation order of the oracle.
// kind 0: float3x3_sym * float3 (tensors.h:201-206); in = 6 metric + 3 vector, out = 3
// kind 1: trace_contra(sym, sym) (tensors.h:241-244); in = 6 + 6, out = 1
// kind 3: (1u << depth) / outer_dx as in __differentiate (AMR.h:1176); in = depth, out = 1
// kind 4: length(float3) (helper_math.h) as in __amr_criterion_1; in = 3, out = 1
// kind 5: float3x3_sym::determinant (tensors.h:208-210); in = 6, out = 1
__global__ void k_ref_probe(int kind, const float* in, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (kind == 0) {
        const float* a = in + 9 * i;
        float3 r = float3x3_sym(a[0], a[1], a[2], a[3], a[4], a[5]) * make_float3(a[6], a[7], a[8]);
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    } else if (kind == 1) {
        const float* a = in + 12 * i;
        out[i] = trace_contra(float3x3_sym(a[0], a[1], a[2], a[3], a[4], a[5]),
                              float3x3_sym(a[6], a[7], a[8], a[9], a[10], a[11]));
    } else if (kind == 3) {
        uint depth = (uint)in[i];
        out[i] = (1u << depth) / outer_dx;
    } else if (kind == 4) {
        const float* a = in + 3 * i;
        out[i] = length(make_float3(a[0], a[1], a[2]));
    } else if (kind == 5) {
        const float* a = in + 6 * i;
        out[i] = float3x3_sym(a[0], a[1], a[2], a[3], a[4], a[5]).determinant();
    }
}
static int blocks_for(int n) { return (n + 255) / 256; }
// Launch errors (e.g. an empty grid) are reported before asynchronous execution errors.
static int launch_status() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    return (int)cudaDeviceSynchronize();
}
REF_API int refd_probe(int kind, const float* in, int n, float* out) {
    if (n <= 0) return 0;
    k_ref_probe<<<(n + 63) / 64, 64>>>(kind, in, n, out);
    return launch_status();
}
REF_API int refd_cf3_encode_seeded(const float* xyz, const int32_t* seeds, int n, uint32_t* out) {
    if (n <= 0) return 0;
    k_ref_cf3_encode_seeded<<<blocks_for(n), 256>>>(xyz, seeds, n, out);
    return launch_status();
}
REF_API int refd_cf3_encode_det(const float* xyz, int n, uint32_t* out) {
    if (n <= 0) return 0;
    k_ref_cf3_encode_det<<<blocks_for(n), 256>>>(xyz, n, out);
    return launch_status();
}
REF_API int refd_cf3_decode(const uint32_t* in, int n, float* xyz) {
    if (n <= 0) return 0;
    k_ref_cf3_decode<<<blocks_for(n), 256>>>(in, n, xyz);
    return launch_status();
}
REF_API int refd_prng_floats(const int32_t* seeds, int n, int draws, float* out) {
    if (n <= 0) return 0;
    k_ref_prng_floats<<<blocks_for(n), 256>>>(seeds, n, draws, out);
    return launch_status();
}
REF_API int refd_sym_inverse(const float* m6, int n, float* out6) {
    if (n <= 0) return 0;
    k_ref_sym_inverse<<<blocks_for(n), 256>>>(m6, n, out6);
    return launch_status();
}

// ------------------------------------------------------------------ device: operator kernels
// Each launcher reproduces the grid/block shape of the reference wrapper named beside it.
static inline dim3 stencil_threads() { return dim3(threadsA3_v, threadsB3_v, threadsD3_v); }
static inline dim3 stencil_blocks(uint32_t used) {
    dim3 t = stencil_threads();
    return dim3(size_domain / t.x, size_domain / t.y, used * size_domain / t.z);
}

// differentiate, AMR.h:1280-1302
REF_API int refd_differentiate(const float* field, uint32_t* dif, uint32_t* d2if, const uint32_t* positions,
                               uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed) {
    if (d2if)
        __differentiate<<<stencil_blocks(used), stencil_threads()>>>(field, (compressed_float3*)dif, (compressed_float3*)d2if,
            (const octree_abs_pos*)positions, substep, max_depth, seed);
    else
        __differentiate<<<stencil_blocks(used), stencil_threads()>>>(field, (compressed_float3*)dif,
            (const octree_abs_pos*)positions, substep, max_depth, seed);
    return launch_status();
}
// mixed_partials, AMR.h:1268-1278
REF_API int refd_mixed_partials(const float* field, uint32_t* off, const uint32_t* positions,
                                uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed) {
    __mixed_partials<<<stencil_blocks(used), stencil_threads()>>>(field, (compressed_float3*)off,
        (const octree_abs_pos*)positions, substep, max_depth, seed);
    return launch_status();
}
// scalar_laplacian_noncovariant's third launch, BSSN.h:31-35
REF_API int refd_deriv_trace(const uint32_t* hess_diag, const uint32_t* hess_off, float* const* metric6, float* out,
                             const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    comp_tensor2_sym_ptrs h((compressed_float3*)hess_diag, (compressed_float3*)hess_off);
    tensor2_sym_ptrs m(metric6[0], metric6[1], metric6[2], metric6[3], metric6[4], metric6[5]);
    __deriv_trace<<<stencil_blocks(used), stencil_threads()>>>(h, m, out, (const octree_abs_pos*)positions, substep, max_depth);
    return launch_status();
}
// compute_raised_christoffel_symbols, BSSN.h:93-102
REF_API int refd_christoffel(float* const* metric6, uint32_t* const* derivs6, int32_t seed, uint32_t* const* out6,
                             const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    tensor2_sym_ptrs m(metric6[0], metric6[1], metric6[2], metric6[3], metric6[4], metric6[5]);
    comp_tensor3_sym_ptrs d((compressed_float3*)derivs6[0], (compressed_float3*)derivs6[1], (compressed_float3*)derivs6[2],
                            (compressed_float3*)derivs6[3], (compressed_float3*)derivs6[4], (compressed_float3*)derivs6[5]);
    comp_tensor3_sym_ptrs o((compressed_float3*)out6[0], (compressed_float3*)out6[1], (compressed_float3*)out6[2],
                            (compressed_float3*)out6[3], (compressed_float3*)out6[4], (compressed_float3*)out6[5]);
    __compute_raised_christoffel_symbols<<<stencil_blocks(used), stencil_threads()>>>(m, d, seed, o,
        (const octree_abs_pos*)positions, substep, max_depth);
    return launch_status();
}
// copy_boundaries, AMR.h:880-889
REF_API int refd_copy_boundaries(float* old_f, float* new_f, const uint64_t* boundaries, uint32_t used,
                                 uint32_t substep, uint32_t max_depth, int copy_only_new) {
    dim3 threads(threadsA_v, threadsB_v, threadsD);
    dim3 blocks(size_domain / threads.x, size_domain / threads.y, (used * 6u * padding_domain) / threads.z);
    __copy_boundaries<float><<<blocks, threads>>>(old_f, new_f, (const domain_boundary*)boundaries, substep, max_depth,
                                                  copy_only_new != 0);
    return launch_status();
}
// copy_new_to_old, AMR.h:998-1007
REF_API int refd_copy_new_to_old(float* old_f, const float* new_f, const uint32_t* positions, const int32_t* children,
                                 uint32_t used, uint32_t substep, uint32_t max_depth) {
    dim3 threads(threadsA2_v, threadsB2_v, threadsD2_v);
    dim3 blocks(total_size_domain / threads.x, total_size_domain / threads.y, used * total_size_domain / threads.z);
    __copy_new_to_old<float><<<blocks, threads>>>(old_f, new_f, (const octree_abs_pos*)positions, children, substep, max_depth);
    return launch_status();
}
// copy_to_child, AMR.h:1075-1082
REF_API int refd_copy_to_child(float* buf, uint32_t offset, int32_t child, int32_t parent) {
    dim3 threads(threadsA2_v, threadsB2_v, threadsD2_v);
    dim3 blocks(total_size_domain / threads.x, total_size_domain / threads.y, total_size_domain / threads.z);
    __copy_to_child<float><<<blocks, threads>>>(buf, offset, child, parent);
    return launch_status();
}
// wave_equation_predictor / _corrector, SimpleWave.h:48-72
REF_API int refd_wave_step(int corrector, const float* old_f, const uint32_t* derivs, const uint32_t* hess, float* new_f,
                           const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    if (corrector)
        __corrector_step<<<stencil_blocks(used), stencil_threads()>>>(old_f, (const compressed_float3*)derivs,
            (const compressed_float3*)hess, new_f, (const octree_abs_pos*)positions, substep, max_depth);
    else
        __predictor_step<<<stencil_blocks(used), stencil_threads()>>>(old_f, (const compressed_float3*)derivs,
            (const compressed_float3*)hess, new_f, (const octree_abs_pos*)positions, substep, max_depth);
    return launch_status();
}
// amr_criterion's two kernels, SimpleWave.h:146-150
REF_API int refd_criterion(const uint32_t* derivs, const uint32_t* hess, float* crit, const uint32_t* positions,
                           uint32_t used, uint32_t substep, uint32_t max_depth) {
    dim3 threads(threadsE_v, threadsF_v, 2u);
    dim3 blocks(size_domain / threads.x, (size_domain >> 1u) / threads.y, used);
    __amr_criterion_1<<<blocks, threads>>>((const compressed_float3*)derivs, (const compressed_float3*)hess, crit,
                                           (const octree_abs_pos*)positions, substep, max_depth);
    __amr_criterion_2<<<used, 8u>>>(crit);
    return launch_status();
}

// rasterise_to_image, AMR.h:1356-1365 (the wrapper's launch shape)
REF_API int refd_rasterise(const float* data, float* raster, const int32_t* children, uint32_t width, uint32_t height,
                           float z_slice) {
    dim3 threads(min_uint(width, 32u), min_uint(height, 32u), 1u);
    dim3 blocks((uint32_t)ceilf(float(width) / threads.x), (uint32_t)ceilf(float(height) / threads.y), 1u);
    __rasterise_to_image<<<blocks, threads>>>(data, (float4*)raster, children, width, height, size_domain,
                                              padding_domain, z_slice);
    return launch_status();
}

// ------------------------------------------------------------------ device: whole plugins
struct RefBssn { AMR<BSSN_AMR_data> amr; explicit RefBssn(uint32_t s) : amr(s) { amr.timer_helper = 0u; } };
REF_API void* refd_bssn_create(uint32_t slots) { return new RefBssn(slots); }
REF_API void refd_bssn_destroy(void* h) { cuda_sync(); delete (RefBssn*)h; }
REF_API void refd_bssn_add_node(void* h, int32_t parent, int32_t offset) { ((RefBssn*)h)->amr.add_node(parent, offset); cuda_sync(); }
REF_API void refd_bssn_remove_node(void* h, int32_t idx) { ((RefBssn*)h)->amr.remove_node(idx); cuda_sync(); }
// which: 0 cyij_old, 1 cyij_new, 2 cRij (inner layout)
REF_API float* refd_bssn_field(void* h, int which, int comp) {
    BSSN_AMR_data& d = ((RefBssn*)h)->amr.sim_data;
    tensor2_sym_field* f = which == 0 ? &d.cyij_old : which == 1 ? &d.cyij_new : &d.cRij;
    smart_gpu_buffer<float>* c[6] = {&f->xx, &f->xy, &f->xz, &f->yy, &f->yz, &f->zz};
    return c[comp]->gpu_buffer_ptr;
}
// which: 0 cyij_k, 1 cGijk (6 comps each)
REF_API uint32_t* refd_bssn_cf3(void* h, int which, int comp) {
    BSSN_AMR_data& d = ((RefBssn*)h)->amr.sim_data;
    comp_tensor3_sym_field* f = which == 0 ? &d.cyij_k : &d.cGijk;
    smart_gpu_buffer<compressed_float3>* c[6] = {&f->xx, &f->xy, &f->xz, &f->yy, &f->yz, &f->zz};
    return (uint32_t*)c[comp]->gpu_buffer_ptr;
}
REF_API int refd_bssn_timestep(void* h) { ((RefBssn*)h)->amr.sim_data.timestep(); return launch_status(); }
REF_API int refd_bssn_copy_bounds(void* h) { ((RefBssn*)h)->amr.sim_data.copy_bounds(); return (int)cuda_sync(); }
REF_API int32_t refd_bssn_rng_seed(void* h) { return ((RefBssn*)h)->amr.sim_data.rng.seed; }
REF_API void refd_bssn_octree_state(void* h, uint32_t* positions, int32_t* parent, int32_t* children, uint64_t* boundaries,
                                    uint32_t* lifetime, uint32_t* scalars) {
    dump_octree(((RefBssn*)h)->amr, positions, parent, children, boundaries, lifetime, scalars);
}

struct RefWave { AMR<wave_AMR_data> amr; explicit RefWave(uint32_t s) : amr(s) { amr.timer_helper = 0u; } };
REF_API void* refd_wave_create(uint32_t slots) { return new RefWave(slots); }
REF_API void refd_wave_destroy(void* h) { cuda_sync(); delete (RefWave*)h; }
REF_API void refd_wave_add_node(void* h, int32_t parent, int32_t offset) { ((RefWave*)h)->amr.add_node(parent, offset); cuda_sync(); }
// which: 0 old_field, 1 new_field
REF_API float* refd_wave_field(void* h, int which) {
    wave_AMR_data& d = ((RefWave*)h)->amr.sim_data;
    return which == 0 ? d.old_field.gpu_buffer_ptr : d.new_field.gpu_buffer_ptr;
}
// which: 0 first_derivs, 1 hessian_diag
REF_API uint32_t* refd_wave_cf3(void* h, int which) {
    wave_AMR_data& d = ((RefWave*)h)->amr.sim_data;
    return (uint32_t*)(which == 0 ? d.first_derivs.gpu_buffer_ptr : d.hessian_diag.gpu_buffer_ptr);
}
REF_API float* refd_wave_criterion_host(void* h) { return ((RefWave*)h)->amr.sim_data.criterion.cpu_buffer_ptr; }
REF_API int refd_wave_timestep(void* h) { ((RefWave*)h)->amr.sim_data.timestep(); return launch_status(); }
REF_API int refd_wave_copy_bounds(void* h) { ((RefWave*)h)->amr.sim_data.copy_bounds(); return (int)cuda_sync(); }
REF_API int32_t refd_wave_rng_seed(void* h) { return ((RefWave*)h)->amr.sim_data.rng.seed; }
REF_API void refd_wave_octree_state(void* h, uint32_t* positions, int32_t* parent, int32_t* children, uint64_t* boundaries,
                                    uint32_t* lifetime, uint32_t* scalars) {
    dump_octree(((RefWave*)h)->amr, positions, parent, children, boundaries, lifetime, scalars);
}


// ------------------------------------------------------------------ parallel.h: scan and reductions
// The reference's apply_incl_cum_sum / find_maximum_val / find_minimum_val on a caller's device
// array (wrapped without taking ownership); dtype 0 uint, 1 int, 2 float; ncomp 1-4 selects the
// scalar or the helper_math vector type.
template <class T>
static smart_gpu_buffer<T> ref_view(void* d, uint32_t n) {
    smart_gpu_buffer<T> b;
    b.dedicated_len = n;
    b.gpu_buffer_ptr = static_cast<T*>(d);
    return b;
}
template <class T>
static void ref_scan(void* d, uint32_t n) {
    smart_gpu_buffer<T> b = ref_view<T>(d, n);
    apply_incl_cum_sum(b);
}
template <class T>
static void ref_extreme(int is_max, void* d, uint32_t n, void* result) {
    smart_gpu_buffer<T> b = ref_view<T>(d, n);
    const T r = is_max ? find_maximum_val(b) : find_minimum_val(b);
    std::memcpy(result, &r, sizeof(T));
}
#define REF_TYPES(F, ...)                                                                                   \
    switch (dtype * 4 + ncomp - 1) {                                                                        \
        case 0: F<uint>(__VA_ARGS__); break;   case 1: F<uint2>(__VA_ARGS__); break;                        \
        case 2: F<uint3>(__VA_ARGS__); break;  case 3: F<uint4>(__VA_ARGS__); break;                        \
        case 4: F<int>(__VA_ARGS__); break;    case 5: F<int2>(__VA_ARGS__); break;                         \
        case 6: F<int3>(__VA_ARGS__); break;   case 7: F<int4>(__VA_ARGS__); break;                         \
        case 8: F<float>(__VA_ARGS__); break;  case 9: F<float2>(__VA_ARGS__); break;                       \
        case 10: F<float3>(__VA_ARGS__); break; case 11: F<float4>(__VA_ARGS__); break;                     \
        default: return -1;                                                                                  \
    }
REF_API int refd_scan(int dtype, int ncomp, void* d, uint32_t n) {
    REF_TYPES(ref_scan, d, n)
    return (int)cudaDeviceSynchronize();
}
REF_API int refd_extreme(int dtype, int ncomp, int is_max, void* d, uint32_t n, void* result) {
    REF_TYPES(ref_extreme, is_max, d, n, result)
    return (int)cudaDeviceSynchronize();
}
