// capi.cu -- extern "C" operator entry points and octree bindings (include/amr_gb300.h).
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>

#include "amr_gb300.h"
#include "capi_internal.h"
#include "kernels.h"
#include "octree.h"

namespace amr {

thread_local int g_last_cuda_error = 0;

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return AMR_OK;
    g_last_cuda_error = (int)e;
    return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? AMR_ERR_NO_DEVICE : AMR_ERR_CUDA;
}

bool config_supported(const amr_config* c) {
    if (!c || !(c->outer_size > 0.f)) return false;
#define AMR_CHECK_CFG(N, P) if (c->size_domain == N && c->padding_domain == P) return true;
    AMR_FOR_EACH_CONFIG(AMR_CHECK_CFG)
#undef AMR_CHECK_CFG
    return false;
}
bool bssn_fused_supported(const amr_config* c) {
#define AMR_CHECK_CFG(N, P) if (c->size_domain == N && c->padding_domain == P) return true;
    AMR_FOR_EACH_BSSN_CONFIG(AMR_CHECK_CFG)
#undef AMR_CHECK_CFG
    return false;
}

cudaError_t launch_stencil(const amr_config& c, int kind, const StencilArgs& a, uint32_t grid, cudaStream_t st) {
#define AMR_DISPATCH(N, P)                                                          \
    if (c.size_domain == N && c.padding_domain == P) {                              \
        switch (kind) {                                                             \
            case SK_GRAD: return launch_stencil_t<N, P, SK_GRAD>(a, grid, st);      \
            case SK_GRAD_HESS: return launch_stencil_t<N, P, SK_GRAD_HESS>(a, grid, st); \
            case SK_MIXED: return launch_stencil_t<N, P, SK_MIXED>(a, grid, st);    \
            default: break;                                                         \
        }                                                                           \
    }
    AMR_FOR_EACH_CONFIG(AMR_DISPATCH)
#undef AMR_DISPATCH
#define AMR_DISPATCH_BSSN(N, P) \
    if (c.size_domain == N && c.padding_domain == P && kind == SK_BSSN) return launch_stencil_t<N, P, SK_BSSN>(a, grid, st);
    AMR_FOR_EACH_BSSN_CONFIG(AMR_DISPATCH_BSSN)
#undef AMR_DISPATCH_BSSN
    return cudaErrorInvalidValue;
}

// Persistent grid for the streaming stencil: as many CTAs as fit on the device at once, but no
// more than there are work items.
uint32_t stencil_grid(const amr_config& c, int kind, uint32_t n_items) {
    int dev = 0, sms = 0;   // the current device's
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    size_t smem = 0;
#define AMR_SMEM(N, P) \
    if (c.size_domain == N && c.padding_domain == P) smem = kind == SK_BSSN ? stencil_smem_bytes<N, P, SK_BSSN>() : stencil_smem_bytes<N, P, SK_GRAD>();
    AMR_FOR_EACH_CONFIG(AMR_SMEM)
#undef AMR_SMEM
    const uint32_t threads = c.size_domain * c.size_domain;
    uint32_t per_sm = (uint32_t)(220u * 1024u / (smem ? smem : 1));
    per_sm = per_sm < 2048u / threads ? per_sm : 2048u / threads;
    if (per_sm < 1) per_sm = 1;
    const uint32_t cap = per_sm * (uint32_t)sms;
    // few items: wider grids than one CTA per item.  The fused kind splits its planes evenly over
    // the CTAs: at least 4 interior planes each (each CTA also streams 2p halo planes), unless
    // that leaves SMs idle, then one CTA per SM down to one plane each.  The others cut items
    // into z-ranges.
    const uint64_t planes = (uint64_t)n_items * c.size_domain;
    const uint64_t one_per_sm = planes < (uint64_t)sms ? planes : (uint64_t)sms;
    const uint64_t want = kind == SK_BSSN ? std::max((planes + 3u) / 4u, one_per_sm)
                                          : (uint64_t)n_items * (c.size_domain / 2u);
    return want < cap ? (uint32_t)want : cap;
}

// Error flag of the current device, shared by the operator entry points and the simulations on
// that device (set by bounded waits that give up); allocated on first use per device.
int* device_error_flag() {
    constexpr int kMaxDevices = 64;
    static int* flag[kMaxDevices] = {};
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!flag[dev]) {
        int* p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) { cudaFree(p); return nullptr; }
        flag[dev] = p;
    }
    return flag[dev];
}

// Read the device error flag and clear it (the caller has synchronised the work that may set
// it): AMR_ERR_TIMEOUT if a bounded wait gave up since the last read.
int take_device_error(int* flag) {
    if (!flag) return AMR_ERR_CUDA;
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && h) e = cudaMemset(flag, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_status(e);
    return h ? AMR_ERR_TIMEOUT : AMR_OK;
}

}  // namespace amr

using namespace amr;

#define AMR_API extern "C" __attribute__((visibility("default")))
#define AMR_REQUIRE(cond) do { if (!(cond)) return AMR_ERR_INVALID; } while (0)
#define AMR_REQUIRE_CFG(c) do { if (!(c)) return AMR_ERR_INVALID; if (!config_supported(c)) return AMR_ERR_UNSUPPORTED; } while (0)

static inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

AMR_API const char* amr_version(void) { return "adaptivemesh_gb300 0.1.0 (sm_103a)"; }
AMR_API int amr_config_supported(const amr_config* cfg) { return config_supported(cfg) ? 1 : 0; }
AMR_API int amr_last_cuda_error(void) { return g_last_cuda_error; }
AMR_API const char* amr_status_string(int s) {
    switch (s) {
        case AMR_OK: return "ok";
        case AMR_ERR_INVALID: return "invalid argument";
        case AMR_ERR_UNSUPPORTED: return "unsupported (size_domain, padding_domain)";
        case AMR_ERR_CUDA: return "CUDA runtime error";
        case AMR_ERR_NO_DEVICE: return "no CUDA device";
        case AMR_ERR_CAPACITY: return "capacity exceeded";
        case AMR_ERR_TIMEOUT: return "a kernel's bounded wait gave up (its results are invalid)";
        default: return "unknown status";
    }
}

AMR_API int amr_device_status(void* stream) {
    const cudaError_t e = cudaStreamSynchronize(S(stream));
    if (e != cudaSuccess) return cuda_status(e);
    return take_device_error(device_error_flag());
}

AMR_API int amr_cf3_encode(const float* xyz, const int32_t* seeds, uint64_t n, uint32_t* out, void* stream) {
    AMR_REQUIRE(n == 0 || (xyz && out));
    return cuda_status(launch_cf3_encode(xyz, seeds, n, out, S(stream)));
}
AMR_API int amr_cf3_decode(const uint32_t* words, uint64_t n, float* xyz, void* stream) {
    AMR_REQUIRE(n == 0 || (words && xyz));
    return cuda_status(launch_cf3_decode(words, n, xyz, S(stream)));
}

static StencilArgs base_args(const amr_config* cfg, const uint32_t* positions, uint32_t used, uint32_t substep,
                             uint32_t max_depth) {
    StencilArgs a;
    std::memset(&a, 0, sizeof(a));
    a.positions = positions;
    a.items = nullptr;
    a.n_items = used;
    a.substep = substep;
    a.max_depth = max_depth;
    a.geo = make_geo(*cfg);
    a.err = device_error_flag();
    return a;
}

AMR_API int amr_differentiate(const amr_config* cfg, const float* field, uint32_t* dif, uint32_t* d2if,
                              const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth,
                              int32_t seed, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(field && dif && positions && max_depth <= kDepthLimit);
    StencilArgs a = base_args(cfg, positions, used, substep, max_depth);
    if (!a.err) return AMR_ERR_CUDA;
    a.field[0] = field;
    a.grad[0] = dif;
    a.hdiag = d2if;
    a.seed_d[0] = seed;
    const int kind = d2if ? SK_GRAD_HESS : SK_GRAD;
    return cuda_status(launch_stencil(*cfg, kind, a, stencil_grid(*cfg, kind, used), S(stream)));
}
AMR_API int amr_mixed_partials(const amr_config* cfg, const float* field, uint32_t* off, const uint32_t* positions,
                               uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(field && off && positions && max_depth <= kDepthLimit);
    StencilArgs a = base_args(cfg, positions, used, substep, max_depth);
    if (!a.err) return AMR_ERR_CUDA;
    a.field[0] = field;
    a.hoff = off;
    a.seed_m[0] = seed;
    return cuda_status(launch_stencil(*cfg, SK_MIXED, a, stencil_grid(*cfg, SK_MIXED, used), S(stream)));
}
AMR_API int amr_deriv_trace(const amr_config* cfg, const uint32_t* hd, const uint32_t* ho, float* const* metric6,
                            float* out, const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth,
                            void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(hd && ho && metric6 && out && positions && max_depth <= kDepthLimit);
    for (int k = 0; k < 6; k++) AMR_REQUIRE(metric6[k]);
    return cuda_status(launch_deriv_trace(make_dims(*cfg), hd, ho, metric6, out, positions, used, substep, max_depth, S(stream)));
}
AMR_API int amr_christoffel(const amr_config* cfg, float* const* metric6, uint32_t* const* derivs6, int32_t seed,
                            uint32_t* const* out6, const uint32_t* positions, uint32_t used, uint32_t substep,
                            uint32_t max_depth, int mode, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(metric6 && derivs6 && out6 && positions && max_depth <= kDepthLimit);
    AMR_REQUIRE(mode == AMR_CHRISTOFFEL_REFERENCE || mode == AMR_CHRISTOFFEL_RAISED);
    for (int k = 0; k < 6; k++) AMR_REQUIRE(metric6[k] && derivs6[k] && out6[k]);
    return cuda_status(launch_christoffel(make_dims(*cfg), metric6, derivs6, seed, out6, positions, used, substep,
                                          max_depth, mode, S(stream)));
}
AMR_API int amr_copy_boundaries(const amr_config* cfg, float* old_f, float* new_f, const uint64_t* boundaries,
                                uint32_t used, uint32_t substep, uint32_t max_depth, int copy_only_new, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(old_f && new_f && boundaries && max_depth <= kDepthLimit);
    const Dims d = make_dims(*cfg);
    FieldSet f;
    std::memset(&f, 0, sizeof(f));
    f.old_f[0] = old_f;
    f.new_f[0] = new_f;
    f.ncomp = 1;
    // staging from the device's stream-ordered pool: nothing is shared between calls, streams or
    // devices, and the memory returns to the pool after the fill
    float* stage = nullptr;
    const size_t bytes = ghost_scratch_floats(d, used, 1) * sizeof(float);
    cudaError_t e = cudaSuccess;
    if (bytes) e = cudaMallocAsync(reinterpret_cast<void**>(&stage), bytes, S(stream));
    if (e != cudaSuccess) return cuda_status(e);
    e = launch_copy_boundaries(d, f, boundaries, used, substep, max_depth, copy_only_new, stage, S(stream));
    if (stage) {
        const cudaError_t e2 = cudaFreeAsync(stage, S(stream));
        if (e == cudaSuccess) e = e2;
    }
    return cuda_status(e);
}
AMR_API int amr_field_norms(const amr_config* cfg, const float* field, const uint32_t* positions, const int32_t* children,
                            uint32_t used, double* out4, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(field && positions && children && out4);
    return field_norms(cfg->size_domain, cfg->padding_domain, field, positions, children, used, out4,
                       static_cast<cudaStream_t>(stream));
}
AMR_API int amr_copy_new_to_old(const amr_config* cfg, float* old_f, const float* new_f, const uint32_t* positions,
                                const int32_t* children, uint32_t used, uint32_t substep, uint32_t max_depth,
                                void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(old_f && new_f && positions && children && max_depth <= kDepthLimit);
    AMR_REQUIRE(cfg->size_domain % 2u == 0u);
    FieldSet f;
    std::memset(&f, 0, sizeof(f));
    f.old_f[0] = old_f;
    f.new_f[0] = const_cast<float*>(new_f);
    f.ncomp = 1;
    return cuda_status(launch_copy_new_to_old(make_dims(*cfg), f, positions, children, nullptr, used, substep, max_depth,
                                              S(stream)));
}
AMR_API int amr_copy_to_child(const amr_config* cfg, float* field, uint32_t offset, int32_t child, int32_t parent,
                              void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(field && offset < 8u && child >= 0 && parent >= 0);
    return cuda_status(launch_copy_to_child(make_dims(*cfg), field, offset, child, parent, S(stream)));
}
AMR_API int amr_wave_predictor(const amr_config* cfg, const float* old_f, const uint32_t* derivs, const uint32_t* hess,
                               float* new_f, const uint32_t* positions, uint32_t used, uint32_t substep,
                               uint32_t max_depth, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(old_f && derivs && hess && new_f && positions && max_depth <= kDepthLimit);
    return cuda_status(launch_wave_step(make_dims(*cfg), make_geo(*cfg), 0, old_f, derivs, hess, new_f, positions, used,
                                        substep, max_depth, S(stream)));
}
AMR_API int amr_wave_corrector(const amr_config* cfg, const float* old_f, const uint32_t* derivs, const uint32_t* hess,
                               float* new_f, const uint32_t* positions, uint32_t used, uint32_t substep,
                               uint32_t max_depth, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(old_f && derivs && hess && new_f && positions && max_depth <= kDepthLimit);
    return cuda_status(launch_wave_step(make_dims(*cfg), make_geo(*cfg), 1, old_f, derivs, hess, new_f, positions, used,
                                        substep, max_depth, S(stream)));
}
AMR_API int amr_criterion(const amr_config* cfg, const uint32_t* derivs, const uint32_t* hess, float* crit,
                          const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(derivs && hess && crit && positions && max_depth <= kDepthLimit);
    AMR_REQUIRE(cfg->size_domain % 4u == 0u);
    return cuda_status(launch_criterion(make_dims(*cfg), make_geo(*cfg), derivs, hess, crit, positions, used, substep,
                                        max_depth, S(stream)));
}

AMR_API int amr_rasterise(const amr_config* cfg, const float* field, const int32_t* children, uint32_t used,
                          uint32_t width, uint32_t height, float z_slice, int bounding_boxes, float* raster_rgba,
                          void* stream) {
    AMR_REQUIRE_CFG(cfg);
    AMR_REQUIRE(field && children && raster_rgba && used >= 1u && width <= 65536u && height <= 65536u);
    AMR_REQUIRE(reinterpret_cast<uintptr_t>(raster_rgba) % 16u == 0u);
    return cuda_status(launch_rasterise(make_dims(*cfg), field, children, used, width, height, z_slice,
                                        bounding_boxes ? 1 : 0, raster_rgba, S(stream)));
}

// ---------------------------------------------------------------- octree
struct amr_octree { Octree tree; explicit amr_octree(uint32_t s) : tree(s) {} };

AMR_API int amr_octree_create(uint32_t node_slots, amr_octree** out) {
    AMR_REQUIRE(out && node_slots >= 1u && node_slots <= (1u << 23));
    *out = new (std::nothrow) amr_octree(node_slots);
    return *out ? AMR_OK : AMR_ERR_CAPACITY;
}
AMR_API int amr_octree_destroy(amr_octree* o) {
    delete o;
    return AMR_OK;
}
AMR_API int amr_octree_add_node(amr_octree* o, int32_t parent, int32_t offset) {
    AMR_REQUIRE(o && parent >= 0 && (uint32_t)parent < o->tree.max_slots() && offset >= 0 && offset < 8);
    o->tree.add_node(parent, offset);
    return AMR_OK;
}
AMR_API int amr_octree_remove_node(amr_octree* o, int32_t node) {
    AMR_REQUIRE(o && node >= -1 && node < (int32_t)o->tree.max_slots());
    o->tree.remove_node(node);
    return AMR_OK;
}
AMR_API int amr_octree_add_nodes(amr_octree* o, const int32_t* parents, const int32_t* offsets, uint32_t n) {
    AMR_REQUIRE(o && (n == 0 || (parents && offsets)));
    for (uint32_t i = 0; i < n; i++)
        AMR_REQUIRE(parents[i] >= 0 && (uint32_t)parents[i] < o->tree.max_slots() && offsets[i] >= 0 && offsets[i] < 8);
    o->tree.begin_batch();
    for (uint32_t i = 0; i < n; i++) o->tree.add_node(parents[i], offsets[i]);
    o->tree.end_batch();
    return AMR_OK;
}
AMR_API int amr_octree_remove_nodes(amr_octree* o, const int32_t* nodes, uint32_t n) {
    AMR_REQUIRE(o && (n == 0 || nodes));
    for (uint32_t i = 0; i < n; i++) AMR_REQUIRE(nodes[i] >= -1 && nodes[i] < (int32_t)o->tree.max_slots());
    o->tree.begin_batch();
    for (uint32_t i = 0; i < n; i++) o->tree.remove_node(nodes[i]);
    o->tree.end_batch();
    return AMR_OK;
}
AMR_API int amr_octree_set_periodic(amr_octree* o, int periodic) {
    AMR_REQUIRE(o);
    o->tree.set_periodic(periodic != 0);
    return AMR_OK;
}
AMR_API int amr_octree_increment_timer(amr_octree* o) {
    AMR_REQUIRE(o);
    o->tree.increment_timer();
    return AMR_OK;
}
AMR_API uint32_t amr_octree_find_node_idx(const amr_octree* o, uint32_t packed, uint32_t max_depth) {
    return o ? o->tree.find_node_idx(packed, max_depth) : 0u;
}
int amr::octree_state_impl(const Octree& t, uint32_t* positions, int32_t* parent, int32_t* children,
                           uint64_t* boundaries, uint32_t* lifetime, uint32_t* scalars) {
    const size_t s = t.max_slots();
    if (positions) std::memcpy(positions, t.positions().data(), s * 4);
    if (parent) std::memcpy(parent, t.parents().data(), s * 4);
    if (children) std::memcpy(children, t.children().data(), s * 32);
    if (boundaries) std::memcpy(boundaries, t.boundaries().data(), s * 48);
    if (lifetime) std::memcpy(lifetime, t.lifetime().data(), s * 4);
    if (scalars) {
        scalars[0] = t.timer();
        scalars[1] = (uint32_t)t.read_max_depth();
        scalars[2] = t.read_first_free_slot();
        scalars[3] = t.curr_used_slots();
        scalars[4] = t.max_slots();
    }
    return AMR_OK;
}
AMR_API int amr_octree_state(const amr_octree* o, uint32_t* positions, int32_t* parent, int32_t* children,
                             uint64_t* boundaries, uint32_t* lifetime, uint32_t* scalars) {
    AMR_REQUIRE(o);
    return octree_state_impl(o->tree, positions, parent, children, boundaries, lifetime, scalars);
}
