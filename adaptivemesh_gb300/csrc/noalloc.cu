// noalloc.cu -- ghost fill that allocates nothing (amr_copy_boundaries_noalloc).
//
// amr_copy_boundaries stages its ghost values in a device buffer that the library allocates on
// first use and grows with cudaMalloc.  Some callers cannot allow that: a host application that
// owns a fixed device-memory budget and hands the library only its field buffers, or a
// time-critical loop that must not block on an allocation (cudaMalloc/cudaFree may synchronise
// the device).  For them, this entry point stages the values in a fixed array compiled into the
// library instead.
//
// The array has room for kNoAllocStageFloats floats (8 MiB).  It is a file-scope __device__
// variable, so every GPU that loads the library holds it until the process exits.  All calls
// share it: two calls whose work overlaps on the GPU (different streams, or different host
// threads) race on it, so callers must order them.  Nothing has to start at zero: each call
// writes every staged value before reading it back.
#include <mutex>

#include "capi_internal.h"

namespace amr {
namespace {

constexpr size_t kNoAllocStageFloats = (size_t)2 << 20;   // 8 MiB of staging space
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_ghost_stage[kNoAllocStageFloats];

// Device address of g_ghost_stage on the current device, looked up once per device.  The lookup
// happens on the first call on each device.
float* stage_address(cudaError_t* err) {
    static float* addr[kMaxDevices] = {};
    static std::mutex mu;
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= kMaxDevices) { *err = cudaErrorInvalidDevice; return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_ghost_stage);
        if (*err != cudaSuccess) return nullptr;
        addr[dev] = static_cast<float*>(p);
    }
    return addr[dev];
}

}  // namespace
}  // namespace amr

using namespace amr;

extern "C" __attribute__((visibility("default")))
int amr_copy_boundaries_noalloc(const amr_config* cfg, float* old_f, float* new_f, const uint64_t* boundaries,
                                uint32_t used_slots, uint32_t substep, uint32_t max_depth, int copy_only_new,
                                void* stream) {
    if (!cfg) return AMR_ERR_INVALID;
    if (!config_supported(cfg)) return AMR_ERR_UNSUPPORTED;
    if (!old_f || !new_f || !boundaries || max_depth > kDepthLimit) return AMR_ERR_INVALID;
    const Dims d = make_dims(*cfg);
    if (ghost_scratch_floats(d, used_slots, 1) > kNoAllocStageFloats) return AMR_ERR_CAPACITY;
    cudaError_t e;
    float* stage = stage_address(&e);
    if (!stage) return cuda_status(e);
    FieldSet f{};
    f.old_f[0] = old_f;
    f.new_f[0] = new_f;
    f.ncomp = 1;
    return cuda_status(launch_copy_boundaries(d, f, boundaries, used_slots, substep, max_depth, copy_only_new, stage,
                                              static_cast<cudaStream_t>(stream)));
}
