// exchange.cu -- packing and unpacking the source boxes of the ghost exchange between ranks.
//
// A box record (8 x uint32, as amr_ghost_exchange_plan writes them) is
// {source slot, source rank, lo x, lo y, lo z, extent x, extent y, extent z} in padded-domain cells.
// Packing copies every box of a field, x fastest, into one contiguous buffer at the box's offset
// (offsets[b], floats); a transport (NCCL send/recv, peer copies) moves the buffer; unpacking writes
// it into the receiver's copy of the field.  One CTA per box.
#include "capi_internal.h"

namespace amr {
namespace {

constexpr int kBlock = 256;

template <bool PACK>
__global__ void __launch_bounds__(kBlock) k_exchange_boxes(float* __restrict__ field, uint32_t t, uint32_t slots,
                                                           const uint32_t* __restrict__ boxes,
                                                           const uint64_t* __restrict__ offsets,
                                                           float* __restrict__ buf) {
    const uint32_t* b = boxes + (size_t)blockIdx.x * 8u;
    const uint32_t ex = b[5], ey = b[6], ez = b[7];
    // a record that leaves the slot range or its cube is skipped (its part of the buffer untouched)
    if (b[0] >= slots || b[2] >= t || b[3] >= t || b[4] >= t || ex == 0u || ey == 0u || ez == 0u ||
        ex > t - b[2] || ey > t - b[3] || ez > t - b[4])
        return;
    const uint32_t count = ex * ey * ez;
    const size_t base = ((size_t)b[0] * t + b[4]) * t * t + (size_t)b[3] * t + b[2];
    float* packed = buf + offsets[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < count; i += kBlock) {
        const uint32_t x = i % ex, y = (i / ex) % ey, z = i / (ex * ey);
        const size_t cell = base + ((size_t)z * t + y) * t + x;
        if (PACK) packed[i] = field[cell];
        else field[cell] = packed[i];
    }
}

}  // namespace
}  // namespace amr

using namespace amr;

extern "C" __attribute__((visibility("default")))
int amr_pack_boxes(const amr_config* cfg, const float* field, uint32_t used_slots, const uint32_t* boxes,
                   const uint64_t* offsets, uint32_t n_boxes, float* out, void* stream) {
    if (!cfg) return AMR_ERR_INVALID;
    if (!config_supported(cfg)) return AMR_ERR_UNSUPPORTED;
    if (n_boxes == 0) return AMR_OK;
    if (!field || !boxes || !offsets || !out) return AMR_ERR_INVALID;
    const uint32_t t = cfg->size_domain + 2u * cfg->padding_domain;
    k_exchange_boxes<true><<<n_boxes, kBlock, 0, static_cast<cudaStream_t>(stream)>>>(
        const_cast<float*>(field), t, used_slots, boxes, offsets, out);
    return cuda_status(cudaGetLastError());
}

extern "C" __attribute__((visibility("default")))
int amr_unpack_boxes(const amr_config* cfg, float* field, uint32_t used_slots, const uint32_t* boxes,
                     const uint64_t* offsets, uint32_t n_boxes, const float* in, void* stream) {
    if (!cfg) return AMR_ERR_INVALID;
    if (!config_supported(cfg)) return AMR_ERR_UNSUPPORTED;
    if (n_boxes == 0) return AMR_OK;
    if (!field || !boxes || !offsets || !in) return AMR_ERR_INVALID;
    const uint32_t t = cfg->size_domain + 2u * cfg->padding_domain;
    k_exchange_boxes<false><<<n_boxes, kBlock, 0, static_cast<cudaStream_t>(stream)>>>(
        field, t, used_slots, boxes, offsets, const_cast<float*>(in));
    return cuda_status(cudaGetLastError());
}
