// kernels_amr.cu -- restriction, prolongation and ghost fill between octree domains.
//
// These kernels move data between domains; each is bound by HBM bandwidth (restriction) or by
// the latency of its gathers (ghost fill, whose sources are L2-resident neighbour cells).
// Several field components are handled per launch so the index and interpolation-weight
// arithmetic is done once per cell for all components.
#include "kernels.h"

#include "amr_device.cuh"

namespace amr {

namespace {

constexpr int kBlock = 256;
inline uint32_t blocks_for(uint64_t n) { return (uint32_t)((n + kBlock - 1) / kBlock); }

// ---------------------------------------------------------------- restriction, AMR.h:961-996
// grid: x = cells of one padded domain, y = work item (domain), z = component
__global__ void k_copy_new_to_old(Dims d, FieldSet f, const uint32_t* __restrict__ positions,
                                  const int32_t* __restrict__ children, const uint32_t* __restrict__ items,
                                  uint32_t substep, uint32_t max_depth) {
    const uint32_t cells = d.t * d.t * d.t;
    const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= cells) return;
    const uint32_t slot = items ? items[blockIdx.y] : blockIdx.y;
    const int depth = pos_depth(positions[slot]);
    if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) return;
    const uint32_t x = cell % d.t, y = (cell / d.t) % d.t, z = cell / (d.t * d.t);
    const uint32_t h = d.n / 2u;
    const uint32_t tx = (x - d.p) / h, ty = (y - d.p) / h, tz = (z - d.p) / h;   // ghosts wrap to >= 2
    const int32_t child = (tx < 2u && ty < 2u && tz < 2u) ? children[tx + ty * 2u + tz * 4u + slot * 8u] : -1;
    const uint64_t o = (uint64_t)slot * cells + cell;
    float* __restrict__ dst = f.old_f[blockIdx.z];
    const float* __restrict__ src = f.new_f[blockIdx.z];
    if (child == -1) {
        dst[o] = src[o];
        return;
    }
    const uint32_t cx = ((x - d.p) * 2u) % d.n + d.p, cy = ((y - d.p) * 2u) % d.n + d.p, cz = ((z - d.p) * 2u) % d.n + d.p;
    const uint64_t ci = (uint64_t)child * cells + ((uint64_t)cz * d.t + cy) * d.t + cx;
    const uint64_t t = d.t, t2 = t * t;
    float s = __fadd_rn(src[ci], src[ci + 1]);
    s = __fadd_rn(s, src[ci + t]);
    s = __fadd_rn(s, src[ci + t + 1]);
    s = __fadd_rn(s, src[ci + t2]);
    s = __fadd_rn(s, src[ci + t2 + 1]);
    s = __fadd_rn(s, src[ci + t2 + t]);
    s = __fadd_rn(s, src[ci + t2 + t + 1]);
    dst[o] = __fmul_rn(s, .125f);
}

// ---------------------------------------------------------------- prolongation, AMR.h:1053-1073
__global__ void k_copy_to_child(Dims d, float inv_n, float* buf, uint32_t offset, int32_t child, int32_t parent) {
    const uint32_t cells = d.t * d.t * d.t;
    const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= cells) return;
    const uint32_t w[3] = {cell % d.t, (cell / d.t) % d.t, cell / (d.t * d.t)};
    const float off[3] = {(float)(offset & 1u), (float)((offset & 2u) >> 1), (float)((offset & 4u) >> 2)};
    uint32_t ri[3];
    float r[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float rp = __fmaf_rn(__fadd_rn(__fsub_rn((float)w[a], (float)d.p), .5f), inv_n, -.5f);
        rp = __fmaf_rn(rp, .5f, __fmul_rn(__fsub_rn(off[a], .5f), .5f));
        rp = __fsub_rn(__fmaf_rn(__fadd_rn(rp, .5f), (float)d.n, (float)d.p), .5f);
        ri[a] = __float2uint_rz(__fadd_rn(rp, .5f));
        r[a] = __fsub_rn(rp, (float)ri[a]);
    }
    const uint64_t rin = (uint64_t)parent * cells + ri[0] + ((uint64_t)ri[1] + (uint64_t)ri[2] * d.t) * d.t;
    float v;
    switch (d.t) {   // interpolation strides are the padded edge
        case 22: v = interp10<22>(buf + rin, r[0], r[1], r[2]); break;
        case 32: v = interp10<32>(buf + rin, r[0], r[1], r[2]); break;
        case 38: v = interp10<38>(buf + rin, r[0], r[1], r[2]); break;
        default: v = interp10<12>(buf + rin, r[0], r[1], r[2]); break;
    }
    buf[(uint64_t)child * cells + cell] = v;
}

// ---------------------------------------------------------------- ghost fill, AMR.h:634-762
// Index of ghost cell (slot, face, layer, v, u) in the staging buffer of one field.
__device__ __forceinline__ uint64_t ghost_index(const Dims& d, uint32_t slot, uint32_t face, uint32_t layer,
                                                uint32_t v, uint32_t u) {
    return ((((uint64_t)slot * 6u + face) * d.p + layer) * d.n + v) * d.n + u;
}
// Padded cell written by ghost (face, layer, u, v) of a domain (AMR.h:715-735).
__device__ __forceinline__ void ghost_cell(const Dims& d, uint32_t face, uint32_t layer, uint32_t u, uint32_t v,
                                           uint32_t* w) {
    switch (face) {
        case 0: w[0] = layer + d.p + d.n; w[1] = u + d.p; w[2] = v + d.p; break;
        case 1: w[0] = u + d.p; w[1] = layer + d.p + d.n; w[2] = v + d.p; break;
        case 2: w[0] = u + d.p; w[1] = v + d.p; w[2] = layer + d.p + d.n; break;
        case 3: w[0] = layer; w[1] = u + d.p; w[2] = v + d.p; break;
        case 4: w[0] = u + d.p; w[1] = layer; w[2] = v + d.p; break;
        default: w[0] = u + d.p; w[1] = v + d.p; w[2] = layer; break;
    }
}
struct GhostJob {
    bool active;
    int32_t target;
    uint32_t dd;
    int cd;
};
__device__ __forceinline__ GhostJob ghost_job(uint64_t bd, uint32_t substep, uint32_t max_depth) {
    GhostJob j;
    j.target = bd_target(bd);
    j.cd = bd_curr_depth(bd);
    j.dd = bd_depth_diff(bd);
    j.active = !(j.target == -1 || j.cd <= 0) && active_depth(substep, (uint32_t)j.cd, max_depth);
    return j;
}

// Phase 1: interpolate every ghost value of every component from the unmodified fields into
// the staging buffer (old values first, then new, per component).
template <int T>
__global__ void k_ghost_gather(Dims d, float inv_n, FieldSet f, const uint64_t* __restrict__ bds, uint32_t used,
                               uint32_t substep, uint32_t max_depth, int copy_only_new, float* __restrict__ stage) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t per_slot = 6ull * d.p * d.n * d.n;
    const uint64_t total = (uint64_t)used * per_slot;
    if (gid >= total) return;
    uint32_t u = (uint32_t)(gid % d.n);
    uint64_t rest = gid / d.n;
    const uint32_t v = (uint32_t)(rest % d.n); rest /= d.n;
    const uint32_t layer = (uint32_t)(rest % d.p); rest /= d.p;
    const uint32_t face = (uint32_t)(rest % 6u);
    const uint32_t slot = (uint32_t)(rest / 6u);
    const uint64_t bd = bds[slot * 6u + face];
    const GhostJob j = ghost_job(bd, substep, max_depth);
    if (!j.active) return;
    uint32_t w[3];
    ghost_cell(d, face, layer, u, v, w);
    const float rel_scale = __uint_as_float((127u - j.dd) << 23);         // 1 / 2^depth_diff
    const float3 rel_pos = cf3_decode((uint32_t)(bd >> 32));
    const float relp[3] = {rel_pos.x, rel_pos.y, rel_pos.z};
    uint32_t ri[3];
    float r[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {                                          // AMR.h:737-753
        float rp = __fmaf_rn(__fadd_rn(__fsub_rn((float)w[a], (float)d.p), .5f), inv_n, -.5f);
        rp = __fmaf_rn(rp, rel_scale, relp[a]);
        rp = __fsub_rn(__fmaf_rn(__fadd_rn(rp, .5f), (float)d.n, (float)d.p), .5f);
        const uint32_t idx = j.target == 0 ? min(__float2uint_rz(__fadd_rn(fmaxf(rp, 0.f), .5f)), d.t - 2u)
                                           : min(__float2uint_rz(__fadd_rn(fmaxf(rp, (float)d.p), .5f)), d.t - d.p - 2u);
        ri[a] = idx;
        r[a] = __fsub_rn(rp, (float)idx);
    }
    const uint64_t cells = (uint64_t)T * T * T;
    const uint64_t rin = (uint64_t)j.target * cells + ri[0] + ((uint64_t)ri[1] + (uint64_t)ri[2] * T) * T;
    const float tm = (float)((substep >> (max_depth - (uint32_t)j.cd)) & ((1u << j.dd) - 1u));   // AMR.h:634-639
    const float t0 = __fmul_rn(tm, rel_scale), t1 = __fmul_rn(__fadd_rn(tm, 1.f), rel_scale);
    const uint64_t gi = ghost_index(d, slot, face, layer, v, u);
    for (int k = 0; k < f.ncomp; k++) {
        const float od = interp10<T>(f.old_f[k] + rin, r[0], r[1], r[2]);
        const float nw = interp10<T>(f.new_f[k] + rin, r[0], r[1], r[2]);
        float* sk = stage + (uint64_t)k * 2u * total;
        if (!copy_only_new) sk[gi] = __fmaf_rn(od, __fsub_rn(1.f, t0), __fmul_rn(nw, t0));
        sk[total + gi] = __fmaf_rn(od, __fsub_rn(1.f, t1), __fmul_rn(nw, t1));
    }
}
// Phase 2: write the staged ghost values into the fields.
__global__ void k_ghost_scatter(Dims d, FieldSet f, const uint64_t* __restrict__ bds, uint32_t used,
                                uint32_t substep, uint32_t max_depth, int copy_only_new, const float* __restrict__ stage) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t per_slot = 6ull * d.p * d.n * d.n;
    const uint64_t total = (uint64_t)used * per_slot;
    if (gid >= total) return;
    uint32_t u = (uint32_t)(gid % d.n);
    uint64_t rest = gid / d.n;
    const uint32_t v = (uint32_t)(rest % d.n); rest /= d.n;
    const uint32_t layer = (uint32_t)(rest % d.p); rest /= d.p;
    const uint32_t face = (uint32_t)(rest % 6u);
    const uint32_t slot = (uint32_t)(rest / 6u);
    const GhostJob j = ghost_job(bds[slot * 6u + face], substep, max_depth);
    if (!j.active) return;
    uint32_t w[3];
    ghost_cell(d, face, layer, u, v, w);
    const uint64_t win = (uint64_t)slot * d.t * d.t * d.t + w[0] + ((uint64_t)w[1] + (uint64_t)w[2] * d.t) * d.t;
    for (int k = 0; k < f.ncomp; k++) {
        const float* sk = stage + (uint64_t)k * 2u * total;
        if (!copy_only_new) f.old_f[k][win] = sk[gid];
        f.new_f[k][win] = sk[total + gid];
    }
}

}  // namespace

// ---------------------------------------------------------------- launchers
cudaError_t launch_copy_new_to_old(Dims d, const FieldSet& f, const uint32_t* positions, const int32_t* children,
                                   const uint32_t* items, uint32_t n_items, uint32_t substep, uint32_t max_depth,
                                   cudaStream_t st) {
    if (n_items == 0 || f.ncomp == 0) return cudaSuccess;
    const dim3 grid(blocks_for((uint64_t)d.t * d.t * d.t), n_items, (uint32_t)f.ncomp);
    k_copy_new_to_old<<<grid, kBlock, 0, st>>>(d, f, positions, children, items, substep, max_depth);
    return cudaGetLastError();
}
cudaError_t launch_copy_to_child(Dims d, float* buf, uint32_t offset, int32_t child, int32_t parent, cudaStream_t st) {
    const float inv_n = 1.f / (float)d.n;
    k_copy_to_child<<<blocks_for((uint64_t)d.t * d.t * d.t), kBlock, 0, st>>>(d, inv_n, buf, offset, child, parent);
    return cudaGetLastError();
}
size_t ghost_scratch_floats(Dims d, uint32_t used, int ncomp) {
    return (size_t)ncomp * 2u * used * 6u * d.p * d.n * d.n;
}
cudaError_t launch_copy_boundaries(Dims d, const FieldSet& f, const uint64_t* boundaries, uint32_t used,
                                   uint32_t substep, uint32_t max_depth, int copy_only_new, float* scratch,
                                   cudaStream_t st) {
    const uint64_t total = (uint64_t)used * 6u * d.p * d.n * d.n;
    if (total == 0 || f.ncomp == 0) return cudaSuccess;
    const float inv_n = 1.f / (float)d.n;
    switch (d.t) {
        case 22: k_ghost_gather<22><<<blocks_for(total), kBlock, 0, st>>>(d, inv_n, f, boundaries, used, substep, max_depth, copy_only_new, scratch); break;
        case 32: k_ghost_gather<32><<<blocks_for(total), kBlock, 0, st>>>(d, inv_n, f, boundaries, used, substep, max_depth, copy_only_new, scratch); break;
        case 38: k_ghost_gather<38><<<blocks_for(total), kBlock, 0, st>>>(d, inv_n, f, boundaries, used, substep, max_depth, copy_only_new, scratch); break;
        case 12: k_ghost_gather<12><<<blocks_for(total), kBlock, 0, st>>>(d, inv_n, f, boundaries, used, substep, max_depth, copy_only_new, scratch); break;
        default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_ghost_scatter<<<blocks_for(total), kBlock, 0, st>>>(d, f, boundaries, used, substep, max_depth, copy_only_new, scratch);
    return cudaGetLastError();
}

}  // namespace amr
