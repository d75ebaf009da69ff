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
// One CTA per (domain, component, slab): the padded cube is cut into gridDim.z contiguous ranges so a
// domain with children (8 gathers per covered cell) spreads over as many CTAs as a leaf.  A domain
// without children is a straight copy of its range (16-byte aligned: 128-bit loads and stores,
// several in flight per thread); otherwise every cell covered by a child becomes the mean of the
// child's 2x2x2 cells and the rest is copied.
constexpr uint32_t kSlabs = 4;          // slabs per domain of a launch over all active domains (at least)
constexpr uint32_t kParentSlabs = 16;   // ... of a launch over domains with children only (gathers)
template <int N, int P>
__global__ void __launch_bounds__(kBlock) k_copy_new_to_old(const __grid_constant__ FieldSet f, const uint32_t* __restrict__ positions,
                                                        const int32_t* __restrict__ children,
                                                        const uint32_t* __restrict__ items, uint32_t substep,
                                                        uint32_t max_depth) {
    constexpr uint32_t T = N + 2 * P, CELLS = T * T * T, H = N / 2;
    static_assert(CELLS % 4 == 0, "padded domains are whole 16-byte vectors");
    const uint32_t slot = items ? items[blockIdx.x] : blockIdx.x;
    const int depth = pos_depth(positions[slot]);
    if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) return;
    float* __restrict__ dst = f.old_f[blockIdx.y] + (size_t)slot * CELLS;
    const float* __restrict__ src = f.new_f[blockIdx.y];
    const float* __restrict__ own = src + (size_t)slot * CELLS;
    int32_t ch[8];
    bool any_child = false;
#pragma unroll
    for (int i = 0; i < 8; i++) { ch[i] = children[slot * 8u + i]; any_child |= ch[i] != -1; }
    if (!any_child) {   // kU vectors per thread in flight before the first store
        constexpr uint32_t V = CELLS / 4, kU = 8;
        const uint32_t end = (blockIdx.z + 1u) * V / gridDim.z;
        const float4* s4 = reinterpret_cast<const float4*>(own);
        float4* d4 = reinterpret_cast<float4*>(dst);
        for (uint32_t base = blockIdx.z * V / gridDim.z + threadIdx.x; base < end; base += kU * kBlock) {
            float4 b[kU];
#pragma unroll
            for (uint32_t i = 0; i < kU; i++)
                if (base + i * kBlock < end) b[i] = __ldcs(s4 + base + i * kBlock);
#pragma unroll
            for (uint32_t i = 0; i < kU; i++)
                if (base + i * kBlock < end) d4[base + i * kBlock] = b[i];
        }
        return;
    }
    const uint32_t end = (blockIdx.z + 1u) * CELLS / gridDim.z;
#pragma unroll 4   // independent cells: several gathers in flight per thread
    for (uint32_t cell = blockIdx.z * CELLS / gridDim.z + threadIdx.x; cell < end; cell += kBlock) {
        const uint32_t x = cell % T, y = (cell / T) % T, z = cell / (T * T);
        const uint32_t tx = (x - P) / H, ty = (y - P) / H, tz = (z - P) / H;   // ghosts wrap to >= 2
        const int32_t child = (tx < 2u && ty < 2u && tz < 2u) ? ch[tx + ty * 2u + tz * 4u] : -1;
        float v;
        if (child == -1) {
            v = own[cell];
        } else {
            const uint32_t cx = ((x - P) * 2u) % N + P, cy = ((y - P) * 2u) % N + P, cz = ((z - P) * 2u) % N + P;
            const float* c = src + (size_t)child * CELLS + (cz * T + cy) * T + cx;
            constexpr uint32_t T2 = T * T;
            float s = __fadd_rn(c[0], c[1]);
            s = __fadd_rn(s, c[T]);
            s = __fadd_rn(s, c[T + 1]);
            s = __fadd_rn(s, c[T2]);
            s = __fadd_rn(s, c[T2 + 1]);
            s = __fadd_rn(s, c[T2 + T]);
            s = __fadd_rn(s, c[T2 + T + 1]);
            v = __fmul_rn(s, .125f);
        }
        dst[cell] = v;
    }
}

// ---------------------------------------------------------------- prolongation, AMR.h:1053-1073
__device__ __forceinline__ void prolongate_cell(Dims d, float inv_n, float* buf, uint32_t offset, int32_t child,
                                                int32_t parent, uint32_t cell);
__global__ void k_copy_to_child(Dims d, float inv_n, float* buf, uint32_t offset, int32_t child, int32_t parent) {
    const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= d.t * d.t * d.t) return;
    prolongate_cell(d, inv_n, buf, offset, child, parent, cell);
}
struct BufList {
    float* p[12];
};
// blockIdx.y: the item, blockIdx.z: the buffer
__global__ void k_copy_to_children(Dims d, float inv_n, const __grid_constant__ BufList bufs, const int32_t* __restrict__ items) {
    const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= d.t * d.t * d.t) return;
    const int32_t* it = items + 3u * blockIdx.y;
    prolongate_cell(d, inv_n, bufs.p[blockIdx.z], (uint32_t)it[2], it[0], it[1], cell);
}
__device__ __forceinline__ void prolongate_cell(Dims d, float inv_n, float* buf, uint32_t offset, int32_t child,
                                                int32_t parent, uint32_t cell) {
    const uint32_t cells = d.t * d.t * d.t;
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
// The fill's result is defined as the interpolation of the fields as they were before the fill
// (the reference's own launch reads cells that it may be writing at the same time).  Which cells
// can a fill read?  For a non-root source the nearest index is clamped to [P, T-P-2]
// (AMR.h:743-750) and the 10-point stencil reaches one cell back (d[-1], d[-T], d[-T^2]) and one
// forward (d[+1], ...), so its reads stay in [P-1, T-P-1] along each axis, with at most one axis
// at P-1: the interior and the innermost layer (P-1) of the -x, -y and -z ghost faces.  The root
// source (target 0) may be read anywhere, but the root is never filled (its depth is 0).  So the
// only ghost cells that a fill both reads and writes are those innermost lower layers.  Phase 1
// writes every other ghost cell directly and stages the innermost lower layers; phase 2 copies the
// staged values into place.  Every cell ends with the value computed from the pre-fill state.
//
// Ghost cells of one field are enumerated per (slot, face) in the order that is contiguous in the
// destination domain: x-faces with the layer (x) fastest, the other faces with u (x) fastest.
template <int N, int P>
struct GhostShape {
    static constexpr uint32_t T = N + 2 * P, FACE = P * N * N, SLOT = 6 * FACE, CELLS = T * T * T;
    static constexpr uint32_t STAGED = 3 * N * N;   // staged cells per slot: one layer of each lower face
};
// padded cell written for layer `layer` and face coordinates (u, v) of a face (AMR.h:715-735)
template <int N, int P>
__device__ __forceinline__ void ghost_cell(uint32_t face, uint32_t layer, uint32_t u, uint32_t v, uint32_t* w) {
    switch (face) {
        case 0: w[0] = layer + P + N; w[1] = u + P; w[2] = v + P; break;
        case 1: w[0] = u + P; w[1] = layer + P + N; w[2] = v + P; break;
        case 2: w[0] = u + P; w[1] = v + P; w[2] = layer + P + N; break;
        case 3: w[0] = layer; w[1] = u + P; w[2] = v + P; break;
        case 4: w[0] = u + P; w[1] = layer; w[2] = v + P; break;
        default: w[0] = u + P; w[1] = v + P; w[2] = layer; break;
    }
}
// slot, face, face coordinates (u, v) and written padded cell of ghost number gid
template <int N, int P>
__device__ __forceinline__ void ghost_decode(uint64_t gid, uint32_t& slot, uint32_t& face, uint32_t& u, uint32_t& v,
                                             uint32_t* w) {
    using G = GhostShape<N, P>;
    slot = (uint32_t)(gid / G::SLOT);
    const uint32_t r = (uint32_t)(gid - (uint64_t)slot * G::SLOT);
    face = r / G::FACE;
    const uint32_t j = r - face * G::FACE;
    uint32_t layer;
    if (face == 0 || face == 3) { layer = j % P; u = (j / P) % N; v = j / (P * N); }
    else { u = j % N; v = (j / N) % N; layer = j / (N * N); }
    ghost_cell<N, P>(face, layer, u, v, w);
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

// Source index (nearest cell) and offset from it along one axis for written coordinate w
// (AMR.h:737-753).  Each step is monotone in w, so over a face the extreme indices come from the
// extreme coordinates.
template <int N, int P>
__device__ __forceinline__ void ghost_source(uint32_t w, float rel_scale, float relp, bool root, uint32_t& ri, float& r) {
    constexpr uint32_t T = N + 2 * P;
    constexpr float inv_n = 1.f / N;
    float rp = __fmaf_rn(__fadd_rn(__fsub_rn((float)w, (float)P), .5f), inv_n, -.5f);
    rp = __fmaf_rn(rp, rel_scale, relp);
    rp = __fsub_rn(__fmaf_rn(__fadd_rn(rp, .5f), (float)N, (float)P), .5f);
    ri = root ? min(__float2uint_rz(__fadd_rn(fmaxf(rp, 0.f), .5f)), T - 2u)
              : min(__float2uint_rz(__fadd_rn(fmaxf(rp, (float)P), .5f)), T - P - 2u);
    r = __fsub_rn(rp, (float)ri);
}
// n / d for n * d < 2^32 with m = ceil(2^32 / d), d >= 2
struct FastDiv {
    uint32_t d, m;
    __device__ void init(uint32_t dv) { d = dv; m = (uint32_t)(0xFFFFFFFFu / dv) + 1u; }
    __device__ __forceinline__ uint32_t div(uint32_t n) const { return __umulhi(n, m); }
};
// 4-byte asynchronous global -> shared copies (completion tracked per thread by commit groups)
__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gsrc) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory"); }
// Largest source box of one face and component: P+2 cells along the normal, N+2 along the others.
template <int N, int P>
struct GhostBox {
    static constexpr uint32_t MAX = (P + 2) * (N + 2) * (N + 2);
    static constexpr size_t SMEM = 4u * MAX * sizeof(float);   // two buffers of (old, new)
    // resident CTAs per SM the register budget is set for: more ghost cells per thread at larger N
    static constexpr int MIN_CTAS = N <= 16 ? 4 : 2;
};

// Phase 1, one CTA per (slot, face).  The source cells that the face's ghost cells interpolate
// from lie in a box one cell wider than the range of their nearest source indices.  Per
// component, the CTA copies the old and new values of that box into shared memory (double
// buffered, asynchronous copies: the next component loads while this one is interpolated), then computes every
// ghost value of the face from there and writes it in place, or to the staging buffer if it lies
// in an innermost lower layer.  The box never holds a cell that phase 1 writes (see above), and the
// arithmetic is the reference's per cell, so the values equal a fill of the pre-fill state.  A
// box that would leave the domain's cube (only a root source can come near) or exceed the
// shared-memory buffer is read from global memory instead.
template <int N, int P>
__global__ void __launch_bounds__(kBlock, GhostBox<N, P>::MIN_CTAS) k_ghost_face(const __grid_constant__ FieldSet f, const uint64_t* __restrict__ bds, uint32_t used,
                                                      uint32_t substep, uint32_t max_depth, int copy_only_new,
                                                      int in_place, float* __restrict__ stage) {
    using G = GhostShape<N, P>;
    constexpr uint32_t T = G::T, BOX = GhostBox<N, P>::MAX;
    extern __shared__ float sbox[];
    __shared__ uint32_t s_off[3][T];   // per axis and written coordinate: box-relative source index
    __shared__ float s_r[3][T];        // and offset from it
    const uint32_t slot = blockIdx.x / 6u, face = blockIdx.x - slot * 6u;
    const uint64_t bd = bds[(size_t)slot * 6u + face];
    const GhostJob j = ghost_job(bd, substep, max_depth);
    if (!j.active) return;   // uniform in the CTA
    const float rel_scale = __uint_as_float((127u - j.dd) << 23);         // 1 / 2^depth_diff
    const float3 rel_pos = cf3_decode((uint32_t)(bd >> 32));
    const float relp[3] = {rel_pos.x, rel_pos.y, rel_pos.z};
    const bool root = j.target == 0;
    const float tm = (float)((substep >> (max_depth - (uint32_t)j.cd)) & ((1u << j.dd) - 1u));   // AMR.h:634-639
    const float t0 = __fmul_rn(tm, rel_scale), t1 = __fmul_rn(__fadd_rn(tm, 1.f), rel_scale);
    const uint32_t normal = face % 3u;
    const uint64_t n_staged = (uint64_t)used * G::STAGED;
    const bool staged_face = face >= 3u && !in_place;
    // In place (see launch_copy_boundaries): new's innermost lower layer of an active source is
    // read from old, which holds its value before this fill.
    const bool redirect = in_place && !root && active_depth(substep, (uint32_t)(j.cd - (int)j.dd), max_depth);

    // written coordinate range and source box per axis
    uint32_t wlo[3], whi[3], ext[3];
    int32_t lo[3];
    bool boxed = true;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        wlo[a] = a == (int)normal ? (face < 3u ? P + N : 0u) : P;
        whi[a] = a == (int)normal ? wlo[a] + P - 1u : P + N - 1u;
        uint32_t r0, r1;
        float unused;
        ghost_source<N, P>(wlo[a], rel_scale, relp[a], root, r0, unused);
        ghost_source<N, P>(whi[a], rel_scale, relp[a], root, r1, unused);
        lo[a] = (int32_t)r0 - 1;
        ext[a] = r1 - r0 + 3u;
        boxed &= lo[a] >= 0;
    }
    boxed &= ext[0] * ext[1] * ext[2] <= BOX;

    if (!boxed) {   // global-memory path, one ghost cell per thread and pass
        for (uint32_t g = threadIdx.x; g < G::FACE; g += kBlock) {
            uint32_t sl, fc, u, v, w[3];
            ghost_decode<N, P>((uint64_t)slot * G::SLOT + (uint64_t)face * G::FACE + g, sl, fc, u, v, w);
            uint32_t ri[3];
            float r[3];
#pragma unroll
            for (int a = 0; a < 3; a++) ghost_source<N, P>(w[a], rel_scale, relp[a], root, ri[a], r[a]);
            const uint64_t rin = (uint64_t)j.target * G::CELLS + ri[0] + (ri[1] + ri[2] * T) * T;
            const bool staged = staged_face && (normal == 0u ? w[0] : normal == 1u ? w[1] : w[2]) == P - 1u;
            const uint64_t out = staged ? ((uint64_t)slot * 3u + (face - 3u)) * (N * N) + u + v * N
                                        : (uint64_t)slot * G::CELLS + w[0] + (w[1] + w[2] * T) * T;
            for (int k = 0; k < f.ncomp; k++) {
                const float od = interp10<T>(f.old_f[k] + rin, r[0], r[1], r[2]);
                const float* o = f.old_f[k] + rin;
                const float* d = f.new_f[k] + rin;
                constexpr uint32_t T2 = T * T;
                const float nw = interp10_taps(d[0], d[1], d[T], d[T2], (redirect && ri[0] == P ? o : d)[-1],
                                               (redirect && ri[1] == P ? o : d)[-(int)T],
                                               (redirect && ri[2] == P ? o : d)[-(int)T2], d[T + 1], d[T2 + 1],
                                               d[T2 + T], r[0], r[1], r[2]);
                float* dst_old = staged ? stage + (uint64_t)k * 2u * n_staged : f.old_f[k];
                float* dst_new = staged ? stage + ((uint64_t)k * 2u + 1u) * n_staged : f.new_f[k];
                if (!copy_only_new) dst_old[out] = __fmaf_rn(od, __fsub_rn(1.f, t0), __fmul_rn(nw, t0));
                dst_new[out] = __fmaf_rn(od, __fsub_rn(1.f, t1), __fmul_rn(nw, t1));
            }
        }
        return;
    }

    for (uint32_t i = threadIdx.x; i < 3u * T; i += kBlock) {
        const uint32_t a = i / T, w = i - a * T;   // selects, not indexing: the arrays stay in registers
        const uint32_t wl = a == 0u ? wlo[0] : a == 1u ? wlo[1] : wlo[2];
        const uint32_t wh = a == 0u ? whi[0] : a == 1u ? whi[1] : whi[2];
        if (w < wl || w > wh) continue;
        uint32_t ri;
        float r;
        ghost_source<N, P>(w, rel_scale, a == 0u ? relp[0] : a == 1u ? relp[1] : relp[2], root, ri, r);
        s_off[a][w] = ri - (uint32_t)(a == 0u ? lo[0] : a == 1u ? lo[1] : lo[2]);
        s_r[a][w] = r;
    }
    const uint32_t sy = ext[0], sz = ext[0] * ext[1], box = sz * ext[2];
    const size_t src0 = (size_t)j.target * G::CELLS + (uint32_t)lo[0] + ((uint32_t)lo[1] + (uint32_t)lo[2] * T) * T;
    // Box element i = tid + n*kBlock as (bx, by, bz) and its cell offset gi from src0; stepping by
    // kBlock adds (A, B, C) with one carry per axis at most.
    FastDiv div_x, div_xy;
    div_x.init(sy);
    div_xy.init(sz);
    const uint32_t bz0 = div_xy.div(threadIdx.x), by0 = div_x.div(threadIdx.x - bz0 * sz), bx0 = threadIdx.x - bz0 * sz - by0 * sy;
    const uint32_t C = div_xy.div(kBlock), B = div_x.div(kBlock - C * sz), A = kBlock - C * sz - B * sy;

    // per ghost cell of this thread: box offset of its nearest source cell, offsets, destination
    constexpr uint32_t CPT = (G::FACE + kBlock - 1) / kBlock;
    uint32_t c_o[CPT], c_dst[CPT];
    float c_rx[CPT], c_ry[CPT], c_rz[CPT];
    const uint64_t stage_base = ((uint64_t)slot * 3u + (face - 3u)) * (N * N);   // used for lower faces only
    const uint64_t slot_base = (uint64_t)slot * G::CELLS;

    // The source offsets of this thread's box elements are the same for every component: at
    // small sizes they are computed once and kept in registers.
    constexpr uint32_t EPT = (BOX + kBlock - 1) / kBlock;   // box elements per thread, at most
    constexpr bool kCached = EPT <= 8;
    uint32_t e_gi[kCached ? EPT : 1];
    uint32_t e_low = 0;   // bit e: element e lies in the source's innermost lower layer (redirect only)
    auto low_layer = [&](uint32_t bx, uint32_t by, uint32_t bz) {
        return (uint32_t)lo[0] + bx == P - 1u || (uint32_t)lo[1] + by == P - 1u || (uint32_t)lo[2] + bz == P - 1u;
    };
    if (kCached) {
        uint32_t bx = bx0, by = by0, bz = bz0;
#pragma unroll
        for (uint32_t e = 0; e < EPT; e++) {
            e_gi[e] = bx + (by + bz * T) * T;
            if (redirect && low_layer(bx, by, bz)) e_low |= 1u << e;
            bx += A; by += B; bz += C;
            if (bx >= sy) { bx -= sy; by++; }
            if (by >= ext[1]) { by -= ext[1]; bz++; }
        }
    }
    // Component k's box goes to buffer k & 1 by asynchronous copies, issued one component ahead.
    // A box element is the pair (old, new), so that one interpolation serves both.
    float2* const sbox2 = reinterpret_cast<float2*>(sbox);
    auto issue = [&](int k) {
        float* buf = reinterpret_cast<float*>(sbox2 + (k & 1) * BOX);
        const float* go = f.old_f[k] + src0;
        const float* gn = f.new_f[k] + src0;
        if (kCached) {
#pragma unroll
            for (uint32_t e = 0; e < EPT; e++) {
                const uint32_t i = threadIdx.x + e * kBlock;
                if (i < box) {
                    cp_async4(buf + 2u * i, go + e_gi[kCached ? e : 0]);
                    cp_async4(buf + 2u * i + 1u, ((e_low >> e) & 1u ? go : gn) + e_gi[kCached ? e : 0]);
                }
            }
        } else {
            uint32_t bx = bx0, by = by0, bz = bz0;
            for (uint32_t i = threadIdx.x; i < box; i += kBlock) {
                const uint32_t gi = bx + (by + bz * T) * T;
                cp_async4(buf + 2u * i, go + gi);
                cp_async4(buf + 2u * i + 1u, (redirect && low_layer(bx, by, bz) ? go : gn) + gi);
                bx += A; by += B; bz += C;
                if (bx >= sy) { bx -= sy; by++; }
                if (by >= ext[1]) { by -= ext[1]; bz++; }
            }
        }
        cp_async_commit();
    };
    issue(0);
    for (int k = 0; k < f.ncomp; k++) {
        const float2* buf = sbox2 + (k & 1) * BOX;
        if (k + 1 < f.ncomp) { issue(k + 1); cp_async_wait<1>(); }
        else cp_async_wait<0>();
        __syncthreads();   // component k's box is complete in every thread's view
        if (k == 0) {
#pragma unroll
            for (uint32_t c = 0; c < CPT; c++) {
                const uint32_t g = threadIdx.x + c * kBlock;
                if (g >= G::FACE) break;
                uint32_t layer, u, v, w[3];
                if (normal == 0u) { layer = g % P; u = (g / P) % N; v = g / (P * N); }
                else { u = g % N; v = (g / N) % N; layer = g / (N * N); }
                ghost_cell<N, P>(face, layer, u, v, w);
                c_o[c] = s_off[0][w[0]] + s_off[1][w[1]] * sy + s_off[2][w[2]] * sz;
                c_rx[c] = s_r[0][w[0]]; c_ry[c] = s_r[1][w[1]]; c_rz[c] = s_r[2][w[2]];
                // destination: bit 31 marks a staged cell, the rest is its offset from the base
                c_dst[c] = staged_face && layer == P - 1u ? 0x80000000u | (u + v * N) : w[0] + (w[1] + w[2] * T) * T;
            }
        }
        float* const stage_old = stage + (uint64_t)k * 2u * n_staged + stage_base;
        float* const stage_new = stage + ((uint64_t)k * 2u + 1u) * n_staged + stage_base;
        float* const field_old = f.old_f[k] + slot_base;
        float* const field_new = f.new_f[k] + slot_base;
#pragma unroll
        for (uint32_t c = 0; c < CPT; c++) {
            if (threadIdx.x + c * kBlock >= G::FACE) break;
            const float2 on = interp10_pair(buf + c_o[c], (int)sy, (int)sz, c_rx[c], c_ry[c], c_rz[c]);
            const float od = on.x, nw = on.y;
            const bool staged = (c_dst[c] & 0x80000000u) != 0u;
            const uint32_t off = c_dst[c] & 0x7FFFFFFFu;
            if (!copy_only_new) (staged ? stage_old : field_old)[off] = __fmaf_rn(od, __fsub_rn(1.f, t0), __fmul_rn(nw, t0));
            (staged ? stage_new : field_new)[off] = __fmaf_rn(od, __fsub_rn(1.f, t1), __fmul_rn(nw, t1));
        }
        __syncthreads();   // everyone is done with buffer k & 1 before component k + 2 is copied into it
    }
}
// Phase 2: write the staged innermost lower layers into the fields.
template <int N, int P>
__global__ void __launch_bounds__(256) k_ghost_commit(const __grid_constant__ FieldSet f, const uint64_t* __restrict__ bds, uint32_t used,
                                                     uint32_t substep, uint32_t max_depth, int copy_only_new,
                                                     const float* __restrict__ stage) {
    using G = GhostShape<N, P>;
    constexpr uint32_t T = G::T;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n_staged = (uint64_t)used * G::STAGED;
    if (gid >= n_staged) return;
    const uint32_t slot = (uint32_t)(gid / G::STAGED);
    const uint32_t r = (uint32_t)(gid - (uint64_t)slot * G::STAGED);
    const uint32_t face = 3u + r / (N * N), u = r % N, v = (r / N) % N;
    if (!ghost_job(bds[slot * 6u + face], substep, max_depth).active) return;
    uint32_t w[3];
    ghost_cell<N, P>(face, P - 1u, u, v, w);
    const uint64_t win = (uint64_t)slot * G::CELLS + w[0] + (w[1] + w[2] * T) * T;
    for (int k = 0; k < f.ncomp; k++) {
        if (!copy_only_new) f.old_f[k][win] = __ldcs(stage + (uint64_t)k * 2u * n_staged + gid);
        f.new_f[k][win] = __ldcs(stage + ((uint64_t)k * 2u + 1u) * n_staged + gid);
    }
}

}  // namespace

// ---------------------------------------------------------------- launchers
cudaError_t launch_copy_new_to_old(Dims d, const FieldSet& f, const uint32_t* positions, const int32_t* children,
                                   const uint32_t* items, uint32_t n_items, uint32_t substep, uint32_t max_depth,
                                   cudaStream_t st, bool parents_only) {
    if (n_items == 0 || f.ncomp == 0) return cudaSuccess;
    // few domains: more slabs per domain, up to about two CTAs per SM in all
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint32_t slabs = parents_only ? kParentSlabs : kSlabs;
    const uint64_t per_slab = (uint64_t)n_items * (uint32_t)f.ncomp;
    while (slabs < 64u && per_slab * slabs * 2u <= 2u * (uint64_t)(sms > 0 ? sms : 1)) slabs *= 2u;
    const dim3 grid(n_items, (uint32_t)f.ncomp, slabs);
#define AMR_RESTRICT(N, P) \
    if (d.n == N && d.p == P) { k_copy_new_to_old<N, P><<<grid, kBlock, 0, st>>>(f, positions, children, items, substep, max_depth); return cudaGetLastError(); }
    AMR_FOR_EACH_CONFIG(AMR_RESTRICT)
#undef AMR_RESTRICT
    return cudaErrorInvalidValue;
}
cudaError_t launch_copy_to_child(Dims d, float* buf, uint32_t offset, int32_t child, int32_t parent, cudaStream_t st) {
    const float inv_n = 1.f / (float)d.n;
    k_copy_to_child<<<blocks_for((uint64_t)d.t * d.t * d.t), kBlock, 0, st>>>(d, inv_n, buf, offset, child, parent);
    return cudaGetLastError();
}
cudaError_t launch_copy_to_children(Dims d, float* const* bufs, int nbuf, const int32_t* items, uint32_t n_items,
                                    cudaStream_t st) {
    if (nbuf < 1 || nbuf > 12) return cudaErrorInvalidValue;
    if (n_items == 0) return cudaSuccess;
    BufList b;
    for (int i = 0; i < 12; i++) b.p[i] = i < nbuf ? bufs[i] : nullptr;
    const float inv_n = 1.f / (float)d.n;
    for (uint32_t i = 0; i < n_items; i += 65535u) {   // grid y holds at most 65535 items
        k_copy_to_children<<<dim3(blocks_for((uint64_t)d.t * d.t * d.t), std::min(n_items - i, 65535u), (uint32_t)nbuf),
                             kBlock, 0, st>>>(d, inv_n, b, items + 3u * (size_t)i);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
size_t ghost_scratch_floats(Dims d, uint32_t used, int ncomp) {
    return (size_t)ncomp * 2u * used * 3u * d.n * d.n;
}
cudaError_t launch_copy_boundaries(Dims d, const FieldSet& f, const uint64_t* boundaries, uint32_t used,
                                   uint32_t substep, uint32_t max_depth, int copy_only_new, float* scratch,
                                   cudaStream_t st, bool sources_restricted) {
    const int in_place = copy_only_new && sources_restricted ? 1 : 0;
#define AMR_GHOST(N, P)                                                                                     \
    if (d.n == N && d.p == P) {                                                                             \
        static std::atomic<uint64_t> configured{0};                                                         \
        if (const cudaError_t e0 = ensure_smem_limit(k_ghost_face<N, P>, GhostBox<N, P>::SMEM, configured))   \
            return e0;                                                                                      \
        if (used == 0 || f.ncomp == 0) return cudaSuccess;                                                  \
        k_ghost_face<N, P><<<used * 6u, kBlock, GhostBox<N, P>::SMEM, st>>>(f, boundaries, used, substep,     \
                                                                          max_depth, copy_only_new, in_place, \
                                                                          scratch);                           \
        cudaError_t e = cudaGetLastError();                                                                 \
        if (e != cudaSuccess || in_place) return e;                                                         \
        k_ghost_commit<N, P><<<blocks_for((uint64_t)used * 3u * N * N), kBlock, 0, st>>>(                   \
            f, boundaries, used, substep, max_depth, copy_only_new, scratch);                               \
        return cudaGetLastError();                                                                          \
    }
    AMR_FOR_EACH_CONFIG(AMR_GHOST)
#undef AMR_GHOST
    return cudaErrorInvalidValue;
}

}  // namespace amr
