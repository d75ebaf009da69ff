// kernels_point.cu -- cell-local kernels (one thread per interior cell or codec word).
#include "kernels.h"

#include "amr_device.cuh"

namespace amr {

namespace {

constexpr int kBlock = 256;

inline uint32_t blocks_for(uint64_t n) { return (uint32_t)((n + kBlock - 1) / kBlock); }

// Decompose an inner-layout index into (slot, x, y, z) and the padded index of the same cell.
struct InnerCell {
    uint32_t slot, x, y, z;
    uint64_t padded;
};
__device__ __forceinline__ InnerCell inner_cell(uint64_t o, const Dims& d) {
    InnerCell c;
    const uint64_t n3 = (uint64_t)d.n * d.n * d.n;
    c.slot = (uint32_t)(o / n3);
    uint32_t r = (uint32_t)(o - (uint64_t)c.slot * n3);
    c.x = r % d.n; r /= d.n;
    c.y = r % d.n;
    c.z = r / d.n;
    c.padded = (((uint64_t)c.slot * d.t + c.z + d.p) * d.t + c.y + d.p) * d.t + c.x + d.p;
    return c;
}
__device__ __forceinline__ bool slot_active(const uint32_t* positions, uint32_t slot, uint32_t substep,
                                            uint32_t max_depth, int* depth_out) {
    const int depth = pos_depth(positions[slot]);
    *depth_out = depth;
    return depth != -1 && active_depth(substep, (uint32_t)depth, max_depth);
}

struct Ptr6f { float* p[6]; };
struct Ptr6u { uint32_t* p[6]; };

// ---------------------------------------------------------------- codec
__global__ void k_cf3_encode(const float* __restrict__ xyz, const int32_t* __restrict__ seeds, uint64_t n,
                             uint32_t* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    if (seeds) {
        int32_t s = seeds[i];
        out[i] = cf3_encode_codec(x, y, z, s);
    } else {
        out[i] = cf3_encode_det(x, y, z);
    }
}
__global__ void k_cf3_decode(const uint32_t* __restrict__ w, uint64_t n, float* __restrict__ xyz) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 v = cf3_decode(w[i]);
    xyz[3 * i] = v.x; xyz[3 * i + 1] = v.y; xyz[3 * i + 2] = v.z;
}

// ---------------------------------------------------------------- g^kl H_kl, BSSN.h:7-22
__global__ void k_deriv_trace(Dims d, const uint32_t* __restrict__ hd, const uint32_t* __restrict__ ho, Ptr6f m,
                              float* __restrict__ out, const uint32_t* __restrict__ positions, uint32_t used,
                              uint32_t substep, uint32_t max_depth) {
    const uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= (uint64_t)used * d.n * d.n * d.n) return;
    const InnerCell c = inner_cell(o, d);
    int depth;
    if (!slot_active(positions, c.slot, substep, max_depth, &depth)) return;
    const Sym g{m.p[0][c.padded], m.p[1][c.padded], m.p[2][c.padded], m.p[3][c.padded], m.p[4][c.padded], m.p[5][c.padded]};
    out[o] = trace_contra(sym_from_cf3(hd[o], ho[o]), sym_inverse(g));
}

// ---------------------------------------------------------------- Christoffel symbols, BSSN.h:55-91
__global__ void k_christoffel(Dims d, Ptr6f m, Ptr6u der, int32_t seed, Ptr6u outp,
                              const uint32_t* __restrict__ positions, uint32_t used, uint32_t substep,
                              uint32_t max_depth, int mode) {
    const uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= (uint64_t)used * d.n * d.n * d.n) return;
    const InnerCell c = inner_cell(o, d);
    int depth;
    if (!slot_active(positions, c.slot, substep, max_depth, &depth)) return;
    int32_t rng = cell_rng(seed, c.x, c.y, c.slot * d.n + c.z);
    uint32_t G[6];
#pragma unroll
    for (int k = 0; k < 6; k++) G[k] = der.p[k][o];
    const Sym g{m.p[0][c.padded], m.p[1][c.padded], m.p[2][c.padded], m.p[3][c.padded], m.p[4][c.padded], m.p[5][c.padded]};
    const Sym M = mode == AMR_CHRISTOFFEL_RAISED ? sym_inverse(g) : g;
    float3 dd[6];
#pragma unroll
    for (int k = 0; k < 6; k++) dd[k] = cf3_decode(G[k]);
    const Sym Sx{dd[0].x, __fmul_rn(__fadd_rn(dd[0].y, dd[1].x), .5f), __fmul_rn(__fadd_rn(dd[0].z, dd[2].x), .5f),
                 dd[1].y, __fmul_rn(__fadd_rn(dd[2].y, dd[1].z), .5f), dd[2].z};
    const Sym Sy{dd[1].x, __fmul_rn(__fadd_rn(dd[1].y, dd[3].x), .5f), __fmul_rn(__fadd_rn(dd[1].z, dd[4].x), .5f),
                 dd[3].y, __fmul_rn(__fadd_rn(dd[4].y, dd[3].z), .5f), dd[4].z};
    const Sym Sz{dd[2].x, __fmul_rn(__fadd_rn(dd[2].y, dd[4].x), .5f), __fmul_rn(__fadd_rn(dd[2].z, dd[5].x), .5f),
                 dd[4].y, __fmul_rn(__fadd_rn(dd[5].y, dd[4].z), .5f), dd[5].z};
    const float sx[6] = {Sx.xx, Sx.xy, Sx.xz, Sx.yy, Sx.yz, Sx.zz};
    const float sy[6] = {Sy.xx, Sy.xy, Sy.xz, Sy.yy, Sy.yz, Sy.zz};
    const float sz[6] = {Sz.xx, Sz.xy, Sz.xz, Sz.yy, Sz.yz, Sz.zz};
#pragma unroll
    for (int jk = 0; jk < 6; jk++) {
        const float3 v = make_float3(__fmaf_rn(-dd[jk].x, .5f, sx[jk]), __fmaf_rn(-dd[jk].y, .5f, sy[jk]),
                                     __fmaf_rn(-dd[jk].z, .5f, sz[jk]));
        const float3 r = sym_times(M, v);
        outp.p[jk][o] = cf3_encode(r.x, r.y, r.z, rng);
    }
}

// ---------------------------------------------------------------- SimpleWave Heun update, SimpleWave.h:7-46
__global__ void k_wave_step(Dims d, float outer_dt, int corrector, const float* __restrict__ old_f,
                            const uint32_t* __restrict__ der, const uint32_t* __restrict__ hess, float* new_f,
                            const uint32_t* __restrict__ positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    const uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= (uint64_t)used * d.n * d.n * d.n) return;
    const InnerCell c = inner_cell(o, d);
    int depth;
    if (!slot_active(positions, c.slot, substep, max_depth, &depth)) return;
    const float visc = 0.01f;                                          // SimpleWave.h:5
    const float gx = cf3_decode(der[o]).x;
    const float3 h = cf3_decode(hess[o]);
    const float lap = __fmaf_rn(h.z, visc, __fmaf_rn(h.x, visc, __fmul_rn(h.y, visc)));
    const float v = old_f[c.padded];
    // (lap - v*gx) * dt / 2^depth; the division by a power of two is exact
    const float upd = __fmul_rn(__fmul_rn(__fmaf_rn(-v, gx, lap), outer_dt), __uint_as_float((127u - (uint32_t)depth) << 23));
    if (!corrector) new_f[c.padded] = __fadd_rn(v, upd);
    else new_f[c.padded] = __fmul_rn(__fadd_rn(new_f[c.padded], __fadd_rn(v, upd)), .5f);
}

// ---------------------------------------------------------------- refinement criterion, SimpleWave.h:91-139
__device__ __forceinline__ float cf3_length(uint32_t w) {
    const float3 v = cf3_decode(w);
    return sqrt_approx(__fmaf_rn(v.z, v.z, __fmaf_rn(v.x, v.x, __fmul_rn(v.y, v.y))));
}
__global__ void k_criterion_columns(Dims d, float outer_dx, const uint32_t* __restrict__ der,
                                    const uint32_t* __restrict__ hess, float* __restrict__ crit,
                                    const uint32_t* __restrict__ positions, uint32_t used, uint32_t substep,
                                    uint32_t max_depth) {
    const uint32_t n = d.n, h = n >> 1, q = n >> 2;
    const uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;   // x + (y + zi*h)*n
    if (o >= (uint64_t)used * n * n) return;
    const uint32_t x = (uint32_t)(o % n);
    const uint32_t rest = (uint32_t)(o / n);
    const uint32_t y = rest % h, zi = rest / h;
    const int depth = pos_depth(positions[zi / 2]);
    if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) { crit[o] = __int_as_float(0x7fc00000); return; }   // NAN, SimpleWave.h:97
    uint64_t ro = x + ((uint64_t)y + ((y >= q) ? q : 0u) + (uint64_t)zi * n * h) * n;
    // |g| * dx / 2^depth and |H| * dx * dx / 4^depth, left to right (the power-of-two scaling is exact)
    const float s1 = __uint_as_float((127u - (uint32_t)depth) << 23);
    const float s2 = __uint_as_float((127u - 2u * (uint32_t)depth) << 23);
    float cr = 0.f;
    for (uint32_t i = 0; i < h; i++) {
        cr = fmaxf(cr, __fmul_rn(__fmul_rn(cf3_length(der[ro]), outer_dx), s1));
        cr = fmaxf(cr, __fmul_rn(__fmul_rn(__fmul_rn(cf3_length(hess[ro]), outer_dx), outer_dx), s2));
        cr = fmaxf(cr, __fmul_rn(__fmul_rn(cf3_length(der[ro + (uint64_t)q * n]), outer_dx), s1));
        cr = fmaxf(cr, __fmul_rn(__fmul_rn(__fmul_rn(cf3_length(hess[ro + (uint64_t)q * n]), outer_dx), outer_dx), s2));
        ro += (uint64_t)n * n;
    }
    crit[o] = cr;
}
// One warp per octant (8 per block of 256).  The reference takes the maximum of the octant's q x h
// column values in order, starting from NaN (SimpleWave.h:117-139); the values are non-negative
// or NaN and fmaxf skips NaN, so the maximum does not depend on the order: the lanes take strided
// parts and combine them in a tree.
__global__ void k_criterion_octants(Dims d, float* __restrict__ crit, uint32_t used) {
    const uint32_t n = d.n, h = n >> 1, q = n >> 2;
    const uint32_t idx = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
    if (idx >= used * 8u) return;   // uniform in the warp
    const uint32_t x = idx & 1u, y = (idx >> 1) & 1u, z = (idx >> 2) & 1u, node = idx >> 3;
    const uint64_t base = (uint64_t)node * n * n + z * (n * n >> 1) + y * (n * n >> 2) + x * h;
    float cr = __int_as_float(0x7fc00000);
    for (uint32_t e = lane; e < q * h; e += 32u) cr = fmaxf(cr, crit[base + e % h + (uint64_t)(e / h) * n]);
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) cr = fmaxf(cr, __shfl_xor_sync(0xFFFFFFFFu, cr, s));
    if (lane == 0) crit[base] = cr;
}


// ---------------------------------------------------------------- slice rasteriser, AMR.h:1313-1352
// One thread per pixel of a z-slice through the unit cube: descend the octree to the leaf holding
// the point, interpolate the padded field there (10-point, AMR.h:672-699) and write grey RGBA, or
// red near the leaf's border when bounding boxes are drawn (the reference's build draws them).
// As the reference's fast-math build computes them, px / width - 0.5 is a fused multiply-add with
// the approximate reciprocal of width, and so is the border threshold.  The descent stops at
// kDepthLimit levels or at a child index outside the used slots.
__global__ void k_rasterise(Dims d, const float* __restrict__ data, const int32_t* __restrict__ children,
                            uint32_t used, uint32_t width, uint32_t height, float z_slice, int boxes,
                            float4* __restrict__ raster) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= width || py >= height) return;
    const float rw = rcp_approx((float)width), rh = rcp_approx((float)height);
    float tp[3] = {__fmaf_rn((float)px, rw, -.5f), __fmaf_rn((float)py, rh, -.5f), z_slice};
    auto octant = [&]() { return (uint32_t)(tp[0] > 0.f) | ((uint32_t)(tp[1] > 0.f) << 1) | ((uint32_t)(tp[2] > 0.f) << 2); };
    uint32_t curr = 0, depth = 0;
    int32_t child = children[octant()];
    for (; child != -1 && (uint32_t)child < used && depth < kDepthLimit; depth++) {
        curr = (uint32_t)child;
#pragma unroll
        for (int a = 0; a < 3; a++) {   // fracf(2 t) - 0.5, helper_math.h:1475-1478
            const float v = __fmul_rn(tp[a], 2.f);
            tp[a] = __fsub_rn(__fsub_rn(v, floorf(v)), .5f);
        }
        child = children[curr * 8u + octant()];
    }
    if (boxes) {   // DISPLAY_BOUNDING_BOXES (AMR.h:1312, 1329-1337): red where the leaf's border is near
        const float threshold = __fmaf_rn(-__fmul_rn(2.f, (float)(1u << depth)), rw, .5f);
        if (fmaxf(fabsf(tp[0]), fabsf(tp[1])) >= threshold) {
            raster[(size_t)py * width + px] = make_float4(1.f, 0.f, 0.f, 1.f);
            return;
        }
    }
    uint32_t ri[3];
    float r[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float q = __fmaf_rn(__fadd_rn(tp[a], .5f), (float)d.n, (float)d.p);
        ri[a] = __float2uint_rz(__fadd_rn(q, .5f));
        r[a] = __fsub_rn(q, (float)ri[a]);
    }
    const uint64_t rin = (((uint64_t)curr * d.t + ri[2]) * d.t + ri[1]) * d.t + ri[0];
    const float v = __fadd_rn(interp10_strided(data + rin, (int)d.t, (int)(d.t * d.t), r[0], r[1], r[2]), .5f);
    raster[(size_t)py * width + px] = make_float4(v, v, v, 1.f);
}

}  // namespace

// ---------------------------------------------------------------- launchers
cudaError_t launch_cf3_encode(const float* xyz, const int32_t* seeds, uint64_t n, uint32_t* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_cf3_encode<<<blocks_for(n), kBlock, 0, st>>>(xyz, seeds, n, out);
    return cudaGetLastError();
}
cudaError_t launch_cf3_decode(const uint32_t* w, uint64_t n, float* xyz, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_cf3_decode<<<blocks_for(n), kBlock, 0, st>>>(w, n, xyz);
    return cudaGetLastError();
}
cudaError_t launch_deriv_trace(Dims d, const uint32_t* hd, const uint32_t* ho, float* const* metric6, float* out,
                               const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth,
                               cudaStream_t st) {
    const uint64_t n = (uint64_t)used * d.n * d.n * d.n;
    if (n == 0) return cudaSuccess;
    Ptr6f m;
    for (int k = 0; k < 6; k++) m.p[k] = metric6[k];
    k_deriv_trace<<<blocks_for(n), kBlock, 0, st>>>(d, hd, ho, m, out, positions, used, substep, max_depth);
    return cudaGetLastError();
}
cudaError_t launch_christoffel(Dims d, float* const* metric6, uint32_t* const* der6, int32_t seed, uint32_t* const* out6,
                               const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, int mode,
                               cudaStream_t st) {
    const uint64_t n = (uint64_t)used * d.n * d.n * d.n;
    if (n == 0) return cudaSuccess;
    Ptr6f m; Ptr6u der, out;
    for (int k = 0; k < 6; k++) { m.p[k] = metric6[k]; der.p[k] = der6[k]; out.p[k] = out6[k]; }
    k_christoffel<<<blocks_for(n), kBlock, 0, st>>>(d, m, der, seed, out, positions, used, substep, max_depth, mode);
    return cudaGetLastError();
}
cudaError_t launch_wave_step(Dims d, const Geo& g, int corrector, const float* old_f, const uint32_t* der,
                             const uint32_t* hess, float* new_f, const uint32_t* positions, uint32_t used,
                             uint32_t substep, uint32_t max_depth, cudaStream_t st) {
    const uint64_t n = (uint64_t)used * d.n * d.n * d.n;
    if (n == 0) return cudaSuccess;
    k_wave_step<<<blocks_for(n), kBlock, 0, st>>>(d, g.outer_dt, corrector, old_f, der, hess, new_f, positions, used,
                                                  substep, max_depth);
    return cudaGetLastError();
}
cudaError_t launch_criterion(Dims d, const Geo& g, const uint32_t* der, const uint32_t* hess, float* crit,
                             const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth,
                             cudaStream_t st) {
    const uint64_t n = (uint64_t)used * d.n * d.n;
    if (n == 0) return cudaSuccess;
    k_criterion_columns<<<blocks_for(n), kBlock, 0, st>>>(d, g.outer_dx, der, hess, crit, positions, used, substep, max_depth);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_criterion_octants<<<(uint32_t)(((uint64_t)used * 8u + kBlock / 32u - 1u) / (kBlock / 32u)), kBlock, 0, st>>>(d, crit, used);
    return cudaGetLastError();
}

cudaError_t launch_rasterise(Dims d, const float* data, const int32_t* children, uint32_t used, uint32_t width,
                             uint32_t height, float z_slice, int boxes, float* raster, cudaStream_t st) {
    if (width == 0 || height == 0) return cudaSuccess;
    const dim3 threads(32, 8), grid((width + 31) / 32, (height + 7) / 8);
    k_rasterise<<<grid, threads, 0, st>>>(d, data, children, used, width, height, z_slice, boxes,
                                          reinterpret_cast<float4*>(raster));
    return cudaGetLastError();
}

// ---------------------------------------------------------------- words carried by a launch
namespace {
struct WordBlock {
    static constexpr uint32_t kMax = 1000;   // 4 KB of parameters
    int32_t v[kMax];
    uint32_t n;
};
__global__ void k_store_words(int32_t* __restrict__ dst, const __grid_constant__ WordBlock b) {
    for (uint32_t i = threadIdx.x; i < b.n; i += blockDim.x) dst[i] = b.v[i];
}
}  // namespace

cudaError_t launch_store_words(int32_t* dst, const int32_t* words, uint32_t n, cudaStream_t st, uint32_t* launched) {
    uint32_t count = 0;
    for (uint32_t at = 0; at < n; at += WordBlock::kMax) {
        WordBlock b;
        b.n = n - at < WordBlock::kMax ? n - at : WordBlock::kMax;
        for (uint32_t i = 0; i < b.n; i++) b.v[i] = words[at + i];
        k_store_words<<<1, 256, 0, st>>>(dst + at, b);
        count++;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { if (launched) *launched = count; return e; }
    }
    if (launched) *launched = count;
    return cudaSuccess;
}

// ---------------------------------------------------------------- device-to-device copy
namespace {
// n4 float4 with four loads in flight per thread, then the n % 4 trailing words
__global__ void __launch_bounds__(kBlock) k_copy_words4(float4* __restrict__ dst, const float4* __restrict__ src,
                                                       uint64_t n4, float* __restrict__ dtail,
                                                       const float* __restrict__ stail, uint32_t ntail) {
    const uint64_t stride = (uint64_t)gridDim.x * kBlock;
    uint64_t i = (uint64_t)blockIdx.x * kBlock + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        const float4 a = __ldcs(src + i), b = __ldcs(src + i + stride), c = __ldcs(src + i + 2 * stride),
                     d = __ldcs(src + i + 3 * stride);
        __stcs(dst + i, a); __stcs(dst + i + stride, b); __stcs(dst + i + 2 * stride, c); __stcs(dst + i + 3 * stride, d);
    }
    for (; i < n4; i += stride) __stcs(dst + i, __ldcs(src + i));
    if (blockIdx.x == 0 && threadIdx.x < ntail) dtail[threadIdx.x] = stail[threadIdx.x];
}
__global__ void __launch_bounds__(kBlock) k_copy_words1(float* __restrict__ dst, const float* __restrict__ src, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kBlock) dst[i] = src[i];
}
}  // namespace

cudaError_t launch_copy_words(void* dst, const void* src, uint64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int dev = 0, sms = 0;   // the current device's
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    const uint32_t cap = (uint32_t)sms * 8u;
    if ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 16u == 0u) {
        const uint64_t n4 = n / 4u;
        const uint32_t want = (uint32_t)((n4 + 4u * kBlock - 1u) / (4u * kBlock));
        const uint32_t grid = want < 1u ? 1u : (want < cap ? want : cap);
        k_copy_words4<<<grid, kBlock, 0, st>>>(static_cast<float4*>(dst), static_cast<const float4*>(src), n4,
                                              static_cast<float*>(dst) + n4 * 4u,
                                              static_cast<const float*>(src) + n4 * 4u, (uint32_t)(n % 4u));
    } else {
        const uint32_t want = blocks_for(n);
        k_copy_words1<<<want < cap ? want : cap, kBlock, 0, st>>>(static_cast<float*>(dst), static_cast<const float*>(src), n);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- many copies in one launch
namespace {
// blockIdx.y: the copy; its CTAs stride over its 16-byte vectors, then its last n % 4 words
__global__ void __launch_bounds__(kBlock) k_copy_many(const __grid_constant__ CopyList l) {
    const CopyList::Item& it = l.item[blockIdx.y];
    const uint64_t n4 = it.n / 4u;
    const float4* __restrict__ s4 = static_cast<const float4*>(it.src);
    float4* __restrict__ d4 = static_cast<float4*>(it.dst);
    for (uint64_t i = (uint64_t)blockIdx.x * kBlock + threadIdx.x; i < n4; i += (uint64_t)gridDim.x * kBlock)
        __stcs(d4 + i, __ldcs(s4 + i));
    if (blockIdx.x == 0 && threadIdx.x < (uint32_t)(it.n % 4u))
        static_cast<float*>(it.dst)[n4 * 4u + threadIdx.x] = static_cast<const float*>(it.src)[n4 * 4u + threadIdx.x];
}
}  // namespace

cudaError_t launch_copy_many(const CopyList& l, cudaStream_t st) {
    if (l.n == 0) return cudaSuccess;
    if (l.n > CopyList::kMax) return cudaErrorInvalidValue;
    uint64_t most = 0;
    for (uint32_t i = 0; i < l.n; i++) {
        if ((reinterpret_cast<uintptr_t>(l.item[i].dst) | reinterpret_cast<uintptr_t>(l.item[i].src)) % 16u != 0u)
            return cudaErrorInvalidValue;   // the callers' buffers are allocations: 256-byte aligned
        most = l.item[i].n > most ? l.item[i].n : most;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    // about 8 CTAs per SM in all, and no more per copy than its largest member's vectors need
    uint64_t per = ((uint64_t)sms * 8u + l.n - 1u) / l.n;
    const uint64_t need = (most / 4u + 4u * kBlock - 1u) / (4u * kBlock);
    per = per < need ? per : need;
    k_copy_many<<<dim3((uint32_t)(per < 1u ? 1u : per), l.n), kBlock, 0, st>>>(l);
    return cudaGetLastError();
}

}  // namespace amr
