// reduce.cu -- the reference's general-purpose scan and reductions (AdaptiveMesh/parallel.h) on
// arrays of 1-4 component elements of uint32, int32 or float32, and FP64 norms of a field over
// the leaf domains (no counterpart in the reference).
//
// The results, including the values these functions leave in the buffer, are the reference's:
// the same multi-pass scheme over 512-element blocks, each block combining its elements in the
// same binary tree, so that float sums are rounded in the same order.
//   inclusive scan (parallel.h:10-82): up passes at strides 1, 512, 512^2, ... build each
//     block's partial-sum tree over the elements (k+1)*stride - 1; down passes from the top
//     stride add the preceding blocks' total to the tree's left spine (nodes 2^i - 1) and sweep it
//     down the tree.
//   maximum / minimum (parallel.h:215-251, 385-421): passes at strides 1, 512, ... reduce each
//     block's elements k*stride in a tree into the block's first element; the answer ends in
//     element 0.  Elements past the end count as the lowest value for the maximum and as zero
//     for the minimum (parallel.h:389), as in the reference.
#include <cfloat>
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "amr_gb300.h"

namespace amr {
namespace {

constexpr uint32_t kPow = 9, kBlk = 1u << kPow;   // 512 elements per block

template <class S, int NC>
struct Elem {
    S v[NC];
};
template <class S, int NC>
__device__ __forceinline__ Elem<S, NC> load(const S* d, uint64_t i) {
    Elem<S, NC> e;
#pragma unroll
    for (int c = 0; c < NC; c++) e.v[c] = d[i * NC + c];
    return e;
}
template <class S, int NC>
__device__ __forceinline__ void store(S* d, uint64_t i, const Elem<S, NC>& e) {
#pragma unroll
    for (int c = 0; c < NC; c++) d[i * NC + c] = e.v[c];
}
template <class S, int NC>
__device__ __forceinline__ Elem<S, NC> filled(S x) {
    Elem<S, NC> e;
#pragma unroll
    for (int c = 0; c < NC; c++) e.v[c] = x;
    return e;
}
template <class S>
__device__ __forceinline__ S add(S a, S b) { return a + b; }
template <>
__device__ __forceinline__ int32_t add<int32_t>(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
template <>
__device__ __forceinline__ float add<float>(float a, float b) { return __fadd_rn(a, b); }
template <class S>
__device__ __forceinline__ S maxv(S a, S b) { return a > b ? a : b; }
template <>
__device__ __forceinline__ float maxv<float>(float a, float b) { return fmaxf(a, b); }
template <class S>
__device__ __forceinline__ S minv(S a, S b) { return a < b ? a : b; }
template <>
__device__ __forceinline__ float minv<float>(float a, float b) { return fminf(a, b); }
template <class S>
__device__ __forceinline__ S lowest();
template <>
__device__ __forceinline__ uint32_t lowest<uint32_t>() { return 0u; }
template <>
__device__ __forceinline__ int32_t lowest<int32_t>() { return INT_MIN; }
template <>
__device__ __forceinline__ float lowest<float>() { return -INFINITY; }

// scan, up pass: block b's slots t hold elements (t + 512 b + 1) * stride - 1
template <class S, int NC>
__global__ void __launch_bounds__(kBlk) k_scan_up(S* data, uint32_t n, uint32_t stride) {
    __shared__ Elem<S, NC> a[kBlk];
    const uint32_t t = threadIdx.x;
    const uint64_t i = ((uint64_t)t + (uint64_t)kBlk * blockIdx.x + 1u) * stride - 1u;
    a[t] = i < n ? load<S, NC>(data, i) : filled<S, NC>(S(0));
    for (uint32_t d = 1; d < kBlk; d <<= 1) {   // node (t+1)*2d - 1 takes in the node d before it
        __syncthreads();
        const uint32_t k = (t + 1u) * 2u * d - 1u;
        if (k < kBlk)
#pragma unroll
            for (int c = 0; c < NC; c++) a[k].v[c] = add(a[k].v[c], a[k - d].v[c]);
        __syncthreads();
    }
    if (i < n) store<S, NC>(data, i, a[t]);
}
// scan, down pass at the same slots: the preceding blocks' total (element 512 b stride - 1, final
// from the pass above) joins the left spine, then each node (t+1)*2d - 1 passes its sum d ahead
template <class S, int NC>
__global__ void __launch_bounds__(kBlk) k_scan_down(S* data, uint32_t n, uint32_t stride) {
    __shared__ Elem<S, NC> a[kBlk];
    const uint32_t t = threadIdx.x;
    const uint64_t i = ((uint64_t)t + (uint64_t)kBlk * blockIdx.x + 1u) * stride - 1u;
    a[t] = i < n ? load<S, NC>(data, i) : filled<S, NC>(S(0));
    const bool spine = ((t + 1u) & t) == 0u && t + 1u <= kBlk / 2u;   // t + 1 = 1, 2, 4, ..., 256
    if (blockIdx.x > 0 && spine) {
        const Elem<S, NC> carry = load<S, NC>(data, (uint64_t)kBlk * blockIdx.x * stride - 1u);
#pragma unroll
        for (int c = 0; c < NC; c++) a[t].v[c] = add(a[t].v[c], carry.v[c]);
    }
    for (uint32_t d = kBlk / 4u; d >= 1u; d >>= 1) {
        __syncthreads();
        const uint32_t m = (t + 1u) * 2u * d - 1u;
        if (m + d < kBlk)
#pragma unroll
            for (int c = 0; c < NC; c++) a[m + d].v[c] = add(a[m + d].v[c], a[m].v[c]);
        __syncthreads();
    }
    if (i < n) store<S, NC>(data, i, a[t]);
}
// maximum (MAX) or minimum: block b's slots t hold elements (t + 512 b) * stride; node t*2d takes in
// node t*2d + d; the block's result goes to its first element
template <class S, int NC, bool MAX>
__global__ void __launch_bounds__(kBlk) k_extreme(S* data, uint32_t n, uint32_t stride) {
    __shared__ Elem<S, NC> a[kBlk];
    const uint32_t t = threadIdx.x;
    const uint64_t i = ((uint64_t)t + (uint64_t)kBlk * blockIdx.x) * stride;
    a[t] = i < n ? load<S, NC>(data, i) : filled<S, NC>(MAX ? lowest<S>() : S(0));
    for (uint32_t d = 1; d < kBlk; d <<= 1) {
        __syncthreads();
        const uint32_t k = t * 2u * d;
        if (k < kBlk)
#pragma unroll
            for (int c = 0; c < NC; c++) a[k].v[c] = MAX ? maxv(a[k].v[c], a[k + d].v[c]) : minv(a[k].v[c], a[k + d].v[c]);
        __syncthreads();
    }
    if (i < n && t == 0u) store<S, NC>(data, i, a[0]);
}

inline uint32_t blocks_of(uint32_t n, uint64_t span) { return (uint32_t)((n + span - 1u) / span); }

template <class S, int NC>
cudaError_t scan(S* data, uint32_t n, cudaStream_t st) {
    uint64_t stride = 1;
    for (; stride < n; stride <<= kPow) {
        k_scan_up<S, NC><<<blocks_of(n, kBlk * stride), kBlk, 0, st>>>(data, n, (uint32_t)stride);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    for (stride >>= kPow; stride > 0; stride >>= kPow) {
        k_scan_down<S, NC><<<blocks_of(n, kBlk * stride), kBlk, 0, st>>>(data, n, (uint32_t)stride);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
template <class S, int NC, bool MAX>
cudaError_t extreme(S* data, uint32_t n, void* result, cudaStream_t st) {
    for (uint64_t stride = 1; stride < n; stride <<= kPow) {
        k_extreme<S, NC, MAX><<<blocks_of(n, kBlk * stride), kBlk, 0, st>>>(data, n, (uint32_t)stride);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemcpyAsync(result, data, sizeof(S) * NC, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// dtype and component count to a typed call
template <template <class, int> class F, class... A>
int dispatch(int dtype, int ncomp, void* data, A... args) {
#define AMR_NC(S)                                                                                           \
    switch (ncomp) {                                                                                        \
        case 1: return F<S, 1>::run(static_cast<S*>(data), args...);                                        \
        case 2: return F<S, 2>::run(static_cast<S*>(data), args...);                                        \
        case 3: return F<S, 3>::run(static_cast<S*>(data), args...);                                        \
        case 4: return F<S, 4>::run(static_cast<S*>(data), args...);                                        \
        default: return AMR_ERR_INVALID;                                                                    \
    }
    switch (dtype) {
        case AMR_DTYPE_UINT32: AMR_NC(uint32_t)
        case AMR_DTYPE_INT32: AMR_NC(int32_t)
        case AMR_DTYPE_FLOAT32: AMR_NC(float)
        default: return AMR_ERR_INVALID;
    }
#undef AMR_NC
}
int status_of(cudaError_t e) { return e == cudaSuccess ? AMR_OK : AMR_ERR_CUDA; }
template <class S, int NC>
struct Scan {
    static int run(S* d, uint32_t n, cudaStream_t st) { return status_of(scan<S, NC>(d, n, st)); }
};
template <class S, int NC>
struct Max {
    static int run(S* d, uint32_t n, void* r, cudaStream_t st) { return status_of(extreme<S, NC, true>(d, n, r, st)); }
};
template <class S, int NC>
struct Min {
    static int run(S* d, uint32_t n, void* r, cudaStream_t st) { return status_of(extreme<S, NC, false>(d, n, r, st)); }
};

// ---------------------------------------------------------------- FP64 norms of a padded field
// Over the interior cells of the leaf domains (live slots without children): sum, sum of squares
// and largest magnitude, in double.  Every cell's value is exact in double and so is its square;
// the sums are taken in a fixed order (a thread's cells in index order, then fixed trees over the
// threads of a domain and over the domains), so a result is the same on every run.
constexpr uint32_t kNormThreads = 256;
struct NormPart {
    double sum, sq, max_abs, cells;
};
__device__ __forceinline__ NormPart norm_join(NormPart a, const NormPart& b) {
    a.sum += b.sum;
    a.sq += b.sq;
    a.max_abs = (a.max_abs != a.max_abs || b.max_abs != b.max_abs) ? __longlong_as_double(0x7FF8000000000000ll)
                                                                  : fmax(a.max_abs, b.max_abs);
    a.cells += b.cells;
    return a;
}
__device__ NormPart norm_block(NormPart v) {   // fixed tree: lanes by xor distance, then warps in order
    __shared__ NormPart warp_part[kNormThreads / 32];
    for (int d = 16; d >= 1; d >>= 1) {
        NormPart o;
        o.sum = __shfl_xor_sync(0xFFFFFFFFu, v.sum, d);
        o.sq = __shfl_xor_sync(0xFFFFFFFFu, v.sq, d);
        o.max_abs = __shfl_xor_sync(0xFFFFFFFFu, v.max_abs, d);
        o.cells = __shfl_xor_sync(0xFFFFFFFFu, v.cells, d);
        v = (threadIdx.x & (uint32_t)d) ? norm_join(o, v) : norm_join(v, o);   // lower lane's value first
    }
    if ((threadIdx.x & 31u) == 0u) warp_part[threadIdx.x >> 5] = v;
    __syncthreads();
    NormPart r = warp_part[0];
    for (uint32_t w = 1; w < kNormThreads / 32; w++) r = norm_join(r, warp_part[w]);
    return r;
}
__global__ void __launch_bounds__(kNormThreads) k_norms_domain(const float* __restrict__ f, const uint32_t* __restrict__ pos,
                                                               const int32_t* __restrict__ children, uint32_t n,
                                                               uint32_t p, NormPart* __restrict__ part) {
    const uint32_t slot = blockIdx.x, t = n + 2u * p;
    bool leaf = pos[slot] != 0xFFFFFFFFu;
    for (int c = 0; c < 8; c++) leaf &= children[(size_t)slot * 8u + c] == -1;
    NormPart v{0.0, 0.0, 0.0, 0.0};
    if (leaf) {   // uniform in the block
        const float* d = f + (size_t)slot * t * t * t;
        for (uint32_t i = threadIdx.x; i < n * n * n; i += kNormThreads) {
            const uint32_t x = i % n, y = (i / n) % n, z = i / (n * n);
            const double a = (double)d[((z + p) * t + y + p) * t + x + p];
            v.sum += a;
            v.sq = fma(a, a, v.sq);
            v.max_abs = (a != a || v.max_abs != v.max_abs) ? a + v.max_abs : fmax(v.max_abs, fabs(a));
            v.cells += 1.0;
        }
    }
    const NormPart r = norm_block(v);
    if (threadIdx.x == 0) part[slot] = r;
}
__global__ void __launch_bounds__(kNormThreads) k_norms_total(const NormPart* __restrict__ part, uint32_t used,
                                                              NormPart* __restrict__ out) {
    NormPart v{0.0, 0.0, 0.0, 0.0};
    for (uint32_t s = threadIdx.x; s < used; s += kNormThreads) v = norm_join(v, part[s]);
    const NormPart r = norm_block(v);
    if (threadIdx.x == 0) *out = r;
}

}  // namespace

int field_norms(uint32_t n, uint32_t p, const float* field, const uint32_t* positions, const int32_t* children,
                uint32_t used, double* out4, cudaStream_t st) {
    if (used == 0) {
        for (int i = 0; i < 4; i++) out4[i] = 0.0;
        return AMR_OK;
    }
    NormPart* part = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&part), sizeof(NormPart) * (used + 1u), st);
    if (e != cudaSuccess) return AMR_ERR_CUDA;
    k_norms_domain<<<used, kNormThreads, 0, st>>>(field, positions, children, n, p, part);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_norms_total<<<1, kNormThreads, 0, st>>>(part, used, part + used);
        e = cudaGetLastError();
    }
    NormPart r{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&r, part + used, sizeof(r), cudaMemcpyDeviceToHost, st);
    const cudaError_t f = cudaFreeAsync(part, st);
    if (e == cudaSuccess) e = f;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return AMR_ERR_CUDA;
    out4[0] = r.sum;
    out4[1] = r.sq;
    out4[2] = r.max_abs;
    out4[3] = r.cells;
    return AMR_OK;
}

}  // namespace amr

#define AMR_API extern "C" __attribute__((visibility("default")))

AMR_API int amr_inclusive_scan(int dtype, int ncomp, void* data, uint64_t count, void* stream) {
    if (!data || count > 0xFFFFFFFFull) return AMR_ERR_INVALID;
    if (count == 0) return AMR_OK;
    return amr::dispatch<amr::Scan>(dtype, ncomp, data, (uint32_t)count, static_cast<cudaStream_t>(stream));
}
AMR_API int amr_reduce_max(int dtype, int ncomp, void* data, uint64_t count, void* result, void* stream) {
    if (!data || !result || count == 0 || count > 0xFFFFFFFFull) return AMR_ERR_INVALID;
    return amr::dispatch<amr::Max>(dtype, ncomp, data, (uint32_t)count, result, static_cast<cudaStream_t>(stream));
}
AMR_API int amr_reduce_min(int dtype, int ncomp, void* data, uint64_t count, void* result, void* stream) {
    if (!data || !result || count == 0 || count > 0xFFFFFFFFull) return AMR_ERR_INVALID;
    return amr::dispatch<amr::Min>(dtype, ncomp, data, (uint32_t)count, result, static_cast<cudaStream_t>(stream));
}
