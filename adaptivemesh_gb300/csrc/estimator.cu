// estimator.cu -- the learned refinement / error estimator: a small 3-D convolutional network run per
// tile (one domain), trained on the GPU by the kernels below.  No counterpart in the reference,
// whose refinement criterion is a per-octant gradient and curvature threshold
// (SimpleWave.h:91-187, 228-248); here that plain criterion stays both the fallback and the judge
// of the network's decisions (evolve_sim.cu, amr_sim_regrid).
//
// Network (per tile, input 3 x 8^3 features):
//   conv1  3 -> 16 channels, 3x3x3, padding 1, stride 1, ReLU      -> 16 x 8^3
//   conv2  16 -> 16 channels, 3x3x3, padding 1, stride 2, ReLU     -> 16 x 4^3 = 1024
//   fc1    1024 -> 32, ReLU
//   fc2    32 -> 1 (the predicted log10 truncation error of the tile)
// The convolutions and fc1 run as GEMMs on the fifth-generation tensor cores (tcgen05.mma kind::f16,
// BF16 operands in shared memory, FP32 accumulation in Tensor Memory) over im2col matrices; the
// backward pass uses the same GEMM for the weight and input gradients.  Master weights, gradients and the Adam moments are FP32; the GEMM operands
// (weights, activations, back-propagated gradients) are rounded to BF16.
//
// Layouts: activations are position-major, channel-last ([tile][position][channel]); im2col column
// j = channel * 27 + (dz * 9 + dy * 3 + dx) for the tap at offset (dx, dy, dz) - 1; conv1's 81
// columns are padded to 96 with zeros.  The flat parameter vector is W1[96][16], b1[16],
// W2[432][16], b2[16], W3[1024][32], b3[32], W4[32], b4[1] (row-major, K rows by N columns).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "capi_internal.h"
#include "tcgen05.cuh"

namespace amr {

namespace {

using bf16 = __nv_bfloat16;

constexpr int kIn = 3, kC1 = 16, kC2 = 16, kF = 32;
constexpr int kP1 = 512, kP2 = 64;                 // positions after conv1 (8^3) and conv2 (4^3)
constexpr int kK1 = 96, kK1Real = kIn * 27, kK2 = kC1 * 27, kK3 = kP2 * kC2;   // 96, 432, 1024
constexpr size_t kOffW1 = 0, kOffB1 = kOffW1 + kK1 * kC1, kOffW2 = kOffB1 + kC1, kOffB2 = kOffW2 + kK2 * kC2,
                 kOffW3 = kOffB2 + kC2, kOffB3 = kOffW3 + (size_t)kK3 * kF, kOffW4 = kOffB3 + kF,
                 kOffB4 = kOffW4 + kF, kParams = kOffB4 + 1;

// ------------------------------------------------------------------ BF16 GEMM on the tensor cores
// C[m][n] (+)= sum_k A(m, k) B(k, n); A(m, k) = A[m * sam + k * sak], B(k, n) = B[k * sbk + n * sbn],
// C[m * scm + n * scn] (FP32).  A CTA of 4 warps computes a 128 x NT tile (NT = 16 or 32) with the
// fifth-generation tensor cores: per K block of 64 the threads stage A (128 x 64) and B (NT x 64)
// into shared memory as K-major core matrices (zero past the edges), one thread issues four
// tcgen05.mma of K = 16 into a TMEM accumulator and commits them to an mbarrier, and after the last
// block each warp reads its 32 rows of the accumulator back with tcgen05.ld.  Every wait is bounded;
// a wait that runs out raises *err, waits once more for the MMAs in flight and frees the TMEM.
struct GemmArgs {
    const bf16* A;
    int64_t sam, sak;
    const bf16* B;
    int64_t sbk, sbn;
    float* C;
    int64_t scm, scn;
    int M, N, K;
    int accumulate;   // 1: C += A B, 0: C = A B
    int* err;         // device flag raised when a wait gives up
};

constexpr int kGemmM = 128, kGemmK = 64;

template <int NT>
__global__ void __launch_bounds__(128) k_gemm_bf16(const GemmArgs g) {
    static_assert(NT == 16 || NT == 32, "M = 128 tiles take N in multiples of 16; 32 TMEM columns");
    constexpr int MT = kGemmM, KT = kGemmK;
    constexpr uint32_t LBO = 128u, SBO = (KT / 8) * 128u;   // bytes between core matrices along K / M
    __shared__ __align__(1024) bf16 As[MT * KT];
    __shared__ __align__(1024) bf16 Bs[NT * KT];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid / 32;
    const int m0 = blockIdx.y * MT, n0 = blockIdx.x * NT;
    if (warp == 0) tmem_alloc(&s_tmem, 32u);   // the 128 x NT FP32 accumulator
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
        s_fail = 0;
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (warp == 0) tmem_relinquish();
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = umma_idesc_bf16_f32(MT, NT);
    const bf16 zero = __float2bfloat16_rn(0.f);
    // element (row r, k) of a K-major operand: core matrix (r / 8, k / 8) of 64 elements, row r % 8
    auto at = [](int r, int k) { return ((r >> 3) * (KT / 8) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7); };
    uint32_t phase = 0;
    const int nkb = (g.K + KT - 1) / KT;
    for (int kb = 0; kb < nkb; kb++) {
        const int k0 = kb * KT;
        for (int e = tid; e < MT * KT; e += 128) {
            const int r = e / KT, c = e % KT, m = m0 + r, k = k0 + c;
            As[at(r, c)] = (m < g.M && k < g.K) ? g.A[(int64_t)m * g.sam + (int64_t)k * g.sak] : zero;
        }
        for (int e = tid; e < NT * KT; e += 128) {
            const int r = e / KT, c = e % KT, n = n0 + r, k = k0 + c;
            Bs[at(r, c)] = (n < g.N && k < g.K) ? g.B[(int64_t)k * g.sbk + (int64_t)n * g.sbn] : zero;
        }
        fence_proxy_async_smem();   // these writes, visible to the tensor core
        __syncthreads();
        if (tid == 0) {
            tc_fence_after_sync();
            const uint32_t a0 = smem_addr(As), b0 = smem_addr(Bs);
#pragma unroll
            for (int kk = 0; kk < KT / 16; kk++)   // K = 16 per MMA: two core matrices along K
                umma_bf16(tmem, umma_desc_kmajor(a0 + kk * 2 * LBO, LBO, SBO), umma_desc_kmajor(b0 + kk * 2 * LBO, LBO, SBO),
                          idesc, kb > 0 || kk > 0);
            umma_commit(&bar);
        }
        // the block's MMAs have read As and Bs once the barrier's phase completes
        const bool ok = mbar_wait(&bar, phase);
        phase ^= 1u;
        if (!ok) s_fail = 1;
        __syncthreads();
        if (s_fail) break;
    }
    if (!s_fail) {
        tc_fence_after_sync();
        float v[NT];
        const uint32_t row_addr = tmem + ((uint32_t)(warp * 32) << 16);   // lanes 32 w .. 32 w + 31
        tmem_ld16(row_addr, v);
        if constexpr (NT == 32) tmem_ld16(row_addr + 16u, v + 16);
        const int m = m0 + warp * 32 + (tid & 31);
        if (m < g.M) {
#pragma unroll
            for (int n = 0; n < NT; n++)
                if (n0 + n < g.N) {
                    float* c = g.C + (int64_t)m * g.scm + (int64_t)(n0 + n) * g.scn;
                    *c = g.accumulate ? *c + v[n] : v[n];
                }
        }
    } else if (tid == 0) {
        atomicExch(g.err, 1);
        mbar_wait(&bar, phase ^ 1u);   // the MMAs of the block whose wait gave up
    }
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after_sync();
        tmem_dealloc(tmem, 32u);
    }
}

cudaError_t gemm(GemmArgs g, cudaStream_t st) {
    if (g.M <= 0 || g.N <= 0) return cudaSuccess;
    if (!g.err) g.err = device_error_flag();
    if (!g.err) return cudaErrorMemoryAllocation;
    const int nt = g.N <= 16 ? 16 : 32;
    const dim3 grid((unsigned)((g.N + nt - 1) / nt), (unsigned)((g.M + kGemmM - 1) / kGemmM));
    if (nt == 16) k_gemm_bf16<16><<<grid, 128, 0, st>>>(g);
    else k_gemm_bf16<32><<<grid, 128, 0, st>>>(g);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ elementwise and layout kernels
__global__ void k_im2col1(const float* __restrict__ x, int B, bf16* __restrict__ a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)B * kP1 * kK1) return;
    const int j = (int)(i % kK1);
    const int64_t row = i / kK1;
    const int b = (int)(row / kP1), pos = (int)(row % kP1);
    float v = 0.f;
    if (j < kK1Real) {
        const int c = j / 27, tap = j % 27;
        const int x0 = pos % 8 + tap % 3 - 1, y0 = (pos / 8) % 8 + (tap / 3) % 3 - 1, z0 = pos / 64 + tap / 9 - 1;
        if (x0 >= 0 && x0 < 8 && y0 >= 0 && y0 < 8 && z0 >= 0 && z0 < 8)
            v = x[((int64_t)b * kIn + c) * kP1 + (z0 * 8 + y0) * 8 + x0];
    }
    a[i] = __float2bfloat16_rn(v);
}
// conv2's im2col: stride 2, padding 1, from H1 [tile][512][16]
__global__ void k_im2col2(const bf16* __restrict__ h1, int B, bf16* __restrict__ a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)B * kP2 * kK2) return;
    const int j = (int)(i % kK2);
    const int64_t row = i / kK2;
    const int b = (int)(row / kP2), o = (int)(row % kP2);
    const int c = j / 27, tap = j % 27;
    const int x0 = 2 * (o % 4) + tap % 3 - 1, y0 = 2 * ((o / 4) % 4) + (tap / 3) % 3 - 1, z0 = 2 * (o / 16) + tap / 9 - 1;
    bf16 v = __float2bfloat16_rn(0.f);
    if (x0 >= 0 && x0 < 8 && y0 >= 0 && y0 < 8 && z0 >= 0 && z0 < 8) v = h1[((int64_t)b * kP1 + (z0 * 8 + y0) * 8 + x0) * kC1 + c];
    a[i] = v;
}
// conv2's col2im (backward): dH1[tile][pos][c] = sum of dA2 over the (output, tap) pairs reading it,
// gathered (a fixed order: no atomics)
__global__ void k_col2im2(const float* __restrict__ da, int B, float* __restrict__ dh1) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)B * kP1 * kC1) return;
    const int c = (int)(i % kC1);
    const int64_t row = i / kC1;
    const int b = (int)(row / kP1), pos = (int)(row % kP1);
    const int px = pos % 8, py = (pos / 8) % 8, pz = pos / 64;
    float s = 0.f;
    for (int dz = 0; dz < 3; dz++) {
        const int tz = pz + 1 - dz;
        if (tz < 0 || (tz & 1) || tz / 2 >= 4) continue;
        for (int dy = 0; dy < 3; dy++) {
            const int ty = py + 1 - dy;
            if (ty < 0 || (ty & 1) || ty / 2 >= 4) continue;
            for (int dx = 0; dx < 3; dx++) {
                const int tx = px + 1 - dx;
                if (tx < 0 || (tx & 1) || tx / 2 >= 4) continue;
                const int o = (tz / 2 * 4 + ty / 2) * 4 + tx / 2;
                s += da[((int64_t)b * kP2 + o) * kK2 + c * 27 + dz * 9 + dy * 3 + dx];
            }
        }
    }
    dh1[i] = s;
}
// z = y + bias (kept for the backward pass), h = bf16(relu(z))
__global__ void k_bias_relu(const float* __restrict__ y, const float* __restrict__ bias, int64_t rows, int cols,
                            float* __restrict__ z, bf16* __restrict__ h) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const float v = y[i] + bias[i % cols];
    z[i] = v;
    h[i] = __float2bfloat16_rn(fmaxf(v, 0.f));
}
// gradient through the ReLU: dz = dh * (z > 0), as FP32 (for the bias gradient) and BF16 (GEMM operand)
__global__ void k_relu_back(const float* __restrict__ dh, const float* __restrict__ z, int64_t n, float* __restrict__ dz,
                            bf16* __restrict__ dzb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = z[i] > 0.f ? dh[i] : 0.f;
    dz[i] = v;
    dzb[i] = __float2bfloat16_rn(v);
}
// column sums (bias gradients), one block per column, fixed reduction order
__global__ void k_colsum(const float* __restrict__ x, int64_t rows, int cols, float* __restrict__ out) {
    const int c = blockIdx.x;
    float s = 0.f;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) s += x[r * cols + c];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}
// fc2 and the loss: out[b] = h3[b] . w4 + b4; with targets, dout = 2 (out - t) / B and the loss terms
__global__ void k_fc2(const bf16* __restrict__ h3, const float* __restrict__ w4, const float* __restrict__ b4, int B,
                      float* __restrict__ out, const float* __restrict__ target, float* __restrict__ dout,
                      float* __restrict__ sq) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float s = b4[0];
    for (int k = 0; k < kF; k++) s = fmaf(__bfloat162float(h3[(int64_t)b * kF + k]), __bfloat162float(__float2bfloat16_rn(w4[k])), s);
    out[b] = s;
    if (target) {
        const float d = s - target[b];
        dout[b] = 2.f * d / (float)B;
        sq[b] = d * d;
    }
}
// fc2 backward: dW4[k] = sum_b h3[b][k] dout[b], db4 = sum dout, dH3[b][k] = dout[b] w4[k]
__global__ void k_fc2_back(const bf16* __restrict__ h3, const float* __restrict__ w4, const float* __restrict__ dout, int B,
                           float* __restrict__ dw4, float* __restrict__ db4, float* __restrict__ dh3) {
    const int t = threadIdx.x;
    if (t < kF) {
        float s = 0.f;
        for (int b = 0; b < B; b++) s = fmaf(__bfloat162float(h3[(int64_t)b * kF + t]), dout[b], s);
        dw4[t] = s;
    } else if (t == kF) {
        float s = 0.f;
        for (int b = 0; b < B; b++) s += dout[b];
        db4[0] = s;
    }
    for (int64_t i = t; i < (int64_t)B * kF; i += blockDim.x)
        dh3[i] = dout[i / kF] * __bfloat162float(__float2bfloat16_rn(w4[i % kF]));
}
__global__ void k_to_bf16(const float* __restrict__ x, int64_t n, bf16* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}
// Adam on the FP32 master parameters
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}
// sum of the squared errors (the loss), fixed order
__global__ void k_sum(const float* __restrict__ x, int n, float* __restrict__ out) {
    __shared__ float red[256];
    float s = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------ the network object
struct Estimator {
    uint32_t max_batch = 0;
    float* params = nullptr;     // FP32 master parameters (kParams)
    float* grads = nullptr;      // FP32 gradients, same layout
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    bf16* wb = nullptr;          // BF16 copies of W1, W2, W3 (GEMM operands)
    // activations and their gradients for max_batch tiles
    bf16 *a1 = nullptr, *h1 = nullptr, *a2 = nullptr, *h2 = nullptr, *h3 = nullptr;
    float *y1 = nullptr, *z1 = nullptr, *y2 = nullptr, *z2 = nullptr, *y3 = nullptr, *z3 = nullptr, *out = nullptr;
    float *dout = nullptr, *sq = nullptr, *dh3 = nullptr, *dz3 = nullptr, *dh2 = nullptr, *dz2 = nullptr,
          *da2 = nullptr, *dh1 = nullptr, *dz1 = nullptr, *loss = nullptr;
    bf16 *dz3b = nullptr, *dz2b = nullptr, *dz1b = nullptr;
    int step = 0;
    cudaStream_t stream = nullptr;

    ~Estimator() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : {(void*)params, (void*)grads, (void*)adam_m, (void*)adam_v, (void*)wb, (void*)a1, (void*)h1,
                        (void*)a2, (void*)h2, (void*)h3, (void*)y1, (void*)z1, (void*)y2, (void*)z2, (void*)y3,
                        (void*)z3, (void*)out, (void*)dout, (void*)sq, (void*)dh3, (void*)dz3, (void*)dh2,
                        (void*)dz2, (void*)da2, (void*)dh1, (void*)dz1, (void*)loss, (void*)dz3b, (void*)dz2b,
                        (void*)dz1b})
            cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
    template <class T>
    static cudaError_t alloc(T** p, size_t n) { return cudaMalloc((void**)p, n * sizeof(T)); }

    cudaError_t init(uint32_t batch, uint64_t seed) {
        max_batch = batch;
        const size_t B = batch;
        cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = alloc(&params, kParams);
        if (e == cudaSuccess) e = alloc(&grads, kParams);
        if (e == cudaSuccess) e = alloc(&adam_m, kParams);
        if (e == cudaSuccess) e = alloc(&adam_v, kParams);
        if (e == cudaSuccess) e = alloc(&wb, (size_t)kK1 * kC1 + (size_t)kK2 * kC2 + (size_t)kK3 * kF);
        if (e == cudaSuccess) e = alloc(&a1, B * kP1 * kK1);
        if (e == cudaSuccess) e = alloc(&h1, B * kP1 * kC1);
        if (e == cudaSuccess) e = alloc(&a2, B * kP2 * kK2);
        if (e == cudaSuccess) e = alloc(&h2, B * kK3);
        if (e == cudaSuccess) e = alloc(&h3, B * kF);
        if (e == cudaSuccess) e = alloc(&y1, B * kP1 * kC1);
        if (e == cudaSuccess) e = alloc(&z1, B * kP1 * kC1);
        if (e == cudaSuccess) e = alloc(&y2, B * kP2 * kC2);
        if (e == cudaSuccess) e = alloc(&z2, B * kP2 * kC2);
        if (e == cudaSuccess) e = alloc(&y3, B * kF);
        if (e == cudaSuccess) e = alloc(&z3, B * kF);
        if (e == cudaSuccess) e = alloc(&out, B);
        if (e == cudaSuccess) e = alloc(&dout, B);
        if (e == cudaSuccess) e = alloc(&sq, B);
        if (e == cudaSuccess) e = alloc(&dh3, B * kF);
        if (e == cudaSuccess) e = alloc(&dz3, B * kF);
        if (e == cudaSuccess) e = alloc(&dh2, B * kK3);
        if (e == cudaSuccess) e = alloc(&dz2, B * kK3);
        if (e == cudaSuccess) e = alloc(&da2, B * kP2 * kK2);
        if (e == cudaSuccess) e = alloc(&dh1, B * kP1 * kC1);
        if (e == cudaSuccess) e = alloc(&dz1, B * kP1 * kC1);
        if (e == cudaSuccess) e = alloc(&loss, 1);
        if (e == cudaSuccess) e = alloc(&dz3b, B * kF);
        if (e == cudaSuccess) e = alloc(&dz2b, B * kK3);
        if (e == cudaSuccess) e = alloc(&dz1b, B * kP1 * kC1);
        if (e != cudaSuccess) return e;
        // He-uniform initial weights from a seeded 64-bit LCG, zero biases
        std::vector<float> h(kParams, 0.f);
        uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
        auto uni = [&]() {
            s = s * 6364136223846793005ull + 1442695040888963407ull;
            return (float)((double)(s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
        };
        auto fill = [&](size_t off, int rows, int real_rows, int cols, int fan_in) {
            const float a = std::sqrt(6.f / (float)fan_in);
            for (int r = 0; r < rows; r++)
                for (int c = 0; c < cols; c++) h[off + (size_t)r * cols + c] = r < real_rows ? a * uni() : 0.f;
        };
        fill(kOffW1, kK1, kK1Real, kC1, kK1Real);
        fill(kOffW2, kK2, kK2, kC2, kK2);
        fill(kOffW3, kK3, kK3, kF, kK3);
        fill(kOffW4, kF, kF, 1, kF);
        e = set_params(h.data());
        if (e == cudaSuccess) e = cudaMemsetAsync(adam_m, 0, kParams * 4, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(adam_v, 0, kParams * 4, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        step = 0;
        return e;
    }
    cudaError_t refresh_bf16() {
        k_to_bf16<<<blocks((int64_t)kK1 * kC1), 256, 0, stream>>>(params + kOffW1, (int64_t)kK1 * kC1, wb);
        k_to_bf16<<<blocks((int64_t)kK2 * kC2), 256, 0, stream>>>(params + kOffW2, (int64_t)kK2 * kC2, wb + kK1 * kC1);
        k_to_bf16<<<blocks((int64_t)kK3 * kF), 256, 0, stream>>>(params + kOffW3, (int64_t)kK3 * kF,
                                                                wb + kK1 * kC1 + kK2 * kC2);
        return cudaGetLastError();
    }
    cudaError_t set_params(const float* host) {
        cudaError_t e = cudaMemcpyAsync(params, host, kParams * 4, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = refresh_bf16();
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        return e;
    }

    // forward pass of B tiles (x: device [B][3][512] FP32); predictions in `out`
    cudaError_t forward(const float* x, int B, const float* target) {
        const bf16* W1 = wb;
        const bf16* W2 = wb + kK1 * kC1;
        const bf16* W3 = wb + kK1 * kC1 + kK2 * kC2;
        k_im2col1<<<blocks((int64_t)B * kP1 * kK1), 256, 0, stream>>>(x, B, a1);
        cudaError_t e = gemm({a1, kK1, 1, W1, kC1, 1, y1, kC1, 1, B * kP1, kC1, kK1, 0}, stream);
        if (e != cudaSuccess) return e;
        k_bias_relu<<<blocks((int64_t)B * kP1 * kC1), 256, 0, stream>>>(y1, params + kOffB1, (int64_t)B * kP1, kC1, z1, h1);
        k_im2col2<<<blocks((int64_t)B * kP2 * kK2), 256, 0, stream>>>(h1, B, a2);
        if ((e = gemm({a2, kK2, 1, W2, kC2, 1, y2, kC2, 1, B * kP2, kC2, kK2, 0}, stream)) != cudaSuccess) return e;
        k_bias_relu<<<blocks((int64_t)B * kK3), 256, 0, stream>>>(y2, params + kOffB2, (int64_t)B * kP2, kC2, z2, h2);
        if ((e = gemm({h2, kK3, 1, W3, kF, 1, y3, kF, 1, B, kF, kK3, 0}, stream)) != cudaSuccess) return e;
        k_bias_relu<<<blocks((int64_t)B * kF), 256, 0, stream>>>(y3, params + kOffB3, B, kF, z3, h3);
        k_fc2<<<blocks(B), 256, 0, stream>>>(h3, params + kOffW4, params + kOffB4, B, out, target, dout, sq);
        return cudaGetLastError();
    }
    // gradients of the mean squared error of the last forward pass (with targets) into `grads`
    cudaError_t backward(int B) {
        const bf16* W2 = wb + kK1 * kC1;
        const bf16* W3 = wb + kK1 * kC1 + kK2 * kC2;
        k_fc2_back<<<1, 256, 0, stream>>>(h3, params + kOffW4, dout, B, grads + kOffW4, grads + kOffB4, dh3);
        k_relu_back<<<blocks((int64_t)B * kF), 256, 0, stream>>>(dh3, z3, (int64_t)B * kF, dz3, dz3b);
        k_colsum<<<kF, 256, 0, stream>>>(dz3, B, kF, grads + kOffB3);
        // dW3 = H2^T dZ3, dH2 = dZ3 W3^T
        cudaError_t e = gemm({h2, 1, kK3, dz3b, kF, 1, grads + kOffW3, kF, 1, kK3, kF, B, 0}, stream);
        if (e == cudaSuccess) e = gemm({dz3b, kF, 1, W3, 1, kF, dh2, kK3, 1, B, kK3, kF, 0}, stream);
        if (e != cudaSuccess) return e;
        k_relu_back<<<blocks((int64_t)B * kK3), 256, 0, stream>>>(dh2, z2, (int64_t)B * kK3, dz2, dz2b);
        k_colsum<<<kC2, 256, 0, stream>>>(dz2, (int64_t)B * kP2, kC2, grads + kOffB2);
        // dW2 = A2^T dY2, dA2 = dY2 W2^T, then col2im
        e = gemm({a2, 1, kK2, dz2b, kC2, 1, grads + kOffW2, kC2, 1, kK2, kC2, B * kP2, 0}, stream);
        if (e == cudaSuccess) e = gemm({dz2b, kC2, 1, W2, 1, kC2, da2, kK2, 1, B * kP2, kK2, kC2, 0}, stream);
        if (e != cudaSuccess) return e;
        k_col2im2<<<blocks((int64_t)B * kP1 * kC1), 256, 0, stream>>>(da2, B, dh1);
        k_relu_back<<<blocks((int64_t)B * kP1 * kC1), 256, 0, stream>>>(dh1, z1, (int64_t)B * kP1 * kC1, dz1, dz1b);
        k_colsum<<<kC1, 256, 0, stream>>>(dz1, (int64_t)B * kP1, kC1, grads + kOffB1);
        // dW1 = A1^T dY1 (rows 81..95 of A1 are zero, so their gradient is too)
        e = gemm({a1, 1, kK1, dz1b, kC1, 1, grads + kOffW1, kC1, 1, kK1, kC1, B * kP1, 0}, stream);
        if (e != cudaSuccess) return e;
        k_sum<<<1, 256, 0, stream>>>(sq, B, loss);
        return cudaGetLastError();
    }
    cudaError_t adam(float lr) {
        step++;
        const float b1 = .9f, b2 = .999f;
        k_adam<<<blocks((int64_t)kParams), 256, 0, stream>>>(params, grads, adam_m, adam_v, (int64_t)kParams, lr, b1, b2,
                                                            1e-8f, 1.f - std::pow(b1, (float)step),
                                                            1.f - std::pow(b2, (float)step));
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? refresh_bf16() : e;
    }
};

size_t estimator_param_count() { return kParams; }

}  // namespace amr

using namespace amr;

#define AMR_API extern "C" __attribute__((visibility("default")))

struct amr_estimator {
    Estimator net;
};

AMR_API int amr_estimator_create(uint32_t max_batch, uint64_t seed, amr_estimator** out) {
    if (!out || max_batch == 0 || max_batch > (1u << 16)) return AMR_ERR_INVALID;
    amr_estimator* e = new (std::nothrow) amr_estimator;
    if (!e) return AMR_ERR_CAPACITY;
    const cudaError_t st = e->net.init(max_batch, seed);
    if (st != cudaSuccess) {
        delete e;
        return cuda_status(st);
    }
    *out = e;
    return AMR_OK;
}
AMR_API int amr_estimator_destroy(amr_estimator* e) {
    delete e;
    return AMR_OK;
}
AMR_API uint64_t amr_estimator_param_count(void) { return kParams; }
AMR_API int amr_estimator_get_params(amr_estimator* e, float* host) {
    if (!e || !host) return AMR_ERR_INVALID;
    cudaError_t st = cudaMemcpyAsync(host, e->net.params, kParams * 4, cudaMemcpyDeviceToHost, e->net.stream);
    if (st == cudaSuccess) st = cudaStreamSynchronize(e->net.stream);
    return cuda_status(st);
}
AMR_API int amr_estimator_set_params(amr_estimator* e, const float* host) {
    if (!e || !host) return AMR_ERR_INVALID;
    return cuda_status(e->net.set_params(host));
}
AMR_API int amr_estimator_forward(amr_estimator* e, const float* features, uint32_t n, float* out) {
    if (!e || (n && (!features || !out))) return AMR_ERR_INVALID;
    for (uint32_t b0 = 0; b0 < n; b0 += e->net.max_batch) {
        const int B = (int)std::min<uint32_t>(e->net.max_batch, n - b0);
        cudaError_t st = e->net.forward(features + (size_t)b0 * kIn * kP1, B, nullptr);
        if (st == cudaSuccess) st = cudaMemcpyAsync(out + b0, e->net.out, (size_t)B * 4, cudaMemcpyDeviceToDevice, e->net.stream);
        if (st != cudaSuccess) return cuda_status(st);
    }
    const int st = cuda_status(cudaStreamSynchronize(e->net.stream));
    return st ? st : take_device_error(device_error_flag());
}
AMR_API int amr_estimator_gradients(amr_estimator* e, const float* features, const float* targets, uint32_t n,
                                    float* grads_host, float* loss) {
    if (!e || !features || !targets || n == 0 || n > e->net.max_batch) return AMR_ERR_INVALID;
    cudaError_t st = e->net.forward(features, (int)n, targets);
    if (st == cudaSuccess) st = e->net.backward((int)n);
    float l = 0.f;
    if (st == cudaSuccess && grads_host)
        st = cudaMemcpyAsync(grads_host, e->net.grads, kParams * 4, cudaMemcpyDeviceToHost, e->net.stream);
    if (st == cudaSuccess) st = cudaMemcpyAsync(&l, e->net.loss, 4, cudaMemcpyDeviceToHost, e->net.stream);
    if (st == cudaSuccess) st = cudaStreamSynchronize(e->net.stream);
    if (loss) *loss = l / (float)n;
    const int status = cuda_status(st);
    return status ? status : take_device_error(device_error_flag());
}
AMR_API int amr_estimator_train_step(amr_estimator* e, const float* features, const float* targets, uint32_t n,
                                     float lr, float* loss) {
    if (!e || !features || !targets || n == 0 || n > e->net.max_batch || !(lr > 0.f)) return AMR_ERR_INVALID;
    cudaError_t st = e->net.forward(features, (int)n, targets);
    if (st == cudaSuccess) st = e->net.backward((int)n);
    if (st == cudaSuccess) st = e->net.adam(lr);
    float l = 0.f;
    if (st == cudaSuccess && loss) st = cudaMemcpyAsync(&l, e->net.loss, 4, cudaMemcpyDeviceToHost, e->net.stream);
    if (st == cudaSuccess) st = cudaStreamSynchronize(e->net.stream);
    if (loss) *loss = l / (float)n;
    const int status = cuda_status(st);
    return status ? status : take_device_error(device_error_flag());
}
