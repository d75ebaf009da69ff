// kernels_evolve.cu -- kernels of the BSSN evolution and of the scalar wave u_tt = Δu (evolve.h).
//
// Compiled with contraction on (-fmad=true): unlike the reference-semantics kernels, these have no
// reference device build to reproduce bit for bit; they are held to the FP64 oracle
// (oracle/bssn_evolve.c) within stated tolerances.
//
//   k_evo_init      analytic initial data on every cell (ghosts included) of every live slot
//   k_evo_derivs    derivative pass: a CTA per (domain, z-slab); each field's padded slab moves into
//                   shared memory with one 1-D bulk copy (two buffers, the next field in flight),
//                   then first / second / mixed derivatives, advection and Kreiss-Oliger terms
//   k_evo_rhs_*     pointwise right-hand side and RK4 stage update (BSSN: every input staged in
//                   shared memory by bulk copies and cp.async first)
//   k_evo_ghost     ghost fill of a stage's state, one face-normal axis per launch (copies from
//                   same-depth neighbours, separable tricubic interpolation from coarser ones)
//   k_evo_restrict  restriction of children into parents (leaves: 16-byte copies)
//   k_evo_prolong   tricubic prolongation of new domains
//   k_evo_constraints, k_evo_norms_*   Hamiltonian and momentum constraints, FP64 norms
#include <cmath>
#include <type_traits>

#include "amr_device.cuh"
#include "evolve.h"
#include "evolve_kernels.h"
#include "evolve_physics.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace amr {

namespace {

// Centre of a slot's domain in units of the root edge (the root spans [-1/2, 1/2]).
__device__ __forceinline__ void slot_centre(uint32_t pos, float c[3]) {
    const int depth = pos_depth(pos);
    c[0] = c[1] = c[2] = 0.f;
    uint32_t path = pos & kPathMask;
    float step = .25f;
    for (int i = 0; i < depth; i++, path >>= 3, step *= .5f)
        for (int a = 0; a < 3; a++) c[a] += (path & (1u << a)) ? step : -step;
}

// ------------------------------------------------------------------ initial data
__global__ void k_evo_init(EvoInitArgs a) {
    const uint32_t t = a.t, cells = t * t * t;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)a.used * cells) return;
    const uint32_t slot = (uint32_t)(gid / cells), c = (uint32_t)(gid % cells);
    const uint32_t pos = a.positions[slot];
    const int depth = pos_depth(pos);
    if (depth == -1) return;
    float ctr[3];
    slot_centre(pos, ctr);   // exact: sums of powers of two
    const double h = (double)a.outer_size / ((double)a.n * (double)(1u << depth));
    const uint32_t idx[3] = {c % t, (c / t) % t, c / (t * t)};
    double x[3];
    for (int k = 0; k < 3; k++) x[k] = (double)ctr[k] * a.outer_size + ((double)idx[k] + .5 - .5 * (double)t) * h;
    double u[kMaxFields];
    evo_initial_values(a.id, a.physics, x, u);
    for (int f = 0; f < a.nf; f++) {
        const float v = (float)(a.physics == 0 ? u[f] - bssn_offset(f) : u[f]);   // stored as the deviation
        a.out1[f][gid] = v;
        a.out2[f][gid] = v;
        a.out3[f][gid] = v;
    }
}

// ------------------------------------------------------------------ derivative pass
// A CTA per (domain, slab of ZS interior z-planes): the slab's padded planes (ZS + 6) of one field
// fit twice in shared memory.  ZS is a launch-shape choice (amr_sim_autotune times the compiled
// ones, DerivZs below); the default takes two cells per thread at 16^3 (one at 8^3 and 32^3): a
// thread keeps, per cell, the shift through the whole pass.
constexpr int deriv_default_zs(int n) { return n == 8 ? 4 : (n == 16 ? 2 : 1); }
template <int N, int ZS_ = deriv_default_zs(N)>
struct DerivShape {
    static constexpr int P = 3, T = N + 2 * P;
    static constexpr int ZS = ZS_;
    static constexpr int THREADS = 256;
    static constexpr int CELLS = N * N * ZS;
    static constexpr int CPT = CELLS / THREADS;          // cells per thread
    static constexpr uint32_t SLAB = (uint32_t)((ZS + 6) * T * T);   // floats
    static constexpr uint32_t SLAB_BYTES = SLAB * 4u;
    // two field slabs, then per cell the inverse conformal metric (6) and the running sums of
    // d_j d_k beta^k (3), which the BSSN pass keeps across its visits
    static constexpr size_t SMEM = 2u * SLAB_BYTES + 9u * CELLS * 4u + 64u;
    static_assert(CELLS % THREADS == 0 && N % ZS == 0, "whole cells per thread and planes per slab");
    // The row of a cell.  At N = 16 a warp would cover rows y and y + 1 of the 22-float padded
    // rows, whose shared-memory banks overlap for 6 lanes; rows y and y + 8 (176 floats = 16 banks
    // apart) make every tap of the warp conflict-free.
    __device__ static uint32_t row(uint32_t cell) {
        const uint32_t r = (cell / N) % N;
        return N == 16 ? (r >> 1) | ((r & 1u) << 3) : r;
    }
    static_assert(SLAB_BYTES % 16u == 0u && (T * T * 4) % 16 == 0, "slabs are aligned bulk copies");
};

// The order in which the derivative pass visits the fields: the shift first, so that the advection
// terms of the others can use it.
__device__ __forceinline__ int deriv_field_order(int physics, int i) {
    if (physics != 0) return i;
    return i < 3 ? F_BETAX + i : (i < 21 ? i - 3 : i);
}

template <int N, int ZS_>
__global__ void __launch_bounds__(DerivShape<N, ZS_>::THREADS, DerivShape<N, ZS_>::CPT <= 2 ? 3 : 2)
    k_evo_derivs(const __grid_constant__ EvoArgs a) {
    using S = DerivShape<N, ZS_>;
    constexpr int T = S::T, ZS = S::ZS, CPT = S::CPT;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* buf = reinterpret_cast<float*>(smem_raw);
    float* s_gi = reinterpret_cast<float*>(smem_raw + 2u * S::SLAB_BYTES);   // [6][CELLS]
    float* s_ddb = s_gi + 6 * S::CELLS;                                         // [3][CELLS]
    uint64_t* bar = reinterpret_cast<uint64_t*>(s_ddb + 3 * S::CELLS);
    __shared__ int s_abort;

    const uint32_t tid = threadIdx.x;
    const uint32_t slabs = N / ZS;
    const uint32_t item = blockIdx.x / slabs, slab = blockIdx.x % slabs;
    if (item >= a.n_items) return;
    const uint32_t slot = a.items[item];
    const int depth = pos_depth(a.positions[slot]);
    const int nf = a.prm.physics == 0 ? BSSN_NF : WAVE_NF;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
        s_abort = 0;
    }
    __syncthreads();
    const size_t src_off = (size_t)slot * T * T * T + (size_t)slab * ZS * T * T;   // padded plane slab*ZS (p = 3)
    auto issue = [&](int i) {   // field of visit i into buffer i % 2
        const int f = deriv_field_order(a.prm.physics, i);
        mbar_arrive_expect_tx(&bar[i & 1], S::SLAB_BYTES);
        bulk_g2s(buf + (size_t)(i & 1) * S::SLAB, a.fields[f] + src_off, S::SLAB_BYTES, &bar[i & 1]);
    };
    if (tid == 0) {
        issue(0);
        if (nf > 1) issue(1);
    }
    const float h = a.prm.outer_size / ((float)N * (float)(1u << depth));
    const float i12h = 1.f / (12.f * h), i12h2 = 1.f / (12.f * h * h), i144h2 = 1.f / (144.f * h * h);
    const float ko = a.prm.ko_sigma / (64.f * h);
    const bool bssn = a.prm.physics == 0;
    const bool shift_on = bssn && a.prm.shift != 0;
    // the shift at each of this thread's cells, for the advection terms of every field, and the
    // inverse conformal metric, for the contracted second derivatives (evolve.h)
    float beta[CPT][3];
#pragma unroll
    for (int c = 0; c < CPT; c++) {
        const uint32_t cell = tid + (uint32_t)c * S::THREADS;
        const uint32_t x = cell % N, y = S::row(cell), z = slab * ZS + cell / (N * N);
        const size_t pi = (size_t)slot * T * T * T + ((size_t)(z + 3) * T + (y + 3)) * T + (x + 3);
#pragma unroll
        for (int k = 0; k < 3; k++) { beta[c][k] = bssn ? a.fields[F_BETAX + k][pi] : 0.f; s_ddb[k * S::CELLS + cell] = 0.f; }
        float g[6], m[3][3];
#pragma unroll
        for (int k = 0; k < 6; k++) g[k] = bssn ? a.fields[F_GXX + k][pi] + bssn_offset(F_GXX + k) : (k == 0 || k == 3 || k == 5 ? 1.f : 0.f);
        inverse_sym(g, m);
        const float gi6[6] = {m[0][0], m[1][1], m[2][2], m[0][1], m[0][2], m[1][2]};   // xx yy zz xy xz yz
#pragma unroll
        for (int k = 0; k < 6; k++) s_gi[k * S::CELLS + cell] = gi6[k];
    }
    float* D = a.deriv;
    const uint64_t ds = a.deriv_stride;

    int stopped = nf;   // the visit at which a wait gave up
    for (int i = 0; i < nf; i++) {
        const int f = deriv_field_order(a.prm.physics, i);
        const bool ok = mbar_wait(&bar[i & 1], (uint32_t)(i >> 1) & 1u);
        if (!ok) s_abort = 1;
        __syncthreads();
        if (s_abort) { stopped = i; break; }
        const float* tile = buf + (size_t)(i & 1) * S::SLAB;
        // what this field keeps (evolve.h), decided once per visit: 0 nothing but its extra term,
        // 1 first derivatives, 2 first and all six second (chi, alpha), 3 first and the metric
        // contraction of the second (gt_ij), 4 as 3 plus d_j d_k beta^k (beta^i), 5 the Laplacian (u)
        int kind = 0, first = -1, second = -1;
        if (bssn) {
            if (f == F_CHI) { kind = 2; first = D_CHI1; second = D_CHI2; }
            else if (f >= F_GXX && f <= F_GZZ) { kind = 3; first = D_G1 + 3 * (f - F_GXX); second = D_GLAP + (f - F_GXX); }
            else if (f == F_K) { kind = 1; first = D_K1; }
            else if (f >= F_AXX && f <= F_AZZ) { if (a.constraints) { kind = 1; first = D_AT1 + 3 * (f - F_AXX); } }
            else if (f >= F_GAMX && f <= F_GAMZ) { kind = 1; first = D_GAM1 + 3 * (f - F_GAMX); }
            else if (f == F_ALPHA) { kind = 2; first = D_AL1; second = D_AL2; }
            else if (f >= F_BETAX && f <= F_BETAZ) { kind = 4; first = D_BE1 + 3 * (f - F_BETAX); second = D_BELAP + (f - F_BETAX); }
        } else if (f == W_U) {
            kind = 5;
        }
        const int bk = f - F_BETAX;   // kind 4: the shift component
        const bool zero_extra = bssn && !shift_on && f >= F_BETAX;   // a frozen shift and its driver
        float* const Dx = D + (uint64_t)((bssn ? D_EXTRA : WD_EXTRA) + f) * ds;
        float* const D1 = D + (uint64_t)(first < 0 ? 0 : first) * ds;
        float* const D2 = D + (uint64_t)(second < 0 ? 0 : second) * ds;
        auto cells = [&](auto KIND) {
            constexpr int K = decltype(KIND)::value;
#pragma unroll
            for (int c = 0; c < CPT; c++) {
                const uint32_t cell = tid + (uint32_t)c * S::THREADS;
                const uint32_t x = cell % N, y = S::row(cell), zl = cell / (N * N);
                const uint32_t z = slab * ZS + zl;
                const float* q = tile + ((zl + 3) * T + (y + 3)) * T + (x + 3);
                const uint64_t o = ((uint64_t)slot * N + z) * N * N + (uint64_t)y * N + x;
                constexpr int st[3] = {1, T, T * T};
                float d1[3], ko_sum = 0.f;
#pragma unroll
                for (int ax = 0; ax < 3; ax++) {
                    const int s = st[ax];
                    d1[ax] = ((q[-2 * s] - q[2 * s]) + 8.f * (q[s] - q[-s])) * i12h;
                    ko_sum += (q[-3 * s] + q[3 * s]) - 6.f * (q[-2 * s] + q[2 * s]) + 15.f * (q[-s] + q[s]) - 20.f * q[0];
                }
                if constexpr (K >= 1 && K <= 4)
#pragma unroll
                    for (int ax = 0; ax < 3; ax++) D1[(uint64_t)ax * ds + o] = d1[ax];
                if constexpr (K >= 2) {
                    float dd[3];
#pragma unroll
                    for (int ax = 0; ax < 3; ax++) {
                        const int s = st[ax];
                        dd[ax] = (16.f * (q[-s] + q[s]) - (q[-2 * s] + q[2 * s]) - 30.f * q[0]) * i12h2;
                    }
                    if constexpr (K == 5) {
                        D[(uint64_t)WD_LAP * ds + o] = dd[0] + dd[1] + dd[2];
                    } else {
                        constexpr int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
                        constexpr float w[4] = {1.f, -8.f, 8.f, -1.f};
                        constexpr int off[4] = {-2, -1, 1, 2};
                        float d2[6] = {dd[0], dd[1], dd[2], 0.f, 0.f, 0.f};   // xx yy zz xy xz yz
#pragma unroll
                        for (int m = 0; m < 3; m++) {
                            const int sa = st[pa[m]], sb = st[pb[m]];
                            float acc = 0.f;
#pragma unroll
                            for (int u = 0; u < 4; u++) {
                                float row = 0.f;
#pragma unroll
                                for (int v = 0; v < 4; v++) row = fmaf(w[v], q[off[u] * sa + off[v] * sb], row);
                                acc = fmaf(w[u], row, acc);
                            }
                            d2[3 + m] = acc * i144h2;
                        }
                        if constexpr (K == 2) {   // all six
#pragma unroll
                            for (int k = 0; k < 6; k++) D2[(uint64_t)k * ds + o] = d2[k];
                        } else {
                            // gt^lm d_l d_m of the field (the metric's and the shift's components)
                            const float* G = s_gi + cell;   // G[k * CELLS]: this cell's inverse metric
                            constexpr int C = S::CELLS;
                            D2[o] = G[0] * d2[0] + G[C] * d2[1] + G[2 * C] * d2[2] +
                                    2.f * (G[3 * C] * d2[3] + G[4 * C] * d2[4] + G[5 * C] * d2[5]);
                            if constexpr (K == 4) {   // d_j d_k beta^k, k = this component
                                float* B = s_ddb + cell;
                                B[0] += bk == 0 ? d2[0] : (bk == 1 ? d2[3] : d2[4]);
                                B[C] += bk == 0 ? d2[3] : (bk == 1 ? d2[1] : d2[5]);
                                B[2 * C] += bk == 0 ? d2[4] : (bk == 1 ? d2[5] : d2[2]);
                                if (bk == 2)
#pragma unroll
                                    for (int j = 0; j < 3; j++) D[(uint64_t)(D_DDIVB + j) * ds + o] = B[j * C];
                            }
                        }
                    }
                }
                // advection along the shift and dissipation
                float extra = ko * ko_sum;
                if (bssn) {
                    extra = fmaf(beta[c][0], d1[0], fmaf(beta[c][1], d1[1], fmaf(beta[c][2], d1[2], extra)));
                    if (zero_extra) extra = 0.f;
                }
                Dx[o] = extra;
            }
        };
        switch (kind) {
            case 1: cells(std::integral_constant<int, 1>{}); break;
            case 2: cells(std::integral_constant<int, 2>{}); break;
            case 3: cells(std::integral_constant<int, 3>{}); break;
            case 4: cells(std::integral_constant<int, 4>{}); break;
            case 5: cells(std::integral_constant<int, 5>{}); break;
            default: cells(std::integral_constant<int, 0>{}); break;
        }
        __syncthreads();   // every thread is done with buffer i % 2
        if (tid == 0 && i + 2 < nf) issue(i + 2);
    }
    // Every copy issued was waited for, except after a wait gave up at visit `stopped`: the copies
    // of visits stopped and stopped + 1 may still be in flight, and the CTA's shared memory must
    // outlive them (bounded waits).
    if (stopped < nf && tid == 0) {
        atomicExch(a.err, 1);
        for (int i = stopped; i < nf && i <= stopped + 1; i++) mbar_wait(&bar[i & 1], (uint32_t)(i >> 1) & 1u);
    }
}

// ------------------------------------------------------------------ right-hand sides and stage update
// RK4: stage 1: acc = old + dt/6 k1, out = old + dt/2 k1; stage 2: acc += dt/3 k2, out = old + dt/2 k2;
// stage 3: acc += dt/3 k3, out = old + dt k3; stage 4: out = acc + dt/6 k4.
// `lo`: the stage outputs' lower bound (the conformal factor's floor; -inf for the other fields).
// A NaN stays a NaN.
__device__ __forceinline__ void rk_update(const EvoArgs& a, int f, uint64_t pi, uint64_t ii, float u_old, float r,
                                          float dt, float lo = -INFINITY) {
    float v;
    switch (a.stage) {
        case 1:
            a.acc[f][ii] = fmaf(dt * (1.f / 6.f), r, u_old);
            v = fmaf(dt * .5f, r, u_old);
            break;
        case 2:
            a.acc[f][ii] = fmaf(dt * (1.f / 3.f), r, a.acc[f][ii]);
            v = fmaf(dt * .5f, r, u_old);
            break;
        case 3:
            a.acc[f][ii] = fmaf(dt * (1.f / 3.f), r, a.acc[f][ii]);
            v = fmaf(dt, r, u_old);
            break;
        default:
            v = fmaf(dt * (1.f / 6.f), r, a.acc[f][ii]);
            break;
    }
    a.out[f][pi] = v < lo ? lo : v;
}

// BSSN right-hand side and RK stage update: a CTA per kRhsCells consecutive interior cells of one
// domain, every input in shared memory before the arithmetic starts.  Thread 0 issues one bulk
// copy per derivative plane (and, after the first stage, per RK-accumulator plane): kRhsCells * 4
// contiguous bytes of the inner layout each, counted on one mbarrier.  Every thread meanwhile
// issues 4-byte asynchronous copies (cp.async) of its cell's fields and their step-start values
// from the padded layout, and waits for its own.  Consecutive threads read consecutive words.
// Stage 1 stages the derivatives and fields, stages 2 and 3 also the step-start values and the
// accumulator, stage 4 the accumulator only (it updates from it): 30, 42 and 36 KB per CTA, so
// 6, 5 and 6 CTAs per SM (128 cells at stages 2-3: 2 CTAs per SM, 539 against 480 us).
constexpr int kRhsCells = 64;
__host__ __device__ constexpr int rhs_planes(int stage) {   // derivatives, fields, [step-start values], [accumulator]
    return BSSN_ND + BSSN_NF + (stage == 2 || stage == 3 ? 2 * BSSN_NF : (stage == 4 ? BSSN_NF : 0));
}
constexpr size_t rhs_smem(int stage) { return (size_t)rhs_planes(stage) * kRhsCells * 4u + 16u; }
constexpr size_t kRhsSmem = rhs_smem(2);   // the largest

__device__ __forceinline__ void cp_async4(float* dst_smem, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst_smem)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

template <int N>
__global__ void __launch_bounds__(kRhsCells) k_evo_rhs_bssn(const __grid_constant__ EvoArgs a) {
    constexpr int P = 3, T = N + 2 * P, C = kRhsCells;
    constexpr uint32_t CHUNKS = (uint32_t)(N * N * N / kRhsCells);
    static_assert((N * N * N) % kRhsCells == 0 && (kRhsCells * 4) % 16 == 0, "whole, aligned chunks per domain");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const bool later = a.stage != 1;                        // stages 2-4 read the accumulator
    const bool start = a.stage == 2 || a.stage == 3;        // stages 2-3 the step-start state
    float* sd = reinterpret_cast<float*>(smem_raw);   // [BSSN_ND][C] derivatives
    float* su = sd + (size_t)BSSN_ND * C;              // [BSSN_NF][C] fields (stored form)
    float* so = su + (size_t)BSSN_NF * C;              // [BSSN_NF][C] step-start values (stages 2-3)
    float* sa = so + (start ? (size_t)BSSN_NF * C : 0u);   // [BSSN_NF][C] RK accumulator (stages 2-4)
    uint64_t* bar = reinterpret_cast<uint64_t*>(sa + (later ? (size_t)BSSN_NF * C : 0u));
    const uint32_t tid = threadIdx.x;
    const uint32_t item = blockIdx.x / CHUNKS, chunk = blockIdx.x % CHUNKS;
    if (item >= a.n_items) return;   // the whole CTA
    const uint32_t slot = a.items[item];
    const uint32_t cell = chunk * (uint32_t)kRhsCells + tid;
    const uint64_t ii0 = (uint64_t)slot * N * N * N + chunk * (uint32_t)kRhsCells;
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, (uint32_t)((BSSN_ND + (later ? BSSN_NF : 0)) * C * 4));
        for (int k = 0; k < BSSN_ND; k++)
            bulk_g2s(sd + k * C, a.deriv + (uint64_t)k * a.deriv_stride + ii0, C * 4u, bar);
        if (later)
            for (int f = 0; f < BSSN_NF; f++) bulk_g2s(sa + f * C, a.acc[f] + ii0, C * 4u, bar);
    }
    const uint32_t x = cell % N, y = (cell / N) % N, z = cell / (N * N);
    const uint64_t pi = (uint64_t)slot * T * T * T + ((uint64_t)(z + P) * T + (y + P)) * T + (x + P);
    const uint64_t ii = ii0 + tid;
#pragma unroll
    for (int f = 0; f < BSSN_NF; f++) {
        cp_async4(su + f * C + tid, a.fields[f] + pi);
        if (start) cp_async4(so + f * C + tid, a.old_f[f] + pi);
    }
    const int depth = pos_depth(a.positions[slot]);
    const float dt = a.dt0 / (float)(1u << depth);
    cp_async_wait_all();   // this thread's own copies (only it reads them)
    // every bulk copy lands before any thread reads them or leaves (bounded waits)
    const bool ok = __syncthreads_and(mbar_wait(bar, 0));
    if (!ok) {
        if (tid == 0) {
            atomicExch(a.err, 1);
            mbar_wait(bar, 0);
        }
        __syncthreads();
        return;
    }
    float u[BSSN_NF];
#pragma unroll
    for (int f = 0; f < BSSN_NF; f++) u[f] = su[f * C + tid] + bssn_offset(f);
    auto dv = [&](int k) { return sd[k * C + tid]; };
    float rhs[BSSN_NF];
    bssn_rhs(u, dv, a.prm, rhs);
    // RK4 (rk_update): stage 1: acc = old + dt/6 k1, out = old + dt/2 k1; stage 2: acc += dt/3 k2,
    // out = old + dt/2 k2; stage 3: acc += dt/3 k3, out = old + dt k3; stage 4: out = acc + dt/6 k4
    const float c_acc = a.stage == 1 ? dt * (1.f / 6.f) : dt * (1.f / 3.f);
    const float c_out = a.stage == 3 ? dt : (a.stage == 4 ? dt * (1.f / 6.f) : dt * .5f);
#pragma unroll
    for (int f = 0; f < BSSN_NF; f++) {
        const float r = rhs[f] + dv(D_EXTRA + f);
        float v;
        if (a.stage == 4) {
            v = fmaf(c_out, r, sa[f * C + tid]);
        } else {
            const float uo = start ? so[f * C + tid] : su[f * C + tid];   // the stored form
            a.acc[f][ii] = fmaf(c_acc, r, later ? sa[f * C + tid] : uo);
            v = fmaf(c_out, r, uo);
        }
        // chi (stored less 1) is kept at or above its floor, as the geometry divides by it
        const float lo = f == F_CHI ? a.prm.chi_floor - 1.f : -INFINITY;
        a.out[f][pi] = v < lo ? lo : v;
    }
}

template <int N>
__global__ void __launch_bounds__(256) k_evo_rhs_wave(const __grid_constant__ EvoArgs a) {
    constexpr int P = 3, T = N + 2 * P;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)a.n_items * N * N * N) return;
    const uint32_t item = (uint32_t)(gid / (N * N * N)), cell = (uint32_t)(gid % (N * N * N));
    const uint32_t slot = a.items[item];
    const uint32_t x = cell % N, y = (cell / N) % N, z = cell / (N * N);
    const int depth = pos_depth(a.positions[slot]);
    const float dt = a.dt0 / (float)(1u << depth);
    const uint64_t pi = (uint64_t)slot * T * T * T + ((uint64_t)(z + P) * T + (y + P)) * T + (x + P);
    const uint64_t ii = (uint64_t)slot * N * N * N + cell;
    const float* D = a.deriv;
    const uint64_t ds = a.deriv_stride;
    const float uu = a.fields[W_U][pi], vv = a.fields[W_V][pi];
    const float r_u = vv + D[(uint64_t)(WD_EXTRA + W_U) * ds + ii];
    const float r_v = D[(uint64_t)WD_LAP * ds + ii] + D[(uint64_t)(WD_EXTRA + W_V) * ds + ii];
    rk_update(a, W_U, pi, ii, a.stage == 1 ? uu : a.old_f[W_U][pi], r_u, dt);
    rk_update(a, W_V, pi, ii, a.stage == 1 ? vv : a.old_f[W_V][pi], r_v, dt);
}

// ------------------------------------------------------------------ ghost fill
// A CTA per (slot, side, group of kGhostFields fields).  A same-depth face is a copy: the geometry of
// a ghost cell is computed once per group and every load of a cell's group is issued before its
// stores.  A face with a coarser source is interpolated separably through shared memory (below).
// Within one launch (one face-normal axis) no cell is both read and written: the fill writes the
// cells whose index along the axis lies in a ghost layer and reads sources inside the interior
// along it.
constexpr int kGhostFields = 4;
constexpr uint32_t kGhostMaxT = 38;   // the largest padded edge (32 + 2 * 3)
// Shared memory of the interpolating faces, in floats, for padded edge t, size n, padding p: the
// per-axis tables, then the largest source box (E_a <= ext_a / 2 + 5 cells along each axis, the
// source being at least twice as coarse) and the two intermediate stages, over the three passes.
inline uint32_t ghost_interp_floats(uint32_t n, uint32_t p, uint32_t t) {
    uint32_t best = 0;
    for (uint32_t d = 0; d < 3; d++) {
        uint32_t ext[3], E[3];
        for (uint32_t a = 0; a < 3; a++) {
            ext[a] = a == d ? p : (a < d ? t : n);
            E[a] = ext[a] / 2u + 5u;
        }
        const uint32_t need = E[0] * E[1] * E[2] + E[2] * E[1] * ext[0] + E[2] * ext[1] * ext[0];
        best = need > best ? need : best;
    }
    return best;
}

__global__ void __launch_bounds__(256, 4) k_evo_ghost(const __grid_constant__ EvoGhostArgs g) {
    const uint32_t item = blockIdx.x >> 1, side = blockIdx.x & 1u;   // side 0: + face, 1: - face
    const int f0 = (int)blockIdx.y * kGhostFields;
    if (item >= g.n_items || f0 >= g.nf) return;
    const uint32_t slot = g.items[item];
    const uint32_t n = g.n, p = g.p, t = g.t, d = (uint32_t)g.axis;
    const uint32_t face = d + 3u * side;
    const uint64_t bd = g.boundaries[(size_t)slot * 6u + face];
    const int32_t src = bd_target(bd);
    const int cd = bd_curr_depth(bd);
    if (src == -1 || cd <= 0) return;
    const uint32_t dd = bd_depth_diff(bd);
    const int sd = cd - (int)dd;
    const bool root_src = src == 0;
    const bool src_evolved = g.evolved[src] != 0;
    const bool src_active = active_depth(g.substep, (uint32_t)sd, g.max_depth);
    // the source's state at the time of the value being filled (evolve.h)
    int mode;      // 0: old only, 1: X only, 2: old..X, 3: old..new
    float frac = 0.f;
    if (!src_evolved) mode = 0;
    else if (src_active) {
        mode = dd == 0u ? 1 : 2;
        frac = 1.f / (float)(1u << dd);
    } else {
        mode = 3;
        const uint32_t kp = (g.substep >> (g.max_depth - (uint32_t)cd)) & ((1u << dd) - 1u);
        frac = ((float)kp + g.c_stage) / (float)(1u << dd);
    }
    const float3 relp = cf3_decode((uint32_t)(bd >> 32));
    const float rel_scale = 1.f / (float)(1u << dd);
    // extents of the fill: axes before d over the whole padded range (their ghosts are filled),
    // axes after d over the interior
    auto lo_of = [&](uint32_t a2) { return a2 == d ? (side == 0 ? p + n : 0u) : (a2 < d ? 0u : p); };
    auto ext_of = [&](uint32_t a2) { return a2 == d ? p : (a2 < d ? t : n); };
    const uint32_t lo0 = lo_of(0), lo1 = lo_of(1), lo2 = lo_of(2);
    const uint32_t ext0 = ext_of(0), ext1 = ext_of(1), ext2 = ext_of(2);
    const int nfg = min(kGhostFields, g.nf - f0);
    // field of group member q (members past the last field repeat it; they are never stored)
    auto fld = [&](int q) { return f0 + min(q, nfg - 1); };
    auto A0 = [&](int q) { return g.old_f[fld(q)]; };
    auto A1 = [&](int q) { return mode == 3 ? g.new_f[fld(q)] : (const float*)g.X[fld(q)]; };
    const uint32_t count = ext0 * ext1 * ext2;
    const uint64_t cells = (uint64_t)t * t * t;
    const bool exact = dd == 0u;
    // k -> (w0, w1, w2) by multiplication: floor(k * ceil(2^21 / e) / 2^21) = floor(k / e) for
    // k < 2^21 / 38^2 and e <= 38 (the error k * (ceil - exact) / 2^21 stays below 1 / e)
    const uint32_t m0 = ((1u << 21) + ext0 - 1u) / ext0, m1 = ((1u << 21) + ext1 - 1u) / ext1;
    // a same-depth source is this domain shifted by rel * n cells (rel = 0 or +-1 per axis, exact)
    const int r0 = __float2int_rn(relp.x * (float)n), r1 = __float2int_rn(relp.y * (float)n),
              r2 = __float2int_rn(relp.z * (float)n);
    if (exact) {
        for (uint32_t k = threadIdx.x; k < count; k += blockDim.x) {
            const uint32_t q = (uint32_t)(((uint64_t)k * m0) >> 21), q2 = (uint32_t)(((uint64_t)q * m1) >> 21);
            const uint32_t w0 = lo0 + (k - q * ext0), w1 = lo1 + (q - q2 * ext1), w2 = lo2 + q2;
            const uint64_t dst = (uint64_t)slot * cells + ((uint64_t)w2 * t + w1) * t + w0;
            // a copy: every load of the group, then the stores
            const int64_t si = (int64_t)src * (int64_t)cells + ((int64_t)((int)w2 + r2) * t + ((int)w1 + r1)) * t +
                               ((int)w0 + r0);
            float v[kGhostFields];
#pragma unroll
            for (int q4 = 0; q4 < kGhostFields; q4++)
                v[q4] = mode == 0 ? A0(q4)[si] : (mode == 1 ? A1(q4)[si] : fmaf(frac, A1(q4)[si], (1.f - frac) * A0(q4)[si]));
#pragma unroll
            for (int q4 = 0; q4 < kGhostFields; q4++)
                if (q4 < nfg) g.X[f0 + q4][dst] = v[q4];
        }
        return;
    }
    // A coarser source: separable tricubic interpolation through shared memory.  Along each axis a
    // the ghost cell's coordinate w_a alone gives the base cell b_a of its four-point stencil
    // b_a - 1 .. b_a + 2 and the four Lagrange weights; b_a is kept inside the cells that are
    // valid (the interior along the normal axis and the later axes, the whole padded range along
    // the earlier axes, which earlier passes filled, and everywhere in the root, whose frozen
    // ghost layer is the outer boundary).  b_a grows with w_a, so the source cells read form a
    // box.  Per field: the box, with the time interpolation applied to each source cell
    // (frac X + (1 - frac) old, or old alone), then the interpolation along x, along y and along z,
    // each stage through shared memory.
    extern __shared__ __align__(16) float gsm[];
    float* W = gsm;                                                  // [3][kGhostMaxT][4] weights
    int* B = reinterpret_cast<int*>(W + 3 * kGhostMaxT * 4);         // [3][kGhostMaxT] base cells
    float* S = reinterpret_cast<float*>(B + 3 * kGhostMaxT);         // source box (time-interpolated)
    for (uint32_t e = threadIdx.x; e < ext0 + ext1 + ext2; e += blockDim.x) {
        const uint32_t a2 = e < ext0 ? 0u : (e < ext0 + ext1 ? 1u : 2u);
        const uint32_t j = e - (a2 == 0u ? 0u : (a2 == 1u ? ext0 : ext0 + ext1));
        const uint32_t wa = (a2 == 0u ? lo0 : (a2 == 1u ? lo1 : lo2)) + j;
        float rp = ((float)wa - (float)p + .5f) / (float)n - .5f;
        rp = rp * rel_scale + (a2 == 0u ? relp.x : (a2 == 1u ? relp.y : relp.z));
        const float ri = (rp + .5f) * (float)n + (float)p - .5f;
        const int lo_c = root_src || a2 < d ? 1 : (int)p + 1;
        const int hi_c = root_src || a2 < d ? (int)t - 3 : (int)(t - p) - 3;
        int b = __float2int_rd(ri);
        b = b < lo_c ? lo_c : (b > hi_c ? hi_c : b);
        const float x = ri - (float)b;
        B[a2 * kGhostMaxT + j] = b;
        float* w = W + (a2 * kGhostMaxT + j) * 4;
        w[0] = -x * (x - 1.f) * (x - 2.f) * (1.f / 6.f);
        w[1] = (x + 1.f) * (x - 1.f) * (x - 2.f) * .5f;
        w[2] = -(x + 1.f) * x * (x - 2.f) * .5f;
        w[3] = (x + 1.f) * x * (x - 1.f) * (1.f / 6.f);
    }
    __syncthreads();
    // the box: from b_min - 1 to b_max + 2 along each axis (the first and the last w_a)
    const int bmin[3] = {B[0], B[kGhostMaxT], B[2 * kGhostMaxT]};
    const int E[3] = {B[ext0 - 1] - bmin[0] + 4, B[kGhostMaxT + ext1 - 1] - bmin[1] + 4,
                      B[2 * kGhostMaxT + ext2 - 1] - bmin[2] + 4};
    const uint32_t nS = (uint32_t)(E[0] * E[1] * E[2]), nT1 = (uint32_t)(E[2] * E[1]) * ext0,
                   nT2 = (uint32_t)E[2] * ext1 * ext0;
    if (nS + nT1 + nT2 > g.interp_floats) {   // larger than the launch provided: report, skip the face
        if (threadIdx.x == 0) atomicExch(g.err, 1);
        return;
    }
    float* T1 = S + nS;    // [E2][E1][ext0]
    float* T2 = T1 + nT1;  // [E2][ext1][ext0]
    const int64_t sbase = (int64_t)src * (int64_t)cells;
    for (int q4 = 0; q4 < nfg; q4++) {
        const float* a0 = A0(q4);
        const float* a1 = A1(q4);
        for (uint32_t e = threadIdx.x; e < nS; e += blockDim.x) {
            const uint32_t i0 = e % (uint32_t)E[0], r = e / (uint32_t)E[0];
            const uint32_t i1 = r % (uint32_t)E[1], i2 = r / (uint32_t)E[1];
            const int64_t si = sbase + ((int64_t)(bmin[2] - 1 + (int)i2) * t + (bmin[1] - 1 + (int)i1)) * t +
                               (bmin[0] - 1 + (int)i0);
            S[e] = mode == 0 ? a0[si] : fmaf(frac, a1[si], (1.f - frac) * a0[si]);
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < nT1; e += blockDim.x) {   // along x
            const uint32_t j0 = e % ext0, r = e / ext0;              // r = i2 * E1 + i1
            const float* w = W + j0 * 4;
            const float* src_row = S + r * (uint32_t)E[0] + (B[j0] - bmin[0]);
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < 4; k++) v = fmaf(w[k], src_row[k], v);
            T1[e] = v;
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < nT2; e += blockDim.x) {   // along y
            const uint32_t j0 = e % ext0, r = e / ext0, j1 = r % ext1, i2 = r / ext1;
            const float* w = W + (kGhostMaxT + j1) * 4;
            const float* col = T1 + ((size_t)i2 * E[1] + (B[kGhostMaxT + j1] - bmin[1])) * ext0 + j0;
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < 4; k++) v = fmaf(w[k], col[(size_t)k * ext0], v);
            T2[e] = v;
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < count; e += blockDim.x) {   // along z, into the ghost cells
            const uint32_t j0 = e % ext0, r = e / ext0, j1 = r % ext1, j2 = r / ext1;
            const float* w = W + (2 * kGhostMaxT + j2) * 4;
            const float* col = T2 + ((size_t)(B[2 * kGhostMaxT + j2] - bmin[2]) * ext1 + j1) * ext0 + j0;
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < 4; k++) v = fmaf(w[k], col[(size_t)k * ext1 * ext0], v);
            g.X[f0 + q4][(uint64_t)slot * cells + ((uint64_t)(lo2 + j2) * t + lo1 + j1) * t + lo0 + j0] = v;
        }
        __syncthreads();   // S, T1, T2 are reused by the next field
    }
}

// ------------------------------------------------------------------ restriction
// old <- new for every listed slot; a cell covered by a child <- the child's new field at the cell's
// centre (the corner shared by 2x2x2 child cells), by the 4-point midpoint rule (-1, 9, 9, -1)/16 along
// each axis (child cells 2c-1 .. 2c+2, the child's ghost layer at its faces included).  The reference
// averages the 2x2x2 block (AMR.h:961-996), a second-order rule.
// A CTA per (slot, plane z, group of g.fgroup fields).
__global__ void __launch_bounds__(256) k_evo_restrict(const __grid_constant__ EvoRestrictArgs g) {
    const uint32_t t = g.t, p = g.p, n = g.n, hn = n / 2;
    const uint32_t item = blockIdx.x / t, z = blockIdx.x % t;
    const int fb = (int)blockIdx.y * g.fgroup, fe = min(g.nf, fb + g.fgroup);   // this CTA's fields
    if (item >= g.n_items || fb >= fe) return;
    const uint32_t slot = g.items[item];
    const uint64_t cells = (uint64_t)t * t * t;
    bool leaf = true;
#pragma unroll
    for (int c = 0; c < 8; c++) leaf &= g.children[slot * 8u + c] == -1;
    if (leaf) {
        // a domain without children: plane z of every field is a straight copy, 16 bytes at a time
        // (planes are t^2 floats, t^2 * 4 a multiple of 16, every plane 16-byte aligned)
        const uint32_t q4 = t * t / 4u;
        const uint64_t base4 = (slot * cells + (uint64_t)z * t * t) / 4u;
        const uint32_t total = (uint32_t)(fe - fb) * q4;
        constexpr uint32_t U = 4;   // loads in flight per thread before their stores
        for (uint32_t e0 = threadIdx.x; e0 < total; e0 += U * blockDim.x) {
            float4 v[U];
#pragma unroll
            for (uint32_t u = 0; u < U; u++) {
                const uint32_t e = e0 + u * blockDim.x;
                if (e < total) v[u] = reinterpret_cast<const float4*>(g.new_f[fb + (int)(e / q4)])[base4 + e % q4];
            }
#pragma unroll
            for (uint32_t u = 0; u < U; u++) {
                const uint32_t e = e0 + u * blockDim.x;
                if (e < total) reinterpret_cast<float4*>(g.old_f[fb + (int)(e / q4)])[base4 + e % q4] = v[u];
            }
        }
        return;
    }
    constexpr float w4[4] = {-1.f / 16.f, 9.f / 16.f, 9.f / 16.f, -1.f / 16.f};
    for (uint32_t k = threadIdx.x; k < t * t; k += blockDim.x) {
        const uint32_t x = k % t, y = k / t;
        const uint32_t tx = (x - p) / hn, ty = (y - p) / hn, tz = (z - p) / hn;   // unsigned wrap for ghosts
        const int32_t ch = (tx < 2u && ty < 2u && tz < 2u) ? g.children[tx + ty * 2u + tz * 4u + slot * 8u] : -1;
        const uint64_t o = slot * cells + ((uint64_t)z * t + y) * t + x;
        // fields in groups, every load of a group before its stores (old and new are distinct buffers)
        constexpr int G = 8;
        if (ch == -1) {
            for (int f0 = fb; f0 < fe; f0 += G) {
                float v[G];
#pragma unroll
                for (int q = 0; q < G; q++)
                    if (f0 + q < fe) v[q] = g.new_f[f0 + q][o];
#pragma unroll
                for (int q = 0; q < G; q++)
                    if (f0 + q < fe) g.old_f[f0 + q][o] = v[q];
            }
            continue;
        }
        const uint32_t cx = ((x - p) * 2u) % n + p, cy = ((y - p) * 2u) % n + p, cz = ((z - p) * 2u) % n + p;
        const uint64_t base = (uint64_t)ch * cells + ((uint64_t)(cz - 1) * t + (cy - 1)) * t + (cx - 1);
        constexpr int GI = 2;
        for (int f0 = fb; f0 < fe; f0 += GI) {
            float acc[GI];
#pragma unroll
            for (int q = 0; q < GI; q++) acc[q] = 0.f;
#pragma unroll
            for (int k2 = 0; k2 < 4; k2++)
#pragma unroll
                for (int k1 = 0; k1 < 4; k1++) {
#pragma unroll
                    for (int q = 0; q < GI; q++) {
                        const float* v = g.new_f[min(f0 + q, fe - 1)];
                        float row = 0.f;
#pragma unroll
                        for (int k0 = 0; k0 < 4; k0++) row = fmaf(w4[k0], v[base + ((uint64_t)k2 * t + k1) * t + k0], row);
                        acc[q] = fmaf(w4[k1] * w4[k2], row, acc[q]);
                    }
                }
#pragma unroll
            for (int q = 0; q < GI; q++)
                if (f0 + q < fe) g.old_f[f0 + q][o] = acc[q];
        }
    }
}

// ------------------------------------------------------------------ constraints and FP64 norms
template <int N>
__global__ void __launch_bounds__(128) k_evo_constraints(const __grid_constant__ EvoArgs a, const ConsPtrs cons) {
    constexpr int P = 3, T = N + 2 * P;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)a.n_items * N * N * N) return;
    const uint32_t item = (uint32_t)(gid / (N * N * N)), cell = (uint32_t)(gid % (N * N * N));
    const uint32_t slot = a.items[item];
    const uint32_t x = cell % N, y = (cell / N) % N, z = cell / (N * N);
    const uint64_t pi = (uint64_t)slot * T * T * T + ((uint64_t)(z + P) * T + (y + P)) * T + (x + P);
    const uint64_t ii = (uint64_t)slot * N * N * N + cell;
    float u[BSSN_NF], uo[BSSN_NF];
#pragma unroll
    for (int f = 0; f < BSSN_NF; f++) {
        const float s = a.fields[f][pi];   // the stored form
        u[f] = s + bssn_offset(f);
        uo[f] = a.stage == 1 ? s : a.old_f[f][pi];
    }
    const float* D = a.deriv;
    const uint64_t ds = a.deriv_stride;
    auto dv = [&](int k) { return D[(uint64_t)k * ds + ii]; };
    float hm[4];
    bssn_constraints(u, dv, a.prm, hm);
    for (int k = 0; k < 4; k++) cons.c[k][ii] = hm[k];
}

// One CTA per live slot: sum of H^2, max |H|, sum of |M|^2, max |M| and the cell count over its
// interior cells that no child covers and that lie outside the excision radius of every puncture, in
// double, with a fixed reduction order.
__device__ __forceinline__ double nan_max(double a, double b) { return (a != a || b != b) ? (a + b) : fmax(a, b); }
__global__ void __launch_bounds__(256) k_evo_norms_domain(const EvoNormArgs g, double* part) {
    const uint32_t b = blockIdx.x;
    if (b >= g.n_items) return;
    const uint32_t slot = g.items[b], n = g.n, hn = n / 2;
    const uint32_t cells = n * n * n;
    const uint32_t pos = g.positions[slot];
    const int depth = pos_depth(pos);
    float ctr[3];
    slot_centre(pos, ctr);
    const float h = g.outer_size / ((float)n * (float)(1u << depth));
    double s[5] = {0, 0, 0, 0, 0};
    for (uint32_t c = threadIdx.x; c < cells; c += blockDim.x) {
        const uint32_t x = c % n, y = (c / n) % n, z = c / (n * n);
        const uint32_t oct = (x / hn) | ((y / hn) << 1) | ((z / hn) << 2);
        if (g.children[slot * 8u + oct] != -1) continue;
        bool excised = false;
        for (int a = 0; a < g.n_punctures; a++) {
            const float dx = ctr[0] * g.outer_size + ((float)x + .5f - .5f * (float)n) * h - g.pos[a][0];
            const float dy = ctr[1] * g.outer_size + ((float)y + .5f - .5f * (float)n) * h - g.pos[a][1];
            const float dz = ctr[2] * g.outer_size + ((float)z + .5f - .5f * (float)n) * h - g.pos[a][2];
            excised |= dx * dx + dy * dy + dz * dz < g.excision2;
        }
        if (excised) continue;
        const uint64_t i = (uint64_t)slot * cells + c;
        const double hv = g.cons.c[0][i];
        const double m2 = (double)g.cons.c[1][i] * g.cons.c[1][i] + (double)g.cons.c[2][i] * g.cons.c[2][i] +
                          (double)g.cons.c[3][i] * g.cons.c[3][i];
        s[0] += hv * hv;
        s[1] = nan_max(s[1], fabs(hv));
        s[2] += m2;
        s[3] = nan_max(s[3], sqrt(m2));
        s[4] += 1.0;
    }
    __shared__ double red[5][256];
    for (int k = 0; k < 5; k++) red[k][threadIdx.x] = s[k];
    __syncthreads();
    for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] = nan_max(red[1][threadIdx.x], red[1][threadIdx.x + w]);
            red[2][threadIdx.x] += red[2][threadIdx.x + w];
            red[3][threadIdx.x] = nan_max(red[3][threadIdx.x], red[3][threadIdx.x + w]);
            red[4][threadIdx.x] += red[4][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; k++) part[(size_t)b * 5 + k] = red[k][0];
}
__global__ void k_evo_norms_total(const double* part, uint32_t n_items, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[5] = {0, 0, 0, 0, 0};
    for (uint32_t b = 0; b < n_items; b++) {
        s[0] += part[(size_t)b * 5];
        s[1] = nan_max(s[1], part[(size_t)b * 5 + 1]);
        s[2] += part[(size_t)b * 5 + 2];
        s[3] = nan_max(s[3], part[(size_t)b * 5 + 3]);
        s[4] += part[(size_t)b * 5 + 4];
    }
    out[0] = s[4] > 0 ? sqrt(s[0] / s[4]) : 0.;
    out[1] = s[1];
    out[2] = s[4] > 0 ? sqrt(s[2] / s[4]) : 0.;
    out[3] = s[3];
    out[4] = s[4];
}

// ------------------------------------------------------------------ prolongation of new domains
// One CTA per (child, buffer).  Child cell w (padded index) lies at parent index coordinate
// o * n/2 + p + (w - p + 1/2) / 2 - 1/2 along each axis (o: the child's octant bit), which stays in
// [1.25, n + 3.75]: the cubic stencil b-1 .. b+2 (b = floor) fits in the parent's padded range.
// Near a puncture chi ~ r^4 and alpha ~ r^2 (precollapsed lapse): a cubic through their values
// undershoots zero, so they are interpolated as chi^(1/4) and alpha^(1/2), which vary like r, and
// raised back; chi is then kept at or above its floor.
__global__ void __launch_bounds__(256) k_evo_prolong(const __grid_constant__ EvoProlongArgs g) {
    const uint32_t item = blockIdx.x, buf = blockIdx.y;
    if (item >= g.n_items || buf >= g.nbuf) return;
    const int32_t node = g.items[3 * item], parent = g.items[3 * item + 1], off = g.items[3 * item + 2];
    const uint32_t n = g.n, p = g.p, t = g.t;
    const uint64_t cells = (uint64_t)t * t * t;
    const float* src = g.bufs[buf] + (uint64_t)parent * cells;
    float* dst = g.bufs[buf] + (uint64_t)node * cells;
    const uint32_t oct[3] = {(uint32_t)off & 1u, ((uint32_t)off >> 1) & 1u, ((uint32_t)off >> 2) & 1u};
    const float lo = (int)buf == g.floor_buf[0] || (int)buf == g.floor_buf[1] ? g.floor_val : -INFINITY;
    const int root = g.root[buf];
    auto fwd = [&](float v) {   // the interpolated quantity of a stored value
        if (root == 0) return v;
        const float u = sqrtf(fmaxf(v + 1.f, 0.f));
        return root == 2 ? u : sqrtf(u);
    };
    for (uint32_t k = threadIdx.x; k < (uint32_t)cells; k += blockDim.x) {
        const uint32_t w[3] = {k % t, (k / t) % t, k / (t * t)};
        int idx[3];
        float wgt[3][4];
        for (int a = 0; a < 3; a++) {
            const float x = (float)(oct[a] * (n / 2u) + p) + ((float)w[a] - (float)p + .5f) * .5f - .5f;
            int b = __float2int_rd(x);
            b = b < 1 ? 1 : (b > (int)t - 3 ? (int)t - 3 : b);
            const float s = x - (float)b;
            idx[a] = b;
            wgt[a][0] = -s * (s - 1.f) * (s - 2.f) * (1.f / 6.f);
            wgt[a][1] = (s + 1.f) * (s - 1.f) * (s - 2.f) * .5f;
            wgt[a][2] = -(s + 1.f) * s * (s - 2.f) * .5f;
            wgt[a][3] = (s + 1.f) * s * (s - 1.f) * (1.f / 6.f);
        }
        const int64_t si = ((int64_t)idx[2] * t + idx[1]) * t + idx[0];
        float v = 0.f;
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++)
#pragma unroll
            for (int k1 = 0; k1 < 4; k1++) {
                const float w12 = wgt[1][k1] * wgt[2][k2];
                const int64_t row = si + ((int64_t)(k2 - 1) * t + (k1 - 1)) * t - 1;
#pragma unroll
                for (int k0 = 0; k0 < 4; k0++) v = fmaf(wgt[0][k0] * w12, fwd(src[row + k0]), v);
            }
        if (root != 0) {
            const float v2 = v * v;
            v = (root == 2 ? v2 : v2 * v2) - 1.f;
        }
        dst[k] = v < lo ? lo : v;
    }
}

// ------------------------------------------------------------------ tile features and the plain criterion
// One CTA of 512 threads per leaf; thread = cell of the 8^3 feature grid, which covers (N/8)^3
// domain cells.  Per domain cell: the undivided gradients |d chi| and |d alpha| (second-order centred
// differences, i.e. the gradient times the cell size) and |d gt| (the norm over the conformal
// metric's components and axes).  Features of a feature cell: the mean conformal factor,
// log10(max (|d chi| + |d alpha|) + 1e-10) / 5 + 1 and log10(rms |d gt| + 1e-10) / 5 + 1.  The plain
// criterion's indicator of the tile is the largest |d chi| + |d alpha| over its cells.
__global__ void __launch_bounds__(512) k_evo_features(const EvoFeatureArgs g) {
    const uint32_t b = blockIdx.x;
    if (b >= g.n_items) return;
    const uint32_t slot = g.items[b], n = g.n, t = g.t, p = g.p, r = n / 8u;
    const uint32_t c = threadIdx.x, cx = c % 8, cy = (c / 8) % 8, cz = c / 64;
    const uint64_t base = (uint64_t)slot * t * t * t;
    const uint64_t st[3] = {1, t, (uint64_t)t * t};
    float chi = 0.f, g2 = 0.f, ind = 0.f;
    for (uint32_t k = 0; k < r * r * r; k++) {
        const uint32_t x = cx * r + k % r + p, y = cy * r + (k / r) % r + p, z = cz * r + k / (r * r) + p;
        const uint64_t o = base + ((uint64_t)z * t + y) * t + x;
        chi += g.state[F_CHI][o] + bssn_offset(F_CHI);
        float dchi = 0.f, dal = 0.f;
        for (int a = 0; a < 3; a++) {
            const float dc = .5f * (g.state[F_CHI][o + st[a]] - g.state[F_CHI][o - st[a]]);
            const float da = .5f * (g.state[F_ALPHA][o + st[a]] - g.state[F_ALPHA][o - st[a]]);
            dchi += dc * dc;
            dal += da * da;
            for (int q = 0; q < 6; q++) {
                const float dg = .5f * (g.state[F_GXX + q][o + st[a]] - g.state[F_GXX + q][o - st[a]]);
                g2 += dg * dg;
            }
        }
        ind = fmaxf(ind, sqrtf(dchi) + sqrtf(dal));   // per-cell differences are already times dx
    }
    const float inv = 1.f / (float)(r * r * r);
    float* f = g.features + (uint64_t)b * 3u * 512u;
    f[c] = chi * inv;
    f[512 + c] = log10f(ind + 1e-10f) * .2f + 1.f;
    f[1024 + c] = log10f(sqrtf(g2 * inv) + 1e-10f) * .2f + 1.f;
    __shared__ float red[512];
    red[c] = ind;
    __syncthreads();
    for (uint32_t w = 256; w > 0; w >>= 1) {
        if (c < w) red[c] = fmaxf(red[c], red[c + w]);
        __syncthreads();
    }
    if (c == 0) g.indicator[b] = red[0];
}

}  // namespace

// ------------------------------------------------------------------ launchers
cudaError_t launch_evo_prolong(const EvoProlongArgs& g, cudaStream_t st) {
    if (g.n_items == 0 || g.nbuf == 0) return cudaSuccess;
    k_evo_prolong<<<dim3(g.n_items, g.nbuf), 256, 0, st>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_evo_features(const EvoFeatureArgs& g, cudaStream_t st) {
    if (g.n_items == 0) return cudaSuccess;
    k_evo_features<<<g.n_items, 512, 0, st>>>(g);
    return cudaGetLastError();
}

bool evo_config_supported(uint32_t n, uint32_t p) { return p == 3u && (n == 8u || n == 16u || n == 32u); }

cudaError_t launch_evo_init(const EvoInitArgs& a, cudaStream_t st) {
    const uint64_t total = (uint64_t)a.used * a.t * a.t * a.t;
    if (total == 0) return cudaSuccess;
    k_evo_init<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

template <int N, int ZS>
static cudaError_t derivs_zs(const EvoArgs& a, cudaStream_t st) {
    using S = DerivShape<N, ZS>;
    static std::atomic<uint64_t> configured{0};
    cudaError_t e = ensure_smem_limit(k_evo_derivs<N, ZS>, S::SMEM, configured);
    if (e != cudaSuccess || a.n_items == 0) return e;
    k_evo_derivs<N, ZS><<<a.n_items * (N / ZS), S::THREADS, S::SMEM, st>>>(a);
    return cudaGetLastError();
}
// The compiled slab depths (a.deriv_zs; 0 = the default): whole cells per thread of 256.
template <int N>
static cudaError_t derivs_t(const EvoArgs& a, cudaStream_t st) {
    const uint32_t zs = a.deriv_zs ? a.deriv_zs : (uint32_t)deriv_default_zs(N);
    if constexpr (N == 8) {
        if (zs == 4) return derivs_zs<8, 4>(a, st);
        if (zs == 8) return derivs_zs<8, 8>(a, st);
    } else if constexpr (N == 16) {
        if (zs == 1) return derivs_zs<16, 1>(a, st);
        if (zs == 2) return derivs_zs<16, 2>(a, st);
        if (zs == 4) return derivs_zs<16, 4>(a, st);
    } else {
        if (zs == 1) return derivs_zs<32, 1>(a, st);   // deeper slabs would spill registers
    }
    return cudaErrorInvalidValue;
}
cudaError_t launch_evo_derivs(const EvoArgs& a, cudaStream_t st) {
    switch (a.n) {
        case 8: return derivs_t<8>(a, st);
        case 16: return derivs_t<16>(a, st);
        case 32: return derivs_t<32>(a, st);
        default: return cudaErrorInvalidValue;
    }
}
uint32_t evo_deriv_zs_candidates(uint32_t n, uint32_t* out) {
    const uint32_t c8[] = {4, 8}, c16[] = {1, 2, 4}, c32[] = {1};
    const uint32_t* c = n == 8 ? c8 : (n == 16 ? c16 : c32);
    const uint32_t k = n == 16 ? 3u : (n == 8 ? 2u : 1u);
    for (uint32_t i = 0; i < k; i++) out[i] = c[i];
    return n == 8 || n == 16 || n == 32 ? k : 0u;
}

template <int N>
static cudaError_t rhs_t(const EvoArgs& a, cudaStream_t st) {
    const uint64_t total = (uint64_t)a.n_items * N * N * N;
    if (total == 0) return cudaSuccess;
    if (a.prm.physics == 0) {
        static std::atomic<uint64_t> configured{0};
        const cudaError_t e = ensure_smem_limit(k_evo_rhs_bssn<N>, kRhsSmem, configured);
        if (e != cudaSuccess) return e;
        if (a.stage < 1 || a.stage > 4) return cudaErrorInvalidValue;
        k_evo_rhs_bssn<N><<<(unsigned)(total / kRhsCells), kRhsCells, rhs_smem(a.stage), st>>>(a);
    } else {
        k_evo_rhs_wave<N><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}
cudaError_t launch_evo_rhs(const EvoArgs& a, cudaStream_t st) {
    switch (a.n) {
        case 8: return rhs_t<8>(a, st);
        case 16: return rhs_t<16>(a, st);
        case 32: return rhs_t<32>(a, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_evo_restrict(const EvoRestrictArgs& g, cudaStream_t st) {
    if (g.n_items == 0) return cudaSuccess;
    if (g.nf <= 0 || g.nf > kMaxFields || g.fgroup <= 0) return cudaErrorInvalidValue;
    k_evo_restrict<<<dim3(g.n_items * g.t, (unsigned)((g.nf + g.fgroup - 1) / g.fgroup)), 256, 0, st>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_evo_ghost(const EvoGhostArgs& g, cudaStream_t st) {
    if (g.n_items == 0) return cudaSuccess;
    if (g.t > kGhostMaxT) return cudaErrorInvalidValue;   // the kernel's index arithmetic and tables cover edges up to 38
    EvoGhostArgs a = g;
    a.interp_floats = ghost_interp_floats(g.n, g.p, g.t);
    const size_t smem = (size_t)(3u * kGhostMaxT * 5u + a.interp_floats) * 4u;
    static std::atomic<uint64_t> configured{0};   // the limit for the largest edge, once per device
    const cudaError_t e = ensure_smem_limit(k_evo_ghost, (size_t)(3u * kGhostMaxT * 5u + ghost_interp_floats(32u, 3u, 38u)) * 4u,
                                            configured);
    if (e != cudaSuccess) return e;
    const dim3 grid(g.n_items * 2u, (unsigned)((g.nf + kGhostFields - 1) / kGhostFields));
    k_evo_ghost<<<grid, 256, smem, st>>>(a);
    return cudaGetLastError();
}

template <int N>
static cudaError_t cons_t(const EvoArgs& a, const ConsPtrs& cons, cudaStream_t st) {
    const uint64_t total = (uint64_t)a.n_items * N * N * N;
    if (total == 0) return cudaSuccess;
    k_evo_constraints<N><<<(unsigned)((total + 127) / 128), 128, 0, st>>>(a, cons);
    return cudaGetLastError();
}
cudaError_t launch_evo_constraints(const EvoArgs& a, const ConsPtrs& cons, cudaStream_t st) {
    switch (a.n) {
        case 8: return cons_t<8>(a, cons, st);
        case 16: return cons_t<16>(a, cons, st);
        case 32: return cons_t<32>(a, cons, st);
        default: return cudaErrorInvalidValue;
    }
}
cudaError_t launch_evo_norms(const EvoNormArgs& g, double* part, double* out, cudaStream_t st) {
    if (g.n_items) k_evo_norms_domain<<<g.n_items, 256, 0, st>>>(g, part);
    k_evo_norms_total<<<1, 32, 0, st>>>(part, g.n_items, out);
    return cudaGetLastError();
}

}  // namespace amr
