// kernels_stencil.cu -- finite-difference stencils on padded domains (sm_103a).
//
// A persistent grid works through units of domains (whole domains, or z-ranges of them to fill the
// last wave of CTAs).  A unit's padded z-planes are streamed through a shared-memory ring with 1-D TMA
// bulk copies (cp.async.bulk, one copy per plane and component, completion on an mbarrier per ring
// slot); thread (x, y) computes the interior cell (x, y, z) of every plane, so each plane is read
// from HBM once per unit and every stencil tap comes from shared memory.  k_stencil (one operator)
// refills the ring from thread 0 behind a CTA barrier per plane; k_stencil_bssn (the fused pass)
// is warp-specialised, with a producer warp and per-slot full/empty barriers.
//
// Kinds:
//   SK_GRAD       gradient                                   __differentiate  (AMR.h:1152-1179)
//   SK_GRAD_HESS  gradient + diagonal Hessian                __differentiate  (AMR.h:1181-1219)
//   SK_MIXED      off-diagonal Hessian, edge rule            __mixed_partials (AMR.h:1221-1266)
//   SK_BSSN       all six metric components in one pass: gradients (written), diagonal and
//                 off-diagonal Hessians quantised through compressed_float3 in registers exactly
//                 as the reference round-trips them through memory, g^kl d_k d_l g_ij (written),
//                 then the Christoffel symbols (written).  Replaces, per predictor/corrector,
//                 the 18 launches of metric_derivatives_noncovariant (BSSN.h:38-53) and the
//                 Christoffel launch (BSSN.h:93-102).
#include "kernels.h"

#include "amr_device.cuh"
#include "tma.cuh"

namespace amr {

template <int N, int P, int KIND>
struct StencilShape {
    static constexpr int T = N + 2 * P;
    static constexpr int NC = KIND == SK_BSSN ? 6 : 1;
    // ring slots: 2P+1 in use and 2 in flight; the fused kind keeps one in flight so that two
    // CTAs (with their generator and gradient tables) fit in one SM's shared memory
    static constexpr int R = KIND == SK_BSSN ? 2 * P + 2 : 2 * P + 3;
    static constexpr uint32_t PLANE = (uint32_t)(T * T);         // floats per plane
    static constexpr uint32_t PLANE_BYTES = PLANE * 4u;
    // SK_BSSN works on y-tiles of TY interior rows: the whole plane, or half of it where six
    // components' rings of whole planes would not fit in shared memory (32^3 domains).  A tile's
    // padded rows (TY + 2P of them) are contiguous in the plane, so it moves as one bulk copy.
    static constexpr int TY = KIND == SK_BSSN && N * N > 1024 - 32 ? N / 2 : N;
    static constexpr int NT = N / TY;                                   // tiles per plane
    static constexpr uint32_t TILE = (uint32_t)((TY + 2 * P) * T);      // floats per tile plane
    static constexpr uint32_t TILE_BYTES = TILE * 4u;
    static constexpr uint32_t CELLS = (uint32_t)(N * TY);               // interior cells per tile plane
    // The leaves' restriction stores tile 0's padded rows [0, OWN0) and tile 1's [OWN0, T): the
    // first row boundary past tile 0's interior at which both parts are 16-byte aligned.
    static constexpr int own0() {
        int r = TY + P;
        while ((r * T * 4) % 16 != 0) r++;
        return r;
    }
    static constexpr int OWN0 = NT == 1 ? T : own0();
    static constexpr size_t RING_BYTES = (size_t)NC * R * (KIND == SK_BSSN ? TILE_BYTES : PLANE_BYTES);
    static constexpr size_t BAR_BYTES = (size_t)R * 8u * (KIND == SK_BSSN ? 2u : 1u);   // full (+ empty) per slot
    // SK_BSSN runs warp-specialised: ceil(CELLS / 32) compute warps (thread (x, y) per column of the
    // tile) and one producer warp that streams the planes
    static constexpr uint32_t CW = (CELLS + 31u) / 32u;
    static constexpr uint32_t THREADS = KIND == SK_BSSN ? 32u * (CW + 1u) : (uint32_t)(N * N);
    // SK_BSSN: per thread, the 13 generator prefixes (d0, m0, d1, m1, ..., c) and the six gradient words
    static constexpr size_t TABLE_BYTES = KIND == SK_BSSN ? (size_t)(13 + 6) * CELLS * 4u : 0u;
    static constexpr size_t SMEM = RING_BYTES + BAR_BYTES + TABLE_BYTES;
    // SK_BSSN: draw the Christoffel encodes' noise inside the unrolled component passes (faster
    // at 32^3; at 16^3 the unrolled code is slower, measured, and at 28^3 it spills registers)
    static constexpr bool kEarlyChristoffelDraws = N >= 32;
    // SK_BSSN: CTAs per SM the launch bounds ask for, and the registers a thread may then use
    static constexpr int CTAS = N * N <= 256 ? 2 : 1;
    static constexpr int REG_BUDGET = 65536 / ((int)THREADS * CTAS);
    // SK_BSSN: draw the mixed partials' noise at the top of a component pass, beside the other
    // generator chains, where the registers allow it (not at 28^3: 72 registers a thread)
    static constexpr bool kEarlyMixedDraws = REG_BUDGET >= 96;
    static_assert(N % TY == 0 && TILE_BYTES % 16u == 0u && (TY * T * 4) % 16 == 0, "tiles are aligned bulk copies");
    static_assert(NT == 1 || (OWN0 <= TY + 2 * P && OWN0 >= TY), "restriction rows lie in their tile");
    static constexpr uint32_t Q = N >= 16 ? 4u : 2u;              // z-ranges per split domain
    static_assert(N % Q == 0, "split domains into whole planes");
    static_assert(PLANE_BYTES % 16u == 0u, "bulk copies move whole planes of 16-byte multiples");
};

template <int N, int P, int KIND>
size_t stencil_smem_bytes() { return StencilShape<N, P, KIND>::SMEM; }

// ---------------------------------------------------------------- per-cell pieces

// Gradient and diagonal second derivative along the three axes.  `pl(j)` is the plane at
// padded z offset j - P from the cell's plane; c0 is the cell's offset inside a plane.
template <int P, int T, class PL>
__device__ __forceinline__ void fd_axes(const PL& pl, int c0, float& gx, float& gy, float& gz,
                                        float& hx, float& hy, float& hz) {
    gx = gy = gz = hx = hy = hz = 0.f;
    const float* m = pl(P);
#pragma unroll
    for (int i = -P; i <= P; i++) {
        const float c1 = FD<P>::d1(i), c2 = FD<P>::d2(i);
        float a = m[c0 + i];
        gx = __fmaf_rn(a, c1, gx); hx = __fmaf_rn(a, c2, hx);
        a = m[c0 + i * T];
        gy = __fmaf_rn(a, c1, gy); hy = __fmaf_rn(a, c2, hy);
        a = pl(P + i)[c0];
        gz = __fmaf_rn(a, c1, gz); hz = __fmaf_rn(a, c2, hz);
    }
}

// Mixed-partial helpers (AMR.h:1221-1230).  Offsets are given as (plane, in-plane offset).
__device__ __forceinline__ float mixed_centre(float a, float b, float c, float d) {
    return __fmul_rn(.25f, __fsub_rn(__fsub_rn(__fadd_rn(a, b), c), d));
}
__device__ __forceinline__ float mixed_edge(float f, float a, float b, float c, float d, float e, float g) {
    float s = __fadd_rn(a, b);
    s = __fsub_rn(s, c); s = __fsub_rn(s, d); s = __fsub_rn(s, e); s = __fsub_rn(s, g);
    return __fmaf_rn(.5f, s, f);
}

// Off-diagonal Hessian (xy, xz, yz) before scaling, with the reference's edge fallback.
template <int N, int P, int T, class PL>
__device__ __forceinline__ float3 mixed_partials(const PL& pl, int c0, uint32_t x, uint32_t y, uint32_t z) {
    const float* zm = pl(P - 1);
    const float* z0 = pl(P);
    const float* zp = pl(P + 1);
    const int ex = (int)x - (int)min(max(x, 1u), (uint32_t)N - 2u);
    const int ey = (int)y - (int)min(max(y, 1u), (uint32_t)N - 2u);
    const int ez = (int)z - (int)min(max(z, 1u), (uint32_t)N - 2u);
    const int cxy = ex * ey, cxz = ex * ez, cyz = ey * ez;
    float vxy, vxz, vyz;
    if (cxy == 0) {
        vxy = mixed_centre(z0[c0 + 1 + T], z0[c0 - 1 - T], z0[c0 + 1 - T], z0[c0 - 1 + T]);
    } else {
        const int dx = -cxy;
        vxy = __fmul_rn((float)(-cxy), mixed_edge(z0[c0], z0[c0 + dx + T], z0[c0 - dx - T], z0[c0 - dx], z0[c0 + dx],
                                                  z0[c0 - T], z0[c0 + T]));
    }
    if (cxz == 0) {
        vxz = mixed_centre(zp[c0 + 1], zm[c0 - 1], zm[c0 + 1], zp[c0 - 1]);
    } else {
        const int dx = -cxz;
        vxz = __fmul_rn((float)(-cxz), mixed_edge(z0[c0], zp[c0 + dx], zm[c0 - dx], z0[c0 - dx], z0[c0 + dx],
                                                  zm[c0], zp[c0]));
    }
    if (cyz == 0) {
        vyz = mixed_centre(zp[c0 + T], zm[c0 - T], zm[c0 + T], zp[c0 - T]);
    } else {
        const int dx = -cyz * T;
        vyz = __fmul_rn((float)(-cyz), mixed_edge(z0[c0], zp[c0 + dx], zm[c0 - dx], z0[c0 - dx], z0[c0 + dx],
                                                  zm[c0], zp[c0]));
    }
    return make_float3(vxy, vxz, vyz);
}

// fd_axes on two components at once: lane x reads the planes at p, lane y the planes OFF floats
// further (the next component's ring).
template <int P, int T, int OFF, class PL>
__device__ __forceinline__ void fd_axes2(const PL& pl, int c0, float2& gx, float2& gy, float2& gz, float2& hx,
                                         float2& hy, float2& hz) {
    gx = gy = gz = hx = hy = hz = splat2(0.f);
    const float* m = pl(P);
#pragma unroll
    for (int i = -P; i <= P; i++) {
        const float2 c1 = splat2(FD<P>::d1(i)), c2 = splat2(FD<P>::d2(i));
        float2 a = make_float2(m[c0 + i], m[c0 + i + OFF]);
        gx = fma2(a, c1, gx); hx = fma2(a, c2, hx);
        a = make_float2(m[c0 + i * T], m[c0 + i * T + OFF]);
        gy = fma2(a, c1, gy); hy = fma2(a, c2, hy);
        const float* q = pl(P + i);
        a = make_float2(q[c0], q[c0 + OFF]);
        gz = fma2(a, c1, gz); hz = fma2(a, c2, hz);
    }
}
__device__ __forceinline__ float2 mixed_centre2(float2 a, float2 b, float2 c, float2 d) {
    return mul2(splat2(.25f), sub2(sub2(add2(a, b), c), d));
}
__device__ __forceinline__ float2 mixed_edge2(float2 f, float2 a, float2 b, float2 c, float2 d, float2 e, float2 g) {
    float2 s = add2(a, b);
    s = sub2(s, c); s = sub2(s, d); s = sub2(s, e); s = sub2(s, g);
    return fma2(splat2(.5f), s, f);
}
// mixed_partials on two components at once (lanes as in fd_axes2); the edge cases depend on the
// cell only, so both lanes take the same branch.
template <int N, int P, int T, int OFF, class PL>
__device__ __forceinline__ void mixed_partials2(const PL& pl, int c0, uint32_t x, uint32_t y, uint32_t z, float2& vxy,
                                                float2& vxz, float2& vyz) {
    const float* zm = pl(P - 1);
    const float* z0 = pl(P);
    const float* zp = pl(P + 1);
    auto ld = [&](const float* q, int i) { return make_float2(q[i], q[i + OFF]); };
    const int ex = (int)x - (int)min(max(x, 1u), (uint32_t)N - 2u);
    const int ey = (int)y - (int)min(max(y, 1u), (uint32_t)N - 2u);
    const int ez = (int)z - (int)min(max(z, 1u), (uint32_t)N - 2u);
    const int cxy = ex * ey, cxz = ex * ez, cyz = ey * ez;
    if (cxy == 0) {
        vxy = mixed_centre2(ld(z0, c0 + 1 + T), ld(z0, c0 - 1 - T), ld(z0, c0 + 1 - T), ld(z0, c0 - 1 + T));
    } else {
        const int dx = -cxy;
        vxy = mul2(splat2((float)(-cxy)), mixed_edge2(ld(z0, c0), ld(z0, c0 + dx + T), ld(z0, c0 - dx - T),
                                                      ld(z0, c0 - dx), ld(z0, c0 + dx), ld(z0, c0 - T), ld(z0, c0 + T)));
    }
    if (cxz == 0) {
        vxz = mixed_centre2(ld(zp, c0 + 1), ld(zm, c0 - 1), ld(zm, c0 + 1), ld(zp, c0 - 1));
    } else {
        const int dx = -cxz;
        vxz = mul2(splat2((float)(-cxz)), mixed_edge2(ld(z0, c0), ld(zp, c0 + dx), ld(zm, c0 - dx), ld(z0, c0 - dx),
                                                      ld(z0, c0 + dx), ld(zm, c0), ld(zp, c0)));
    }
    if (cyz == 0) {
        vyz = mixed_centre2(ld(zp, c0 + T), ld(zm, c0 - T), ld(zm, c0 + T), ld(zp, c0 - T));
    } else {
        const int dx = -cyz * T;
        vyz = mul2(splat2((float)(-cyz)), mixed_edge2(ld(z0, c0), ld(zp, c0 + dx), ld(zm, c0 - dx), ld(z0, c0 - dx),
                                                      ld(z0, c0 + dx), ld(zm, c0), ld(zp, c0)));
    }
}

// Christoffel symbols of one cell from the six compressed metric gradients (BSSN.h:72-90).
// `M` multiplies the lowered symbols: the metric itself (reference) or its inverse.
// `noise` holds the encodes' noise pairs in draw order (noise_pairs1 per symbol pair).
__device__ __forceinline__ void christoffel_cell(const uint32_t* G, const Sym& M, const float2* noise, uint32_t* out) {
    float3 d[6];
#pragma unroll
    for (int k = 0; k < 6; k++) d[k] = cf3_decode(G[k]);
    // rows of float3x3_sym(float3, float3, float3), tensors.h:138: S_l(j,k) = (d_j g_lk + d_k g_lj)/2
    const Sym Sx{d[0].x, __fmul_rn(__fadd_rn(d[0].y, d[1].x), .5f), __fmul_rn(__fadd_rn(d[0].z, d[2].x), .5f),
                 d[1].y, __fmul_rn(__fadd_rn(d[2].y, d[1].z), .5f), d[2].z};
    const Sym Sy{d[1].x, __fmul_rn(__fadd_rn(d[1].y, d[3].x), .5f), __fmul_rn(__fadd_rn(d[1].z, d[4].x), .5f),
                 d[3].y, __fmul_rn(__fadd_rn(d[4].y, d[3].z), .5f), d[4].z};
    const Sym Sz{d[2].x, __fmul_rn(__fadd_rn(d[2].y, d[4].x), .5f), __fmul_rn(__fadd_rn(d[2].z, d[5].x), .5f),
                 d[4].y, __fmul_rn(__fadd_rn(d[5].y, d[4].z), .5f), d[5].z};
    const float sx[6] = {Sx.xx, Sx.xy, Sx.xz, Sx.yy, Sx.yz, Sx.zz};
    const float sy[6] = {Sy.xx, Sy.xy, Sy.xz, Sy.yy, Sy.yz, Sy.zz};
    const float sz[6] = {Sz.xx, Sz.xy, Sz.xz, Sz.yy, Sz.yz, Sz.zz};
    // symbols jk and jk+1 as the two lanes of a pair; fma(-d, .5, s) = fma(d, -.5, s) exactly
#pragma unroll
    for (int jk = 0; jk < 6; jk += 2) {
        const float2 vx = fma2(make_float2(d[jk].x, d[jk + 1].x), splat2(-.5f), make_float2(sx[jk], sx[jk + 1]));
        const float2 vy = fma2(make_float2(d[jk].y, d[jk + 1].y), splat2(-.5f), make_float2(sy[jk], sy[jk + 1]));
        const float2 vz = fma2(make_float2(d[jk].z, d[jk + 1].z), splat2(-.5f), make_float2(sz[jk], sz[jk + 1]));
        // M * v (sym_times)
        const float2 rx = fma2(vz, splat2(M.xz), fma2(vx, splat2(M.xx), mul2(vy, splat2(M.xy))));
        const float2 ry = fma2(vz, splat2(M.yz), fma2(vx, splat2(M.xy), mul2(vy, splat2(M.yy))));
        const float2 rz = fma2(vz, splat2(M.zz), fma2(vx, splat2(M.xz), mul2(vy, splat2(M.yz))));
        const Cf3Pair w = cf3_encode2<false>(rx, ry, rz, noise[3 * (jk / 2)], noise[3 * (jk / 2) + 1],
                                             noise[3 * (jk / 2) + 2]);
        out[jk] = w.w0;
        out[jk + 1] = w.w1;
    }
}

// ---------------------------------------------------------------- the streaming kernel
template <int N, int P, int KIND>
__global__ void __launch_bounds__(N * N, N * N <= 256 ? 2 : 1) k_stencil(const __grid_constant__ StencilArgs a) {
    static_assert(KIND != SK_BSSN, "the fused kind is k_stencil_bssn");
    using S = StencilShape<N, P, KIND>;
    constexpr int T = S::T, NC = S::NC, R = S::R;
    constexpr uint32_t PLANE = S::PLANE;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + S::RING_BYTES);
    __shared__ int s_abort;

    const uint32_t tid = threadIdx.x;
    // Thread -> (x, y).  At N = 16 a warp would cover rows y and y+1 of the 22-float plane rows,
    // whose banks overlap for 6 lanes; pairing rows y and y+8 (176 floats apart = 16 banks)
    // makes every shared-memory access of the warp conflict-free.
    const uint32_t x = tid % N;
    const uint32_t y = N == 16 ? ((tid / N) >> 1) | (((tid / N) & 1u) << 3) : tid / N;
    const int c0 = (int)((y + P) * T + (x + P));

    if (tid == 0) {
        for (int r = 0; r < R; r++) mbar_init(&bars[r], 1);
        mbar_fence_init();
        s_abort = 0;
    }
    __syncthreads();

    // per-cell generators: the part that depends on (seed, x, y) only, once per thread
    int32_t pre_d[NC], pre_m[NC], pre_c;
    {
        int32_t seed_d[NC], seed_m[NC], seed_c = a.seed_c;
#pragma unroll
        for (int k = 0; k < NC; k++) { seed_d[k] = a.seed_d[k]; seed_m[k] = a.seed_m[k]; }
        if (a.seed_ptr) {
#pragma unroll
            for (int k = 0; k < NC; k++) { seed_d[k] = a.seed_ptr[2 * k]; seed_m[k] = a.seed_ptr[2 * k + 1]; }
            seed_c = a.seed_ptr[12];
        }
#pragma unroll
        for (int k = 0; k < NC; k++) { pre_d[k] = cell_rng_prefix(seed_d[k], x, y); pre_m[k] = cell_rng_prefix(seed_m[k], x, y); }
        pre_c = cell_rng_prefix(seed_c, x, y);
    }
    (void)pre_c;

    // Work units, assigned round-robin.  Items are processed whole, except that when the last
    // round would leave a quarter or more of the CTAs idle (rem <= 3/4 of the grid), its items are
    // cut into Q z-ranges of N/Q interior planes so that it spreads over every CTA.  A unit streams
    // its nz + 2P padded planes through the ring; thread 0 keeps the ring R planes ahead of the
    // plane being computed, across unit boundaries.
    // With a.zsplit > 1 every item is cut that way instead (few items, launched on a wider grid).
    const uint32_t G = gridDim.x;
    const uint32_t rem = a.n_items % G;
    const bool all_split = a.zsplit > 1u;
    const uint32_t Q = all_split ? a.zsplit : S::Q, NZQ = N / Q;
    const bool split = all_split || (rem != 0u && Q * rem <= (Q - 1u) * G);
    const uint32_t n_whole = all_split ? 0u : split ? a.n_items - rem : a.n_items;
    const uint32_t n_units = n_whole + (all_split ? a.n_items * Q : split ? rem * Q : 0u);
    auto unit_of = [&](uint32_t u, uint32_t& item, uint32_t& z0, uint32_t& nz) {
        if (u < n_whole) { item = u; z0 = 0; nz = N; }
        else { const uint32_t v = u - n_whole; item = n_whole + v / Q; z0 = (v % Q) * NZQ; nz = NZQ; }
    };
    auto active_node = [&](uint32_t item, uint32_t& node, int& depth) {
        node = a.items ? a.items[item] : item;
        depth = pos_depth(a.positions[node]);
        return depth != -1 && active_depth(a.substep, (uint32_t)depth, a.max_depth);
    };
    auto next_unit = [&](uint32_t u) {   // this CTA's next unit at or after u with an active domain
        for (; u < n_units; u += G) {
            uint32_t item, z0, nz, node;
            int depth;
            unit_of(u, item, z0, nz);
            if (active_node(item, node, depth)) break;
        }
        return u;
    };
    // thread 0's request state: unit p_unit (its domain's first plane p_src and its plane count
    // p_np), the next of its planes p_j, and the planes requested so far
    uint32_t p_unit = n_units, p_j = 0, p_np = 0, issued = 0;
    size_t p_src = 0;
    auto open_unit = [&](uint32_t u) {
        p_unit = next_unit(u);
        if (p_unit < n_units) {
            uint32_t item, z0, nz, node;
            int depth;
            unit_of(p_unit, item, z0, nz);
            active_node(item, node, depth);
            p_src = ((size_t)node * T + z0) * PLANE;
            p_np = nz + 2u * P;
        }
    };
    if (tid == 0) open_unit(blockIdx.x);
    auto issue_upto = [&](uint32_t limit) {
        while (issued < limit && p_unit < n_units) {
            const uint32_t s = issued % R;
            mbar_arrive_expect_tx(&bars[s], NC * S::PLANE_BYTES);
#pragma unroll
            for (int k = 0; k < NC; k++)
                bulk_g2s(ring + ((size_t)k * R + s) * PLANE, a.field[k] + p_src + (size_t)p_j * PLANE, S::PLANE_BYTES,
                         &bars[s]);
            issued++;
            if (++p_j == p_np) { p_j = 0; open_unit(p_unit + G); }
        }
    };

    uint32_t g_base = 0;   // stream index of the current unit's first padded plane
    for (uint32_t cu = next_unit(blockIdx.x); cu < n_units; cu = next_unit(cu + G)) {
        uint32_t item, z0, nz, node;
        int depth;
        unit_of(cu, item, z0, nz);
        active_node(item, node, depth);
        const float dx1 = a.geo.inv_dx[depth], dx2 = a.geo.inv_dx2[depth];
#pragma unroll 1
        for (uint32_t zl = 0; zl < nz; zl++) {
            const uint32_t g = g_base + zl, z = z0 + zl;   // planes g .. g+2P hold padded z .. z+2P
            if (tid == 0) issue_upto(g + R);               // every plane below g is finished
            // a unit's first window needs all its planes, later windows one more
            bool ok = true;
            for (int j = zl == 0 ? 0 : 2 * P; j <= 2 * P; j++) {
                const uint32_t sq = g + j;
                ok &= mbar_wait(&bars[sq % R], (sq / R) & 1u);
            }
            if (!ok) s_abort = 1;
            if (ok) {
                const uint32_t base = g % R;
                uint32_t slot[2 * P + 1];
#pragma unroll
                for (int j = 0; j <= 2 * P; j++) slot[j] = base + j >= (uint32_t)R ? base + j - R : base + j;
                const uint32_t zg = node * N + z;
                const size_t o = ((size_t)zg * N + y) * N + x;   // inner-layout index

                if (KIND == SK_GRAD || KIND == SK_GRAD_HESS) {
                    auto pl = [&](int j) { return (const float*)(ring + (size_t)slot[j] * PLANE); };
                    float gx, gy, gz, hx, hy, hz;
                    fd_axes<P, T>(pl, c0, gx, gy, gz, hx, hy, hz);
                    int32_t rng = cell_rng_at(pre_d[0], zg);
                    if (KIND == SK_GRAD_HESS)
                        a.hdiag[o] = cf3_encode(__fmul_rn(hx, dx2), __fmul_rn(hy, dx2), __fmul_rn(hz, dx2), rng);
                    a.grad[0][o] = cf3_encode(__fmul_rn(gx, dx1), __fmul_rn(gy, dx1), __fmul_rn(gz, dx1), rng);
                } else if (KIND == SK_MIXED) {
                    auto pl = [&](int j) { return (const float*)(ring + (size_t)slot[j] * PLANE); };
                    const float3 m = mixed_partials<N, P, T>(pl, c0, x, y, z);
                    int32_t rng = cell_rng_at(pre_m[0], zg);
                    a.hoff[o] = cf3_encode(__fmul_rn(m.x, dx2), __fmul_rn(m.y, dx2), __fmul_rn(m.z, dx2), rng);
                }
            }
            __syncthreads();   // every thread is done with plane g: its slot may be refilled
            if (s_abort) {
                if (tid == 0) {
                    atomicExch(a.err, 1);
                    for (uint32_t sq = g; sq < issued; sq++) mbar_wait(&bars[sq % R], (sq / R) & 1u);   // drain (bounded)
                }
                return;
            }
        }
        g_base += nz + 2u * P;
    }
}

// ---------------------------------------------------------------- the fused BSSN pass, warp-specialised
// Work units and plane stream as in k_stencil, but the planes are requested by a producer warp:
// ring slot s has a `full` barrier (the producer's expected bytes, completed by the copies) and an
// `empty` barrier (one arrival per compute warp when it is done with the plane in it).  Compute
// warps never wait for each other, only for data; the producer waits only for the slot it refills.
template <int N, int P>
__device__ __forceinline__ void bssn_cell(const StencilArgs& a, const float* ring, const uint32_t* slot, int c0,
                                          uint32_t x, uint32_t y, uint32_t z, uint32_t zg, size_t o, float dx1,
                                          float dx2, uint32_t tid, const int32_t* s_pre, uint32_t* s_grad) {
    using S = StencilShape<N, P, SK_BSSN>;
    constexpr int T = S::T, R = S::R;
    constexpr uint32_t PLANE = S::TILE, NN = S::CELLS;   // ring slots hold tile planes
    const size_t cz = (size_t)slot[P] * PLANE + c0;
    const Sym g{ring[0 * R * PLANE + cz], ring[1 * (size_t)R * PLANE + cz], ring[2 * (size_t)R * PLANE + cz],
                ring[3 * (size_t)R * PLANE + cz], ring[4 * (size_t)R * PLANE + cz], ring[5 * (size_t)R * PLANE + cz]};
    const Sym ginv = sym_inverse(g);
    // components two at a time, as the lanes of packed pairs (every lane the scalar operation
    // sequence); component 2j+1's ring lies R planes after component 2j's
    constexpr int OFF = R * (int)PLANE;
    const float2 DX1 = splat2(dx1), DX2 = splat2(dx2);
    // One pass: components 2j and 2j+1.
    auto pass = [&](int j) {
        const int k0 = 2 * j, k1 = 2 * j + 1;
        const float* base = ring + (size_t)k0 * R * PLANE;
        auto pl = [&](int jj) { return base + (size_t)slot[jj] * PLANE; };
        // the mixed partials' draws are independent of the others: drawn here, in the same
        // straight-line block, the four generator chains interleave
        float2 mnx, mny, mnz;
        auto mixed_draws = [&] {
            int32_t rm0 = cell_rng_at(s_pre[(2 * k0 + 1) * NN + tid], zg), rm1 = cell_rng_at(s_pre[(2 * k1 + 1) * NN + tid], zg);
            noise_pairs2(rm0, rm1, mnx, mny, mnz);
        };
        if constexpr (S::kEarlyMixedDraws) mixed_draws();
        float2 gx, gy, gz, hx, hy, hz;
        fd_axes2<P, T, OFF>(pl, c0, gx, gy, gz, hx, hy, hz);
        int32_t rd0 = cell_rng_at(s_pre[(2 * k0) * NN + tid], zg), rd1 = cell_rng_at(s_pre[(2 * k1) * NN + tid], zg);
        float2 nx, ny, nz;
        // the Hessians are quantised exactly as the reference writes and re-reads them
        noise_pairs2(rd0, rd1, nx, ny, nz);
        const Cf3Pair hq = cf3_encode2<true>(mul2(hx, DX2), mul2(hy, DX2), mul2(hz, DX2), nx, ny, nz);
        noise_pairs2(rd0, rd1, nx, ny, nz);
        const Cf3Pair gk = cf3_encode2<false>(mul2(gx, DX1), mul2(gy, DX1), mul2(gz, DX1), nx, ny, nz);
        a.grad[k0][o] = gk.w0;
        a.grad[k1][o] = gk.w1;
        s_grad[k0 * NN + tid] = gk.w0;
        s_grad[k1 * NN + tid] = gk.w1;
        float2 mxy, mxz, myz;
        mixed_partials2<N, P, T, OFF>(pl, c0, x, y, z, mxy, mxz, myz);
        if constexpr (!S::kEarlyMixedDraws) mixed_draws();
        const Cf3Pair oq = cf3_encode2<true>(mul2(mxy, DX2), mul2(mxz, DX2), mul2(myz, DX2), mnx, mny, mnz);
        // trace_contra(H, ginv) with H = (hq.x, oq.x, oq.y, hq.y, oq.z, hq.z) (tensors.h:430-435)
        float2 ta = fma2(hq.vx, splat2(ginv.xx), mul2(hq.vy, splat2(ginv.yy)));
        ta = fma2(hq.vz, splat2(ginv.zz), ta);
        float2 tb = fma2(oq.vx, splat2(ginv.xy), mul2(oq.vy, splat2(ginv.xz)));
        tb = fma2(oq.vz, splat2(ginv.yz), tb);
        const float2 lap = fma2(tb, splat2(2.f), ta);
        a.lap[k0][o] = lap.x;
        a.lap[k1][o] = lap.y;
    };
    // The Christoffel encodes' generator is one chain of 18 draws.  With kEarlyChristoffelDraws
    // the three passes are unrolled and each advances it by 6 draws alongside its own chains;
    // otherwise the passes share one loop body (smaller code: faster at 16^3, measured) and the
    // chain runs after them.
    int32_t rc = cell_rng_at(s_pre[12 * NN + tid], zg);
    float2 cn[9];
    if constexpr (S::kEarlyChristoffelDraws) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            noise_pairs1(rc, cn[3 * j], cn[3 * j + 1], cn[3 * j + 2]);
            pass(j);
        }
    } else {
#pragma unroll 1
        for (int j = 0; j < 3; j++) pass(j);
#pragma unroll
        for (int j = 0; j < 3; j++) noise_pairs1(rc, cn[3 * j], cn[3 * j + 1], cn[3 * j + 2]);
    }
    uint32_t G[6];
#pragma unroll
    for (int k = 0; k < 6; k++) G[k] = s_grad[k * NN + tid];
    uint32_t out[6];
    christoffel_cell(G, a.christoffel_mode == AMR_CHRISTOFFEL_RAISED ? ginv : g, cn, out);
#pragma unroll
    for (int k = 0; k < 6; k++) a.chr[k][o] = out[k];
}

template <int N, int P>
__global__ void __launch_bounds__(StencilShape<N, P, SK_BSSN>::THREADS, StencilShape<N, P, SK_BSSN>::CTAS)
    k_stencil_bssn(const __grid_constant__ StencilArgs a) {
    using S = StencilShape<N, P, SK_BSSN>;
    constexpr int T = S::T, NC = 6, R = S::R;
    constexpr uint32_t PLANE = S::PLANE, TILE = S::TILE, NN = S::CELLS, CW = S::CW;
    constexpr uint32_t TY = S::TY, NT = S::NT;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);   // [component][slot] tile planes
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + S::RING_BYTES);
    uint64_t* empty = full + R;
    int32_t* s_pre = reinterpret_cast<int32_t*>(smem_raw + S::RING_BYTES + S::BAR_BYTES);   // [13][NN]
    uint32_t* s_grad = reinterpret_cast<uint32_t*>(s_pre + 13 * NN);                       // [6][NN]
    __shared__ volatile int s_abort;

    const uint32_t tid = threadIdx.x, warp = tid / 32u, lane = tid % 32u;
    if (tid == 0) {
        for (int r = 0; r < R; r++) { mbar_init(&full[r], 1); mbar_init(&empty[r], CW); }
        mbar_fence_init();
        s_abort = 0;
    }
    __syncthreads();   // the only CTA-wide barrier: the producer warp leaves the compute loop

    // Work: the items' interior tile planes (item after item, tile after tile, z last), cut into
    // gridDim.x contiguous ranges of equal length (to a plane), one per CTA.  A range is walked as
    // units -- consecutive planes of one tile of one domain -- whose padded planes (the unit's
    // planes and P more on either side) stream through the ring.
    const uint64_t n_planes = (uint64_t)a.n_items * NT * N;
    const uint32_t p_begin = (uint32_t)((uint64_t)blockIdx.x * n_planes / gridDim.x);
    const uint32_t p_end = (uint32_t)(((uint64_t)blockIdx.x + 1u) * n_planes / gridDim.x);
    auto unit_of = [&](uint32_t p, uint32_t& item, uint32_t& tile, uint32_t& z0, uint32_t& nz) {
        item = p / (NT * N);
        const uint32_t r = p - item * (NT * N);
        tile = r / N;
        z0 = r - tile * N;
        nz = min((uint32_t)N - z0, p_end - p);
    };
    auto active_node = [&](uint32_t item, uint32_t& node, int& depth) {
        node = a.items ? a.items[item] : item;
        depth = pos_depth(a.positions[node]);
        return depth != -1 && active_depth(a.substep, (uint32_t)depth, a.max_depth);
    };
    auto next_unit = [&](uint32_t p) {   // the first plane at or after p of an active domain, or p_end
        while (p < p_end) {
            uint32_t node;
            int depth;
            if (active_node(p / (NT * N), node, depth)) break;
            p = (p / (NT * N) + 1u) * (NT * N);
        }
        return min(p, p_end);
    };
    auto fused_leaf = [&](uint32_t node) {   // restriction fused: a domain without children
        if (!a.children) return false;
        bool leaf = true;
#pragma unroll
        for (int c = 0; c < 8; c++) leaf &= a.children[node * 8u + c] == -1;
        return leaf;
    };

    const uint32_t spins = a.spin_limit ? a.spin_limit : kMaxSpins;
    if (warp == CW) {   // ---------------- producer warp: one thread requests every plane
        if (lane != 0) return;
        uint32_t q = 0;   // planes requested
        bool ok = true;
        for (uint32_t u = next_unit(p_begin), nz = 0; ok && u < p_end; u = next_unit(u + nz)) {
            uint32_t item, tile, z0, node;
            int depth;
            unit_of(u, item, tile, z0, nz);
            active_node(item, node, depth);
            const bool leaf = fused_leaf(node);
            const size_t src = ((size_t)node * T + z0) * PLANE + (size_t)tile * TY * T;
            for (uint32_t j = 0; j < nz + 2u * P; j++, q++) {
                const uint32_t s = q % R;
                // the slot's previous plane (q - R) must have been released by every compute warp
                if (q >= (uint32_t)R && !mbar_wait(&empty[s], ((q / R) - 1u) & 1u, spins)) { ok = false; break; }
                if (s_abort) { ok = false; break; }
                if (q + 1u == a.withhold) continue;   // failure-path test: this plane never arrives
                mbar_arrive_expect_tx(&full[s], NC * S::TILE_BYTES);
#pragma unroll
                for (int k = 0; k < NC; k++)
                    bulk_g2s(ring + ((size_t)k * R + s) * TILE, (leaf ? a.leaf_src[k] : a.field[k]) + src + (size_t)j * PLANE,
                             S::TILE_BYTES, &full[s]);
            }
        }
        if (!ok) {
            s_abort = 1;
            atomicExch(a.err, 1);
        }
        // The CTA's shared memory must outlive every copy issued into it: wait for the last R
        // requests to land (the earlier ones were consumed before their slots were reused).  In a
        // normal run they land anyway; after an abort, compute warps may have left without them.
        for (uint32_t p = q > (uint32_t)R ? q - R : 0u; p < q; p++)
            if (p + 1u != a.withhold) mbar_wait(&full[p % R], (p / R) & 1u);
        return;
    }

    // ---------------- compute warps: thread (x, ty) per column of the tile; the last warp may be
    // partial.  At N = 16 a warp takes rows ty and ty + 8 (176 floats = 16 banks apart), so that
    // every shared-memory access of the warp is conflict-free.
    const bool lane_active = tid < NN;
    const uint32_t t = lane_active ? tid : 0u;
    const uint32_t x = t % N;
    const uint32_t ty = N == 16 ? ((t / N) >> 1) | (((t / N) & 1u) << 3) : t / N;
    const int c0 = (int)((ty + P) * T + (x + P));   // in a ring slot's tile plane
    uint32_t g_base = 0;   // stream index of the current unit's first padded plane
    uint32_t pre_tile = NT;   // the tile the generator prefixes below are for
    for (uint32_t cu = next_unit(p_begin), nz = 0; cu < p_end; cu = next_unit(cu + nz)) {
        uint32_t item, tile, z0, node;
        int depth;
        unit_of(cu, item, tile, z0, nz);
        active_node(item, node, depth);
        const uint32_t y = tile * TY + ty;   // the cell's row in the domain
        if (tile != pre_tile && lane_active) {   // per-cell generators: the part that depends on (seed, x, y) only
            const int32_t* sp = a.seed_ptr;
#pragma unroll
            for (int k = 0; k < NC; k++) {
                s_pre[(2 * k) * NN + tid] = cell_rng_prefix(sp ? sp[2 * k] : a.seed_d[k], x, y);
                s_pre[(2 * k + 1) * NN + tid] = cell_rng_prefix(sp ? sp[2 * k + 1] : a.seed_m[k], x, y);
            }
            s_pre[12 * NN + tid] = cell_rng_prefix(sp ? sp[12] : a.seed_c, x, y);
        }
        pre_tile = tile;
        const float dx1 = a.geo.inv_dx[depth], dx2 = a.geo.inv_dx2[depth];
        const bool leaf = fused_leaf(node);
#pragma unroll 1
        for (uint32_t zl = 0; zl < nz; zl++) {
            const uint32_t g = g_base + zl, z = z0 + zl;   // planes g .. g+2P hold padded z .. z+2P
            bool ok = true;
            for (int j = zl == 0 ? 0 : 2 * P; j <= 2 * P; j++) {   // a unit's first window needs all
                const uint32_t sq = g + j;
                ok &= mbar_wait(&full[sq % R], (sq / R) & 1u, spins);
            }
            if (!ok) {   // this warp's wait gave up: report it (the producer may have nothing left to wait for)
                s_abort = 1;
                if (lane == 0) atomicExch(a.err, 1);
            }
            if (s_abort) { bulk_wait(); return; }
            const uint32_t base_s = g % R;
            uint32_t slot[2 * P + 1];
#pragma unroll
            for (int j = 0; j <= 2 * P; j++) slot[j] = base_s + j >= (uint32_t)R ? base_s + j - R : base_s + j;
            // fused restriction: each padded plane of a leaf goes to field[k] once -- by the unit
            // whose interior it is, the end units also taking the ghost planes beyond; of a plane,
            // each tile stores its rows [row0, row1) -- stored out of the ring by lane 0 of one
            // compute warp per plane, in turn
            const bool storer = leaf && tid == 32u * (g % CW);
            if (storer) {
                const uint32_t row0 = tile == 0u ? 0u : (uint32_t)S::OWN0;
                const uint32_t row1 = tile + 1u == NT ? (uint32_t)T : (uint32_t)S::OWN0;
                for (int j = zl == 0 ? 0 : 2 * P; j <= 2 * P; j++) {
                    const uint32_t jj = zl + (uint32_t)j;   // plane index within the unit
                    const bool own = (jj >= P && jj < nz + P) || (z0 == 0 && jj < P) || (z0 + nz == N && jj >= nz + P);
                    if (!own) continue;
                    const uint32_t sl = base_s + (uint32_t)j >= (uint32_t)R ? base_s + j - R : base_s + j;
#pragma unroll
                    for (int k = 0; k < NC; k++)
                        bulk_s2g(const_cast<float*>(a.field[k]) + ((size_t)node * T + z0 + jj) * PLANE + (size_t)row0 * T,
                                 ring + ((size_t)k * R + sl) * TILE + (size_t)(row0 - tile * TY) * T, (row1 - row0) * T * 4u);
                }
                bulk_commit();
            }
            if (lane_active) {
                const uint32_t zg = node * N + z;
                bssn_cell<N, P>(a, ring, slot, c0, x, y, z, zg, ((size_t)zg * N + y) * N + x, dx1, dx2, tid, s_pre,
                                s_grad);
            }
            // this warp is done with plane g (a storer first waits for its stores to read the ring)
            if (storer) bulk_wait_read();
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[base_s]);
        }
        // the unit's trailing 2P planes start no window: release them too
        __syncwarp();
        if (lane == 0)
            for (uint32_t p = g_base + nz; p < g_base + nz + 2u * P; p++) mbar_arrive(&empty[p % R]);
        g_base += nz + 2u * P;
    }
    bulk_wait();   // this thread's stores out of the ring are complete
}

// ---------------------------------------------------------------- launch
template <int N, int P, int KIND>
cudaError_t launch_stencil_t(const StencilArgs& a, uint32_t grid, cudaStream_t st) {
    using S = StencilShape<N, P, KIND>;
    static std::atomic<uint64_t> configured{0};
    void (*kernel)(const StencilArgs);
    if constexpr (KIND == SK_BSSN) kernel = k_stencil_bssn<N, P>;
    else kernel = k_stencil<N, P, KIND>;
    const cudaError_t e = ensure_smem_limit(kernel, S::SMEM, configured);
    if (e != cudaSuccess) return e;
    if (grid == 0) return cudaSuccess;
    if constexpr (KIND != SK_BSSN) {
        // a grid wider than the items (few domains): cut each into the most z-ranges of at
        // least two planes that the grid holds
        if (a.n_items > 0u && grid > a.n_items) {
            uint32_t q = 1;
            for (uint32_t d = 2; d <= (uint32_t)N / 2u; d++)
                if (N % d == 0 && (uint64_t)d * a.n_items <= grid) q = d;
            StencilArgs b = a;
            b.zsplit = q;
            kernel<<<a.n_items * q, S::THREADS, S::SMEM, st>>>(b);
            return cudaGetLastError();
        }
    }
    kernel<<<grid, S::THREADS, S::SMEM, st>>>(a);
    return cudaGetLastError();
}

#define AMR_STENCIL_INSTANCES(N, P)                                                                      \
    template cudaError_t launch_stencil_t<N, P, SK_GRAD>(const StencilArgs&, uint32_t, cudaStream_t);      \
    template cudaError_t launch_stencil_t<N, P, SK_GRAD_HESS>(const StencilArgs&, uint32_t, cudaStream_t); \
    template cudaError_t launch_stencil_t<N, P, SK_MIXED>(const StencilArgs&, uint32_t, cudaStream_t);     \
    template size_t stencil_smem_bytes<N, P, SK_GRAD>();                                                   \
    template size_t stencil_smem_bytes<N, P, SK_BSSN>();
AMR_FOR_EACH_CONFIG(AMR_STENCIL_INSTANCES)

#define AMR_STENCIL_BSSN_INSTANCES(N, P) \
    template cudaError_t launch_stencil_t<N, P, SK_BSSN>(const StencilArgs&, uint32_t, cudaStream_t);
AMR_FOR_EACH_BSSN_CONFIG(AMR_STENCIL_BSSN_INSTANCES)

}  // namespace amr
