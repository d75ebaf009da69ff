// amr_device.cuh -- device building blocks shared by the GB300 kernels.
//
// Compiled with -fmad=false -ftz=true: every fused multiply-add below is written out
// (__fmaf_rn) and every other product/sum is rounded on its own, so the arithmetic is the
// operation sequence the reference's fast-math device build performs (pinned against that
// build's outputs by the tests), and subnormals flush to zero as they do there.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "amr_types.h"

namespace amr {

// ------------------------------------------------------------------ packed pairs (f32x2, sm_100+)
// One instruction performs the same operation on two independent floats.  Each lane rounds as the
// scalar operation does and flushes subnormals as the -ftz=true scalar code.  One difference: the
// code generator fuses a packed product that feeds a packed add or subtract into one packed
// fused multiply-add (it never does so with the scalar __fmul_rn), so a packed product must only
// feed a multiply or a fused multiply-add, or be exact; where a rounded product is added, the
// product and the sum are done as scalars.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 add2_rz(float2 a, float2 b) { return __fadd2_rz(a, b); }
// a - b as fma(b, -1, a): the product is exact, so this is the rounded difference, signed zeros
// included (x - x = +0 = -x + x), and needs no separate negation of b
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 splat2(float v) { return make_float2(v, v); }

// ------------------------------------------------------------------ fast_prng (tensors.h:276-304)
__device__ __forceinline__ int32_t prng_next(int32_t& s) {
    uint32_t v = (uint32_t)s + 1124781675u;
    v ^= (uint32_t)((int32_t)v >> 7);
    v *= 1246477263u;
    s = (int32_t)v;
    return s;
}
// generate_float() * 0.95f, the encoder's noise (tensors.h:359-361).  The float 2.3283064E-10f is
// exactly 2^-32, so generate_float() is an exact power-of-two scaling of the converted integer
// (nonzero results are at least 2^-32, far from the subnormal range) and the two products round
// once: as the single product by 0.95f * 2^-32, which is exact as a float constant.
constexpr float kNoiseScale = 0.95f * 0x1p-32f;
__device__ __forceinline__ float prng_noise(int32_t& s) {
    return __fmul_rn(__int2float_rn(prng_next(s)), kNoiseScale);
}
// The draw itself as a float (generate_float() / 2^-32, exact): the stencil kernels' encoder adds
// the noise with one fused multiply-add of it by 0.95f * 2^-32 (below).
__device__ __forceinline__ float prng_noise_raw(int32_t& s) { return __int2float_rn(prng_next(s)); }
// Per-cell generator of the stencil kernels, keyed by (launch seed, x, y, slot*N + z)
// (AMR.h:1160-1162, BSSN.h:64-66):
//   s = seed + x*2178614;  s ^= next(s) * y;  s ^= next(s) * zg
// next() leaves its result in s, so the first three steps give s = g ^ (g*y) with g = next(seed +
// x*2178614) and the last one s = h ^ (h*zg) with h = next(that): everything but the final
// multiply and xor depends on (seed, x, y) only.  cell_rng_prefix computes h once per thread;
// cell_rng_at finishes the generator for one cell.
__device__ __forceinline__ int32_t cell_rng_prefix(int32_t seed, uint32_t x, uint32_t y) {
    int32_t s = (int32_t)((uint32_t)seed + x * 2178614u);
    const int32_t g = prng_next(s);
    s = (int32_t)((uint32_t)g ^ ((uint32_t)g * y));
    return prng_next(s);
}
__device__ __forceinline__ int32_t cell_rng_at(int32_t prefix, uint32_t zg) {
    return (int32_t)((uint32_t)prefix ^ ((uint32_t)prefix * zg));
}
__device__ __forceinline__ int32_t cell_rng(int32_t seed, uint32_t x, uint32_t y, uint32_t zg) {
    return cell_rng_at(cell_rng_prefix(seed, x, y), zg);
}

// ------------------------------------------------------------------ compressed_float3 (tensors.h:305-394)
// word = E<<27 | s3<<26 | m3<<18 | s2<<17 | m2<<9 | s1<<8 | m1 ;  value_i = (1 - 2 s_i) m_i 2^(E-22)
// One component's 9-bit field, sign << 8 | mantissa, from the scaled (and noised) value v:
// mantissa = trunc(|clamp(v, -255, 255)| + 0.5), sign = (clamped v < 0) (tensors.h:369-372).  For
// every v -- NaN and +-Inf included -- |clamp(v)| = fminf(|v|, 255) (NaN gives 255, as clamp's
// fminf/fmaxf do) and the sign is (v < 0), false for NaN.  q = fminf(|v|, 255) + 0.5 lies in
// [0.5, 255.5], so adding k = 2^23 + 256*sign with round-toward-zero leaves
// 2^23 + 256*sign + trunc(q) in the float's bits: the field is the low 9 bits.  Returns those bits
// and k (so that bits - k is the mantissa).
struct Cf3Field {
    uint32_t bits;   // 0x4B000000 + field
    float k;         // 2^23 + 256 * sign
    float sign;      // 1.0 or 0.0
};
__device__ __forceinline__ Cf3Field cf3_field(float v) {
    Cf3Field c;
    const float q = __fadd_rn(fminf(fabsf(v), 255.f), .5f);
    asm("set.lt.f32.f32 %0, %1, 0f00000000;" : "=f"(c.sign) : "f"(v));   // 1.0 if v < 0 (false for NaN)
    c.k = __fmaf_rn(c.sign, 256.f, 8388608.f);
    c.bits = __float_as_uint(__fadd_rz(q, c.k));
    return c;
}
// The largest biased exponent of three floats, as the integer maximum of their exponent fields
// would give it: a NaN among them (exponent field 255) wins, which max.NaN reproduces by
// returning a NaN; otherwise |x| orders as its bits do.
__device__ __forceinline__ uint32_t max_exponent3(float x, float y, float z) {
    float m;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(m) : "f"(fabsf(x)), "f"(fabsf(y)));
    asm("max.NaN.f32 %0, %0, %1;" : "+f"(m) : "f"(fabsf(z)));
    return (__float_as_uint(m) >> 23) & 255u;
}
struct Cf3Quantised {
    uint32_t word;
    float3 value;   // the decoded value of `word`
};
// word = E<<27 | s3<<26 | m3<<18 | s2<<17 | m2<<9 | s1<<8 | m1 ;  value_i = (1 - 2 s_i) m_i 2^(E-22)
// The reference's device build adds the noise in two ways (pinned on a GB300 against its own
// kernels): its standalone encoder rounds the noise product first (ROUNDED_NOISE, the codec entry
// point), while the encodes inlined into its stencil and Christoffel kernels fuse the product into
// the add, x * scale + draw * 0.95f as one fused multiply-add (the default).
template <bool STOCHASTIC, bool WANT_VALUE, bool ROUNDED_NOISE = false>
__device__ __forceinline__ Cf3Quantised cf3_encode_impl(float x, float y, float z, int32_t& rng) {
    const uint32_t E = min(max(max_exponent3(x, y, z), 112u) - 112u, 31u);
    const float scale = __uint_as_float((149u - E) << 23);          // 2^(22-E), exact
    if (STOCHASTIC && ROUNDED_NOISE) {
        // The noise product rounded before it is added.  x * scale is exact (a power-of-two
        // scaling), so one fused multiply-add gives the reference's rounded sum x * scale + noise,
        // except where x * scale is subnormal: flushed first, it leaves the sum +0, while fused it
        // can leave -0 (when the noise is 0); the field below reads |v| and (v < 0) only, the same
        // for both zeros.
        x = __fmaf_rn(x, scale, prng_noise(rng));
        y = __fmaf_rn(y, scale, prng_noise(rng));
        z = __fmaf_rn(z, scale, prng_noise(rng));
    } else if (STOCHASTIC) {
        // x * scale (exact, flushed if subnormal) + draw * 0.95 * 2^-32 rounded once
        x = __fmaf_rn(prng_noise_raw(rng), kNoiseScale, __fmul_rn(x, scale));
        y = __fmaf_rn(prng_noise_raw(rng), kNoiseScale, __fmul_rn(y, scale));
        z = __fmaf_rn(prng_noise_raw(rng), kNoiseScale, __fmul_rn(z, scale));
    } else {
        x = __fmul_rn(x, scale);
        y = __fmul_rn(y, scale);
        z = __fmul_rn(z, scale);
    }
    const Cf3Field fx = cf3_field(x), fy = cf3_field(y), fz = cf3_field(z);
    Cf3Quantised r;
    // (0x4B000000 + f) * 2^9 and * 2^18 wrap to f << 9 and f << 18: the high bits fall off
    r.word = (E << 27) + (fx.bits & 511u) + fy.bits * 512u + fz.bits * 262144u;
    if (WANT_VALUE) {   // (bits - k) = m exactly; times +-2^(E-22), the sign applied by the factor
        const float back = __uint_as_float((105u + E) << 23);
        r.value = make_float3(__fmul_rn(__fsub_rn(__uint_as_float(fx.bits), fx.k), __fmaf_rn(fx.sign, -2.f * back, back)),
                              __fmul_rn(__fsub_rn(__uint_as_float(fy.bits), fy.k), __fmaf_rn(fy.sign, -2.f * back, back)),
                              __fmul_rn(__fsub_rn(__uint_as_float(fz.bits), fz.k), __fmaf_rn(fz.sign, -2.f * back, back)));
    }
    return r;
}
__device__ __forceinline__ uint32_t cf3_encode(float x, float y, float z, int32_t& rng) {
    return cf3_encode_impl<true, false>(x, y, z, rng).word;
}
// The reference's standalone encoder (compressed_float3(float3, fast_prng&) in its own kernel).
__device__ __forceinline__ uint32_t cf3_encode_codec(float x, float y, float z, int32_t& rng) {
    return cf3_encode_impl<true, false, true>(x, y, z, rng).word;
}
// Encode and also return the decoded (quantised) value, as a consumer reading the word back sees it.
__device__ __forceinline__ Cf3Quantised cf3_encode_quantised(float x, float y, float z, int32_t& rng) {
    return cf3_encode_impl<true, true>(x, y, z, rng);
}
__device__ __forceinline__ uint32_t cf3_encode_det(float x, float y, float z) {
    int32_t unused = 0;
    return cf3_encode_impl<false, false>(x, y, z, unused).word;
}
// ------------------------------------------------------------------ the encoder on pairs
// Two independent stochastic encodes (lanes x and y) with their floating-point steps done as
// packed pairs; each lane is cf3_encode_impl<true, WANT_VALUE> bit for bit.  The noise pairs
// (nx, ny, nz) are the lanes' three draws (unscaled) in the order the scalar encoder takes them.
struct Cf3Pair {
    uint32_t w0, w1;        // the words of lanes x and y
    float2 vx, vy, vz;      // WANT_VALUE: the decoded components (lane x of each: the first word)
};
__device__ __forceinline__ float2 noise_pair(int32_t s0, int32_t s1) {   // the draws, unscaled
    return make_float2(__int2float_rn(s0), __int2float_rn(s1));
}
// Noise pairs of two generators, one per lane.
__device__ __forceinline__ void noise_pairs2(int32_t& r0, int32_t& r1, float2& nx, float2& ny, float2& nz) {
    nx = noise_pair(prng_next(r0), prng_next(r1));
    ny = noise_pair(prng_next(r0), prng_next(r1));
    nz = noise_pair(prng_next(r0), prng_next(r1));
}
// Noise pairs of one generator: lane x takes its next three draws, lane y the three after.
__device__ __forceinline__ void noise_pairs1(int32_t& r, float2& nx, float2& ny, float2& nz) {
    const int32_t a0 = prng_next(r), a1 = prng_next(r), a2 = prng_next(r);
    const int32_t b0 = prng_next(r), b1 = prng_next(r), b2 = prng_next(r);
    nx = noise_pair(a0, b0);
    ny = noise_pair(a1, b1);
    nz = noise_pair(a2, b2);
}
struct Cf3Field2 {
    float2 bits, k, sign;   // per lane as Cf3Field (bits as a float)
};
__device__ __forceinline__ Cf3Field2 cf3_field2(float2 v) {
    Cf3Field2 c;
    const float2 q = add2(make_float2(fminf(fabsf(v.x), 255.f), fminf(fabsf(v.y), 255.f)), splat2(.5f));
    asm("set.lt.f32.f32 %0, %1, 0f00000000;" : "=f"(c.sign.x) : "f"(v.x));
    asm("set.lt.f32.f32 %0, %1, 0f00000000;" : "=f"(c.sign.y) : "f"(v.y));
    c.k = fma2(c.sign, splat2(256.f), splat2(8388608.f));
    c.bits = add2_rz(q, c.k);
    return c;
}
template <bool WANT_VALUE>
__device__ __forceinline__ Cf3Pair cf3_encode2(float2 x, float2 y, float2 z, float2 nx, float2 ny, float2 nz) {
    const uint32_t E0 = min(max(max_exponent3(x.x, y.x, z.x), 112u) - 112u, 31u);
    const uint32_t E1 = min(max(max_exponent3(x.y, y.y, z.y), 112u) - 112u, 31u);
    const float2 scale = make_float2(__uint_as_float((149u - E0) << 23), __uint_as_float((149u - E1) << 23));
    // x * scale (exact) + draw * 0.95 * 2^-32, one rounding (the stencil kernels' fused noise)
    x = fma2(nx, splat2(kNoiseScale), mul2(x, scale));
    y = fma2(ny, splat2(kNoiseScale), mul2(y, scale));
    z = fma2(nz, splat2(kNoiseScale), mul2(z, scale));
    const Cf3Field2 fx = cf3_field2(x), fy = cf3_field2(y), fz = cf3_field2(z);
    Cf3Pair r;
    r.w0 = (E0 << 27) + (__float_as_uint(fx.bits.x) & 511u) + __float_as_uint(fy.bits.x) * 512u +
           __float_as_uint(fz.bits.x) * 262144u;
    r.w1 = (E1 << 27) + (__float_as_uint(fx.bits.y) & 511u) + __float_as_uint(fy.bits.y) * 512u +
           __float_as_uint(fz.bits.y) * 262144u;
    if (WANT_VALUE) {
        const float2 back = make_float2(__uint_as_float((105u + E0) << 23), __uint_as_float((105u + E1) << 23));
        const float2 back2 = mul2(back, splat2(-2.f));
        r.vx = mul2(sub2(fx.bits, fx.k), fma2(fx.sign, back2, back));
        r.vy = mul2(sub2(fy.bits, fy.k), fma2(fy.sign, back2, back));
        r.vz = mul2(sub2(fz.bits, fz.k), fma2(fz.sign, back2, back));
    }
    return r;
}

// Exact: m * 2^(E-22) is representable, the sign bit is applied last (so m = 0 keeps its sign).
__device__ __forceinline__ float cf3_component(uint32_t w, uint32_t mpos, uint32_t spos) {
    const float scale = __uint_as_float((105u + (w >> 27)) << 23);  // 2^(E-22)
    const float m = __uint2float_rn((w >> mpos) & 255u);
    return __uint_as_float(__float_as_uint(__fmul_rn(m, scale)) | (((w >> spos) & 1u) << 31));
}
__device__ __forceinline__ float3 cf3_decode(uint32_t w) {
    return make_float3(cf3_component(w, 0u, 8u), cf3_component(w, 9u, 17u), cf3_component(w, 18u, 26u));
}

// ------------------------------------------------------------------ fast-math primitives
// The reference is built with --use_fast_math; its divisions and square roots are the
// hardware approximations, which these wrappers issue directly.
__device__ __forceinline__ float rcp_approx(float a) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float sqrt_approx(float a) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// ------------------------------------------------------------------ symmetric 3x3 algebra (tensors.h:133-244)
// Stored as s[0..5] = xx, xy, xz, yy, yz, zz.
struct Sym { float xx, xy, xz, yy, yz, zz; };

__device__ __forceinline__ float sym_determinant(const Sym& m) {          // tensors.h:208-210
    float d = __fmul_rn(__fmul_rn(-m.xz, m.yy), m.xz);
    d = __fmaf_rn(__fmul_rn(m.xy, m.yz), m.xz, d);
    d = __fmaf_rn(__fmul_rn(m.xz, m.xy), m.yz, d);
    d = __fmaf_rn(-__fmul_rn(m.xx, m.yz), m.yz, d);
    d = __fmaf_rn(-__fmul_rn(m.xy, m.xy), m.zz, d);
    d = __fmaf_rn(__fmul_rn(m.xx, m.yy), m.zz, d);
    return d;
}
// Cofactor inverse (tensors.h:211-225).  The products shared with the determinant stay rounded.
__device__ __forceinline__ Sym sym_inverse(const Sym& m) {
    Sym r;
    r.xx = __fmaf_rn(m.yy, m.zz, -__fmul_rn(m.yz, m.yz));
    r.xy = __fmaf_rn(m.yz, m.xz, -__fmul_rn(m.xy, m.zz));
    r.xz = __fsub_rn(__fmul_rn(m.xy, m.yz), __fmul_rn(m.yy, m.xz));
    r.yy = __fmaf_rn(m.xx, m.zz, -__fmul_rn(m.xz, m.xz));
    r.yz = __fsub_rn(__fmul_rn(m.xy, m.xz), __fmul_rn(m.xx, m.yz));
    r.zz = __fsub_rn(__fmul_rn(m.xx, m.yy), __fmul_rn(m.xy, m.xy));
    const float inv_det = rcp_approx(sym_determinant(m));
    r.xx = __fmul_rn(r.xx, inv_det); r.xy = __fmul_rn(r.xy, inv_det); r.xz = __fmul_rn(r.xz, inv_det);
    r.yy = __fmul_rn(r.yy, inv_det); r.yz = __fmul_rn(r.yz, inv_det); r.zz = __fmul_rn(r.zz, inv_det);
    return r;
}
// c^ij m_ij for symmetric c, m (tensors.h:241-244)
__device__ __forceinline__ float trace_contra(const Sym& c, const Sym& m) {
    float a = __fmaf_rn(c.xx, m.xx, __fmul_rn(c.yy, m.yy));
    a = __fmaf_rn(c.zz, m.zz, a);
    float b = __fmaf_rn(c.xy, m.xy, __fmul_rn(c.xz, m.xz));
    b = __fmaf_rn(c.yz, m.yz, b);
    return __fmaf_rn(b, 2.f, a);
}
// m * v (tensors.h:201-206)
__device__ __forceinline__ float3 sym_times(const Sym& m, float3 a) {
    return make_float3(__fmaf_rn(a.z, m.xz, __fmaf_rn(a.x, m.xx, __fmul_rn(a.y, m.xy))),
                       __fmaf_rn(a.z, m.yz, __fmaf_rn(a.x, m.xy, __fmul_rn(a.y, m.yy))),
                       __fmaf_rn(a.z, m.zz, __fmaf_rn(a.x, m.xz, __fmul_rn(a.y, m.yz))));
}
__device__ __forceinline__ Sym sym_from_cf3(uint32_t diag, uint32_t off) {   // tensors.h:430-435
    const float3 d = cf3_decode(diag), o = cf3_decode(off);
    return Sym{d.x, o.x, o.y, d.y, o.z, d.z};
}

// ------------------------------------------------------------------ octree words (AMR.h:22-100)
__device__ __forceinline__ int pos_depth(uint32_t pos) { return (~pos) ? (int)(pos >> 27) : -1; }
__device__ __forceinline__ bool active_depth(uint32_t substep, uint32_t depth, uint32_t max_depth) {
    return (substep & ((1u << (max_depth - depth)) - 1u)) == 0u;
}
__device__ __forceinline__ int32_t bd_target(uint64_t b) {
    const uint32_t nd = (uint32_t)b;
    return (int32_t)((nd & 16777215u) | ((nd & (1u << 23)) ? 4278190080u : 0u));
}
__device__ __forceinline__ uint32_t bd_depth_diff(uint64_t b) { return ((uint32_t)b >> 24) & 15u; }
__device__ __forceinline__ int bd_curr_depth(uint64_t b) {
    const uint32_t nd = (uint32_t)b;
    return ((nd >> 28) == 15u) ? -1 : (int)(nd >> 28);
}

// ------------------------------------------------------------------ finite-difference weights (AMR.h:1144-1150)
// Centred (2p+1)-point weights of the first and second derivative, index i = -p..p.
template <int P> struct FD;
template <> struct FD<1> {
    static __device__ __forceinline__ float d1(int i) { return i == -1 ? -.5f : i == 1 ? .5f : 0.f; }
    static __device__ __forceinline__ float d2(int i) { return i == 0 ? -2.f : 1.f; }
};
template <> struct FD<2> {
    static __device__ __forceinline__ float d1(int i) {
        return i == -2 ? 1.f / 12 : i == -1 ? -2.f / 3 : i == 0 ? 0.f : i == 1 ? 2.f / 3 : -1.f / 12;
    }
    static __device__ __forceinline__ float d2(int i) {
        return i == -2 ? -1.f / 12 : i == -1 ? 4.f / 3 : i == 0 ? -5.f / 2 : i == 1 ? 4.f / 3 : -1.f / 12;
    }
};
template <> struct FD<3> {
    static __device__ __forceinline__ float d1(int i) {
        return i == -3 ? -1.f / 60 : i == -2 ? 3.f / 20 : i == -1 ? -3.f / 4 : i == 0 ? 0.f
             : i == 1 ? 3.f / 4 : i == 2 ? -3.f / 20 : 1.f / 60;
    }
    static __device__ __forceinline__ float d2(int i) {
        return i == -3 ? 1.f / 90 : i == -2 ? -3.f / 20 : i == -1 ? 3.f / 2 : i == 0 ? -49.f / 18
             : i == 1 ? 3.f / 2 : i == 2 ? -3.f / 20 : 1.f / 90;
    }
};

// ------------------------------------------------------------------ 10-point interpolation (AMR.h:672-699)
// d points at the nearest source cell; strides 1, sy, sz; r = offset from it in cells.
// The arithmetic of the 10-point interpolation on its loaded taps: f at the nearest cell, fx/fy/fz
// one cell up and fxx/fyy/fzz one cell down each axis, fxy/fxz/fyz the three upper diagonals.
__device__ __forceinline__ float interp10_taps(float f, float fx, float fy, float fz, float fxx, float fyy, float fzz,
                                              float fxy, float fxz, float fyz, float rx, float ry, float rz) {
    fxy = __fadd_rn(fxy, __fsub_rn(__fsub_rn(f, fx), fy));
    fxz = __fadd_rn(fxz, __fsub_rn(__fsub_rn(f, fx), fz));
    fyz = __fadd_rn(fyz, __fsub_rn(__fsub_rn(f, fy), fz));
    fx = __fmul_rn(__fsub_rn(fx, fxx), .5f);
    fy = __fmul_rn(__fsub_rn(fy, fyy), .5f);
    fz = __fmul_rn(__fsub_rn(fz, fzz), .5f);
    fxx = __fsub_rn(__fadd_rn(fx, fxx), f);
    fyy = __fsub_rn(__fadd_rn(fy, fyy), f);
    fzz = __fsub_rn(__fadd_rn(fz, fzz), f);
    float acc = __fmaf_rn(__fadd_rn(fx, __fmul_rn(fxx, rx)), rx, f);
    acc = __fmaf_rn(__fadd_rn(fy, __fmul_rn(fyy, ry)), ry, acc);
    acc = __fmaf_rn(__fadd_rn(fz, __fmul_rn(fzz, rz)), rz, acc);
    acc = __fmaf_rn(__fmul_rn(fxy, rx), ry, acc);
    acc = __fmaf_rn(__fmul_rn(fxz, rx), rz, acc);
    acc = __fmaf_rn(__fmul_rn(fyz, ry), rz, acc);
    return acc;
}
template <class S>
__device__ __forceinline__ float interp10_strided(const float* __restrict__ d, S sy, S sz, float rx, float ry, float rz) {
    return interp10_taps(d[0], d[1], d[sy], d[sz], d[-1], d[-sy], d[-sz], d[sy + 1], d[sz + 1], d[sz + sy], rx, ry, rz);
}
// interp10_strided on two fields at once: d holds (a, b) pairs, the result is
// (interp10_strided(a), interp10_strided(b)), each lane the same operation sequence.
template <class S>
__device__ __forceinline__ float2 interp10_pair(const float2* __restrict__ d, S sy, S sz, float rx, float ry, float rz) {
    const float2 f = d[0];
    float2 fx = d[1], fy = d[sy], fz = d[sz];
    float2 fxx = d[-1], fyy = d[-sy], fzz = d[-sz];
    float2 fxy = d[sy + 1], fxz = d[sz + 1], fyz = d[sz + sy];
    fxy = add2(fxy, sub2(sub2(f, fx), fy));
    fxz = add2(fxz, sub2(sub2(f, fx), fz));
    fyz = add2(fyz, sub2(sub2(f, fy), fz));
    // the halving is exact (bar a subnormal product), fused into the next add or not
    const float2 half = splat2(.5f);
    fx = mul2(sub2(fx, fxx), half);
    fy = mul2(sub2(fy, fyy), half);
    fz = mul2(sub2(fz, fzz), half);
    fxx = sub2(add2(fx, fxx), f);
    fyy = sub2(add2(fy, fyy), f);
    fzz = sub2(add2(fz, fzz), f);
    const float2 Rx = splat2(rx), Ry = splat2(ry), Rz = splat2(rz);
    // fx + fxx * rx with the product rounded: scalar (a packed product would be fused into the add)
    auto axis = [](float2 g, float2 h, float r) {
        return make_float2(__fadd_rn(g.x, __fmul_rn(h.x, r)), __fadd_rn(g.y, __fmul_rn(h.y, r)));
    };
    float2 acc = fma2(axis(fx, fxx, rx), Rx, f);
    acc = fma2(axis(fy, fyy, ry), Ry, acc);
    acc = fma2(axis(fz, fzz, rz), Rz, acc);
    acc = fma2(mul2(fxy, Rx), Ry, acc);
    acc = fma2(mul2(fxz, Rx), Rz, acc);
    acc = fma2(mul2(fyz, Ry), Rz, acc);
    return acc;
}
// The same on a padded domain (strides T, T^2).
template <int T>
__device__ __forceinline__ float interp10(const float* __restrict__ d, float rx, float ry, float rz) {
    return interp10_strided(d, T, T * T, rx, ry, rz);
}

}  // namespace amr
