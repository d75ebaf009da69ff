/* amr_oracle.c -- CPU restatement of AdaptiveMesh's per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see amr_oracle.h).  Compiled with -ffp-contract=off so that
 * every fused multiply-add below is an explicit fmaf() call: the operation order is the
 * one the reference's device build uses, pinned against that build's own outputs by the
 * fixtures under tests/golden/.
 */
#include "amr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ small helpers */
static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
/* flush a subnormal to a zero of the same sign (the device build runs with -ftz=true) */
static inline float ftz(float f) { return ((fbits(f) & 0x7F800000u) == 0u) ? bitsf(fbits(f) & 0x80000000u) : f; }
static inline uint32_t umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
static inline uint32_t umax(uint32_t a, uint32_t b) { return a > b ? a : b; }
/* float -> uint conversion of a non-negative value, truncating (C semantics, as cvt.rzi) */
static inline uint32_t f2u(float f) { return (uint32_t)f; }

void orc_cfg_init(orc_cfg* c, uint32_t n, uint32_t p, float outer_size, uint32_t flags) {
    c->n = n; c->p = p; c->outer_size = outer_size; c->flags = flags;
    c->outer_dx = outer_size / (float)n;            /* AMR.h:16 */
    c->outer_dt = c->outer_dx * .4f;                /* AMR.h:17 */
    for (int d = 0; d <= 8; d++) c->inv_dx[d] = (float)(1u << d) / c->outer_dx;  /* AMR.h:1176 */
}

/* ------------------------------------------------------------------ fast_prng, tensors.h:276-304 */
int32_t orc_prng_int(int32_t* s) {
    uint32_t v = (uint32_t)*s + 1124781675u;
    v ^= (uint32_t)((int32_t)v >> 7);           /* arithmetic shift of the signed state */
    v *= 1246477263u;
    *s = (int32_t)v;
    return (int32_t)v;
}
float orc_prng_float(int32_t* s) { return (float)orc_prng_int(s) * 2.3283064E-10f; }
int32_t orc_prng_ranged(int32_t* s, int32_t lo, int32_t hi) {
    uint32_t v = (uint32_t)orc_prng_int(s);
    uint64_t span = (uint64_t)(int64_t)(hi - lo);
    return (int32_t)(uint32_t)(((uint64_t)v * span) >> 32) + lo;
}

/* ------------------------------------------------------------------ compressed_float3, tensors.h:305-394
 * word = E<<27 | s3<<26 | m3<<18 | s2<<17 | m2<<9 | s1<<8 | m1 ; value_i = (1-2 s_i) m_i 2^(E-22) */
uint32_t orc_cf3_encode(float x, float y, float z, int32_t* rng, uint32_t flags) {
    const int do_ftz = (flags & ORC_FTZ) != 0;
    float v[3] = {x, y, z};
    uint32_t e = 0;
    for (int i = 0; i < 3; i++) e = umax(e, (fbits(v[i]) >> 23) & 255u);
    uint32_t E = umin(umax(e, 112u) - 112u, 31u);                     /* tensors.h:355-359 */
    float scale = 4194304.f / (float)(1u << E);                       /* 2^15 / (1/128) / 2^E, exact */
    for (int i = 0; i < 3; i++) {
        float a = do_ftz ? ftz(v[i]) : v[i];
        a = a * scale;
        if (do_ftz) a = ftz(a);
        v[i] = a;
    }
    if (rng) {                                                        /* tensors.h:365-367 */
        for (int i = 0; i < 3; i++) {
            float r = orc_prng_float(rng);
            float s = (flags & ORC_FUSED_NOISE) ? fmaf(r, .95f, v[i]) : v[i] + r * .95f;
            v[i] = do_ftz ? ftz(s) : s;
        }
    }
    uint32_t w = E << 27;
    const int mpos[3] = {0, 9, 18}, spos[3] = {8, 17, 26};
    for (int i = 0; i < 3; i++) {
        float c = fmaxf(-255.f, fminf(v[i], 255.f));                /* clamp, tensors.h:369 */
        w |= (f2u(fabsf(c) + .5f) << mpos[i]) | ((uint32_t)(c < 0.f) << spos[i]);
    }
    return w;
}
void orc_cf3_decode(uint32_t w, float* xyz) {                           /* tensors.h:335-348 */
    float base = bitsf((112u + (w >> 27)) << 23);
    const int mpos[3] = {0, 9, 18}, spos[3] = {8, 17, 26};
    for (int i = 0; i < 3; i++) {
        float m = (float)((w >> mpos[i]) & 255u);
        float sg = 1.f - 2.f * (float)((w >> spos[i]) & 1u);
        xyz[i] = base * ((m * sg) * 0.0078125f);
    }
}
void orc_cf3_encode_seeded(const float* xyz, const int32_t* seeds, int64_t n, uint32_t* out, uint32_t flags) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        int32_t s = seeds[i];
        out[i] = orc_cf3_encode(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], &s, flags);
    }
}
int32_t orc_cf3_encode_stream(const float* xyz, int64_t n, int32_t seed, uint32_t* out, uint32_t flags) {
    for (int64_t i = 0; i < n; i++) out[i] = orc_cf3_encode(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], &seed, flags);
    return seed;
}
void orc_cf3_encode_det(const float* xyz, int64_t n, uint32_t* out, uint32_t flags) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = orc_cf3_encode(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], NULL, flags);
}
void orc_cf3_decode_n(const uint32_t* in, int64_t n, float* xyz) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) orc_cf3_decode(in[i], xyz + 3 * i);
}

/* ------------------------------------------------------------------ tensor algebra, tensors.h:133-244
 * Symmetric 3x3 stored (xx, xy, xz, yy, yz, zz). */
float orc_sym_determinant(const float* m) {                             /* tensors.h:208-210 */
    const float xx = m[0], xy = m[1], xz = m[2], yy = m[3], yz = m[4], zz = m[5];
    float d = (-xz * yy) * xz;
    d = fmaf(xy * yz, xz, d);
    d = fmaf(xz * xy, yz, d);
    d = fmaf(-(xx * yz), yz, d);
    d = fmaf(-(xy * xy), zz, d);
    d = fmaf(xx * yy, zz, d);
    return d;
}
void orc_sym_inverse(const float* m, float* r) {                       /* tensors.h:211-225 */
    const float xx = m[0], xy = m[1], xz = m[2], yy = m[3], yz = m[4], zz = m[5];
    /* Cofactors.  The products xy*yz, yy*xz, xy*xz, xx*yz, xy*xy and xx*yy are shared with the
     * determinant, so the device build keeps them rounded; the others fuse into the sum. */
    r[0] = fmaf(yy, zz, -(yz * yz));
    r[1] = fmaf(yz, xz, -(xy * zz));
    r[2] = xy * yz - yy * xz;
    r[3] = fmaf(xx, zz, -(xz * xz));
    r[4] = xy * xz - xx * yz;
    r[5] = xx * yy - xy * xy;
    /* The device build divides with an approximate reciprocal (fast-math); this restatement
     * divides exactly, so results may differ from it by up to 2 ulp. */
    const float det = orc_sym_determinant(m);
    for (int i = 0; i < 6; i++) r[i] = r[i] / det;
}
float orc_trace_contra_sym(const float* c, const float* m) {           /* tensors.h:241-244 */
    float a = fmaf(c[0], m[0], c[3] * m[3]);
    a = fmaf(c[5], m[5], a);
    float b = fmaf(c[1], m[1], c[2] * m[2]);
    b = fmaf(c[4], m[4], b);
    return fmaf(b, 2.f, a);
}
void orc_sym_times_vec(const float* m, const float* a, float* o) {     /* tensors.h:201-206 */
    /* a.x*m0 + a.y*m1 fuses the left product; the third product is fused into that sum */
    o[0] = fmaf(a[2], m[2], fmaf(a[0], m[0], a[1] * m[1]));
    o[1] = fmaf(a[2], m[4], fmaf(a[0], m[1], a[1] * m[3]));
    o[2] = fmaf(a[2], m[5], fmaf(a[0], m[2], a[1] * m[4]));
}

/* ------------------------------------------------------------------ octree helpers, AMR.h:22-116 */
uint32_t orc_reverse_bits(uint32_t a) {                                 /* bit reversal of a 32-bit word */
    uint32_t r = 0;
    for (int i = 0; i < 32; i++) r |= ((a >> i) & 1u) << (31 - i);
    return r;
}
/* Per-axis addition / subtraction of interleaved (Morton) coordinates, AMR.h:102-115.
 * Each axis occupies every third bit of a 27-bit path; the result's bits 27..29 catch a carry
 * (or borrow) out of the top level, which means the neighbour lies outside the root. */
#define ORC_LANE 0x1249249u          /* bits 0, 3, ..., 24: one axis of a 27-bit path */
#define ORC_LANE_OUT 0x9249249u      /* the same plus bit 27, where an overflow lands */
uint32_t orc_sum_coordinates(uint32_t a, uint32_t b, int overflow) {
    uint32_t res = 0;
    for (int axis = 0; axis < 3; axis++) {
        const uint32_t lane = ORC_LANE << axis;
        const uint32_t gaps = (0x7FFFFFFu & ~ORC_LANE) << axis;    /* ones between lane bits carry through */
        res |= ((a | gaps) + (b & lane)) & (ORC_LANE_OUT << axis);
    }
    if ((res & (7u << 27)) && overflow) return ~0u;
    return res & ((1u << 27) - 1u);
}
uint32_t orc_diff_coordinates(uint32_t a, uint32_t b, int overflow) {
    uint32_t res = 0;
    for (int axis = 0; axis < 3; axis++) {
        const uint32_t lane = ORC_LANE << axis;                    /* zeros between lane bits borrow through */
        res |= ((a & lane) - (b & lane)) & (ORC_LANE_OUT << axis);
    }
    if ((res & (7u << 27)) && overflow) return ~0u;
    return res & ((1u << 27) - 1u);
}
static int pos_depth(uint32_t pos) { return (~pos) ? (int)(pos >> 27) : -1; }   /* AMR.h:27-29 */
uint64_t orc_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx) { /* AMR.h:64-86 */
    const int td = pos_depth(this_pos), od = pos_depth(other_pos);
    uint32_t node_data = ((uint32_t)other_idx & 16777215u) | (((uint32_t)(td - od) & 15u) << 24) | (((uint32_t)td & 15u) << 28);
    float r[3] = {0.f, 0.f, 0.f};
    const float mult = .25f * (float)(1u << od);
    uint32_t s = this_pos & 134217727u;
    for (int i = 0; i < td; i++, s >>= 3)
        for (int a = 0; a < 3; a++) r[a] += ((s & (1u << a)) ? mult : -mult) / (float)(1 << i);
    s = other_pos & 134217727u;
    for (int i = 0; i < od; i++, s >>= 3)
        for (int a = 0; a < 3; a++) r[a] -= ((s & (1u << a)) ? mult : -mult) / (float)(1 << i);
    uint32_t rel = orc_cf3_encode(r[0], r[1], r[2], NULL, 0);
    return (uint64_t)node_data | ((uint64_t)rel << 32);
}
static inline int32_t bd_target(uint64_t b) {                            /* AMR.h:87-89 */
    uint32_t nd = (uint32_t)b;
    return (int32_t)((nd & 16777215u) | ((nd & (1u << 23)) ? 4278190080u : 0u));
}
static inline uint32_t bd_depth_diff(uint64_t b) { return ((uint32_t)b >> 24) & 15u; }
static inline int bd_curr_depth(uint64_t b) { uint32_t nd = (uint32_t)b; return ((nd >> 28) == 15u) ? -1 : (int)(nd >> 28); }
static inline int active_depth(uint32_t substep, uint32_t depth, uint32_t max_depth) {   /* AMR.h:640-644 */
    return (substep & ((1u << (max_depth - depth)) - 1u)) == 0u;
}

/* ------------------------------------------------------------------ FD tables, AMR.h:1144-1150 */
static const float FD1[15] = {-.5f, 0.f, .5f,
                              1.f / 12, -2.f / 3, 0.f, 2.f / 3, -1.f / 12,
                              -1.f / 60, 3.f / 20, -3.f / 4, 0.f, 3.f / 4, -3.f / 20, 1.f / 60};
static const float FD2[15] = {1.f, -2.f, 1.f,
                              -1.f / 12, 4.f / 3, -5.f / 2, 4.f / 3, -1.f / 12,
                              1.f / 90, -3.f / 20, 3.f / 2, -49.f / 18, 3.f / 2, -3.f / 20, 1.f / 90};

/* Per-thread generator of the stencil kernels: keyed by (seed, x, y, global z = slot*n + z),
 * AMR.h:1160-1162 (same in __mixed_partials and the Christoffel kernel). */
static inline int32_t cell_rng(int32_t seed, uint32_t x, uint32_t y, uint32_t zg) {
    int32_t s = (int32_t)((uint32_t)seed + x * 2178614u);
    int32_t g = orc_prng_int(&s);
    s = (int32_t)((uint32_t)s ^ ((uint32_t)g * y));
    g = orc_prng_int(&s);
    s = (int32_t)((uint32_t)s ^ ((uint32_t)g * zg));
    return s;
}

static inline uint64_t padded_center(const orc_cfg* c, uint32_t slot, uint32_t x, uint32_t y, uint32_t z) {
    const uint64_t t = c->n + 2 * c->p;
    return ((slot * t + z) * t + y) * t + x + c->p * (1 + t + t * t);
}

/* ------------------------------------------------------------------ __differentiate, AMR.h:1152-1219 */
void orc_differentiate(const orc_cfg* c, const float* f, uint32_t* dif, uint32_t* d2if,
                       const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const int k0 = (int)(p * p + p - 1);
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) continue;
        const float dx1 = c->inv_dx[depth];
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                int32_t rng = cell_rng(seed, x, y, slot * n + z);
                const uint64_t rw = padded_center(c, slot, x, y, z);
                float gx = 0.f, gy = 0.f, gz = 0.f, hx = 0.f, hy = 0.f, hz = 0.f;
                for (int i = -(int)p; i <= (int)p; i++) {
                    const float c1 = FD1[k0 + i], c2 = FD2[k0 + i];
                    float a = f[rw + i];
                    gx = fmaf(a, c1, gx); hx = fmaf(a, c2, hx);
                    a = f[rw + (int64_t)i * t];
                    gy = fmaf(a, c1, gy); hy = fmaf(a, c2, hy);
                    a = f[rw + (int64_t)i * t * t];
                    gz = fmaf(a, c1, gz); hz = fmaf(a, c2, hz);
                }
                gx *= dx1; gy *= dx1; gz *= dx1;
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                if (d2if) {
                    const float dd = dx1 * dx1;
                    hx *= dd; hy *= dd; hz *= dd;
                    d2if[o] = orc_cf3_encode(hx, hy, hz, &rng, c->flags);
                }
                dif[o] = orc_cf3_encode(gx, gy, gz, &rng, c->flags);
            }
    }
}

/* ------------------------------------------------------------------ __mixed_partials, AMR.h:1221-1266 */
static inline float mixed_c(const float* f, int64_t i, int64_t dx, int64_t dy) {          /* AMR.h:1221-1225 */
    return .25f * (((f[i + dx + dy] + f[i - dx - dy]) - f[i + dx - dy]) - f[i - dx + dy]);
}
static inline float mixed_bd(const float* f, int64_t i, int64_t dx, int64_t dy) {         /* AMR.h:1226-1230 */
    float s = f[i + dx + dy] + f[i - dx - dy];
    s = s - f[i - dx]; s = s - f[i + dx]; s = s - f[i - dy]; s = s - f[i + dy];
    return fmaf(.5f, s, f[i]);
}
void orc_mixed_partials(const orc_cfg* c, const float* f, uint32_t* off,
                        const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth, int32_t seed) {
    const uint32_t n = c->n, p = c->p;
    const int64_t t = n + 2 * p;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) continue;
        float dx1 = c->inv_dx[depth];
        dx1 = dx1 * dx1;
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                int32_t rng = cell_rng(seed, x, y, slot * n + z);
                const int64_t rw = (int64_t)padded_center(c, slot, x, y, z);
                const int ex = (int)x - (int)umin(umax(x, 1u), n - 2u);
                const int ey = (int)y - (int)umin(umax(y, 1u), n - 2u);
                const int ez = (int)z - (int)umin(umax(z, 1u), n - 2u);
                const int cxy = ex * ey, cxz = ex * ez, cyz = ey * ez;
                const float vxy = cxy == 0 ? mixed_c(f, rw, 1, t) : (float)(-cxy) * mixed_bd(f, rw, -cxy, t);
                const float vxz = cxz == 0 ? mixed_c(f, rw, 1, t * t) : (float)(-cxz) * mixed_bd(f, rw, -cxz, t * t);
                const float vyz = cyz == 0 ? mixed_c(f, rw, t, t * t) : (float)(-cyz) * mixed_bd(f, rw, -cyz * t, t * t);
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                off[o] = orc_cf3_encode(vxy * dx1, vxz * dx1, vyz * dx1, &rng, c->flags);
            }
    }
}

/* ------------------------------------------------------------------ __deriv_trace, BSSN.h:7-22 */
static inline void sym_from_cf3(uint32_t diag, uint32_t off, float* s) {                 /* tensors.h:430-435 */
    float d[3], o[3];
    orc_cf3_decode(diag, d); orc_cf3_decode(off, o);
    s[0] = d[0]; s[1] = o[0]; s[2] = o[1]; s[3] = d[1]; s[4] = o[2]; s[5] = d[2];
}
void orc_deriv_trace(const orc_cfg* c, const uint32_t* hd, const uint32_t* ho, const float* const* met,
                     float* out, const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    const uint32_t n = c->n;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) continue;
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                const uint64_t rw = padded_center(c, slot, x, y, z);
                float m[6], inv[6], h[6];
                for (int k = 0; k < 6; k++) m[k] = met[k][rw];
                orc_sym_inverse(m, inv);
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                sym_from_cf3(hd[o], ho[o], h);
                out[o] = orc_trace_contra_sym(h, inv);
            }
    }
}

/* ------------------------------------------------------------------ Christoffel symbols, BSSN.h:55-91 */
void orc_christoffel(const orc_cfg* c, const float* const* met, const uint32_t* const* der, int32_t seed,
                     uint32_t* const* out, const uint32_t* positions, uint32_t used, uint32_t substep,
                     uint32_t max_depth, int mode) {
    const uint32_t n = c->n;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) continue;
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                int32_t rng = cell_rng(seed, x, y, slot * n + z);
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                float d[6][3];                      /* d[k] = gradient of metric component k */
                for (int k = 0; k < 6; k++) orc_cf3_decode(der[k][o], d[k]);
                /* S_l(j,k) = (d_j g_lk + d_k g_lj) / 2 for l = x, y, z  (float3x3_sym(float3,float3,float3)) */
                const int row[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};    /* component index of g_ab */
                float S[3][6];
                for (int l = 0; l < 3; l++) {
                    const float* rx = d[row[l][0]]; const float* ry = d[row[l][1]]; const float* rz = d[row[l][2]];
                    S[l][0] = rx[0];
                    S[l][1] = (rx[1] + ry[0]) * .5f;
                    S[l][2] = (rx[2] + rz[0]) * .5f;
                    S[l][3] = ry[1];
                    S[l][4] = (rz[1] + ry[2]) * .5f;
                    S[l][5] = rz[2];
                }
                const uint64_t rw = padded_center(c, slot, x, y, z);
                float m[6], inv[6];
                for (int k = 0; k < 6; k++) m[k] = met[k][rw];
                const float* M = m;
                if (mode == 1) { orc_sym_inverse(m, inv); M = inv; }
                for (int jk = 0; jk < 6; jk++) {
                    float v[3], r[3];
                    for (int l = 0; l < 3; l++) v[l] = fmaf(-d[jk][l], .5f, S[l][jk]);
                    orc_sym_times_vec(M, v, r);
                    out[jk][o] = orc_cf3_encode(r[0], r[1], r[2], &rng, c->flags);
                }
            }
    }
}

/* ------------------------------------------------------------------ ghost fill, AMR.h:634-762 */
/* 10-point quadratic + cross-term interpolation around the nearest cell, AMR.h:672-699 */
static inline float interp10(const float* d, int64_t i, int64_t t, const float* r) {
    const int64_t t2 = t * t;
    float f = d[i], fx = d[i + 1], fy = d[i + t], fz = d[i + t2];
    float fxx = d[i - 1], fyy = d[i - t], fzz = d[i - t2];
    float fxy = d[i + t + 1], fxz = d[i + t2 + 1], fyz = d[i + t2 + t];
    fxy = fxy + ((f - fx) - fy);
    fxz = fxz + ((f - fx) - fz);
    fyz = fyz + ((f - fy) - fz);
    fx = (fx - fxx) * .5f; fy = (fy - fyy) * .5f; fz = (fz - fzz) * .5f;
    fxx = (fx + fxx) - f; fyy = (fy + fyy) - f; fzz = (fz + fzz) - f;
    /* fx is itself a (halving) product, so in `fx + fxx*rx` the device build fuses fx's exact
     * product and rounds fxx*rx: the sum below is an ordinary add of a rounded product. */
    float acc = fmaf(fx + fxx * r[0], r[0], f);
    acc = fmaf(fy + fyy * r[1], r[1], acc);
    acc = fmaf(fz + fzz * r[2], r[2], acc);
    acc = fmaf(fxy * r[0], r[1], acc);
    acc = fmaf(fxz * r[0], r[2], acc);
    acc = fmaf(fyz * r[1], r[2], acc);
    return acc;
}
/* Map a padded cell index of a domain to the (nearest-cell index, fractional offset) of a source
 * domain, AMR.h:737-753.  is_root selects the clamp that allows reading the root's ghosts. */
static inline void map_to_source(const orc_cfg* c, const uint32_t* w, float rel_scale, const float* rel_pos,
                                 int is_root, uint32_t* ri, float* r) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const float inv_n = 1.f / (float)n;
    for (int a = 0; a < 3; a++) {
        float rp = fmaf(((float)w[a] - (float)p) + .5f, inv_n, -.5f);
        rp = fmaf(rp, rel_scale, rel_pos[a]);
        rp = fmaf(rp + .5f, (float)n, (float)p) - .5f;
        uint32_t idx = is_root ? umin(f2u(fmaxf(rp, 0.f) + .5f), t - 2u)
                               : umin(f2u(fmaxf(rp, (float)p) + .5f), t - p - 2u);
        ri[a] = idx;
        r[a] = rp - (float)idx;
    }
}
/* All reads see the fields as they were before the fill: a domain next to a coarser one reads
 * the coarser domain's innermost ghost layer (the clamp keeps the index >= p, the stencil reaches
 * p-1), and that layer may be rewritten by the same fill.  The ghost values are therefore first
 * computed into a staging buffer (slot, face, layer, v, u) and written back afterwards. */
static inline void ghost_write_index(uint32_t dir, uint32_t n, uint32_t p, uint32_t layer, uint32_t u, uint32_t v,
                                     uint32_t* w) {                                           /* AMR.h:715-735 */
    switch (dir) {
        case 0: w[0] = layer + p + n; w[1] = u + p; w[2] = v + p; break;
        case 1: w[0] = u + p; w[1] = layer + p + n; w[2] = v + p; break;
        case 2: w[0] = u + p; w[1] = v + p; w[2] = layer + p + n; break;
        case 3: w[0] = layer; w[1] = u + p; w[2] = v + p; break;
        case 4: w[0] = u + p; w[1] = layer; w[2] = v + p; break;
        default: w[0] = u + p; w[1] = v + p; w[2] = layer; break;
    }
}
static inline int ghost_active(uint64_t bd, uint32_t substep, uint32_t max_depth) {
    const int32_t target = bd_target(bd);
    const int cd = bd_curr_depth(bd);
    return !(target == -1 || cd <= 0) && active_depth(substep, (uint32_t)cd, max_depth);
}
void orc_copy_boundaries(const orc_cfg* c, float* old_f, float* new_f, const uint64_t* bds, uint32_t used,
                         uint32_t substep, uint32_t max_depth, int copy_only_new) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const uint64_t cells = (uint64_t)t * t * t;
    const uint64_t face_cells = (uint64_t)p * n * n;
    float* stage = (float*)calloc((size_t)used * 6u * face_cells * 2u, sizeof(float));   /* untouched pages stay free */
    float* const src_old = old_f;
    float* const src_new = new_f;
    {
        #pragma omp parallel for schedule(dynamic)
        for (int64_t nd = 0; nd < (int64_t)used * 6; nd++) {
            const uint32_t node = (uint32_t)(nd / 6), dir = (uint32_t)(nd % 6);
            const uint64_t bd = bds[node * 6 + dir];
            const int32_t target = bd_target(bd);
            const int cd = bd_curr_depth(bd);
            if (target == -1 || cd <= 0) continue;
            if (!active_depth(substep, (uint32_t)cd, max_depth)) continue;
            const uint32_t dd = bd_depth_diff(bd);
            const float rel_scale = 1.f / (float)(1u << dd);
            float rel_pos[3];
            orc_cf3_decode((uint32_t)(bd >> 32), rel_pos);
            float tm = (float)((substep >> (max_depth - (uint32_t)cd)) & ((1u << dd) - 1u));   /* AMR.h:634-639 */
            const float t0 = tm / (float)(1u << dd), t1 = (tm + 1.f) / (float)(1u << dd);
            float* st = stage + (uint64_t)nd * face_cells * 2u;
            for (uint32_t layer = 0; layer < p; layer++)
                for (uint32_t v = 0; v < n; v++)
                    for (uint32_t u = 0; u < n; u++) {
                        uint32_t w[3];
                        ghost_write_index(dir, n, p, layer, u, v, w);
                        uint32_t ri[3]; float r[3];
                        map_to_source(c, w, rel_scale, rel_pos, target == 0, ri, r);
                        const int64_t rin = (int64_t)target * cells + ri[0] + ((int64_t)ri[1] + (int64_t)ri[2] * t) * t;
                        const float od = interp10(src_old, rin, t, r);
                        const float nw = interp10(src_new, rin, t, r);
                        const uint64_t g = ((uint64_t)layer * n + v) * n + u;
                        st[g] = fmaf(od, 1.f - t0, nw * t0);
                        st[face_cells + g] = fmaf(od, 1.f - t1, nw * t1);
                    }
        }
        /* write back once every value has been computed from the unmodified fields */
        #pragma omp parallel for schedule(dynamic)
        for (int64_t nd = 0; nd < (int64_t)used * 6; nd++) {
            const uint32_t node = (uint32_t)(nd / 6), dir = (uint32_t)(nd % 6);
            if (!ghost_active(bds[node * 6 + dir], substep, max_depth)) continue;
            const float* st = stage + (uint64_t)nd * face_cells * 2u;
            for (uint32_t layer = 0; layer < p; layer++)
                for (uint32_t v = 0; v < n; v++)
                    for (uint32_t u = 0; u < n; u++) {
                        uint32_t w[3];
                        ghost_write_index(dir, n, p, layer, u, v, w);
                        const uint64_t win = node * cells + w[0] + ((uint64_t)w[1] + (uint64_t)w[2] * t) * t;
                        const uint64_t g = ((uint64_t)layer * n + v) * n + u;
                        if (!copy_only_new) old_f[win] = st[g];
                        new_f[win] = st[face_cells + g];
                    }
        }
    }
    free(stage);
}

/* ------------------------------------------------------------------ restriction, AMR.h:961-996 */
void orc_copy_new_to_old(const orc_cfg* c, float* old_f, const float* new_f, const uint32_t* positions,
                         const int32_t* children, uint32_t used, uint32_t substep, uint32_t max_depth) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p, h = n / 2;
    const uint64_t cells = (uint64_t)t * t * t;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t sz = 0; sz < (int64_t)used * t; sz++) {
        const uint32_t slot = (uint32_t)(sz / t), z = (uint32_t)(sz % t);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) continue;
        for (uint32_t y = 0; y < t; y++)
            for (uint32_t x = 0; x < t; x++) {
                const uint32_t tx = (x - p) / h, ty = (y - p) / h, tz = (z - p) / h;   /* unsigned wrap for ghosts */
                const int32_t child = (tx < 2u && ty < 2u && tz < 2u) ? children[tx + ty * 2u + tz * 4u + slot * 8u] : -1;
                const uint64_t o = slot * cells + ((uint64_t)z * t + y) * t + x;
                if (child == -1) { old_f[o] = new_f[o]; continue; }
                const uint32_t cx = ((x - p) * 2u) % n + p, cy = ((y - p) * 2u) % n + p, cz = ((z - p) * 2u) % n + p;
                const uint64_t ci = (uint64_t)child * cells + ((uint64_t)cz * t + cy) * t + cx;
                const uint64_t t2 = (uint64_t)t * t;
                float s = new_f[ci] + new_f[ci + 1];
                s = s + new_f[ci + t]; s = s + new_f[ci + t + 1];
                s = s + new_f[ci + t2]; s = s + new_f[ci + t2 + 1];
                s = s + new_f[ci + t2 + t]; s = s + new_f[ci + t2 + t + 1];
                old_f[o] = s * .125f;
            }
    }
}

/* ------------------------------------------------------------------ prolongation, AMR.h:1053-1073 */
void orc_copy_to_child(const orc_cfg* c, float* buf, uint32_t offset, int32_t child, int32_t parent) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const uint64_t cells = (uint64_t)t * t * t;
    const float inv_n = 1.f / (float)n;
    const float off[3] = {(float)(offset & 1u), (float)((offset & 2u) >> 1), (float)((offset & 4u) >> 2)};
    #pragma omp parallel for schedule(static)
    for (int64_t zz = 0; zz < (int64_t)t; zz++) {
        const uint32_t z = (uint32_t)zz;
        for (uint32_t y = 0; y < t; y++)
            for (uint32_t x = 0; x < t; x++) {
                const uint32_t w[3] = {x, y, z};
                uint32_t ri[3]; float r[3];
                for (int a = 0; a < 3; a++) {
                    float rp = fmaf(((float)w[a] - (float)p) + .5f, inv_n, -.5f);
                    rp = fmaf(rp, .5f, (off[a] - .5f) * .5f);
                    rp = fmaf(rp + .5f, (float)n, (float)p) - .5f;
                    ri[a] = f2u(rp + .5f);
                    r[a] = rp - (float)ri[a];
                }
                const int64_t rin = (int64_t)parent * cells + ri[0] + ((int64_t)ri[1] + (int64_t)ri[2] * t) * t;
                buf[(uint64_t)child * cells + x + ((uint64_t)y + (uint64_t)z * t) * t] = interp10(buf, rin, t, r);
            }
    }
}

/* ------------------------------------------------------------------ slice rasteriser, AMR.h:1313-1352 */
/* The device build computes px / width - 0.5 (and the bounding-box threshold) as a fused
 * multiply-add with the approximate reciprocal of width; this restatement divides exactly, which is
 * the same for power-of-two widths and heights. */
void orc_rasterise(const orc_cfg* c, const float* data, const int32_t* children, uint32_t width, uint32_t height,
                   float z_slice, int boxes, float* rgba) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    #pragma omp parallel for schedule(static)
    for (int64_t yy = 0; yy < (int64_t)height; yy++) {
        const uint32_t py = (uint32_t)yy;
        for (uint32_t px = 0; px < width; px++) {
            float tp[3] = {(float)px / (float)width - .5f, (float)py / (float)height - .5f, z_slice};
            uint32_t curr = 0, depth = 0;
            uint32_t off = (uint32_t)(tp[0] > 0.f) | ((uint32_t)(tp[1] > 0.f) << 1) | ((uint32_t)(tp[2] > 0.f) << 2);
            int32_t child = children[off];
            for (; child != -1; depth++) {
                curr = (uint32_t)child;
                for (int a = 0; a < 3; a++) {       /* fracf(2 t) - 0.5, helper_math.h:1475-1478 */
                    const float v = tp[a] * 2.f;
                    tp[a] = (v - floorf(v)) - .5f;
                }
                off = (uint32_t)(tp[0] > 0.f) | ((uint32_t)(tp[1] > 0.f) << 1) | ((uint32_t)(tp[2] > 0.f) << 2);
                child = children[curr * 8u + off];
            }
            float* o = rgba + 4 * ((uint64_t)py * width + px);
            if (boxes) {                             /* DISPLAY_BOUNDING_BOXES, AMR.h:1312, 1329-1337 */
                const float threshold = .5f - 2.f * (float)(1u << depth) / (float)width;
                if (fmaxf(fabsf(tp[0]), fabsf(tp[1])) >= threshold) {
                    o[0] = 1.f; o[1] = 0.f; o[2] = 0.f; o[3] = 1.f;
                    continue;
                }
            }
            uint32_t ri[3]; float r[3];
            for (int a = 0; a < 3; a++) {           /* nearest cell, USE_LAGRANGE_POLYNOMIAL (AMR.h:4, 1340-1344) */
                const float q = fmaf(tp[a] + .5f, (float)n, (float)p);
                ri[a] = f2u(q + .5f);
                r[a] = q - (float)ri[a];
            }
            const int64_t rin = (((int64_t)curr * t + ri[2]) * t + ri[1]) * t + ri[0];
            const float v = interp10(data, rin, t, r) + .5f;
            o[0] = v; o[1] = v; o[2] = v; o[3] = 1.f;
        }
    }
}

/* ------------------------------------------------------------------ SimpleWave update, SimpleWave.h:7-46 */
void orc_wave_step(const orc_cfg* c, int corrector, const float* old_f, const uint32_t* derivs, const uint32_t* hess,
                   float* new_f, const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    const uint32_t n = c->n;
    const float visc = 0.01f;                                               /* SimpleWave.h:5 */
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) continue;
        const float dtd = (float)(1u << depth);
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                float g[3], h[3];
                orc_cf3_decode(derivs[o], g);
                orc_cf3_decode(hess[o], h);
                const float lap = fmaf(h[2], visc, fmaf(h[0], visc, h[1] * visc));
                const uint64_t rw = padded_center(c, slot, x, y, z);
                const float v = old_f[rw];
                const float upd = (fmaf(-v, g[0], lap) * c->outer_dt) / dtd;
                if (!corrector) new_f[rw] = v + upd;
                else new_f[rw] = (new_f[rw] + (v + upd)) * .5f;
            }
    }
}

/* ------------------------------------------------------------------ refinement criterion, SimpleWave.h:91-139 */
void orc_criterion(const orc_cfg* c, const uint32_t* derivs, const uint32_t* hess, float* crit,
                   const uint32_t* positions, uint32_t used, uint32_t substep, uint32_t max_depth) {
    const uint32_t n = c->n, h = n >> 1, q = n >> 2;
    for (uint32_t zi = 0; zi < 2 * used; zi++)                         /* __amr_criterion_1 */
        for (uint32_t y = 0; y < h; y++)
            for (uint32_t x = 0; x < n; x++) {
                const int depth = pos_depth(positions[zi / 2]);
                const uint64_t o = x + ((uint64_t)y + (uint64_t)zi * h) * n;
                if (depth == -1 || !active_depth(substep, (uint32_t)depth, max_depth)) { crit[o] = NAN; continue; }
                uint64_t ro = x + ((uint64_t)y + ((y >= q) ? q : 0u) + (uint64_t)zi * n * h) * n;
                float cr = 0.f;
                for (uint32_t i = 0; i < h; i++) {
                    const uint32_t w[4] = {derivs[ro], hess[ro], derivs[ro + q * n], hess[ro + q * n]};
                    for (int k = 0; k < 4; k++) {
                        float v[3];
                        orc_cf3_decode(w[k], v);
                        /* the device build takes sqrt with the hardware approximation; this one is exact */
                        const float len = sqrtf(fmaf(v[2], v[2], fmaf(v[0], v[0], v[1] * v[1])));
                        /* |g| * dx / 2^depth and |H| * dx * dx / 4^depth, left to right (SimpleWave.h:108-115) */
                        const float s = (k & 1) ? (len * c->outer_dx) * c->outer_dx / (float)(1u << (depth * 2u))
                                                : len * c->outer_dx / (float)(1u << depth);
                        cr = fmaxf(cr, s);
                    }
                    ro += (uint64_t)n * n;
                }
                crit[o] = cr;
            }
    for (uint32_t idx = 0; idx < used * 8; idx++) {                    /* __amr_criterion_2 */
        const uint32_t x = idx & 1u, y = (idx >> 1) & 1u, z = (idx >> 2) & 1u, node = idx >> 3;
        const uint64_t base = (uint64_t)node * n * n + z * (n * n >> 1) + y * (n * n >> 2) + x * h;
        float cr = NAN;
        for (uint32_t yy = 0; yy < q; yy++)
            for (uint32_t xx = 0; xx < h; xx++) cr = fmaxf(cr, crit[base + xx + (uint64_t)yy * n]);
        crit[base] = cr;
    }
}

/* ------------------------------------------------------------------ FP64 derivatives (no quantisation) */
void orc_differentiate_f64(const orc_cfg* c, const float* f, double* g3, double* hd3, double* ho3,
                           const uint32_t* positions, uint32_t used) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const int k0 = (int)(p * p + p - 1);
    /* exact-rational coefficients of the same stencils */
    static const double D1[15] = {-.5, 0, .5, 1. / 12, -2. / 3, 0, 2. / 3, -1. / 12,
                                  -1. / 60, 3. / 20, -3. / 4, 0, 3. / 4, -3. / 20, 1. / 60};
    static const double D2[15] = {1, -2, 1, -1. / 12, 4. / 3, -5. / 2, 4. / 3, -1. / 12,
                                  1. / 90, -3. / 20, 3. / 2, -49. / 18, 3. / 2, -3. / 20, 1. / 90};
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int depth = pos_depth(positions[slot]);
        if (depth == -1) continue;
        const double dx1 = (double)(1u << depth) / ((double)c->outer_size / (double)n);
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                const int64_t rw = (int64_t)padded_center(c, slot, x, y, z);
                const int64_t st[3] = {1, (int64_t)t, (int64_t)t * t};
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                for (int a = 0; a < 3; a++) {
                    double g = 0, h = 0;
                    for (int i = -(int)p; i <= (int)p; i++) {
                        g += D1[k0 + i] * f[rw + i * st[a]];
                        h += D2[k0 + i] * f[rw + i * st[a]];
                    }
                    if (g3) g3[3 * o + a] = g * dx1;
                    if (hd3) hd3[3 * o + a] = h * dx1 * dx1;
                }
                if (ho3) {
                    const int64_t pr[3][2] = {{1, t}, {1, (int64_t)t * t}, {t, (int64_t)t * t}};
                    for (int k = 0; k < 3; k++) {
                        const int64_t a = pr[k][0], b = pr[k][1];
                        ho3[3 * o + k] = .25 * ((double)f[rw + a + b] + f[rw - a - b] - f[rw + a - b] - f[rw - a + b]) * dx1 * dx1;
                    }
                }
            }
    }
}

/* ------------------------------------------------------------------ BSSN_AMR_data::timestep, BSSN.h:104-170 */
static void range_positions(const uint32_t* positions, uint32_t used, uint32_t b, uint32_t e, uint32_t* out) {
    for (uint32_t i = 0; i < used; i++) out[i] = (i >= b && i < e) ? positions[i] : ~0u;
}
void orc_bssn_timestep(const orc_cfg* c, float* const* old6, float* const* new6, uint32_t* const* dmet6,
                       uint32_t* const* chr6, float* const* ricci6, const uint32_t* positions, const int32_t* children,
                       const uint64_t* bds, uint32_t used, uint32_t max_depth, uint32_t* timer, int32_t* rng,
                       uint32_t sb, uint32_t se) {
    const uint32_t n = c->n;
    uint32_t* pos = (uint32_t*)malloc(sizeof(uint32_t) * used);
    uint64_t* bd = (uint64_t*)malloc(sizeof(uint64_t) * used * 6);
    range_positions(positions, used, sb, se, pos);
    for (uint32_t i = 0; i < used * 6; i++) bd[i] = (i / 6 >= sb && i / 6 < se) ? bds[i] : ~0ull;
    uint32_t* hd = (uint32_t*)calloc((size_t)used * n * n * n, 4);
    uint32_t* ho = (uint32_t*)calloc((size_t)used * n * n * n, 4);
    do {
        const uint32_t s = *timer;
        for (int k = 0; k < 6; k++)                                         /* copy_back, BSSN.h:126-130 */
            orc_copy_new_to_old(c, old6[k], new6[k], pos, children, used, s, max_depth);
        for (int phase = 0; phase < 2; phase++) {                           /* predictor / corrector */
            float* const* g = phase == 0 ? old6 : new6;
            for (int k = 0; k < 6; k++) {                                   /* BSSN.h:46-51 */
                const int32_t s_d = orc_prng_int(rng), s_m = orc_prng_int(rng);
                orc_differentiate(c, g[k], dmet6[k], hd, pos, used, s, max_depth, s_d);
                orc_mixed_partials(c, g[k], ho, pos, used, s, max_depth, s_m);
                orc_deriv_trace(c, hd, ho, (const float* const*)g, ricci6[k], pos, used, s, max_depth);
            }
            orc_christoffel(c, (const float* const*)g, (const uint32_t* const*)dmet6, orc_prng_int(rng), chr6,
                            pos, used, s, max_depth, 0);
            if (phase == 0)                                                 /* copy_bounds, BSSN.h:149-153 */
                for (int k = 0; k < 6; k++) orc_copy_boundaries(c, old6[k], new6[k], bd, used, s, max_depth, 1);
        }
        *timer = (*timer + 1u) & ((1u << max_depth) - 1u);                 /* AMR.h:180-188 */
    } while (*timer != 0u);
    free(pos); free(bd); free(hd); free(ho);
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}


/* ------------------------------------------------------------------ scan and reductions, parallel.h
 * Multi-pass over blocks of 512 slots.  The scan's slot t of block b at stride s is element
 * (t + 512 b + 1) s - 1; its up pass (parallel.h:10-27) adds node k - d into node k = (t+1) 2d - 1
 * for d = 1 .. 256, its down pass (parallel.h:29-60) first adds element 512 b s - 1 to the nodes
 * 2^i - 1 (i = 0..8) of blocks b > 0, then for d = 128 .. 1 adds node m = (t+1) 2d - 1 into m + d.
 * The reductions' slot t is element (t + 512 b) s; node 2td takes in node 2td + d (d = 1 .. 256)
 * and the block's result is written to its first element (parallel.h:215-237, 385-407); missing
 * elements are the lowest value (maximum) or 0 (minimum, parallel.h:389). */
enum { SCAN_POW = 9, SCAN_BLK = 1 << SCAN_POW };

typedef union { uint32_t u; int32_t i; float f; } orc_word;

/* the device's floating-point arithmetic returns one NaN, 0x7FFFFFFF, whatever the operands' */
static inline float canonical_nan(float f) { return f != f ? bitsf(0x7FFFFFFFu) : f; }
static orc_word word_add(int dtype, orc_word a, orc_word b) {
    orc_word r;
    if (dtype == 2) r.f = canonical_nan(ftz(ftz(a.f) + ftz(b.f)));
    else r.u = a.u + b.u;   /* int32 and uint32 both wrap */
    return r;
}
static orc_word word_extreme(int dtype, int is_max, orc_word a, orc_word b) {
    orc_word r;
    if (dtype == 2) {
        const float x = ftz(a.f), y = ftz(b.f);
        /* fmaxf / fminf: a NaN operand yields the other; of two zeros the maximum is +0 and the
           minimum -0 */
        if (x != x) r.f = canonical_nan(y);
        else if (y != y) r.f = x;
        else if (x == y) r.f = is_max ? (signbit(x) ? y : x) : (signbit(x) ? x : y);
        else r.f = is_max ? (x > y ? x : y) : (x < y ? x : y);
    } else if (dtype == 1) {
        r.i = is_max ? (a.i > b.i ? a.i : b.i) : (a.i < b.i ? a.i : b.i);
    } else {
        r.u = is_max ? (a.u > b.u ? a.u : b.u) : (a.u < b.u ? a.u : b.u);
    }
    return r;
}

void orc_scan(int dtype, int ncomp, void* data, uint32_t n) {
    orc_word* d = (orc_word*)data;
    static orc_word a[SCAN_BLK][4];
    uint64_t stride = 1;
    for (; stride < n; stride <<= SCAN_POW) {
        const uint64_t blocks = (n + SCAN_BLK * stride - 1) / (SCAN_BLK * stride);
        for (uint64_t b = 0; b < blocks; b++) {
            for (uint32_t t = 0; t < SCAN_BLK; t++) {
                const uint64_t i = (t + SCAN_BLK * b + 1) * stride - 1;
                for (int c = 0; c < ncomp; c++) a[t][c].u = i < n ? d[i * ncomp + c].u : 0u;
            }
            for (uint32_t dd = 1; dd < SCAN_BLK; dd <<= 1)
                for (uint32_t t = 0; t < SCAN_BLK; t++) {
                    const uint64_t k = (uint64_t)(t + 1) * 2 * dd - 1;
                    if (k < SCAN_BLK)
                        for (int c = 0; c < ncomp; c++) a[k][c] = word_add(dtype, a[k][c], a[k - dd][c]);
                }
            for (uint32_t t = 0; t < SCAN_BLK; t++) {
                const uint64_t i = (t + SCAN_BLK * b + 1) * stride - 1;
                if (i < n) for (int c = 0; c < ncomp; c++) d[i * ncomp + c] = a[t][c];
            }
        }
    }
    for (stride >>= SCAN_POW; stride > 0; stride >>= SCAN_POW) {
        const uint64_t blocks = (n + SCAN_BLK * stride - 1) / (SCAN_BLK * stride);
        /* blocks read their carry before any block of this pass writes (on the device the carry
           element is final already and rewritten unchanged) */
        for (uint64_t b = blocks; b-- > 0;) {
            for (uint32_t t = 0; t < SCAN_BLK; t++) {
                const uint64_t i = (t + SCAN_BLK * b + 1) * stride - 1;
                for (int c = 0; c < ncomp; c++) a[t][c].u = i < n ? d[i * ncomp + c].u : 0u;
            }
            if (b > 0)
                for (uint32_t t = 0; t < SCAN_BLK / 2; t = 2 * t + 1)   /* t + 1 = 1, 2, 4, ..., 256 */
                    for (int c = 0; c < ncomp; c++)
                        a[t][c] = word_add(dtype, a[t][c], d[(SCAN_BLK * b * stride - 1) * ncomp + c]);
            for (uint32_t dd = SCAN_BLK / 4; dd >= 1; dd >>= 1)
                for (uint32_t t = 0; t < SCAN_BLK; t++) {
                    const uint64_t m = (uint64_t)(t + 1) * 2 * dd - 1;
                    if (m + dd < SCAN_BLK)
                        for (int c = 0; c < ncomp; c++) a[m + dd][c] = word_add(dtype, a[m + dd][c], a[m][c]);
                }
            for (uint32_t t = 0; t < SCAN_BLK; t++) {
                const uint64_t i = (t + SCAN_BLK * b + 1) * stride - 1;
                if (i < n) for (int c = 0; c < ncomp; c++) d[i * ncomp + c] = a[t][c];
            }
        }
    }
}

void orc_extreme(int dtype, int ncomp, int is_max, void* data, uint32_t n, void* result) {
    orc_word* d = (orc_word*)data;
    static orc_word a[SCAN_BLK][4];
    orc_word pad;
    if (!is_max) pad.u = 0u;
    else if (dtype == 2) pad.f = -INFINITY;
    else if (dtype == 1) pad.i = INT32_MIN;
    else pad.u = 0u;
    for (uint64_t stride = 1; stride < n; stride <<= SCAN_POW) {
        const uint64_t blocks = (n + SCAN_BLK * stride - 1) / (SCAN_BLK * stride);
        for (uint64_t b = 0; b < blocks; b++) {
            for (uint32_t t = 0; t < SCAN_BLK; t++) {
                const uint64_t i = (t + SCAN_BLK * b) * stride;
                for (int c = 0; c < ncomp; c++) a[t][c] = i < n ? d[i * ncomp + c] : pad;
            }
            for (uint32_t dd = 1; dd < SCAN_BLK; dd <<= 1)
                for (uint32_t t = 0; t < SCAN_BLK; t++) {
                    const uint64_t k = (uint64_t)t * 2 * dd;
                    if (k < SCAN_BLK)
                        for (int c = 0; c < ncomp; c++) a[k][c] = word_extreme(dtype, is_max, a[k][c], a[k + dd][c]);
                }
            const uint64_t i0 = SCAN_BLK * b * stride;
            if (i0 < n) for (int c = 0; c < ncomp; c++) d[i0 * ncomp + c] = a[0][c];
        }
    }
    memcpy(result, d, sizeof(orc_word) * (size_t)ncomp);
}
