/* fp64_path.c -- the reference's BSSN timestep (BSSN_AMR_data::timestep, BSSN.h:104-170) in
 * double precision, with no compressed_float3 quantisation.
 *
 * TEST INFRASTRUCTURE ONLY (see amr_oracle.h): it is the FP64 host oracle against which the
 * single-precision results (this library's kernels, bit-identical to the reference's device
 * build) report their error, and the FP64 CPU stencil path the benchmark times on the host
 * cores.  Same operators and order as the single-precision restatement:
 *   copy_back    old <- new, child-covered cells <- mean of the child's 2x2x2 cells (AMR.h:961-996)
 *   predictor    per metric component: gradient, diagonal and mixed Hessian (AMR.h:1152-1266,
 *                centred (2p+1)-point and 4-point cross stencils with the edge fallback),
 *                g^kl d_k d_l g_ij (BSSN.h:7-22), then the Christoffel symbols (BSSN.h:55-91,
 *                multiplied by the metric as BSSN.h:82 does)
 *   copy_bounds  face ghosts by 10-point interpolation and linear time blend (AMR.h:634-762),
 *                every value computed from the fields before the fill
 *   corrector    the predictor's operators on new
 * Outputs per inner cell: grad[k] and chr[k] as 3 doubles, ricci[k] 1 double. */
#include "amr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int depth_of(uint32_t pos) { return (~pos) ? (int)(pos >> 27) : -1; }
static int is_active(uint32_t s, uint32_t d, uint32_t md) { return (s & ((1u << (md - d)) - 1u)) == 0u; }

static const double D1[15] = {-.5, 0, .5, 1. / 12, -2. / 3, 0, 2. / 3, -1. / 12,
                              -1. / 60, 3. / 20, -3. / 4, 0, 3. / 4, -3. / 20, 1. / 60};
static const double D2[15] = {1, -2, 1, -1. / 12, 4. / 3, -5. / 2, 4. / 3, -1. / 12,
                              1. / 90, -3. / 20, 3. / 2, -49. / 18, 3. / 2, -3. / 20, 1. / 90};

static void inverse6(const double* m, double* r) {                       /* tensors.h:208-225 */
    const double a = m[3] * m[5] - m[4] * m[4], b = m[2] * m[4] - m[1] * m[5], c = m[1] * m[4] - m[2] * m[3];
    const double det = m[0] * a + m[1] * b + m[2] * c;
    r[0] = a / det; r[1] = b / det; r[2] = c / det;
    r[3] = (m[0] * m[5] - m[2] * m[2]) / det;
    r[4] = (m[2] * m[1] - m[0] * m[4]) / det;
    r[5] = (m[0] * m[3] - m[1] * m[1]) / det;
}

static void copy_back64(const orc_cfg* c, double* old_f, const double* new_f, const uint32_t* pos,
                        const int32_t* children, uint32_t used, uint32_t s, uint32_t md) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p, h = n / 2;
    const uint64_t cells = (uint64_t)t * t * t, t2 = (uint64_t)t * t;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t sz = 0; sz < (int64_t)used * t; sz++) {
        const uint32_t slot = (uint32_t)(sz / t), z = (uint32_t)(sz % t);
        const int d = depth_of(pos[slot]);
        if (d == -1 || !is_active(s, (uint32_t)d, md)) continue;
        for (uint32_t y = 0; y < t; y++)
            for (uint32_t x = 0; x < t; x++) {
                const uint32_t tx = (x - p) / h, ty = (y - p) / h, tz = (z - p) / h;
                const int32_t ch = (tx < 2u && ty < 2u && tz < 2u) ? children[tx + ty * 2u + tz * 4u + slot * 8u] : -1;
                const uint64_t o = slot * cells + ((uint64_t)z * t + y) * t + x;
                if (ch == -1) { old_f[o] = new_f[o]; continue; }
                const uint32_t cx = ((x - p) * 2u) % n + p, cy = ((y - p) * 2u) % n + p, cz = ((z - p) * 2u) % n + p;
                const uint64_t ci = (uint64_t)ch * cells + ((uint64_t)cz * t + cy) * t + cx;
                old_f[o] = (new_f[ci] + new_f[ci + 1] + new_f[ci + t] + new_f[ci + t + 1] + new_f[ci + t2] +
                            new_f[ci + t2 + 1] + new_f[ci + t2 + t] + new_f[ci + t2 + t + 1]) * .125;
            }
    }
}

static double interp10_64(const double* d, int64_t i, int64_t t, const double* r) {   /* AMR.h:672-699 */
    const int64_t t2 = t * t;
    const double f = d[i];
    double fx = d[i + 1], fy = d[i + t], fz = d[i + t2];
    double fxx = d[i - 1], fyy = d[i - t], fzz = d[i - t2];
    const double fxy = d[i + t + 1] + f - fx - fy, fxz = d[i + t2 + 1] + f - fx - fz, fyz = d[i + t2 + t] + f - fy - fz;
    fx = (fx - fxx) * .5; fy = (fy - fyy) * .5; fz = (fz - fzz) * .5;
    fxx = fx + fxx - f; fyy = fy + fyy - f; fzz = fz + fzz - f;
    return f + (fx + fxx * r[0]) * r[0] + (fy + fyy * r[1]) * r[1] + (fz + fzz * r[2]) * r[2] + fxy * r[0] * r[1] +
           fxz * r[0] * r[2] + fyz * r[1] * r[2];
}

static void ghost64(const orc_cfg* c, double* old_f, double* new_f, const uint64_t* bds, uint32_t used, uint32_t s,
                    uint32_t md, int copy_only_new) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const uint64_t cells = (uint64_t)t * t * t, fc = (uint64_t)p * n * n;
    double* stage = (double*)calloc((size_t)used * 6u * fc * 2u, sizeof(double));
    for (int pass = 0; pass < 2; pass++) {
        #pragma omp parallel for schedule(dynamic)
        for (int64_t nd = 0; nd < (int64_t)used * 6; nd++) {
            const uint32_t node = (uint32_t)(nd / 6), dir = (uint32_t)(nd % 6);
            const uint64_t bd = bds[node * 6 + dir];
            const uint32_t w32 = (uint32_t)bd;
            const int32_t target = (int32_t)((w32 & 16777215u) | ((w32 & (1u << 23)) ? 4278190080u : 0u));
            const int cd = (w32 >> 28) == 15u ? -1 : (int)(w32 >> 28);
            if (target == -1 || cd <= 0 || !is_active(s, (uint32_t)cd, md)) continue;
            const uint32_t dd = (w32 >> 24) & 15u;
            float relf[3];
            orc_cf3_decode((uint32_t)(bd >> 32), relf);
            const double tm = (double)((s >> (md - (uint32_t)cd)) & ((1u << dd) - 1u));
            const double t0 = tm / (double)(1u << dd), t1 = (tm + 1.) / (double)(1u << dd);
            double* st = stage + (uint64_t)nd * fc * 2u;
            for (uint32_t layer = 0; layer < p; layer++)
                for (uint32_t v = 0; v < n; v++)
                    for (uint32_t u = 0; u < n; u++) {
                        uint32_t w[3];
                        switch (dir) {                                              /* AMR.h:715-735 */
                            case 0: w[0] = layer + p + n; w[1] = u + p; w[2] = v + p; break;
                            case 1: w[0] = u + p; w[1] = layer + p + n; w[2] = v + p; break;
                            case 2: w[0] = u + p; w[1] = v + p; w[2] = layer + p + n; break;
                            case 3: w[0] = layer; w[1] = u + p; w[2] = v + p; break;
                            case 4: w[0] = u + p; w[1] = layer; w[2] = v + p; break;
                            default: w[0] = u + p; w[1] = v + p; w[2] = layer; break;
                        }
                        const uint64_t g = ((uint64_t)layer * n + v) * n + u;
                        const uint64_t win = node * cells + w[0] + ((uint64_t)w[1] + (uint64_t)w[2] * t) * t;
                        if (pass == 1) {
                            if (!copy_only_new) old_f[win] = st[g];
                            new_f[win] = st[fc + g];
                            continue;
                        }
                        uint32_t ri[3];
                        double r[3];
                        for (int a = 0; a < 3; a++) {                               /* AMR.h:737-753 */
                            double rp = (((double)w[a] - p) + .5) / n - .5;
                            rp = rp / (double)(1u << dd) + relf[a];
                            rp = (rp + .5) * n + p - .5;
                            const double lo = target == 0 ? 0. : (double)p;
                            const uint32_t hi = target == 0 ? t - 2u : t - p - 2u;
                            uint32_t idx = (uint32_t)(fmax(rp, lo) + .5);
                            idx = idx < hi ? idx : hi;
                            ri[a] = idx;
                            r[a] = rp - idx;
                        }
                        const int64_t rin = (int64_t)target * cells + ri[0] + ((int64_t)ri[1] + (int64_t)ri[2] * t) * t;
                        const double od = interp10_64(old_f, rin, t, r), nw = interp10_64(new_f, rin, t, r);
                        st[g] = od * (1. - t0) + nw * t0;
                        st[fc + g] = od * (1. - t1) + nw * t1;
                    }
        }
    }
    free(stage);
}

/* Gradient, Hessian, trace and Christoffel symbols of the six components g[k] at active slots. */
static void derivs64(const orc_cfg* c, double* const* g, double* const* grad6, double* const* chr6,
                     double* const* ric6, const uint32_t* pos, uint32_t used, uint32_t s, uint32_t md) {
    const uint32_t n = c->n, p = c->p, t = n + 2 * p;
    const int k0 = (int)(p * p + p - 1);
    const int64_t st[3] = {1, (int64_t)t, (int64_t)t * t};
    #pragma omp parallel for schedule(dynamic)
    for (int64_t nz = 0; nz < (int64_t)used * n; nz++) {
        const uint32_t slot = (uint32_t)(nz / n), z = (uint32_t)(nz % n);
        const int d = depth_of(pos[slot]);
        if (d == -1 || !is_active(s, (uint32_t)d, md)) continue;
        const double dx1 = (double)(1u << d) / ((double)c->outer_size / (double)n), dx2 = dx1 * dx1;
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                const int64_t rw = (int64_t)((((uint64_t)slot * t + z + p) * t + y + p) * t + x + p);
                const uint64_t o = ((uint64_t)(slot * n + z) * n + y) * n + x;
                const int e[3] = {(int)x - (int)(x < 1u ? 1u : x > n - 2u ? n - 2u : x),
                                  (int)y - (int)(y < 1u ? 1u : y > n - 2u ? n - 2u : y),
                                  (int)z - (int)(z < 1u ? 1u : z > n - 2u ? n - 2u : z)};
                double m[6], inv[6], dg[6][3];
                for (int k = 0; k < 6; k++) m[k] = g[k][rw];
                inverse6(m, inv);
                for (int k = 0; k < 6; k++) {
                    const double* f = g[k];
                    double h[6];
                    for (int a = 0; a < 3; a++) {
                        double g1 = 0, g2 = 0;
                        for (int i = -(int)p; i <= (int)p; i++) {
                            g1 += D1[k0 + i] * f[rw + i * st[a]];
                            g2 += D2[k0 + i] * f[rw + i * st[a]];
                        }
                        dg[k][a] = g1 * dx1;
                        h[a == 0 ? 0 : a == 1 ? 3 : 5] = g2 * dx2;
                    }
                    /* mixed partials xy, xz, yz with the reference's edge rule (AMR.h:1221-1254) */
                    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}}, hi[3] = {1, 2, 4};
                    for (int q = 0; q < 3; q++) {
                        const int a = pr[q][0], b = pr[q][1];
                        const int cr = e[a] * e[b];
                        const int64_t sa = st[a], sb = st[b];
                        double v;
                        if (cr == 0) {
                            v = .25 * (f[rw + sa + sb] + f[rw - sa - sb] - f[rw + sa - sb] - f[rw - sa + sb]);
                        } else {
                            const int64_t da = -cr * sa;
                            v = -cr * (.5 * (f[rw + da + sb] + f[rw - da - sb] - f[rw - da] - f[rw + da] - f[rw - sb] -
                                              f[rw + sb]) + f[rw]);
                        }
                        h[hi[q]] = v * dx2;
                    }
                    for (int a = 0; a < 3; a++) grad6[k][3 * o + a] = dg[k][a];
                    ric6[k][o] = h[0] * inv[0] + h[3] * inv[3] + h[5] * inv[5] +
                                 2. * (h[1] * inv[1] + h[2] * inv[2] + h[4] * inv[4]);
                }
                /* Christoffel symbols, BSSN.h:72-90: S_l(j,k) = (d_j g_lk + d_k g_lj)/2, v_l = S_l(jk) - d_l g_jk / 2,
                 * multiplied by the metric (BSSN.h:82) */
                static const int row[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
                static const int jk_a[6] = {0, 0, 0, 1, 1, 2}, jk_b[6] = {0, 1, 2, 1, 2, 2};
                for (int jk = 0; jk < 6; jk++) {
                    const int j = jk_a[jk], kk = jk_b[jk];
                    double v[3];
                    for (int l = 0; l < 3; l++)
                        v[l] = .5 * (dg[row[l][kk]][j] + dg[row[l][j]][kk]) - .5 * dg[jk][l];
                    chr6[jk][3 * o + 0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
                    chr6[jk][3 * o + 1] = m[1] * v[0] + m[3] * v[1] + m[4] * v[2];
                    chr6[jk][3 * o + 2] = m[2] * v[0] + m[4] * v[1] + m[5] * v[2];
                }
            }
    }
}

void orc_bssn_timestep_f64(const orc_cfg* c, double* const* old6, double* const* new6, double* const* grad6,
                           double* const* chr6, double* const* ric6, const uint32_t* pos, const int32_t* children,
                           const uint64_t* bds, uint32_t used, uint32_t max_depth, uint32_t* timer) {
    do {
        const uint32_t s = *timer;
        for (int k = 0; k < 6; k++) copy_back64(c, old6[k], new6[k], pos, children, used, s, max_depth);
        derivs64(c, old6, grad6, chr6, ric6, pos, used, s, max_depth);
        for (int k = 0; k < 6; k++) ghost64(c, old6[k], new6[k], bds, used, s, max_depth, 1);
        derivs64(c, new6, grad6, chr6, ric6, pos, used, s, max_depth);
        *timer = (*timer + 1u) & ((1u << max_depth) - 1u);
    } while (*timer != 0u);
}
