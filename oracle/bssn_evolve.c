/* bssn_evolve.c -- FP64 restatement of the evolution (adaptivemesh_gb300/csrc/evolve.h): the full
 * BSSN system in moving-puncture form and the scalar wave u_tt = Δu, RK4 on the octree of domains
 * with the reference's 2:1 subcycling counter (AMR.h:180-188, 634-644), restriction
 * (AMR.h:961-996) and ghost fill with space / time interpolation (AMR.h:701-762), extended to edges
 * and corners by three axis passes and, from coarser neighbours, with tricubic instead of the
 * reference's 10-point quadratic interpolation (AMR.h:672-699): second-derivative stencils amplify an
 * O(h^3) ghost error into an O(h) one.
 *
 * TEST INFRASTRUCTURE ONLY (see amr_oracle.h).  The reference has no evolution of its own to pin this
 * against ("parity unpinned by the reference"): this file is the FP64 host oracle the GPU's FP32
 * evolution is held to, written from the equations (Baumgarte & Shapiro; Campanelli et al. 2006,
 * Baker et al. 2006 for the puncture gauge; Alcubierre et al. 2004 for the gauge wave), and checked
 * on its own by convergence of the constraints on exact solutions.  State arrays are padded slots
 * (slot*t^3 + (z*t + y)*t + x), one double array per field.
 */
#include "amr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { NF_BSSN = 24, NF_WAVE = 2 };
enum { CHI = 0, GXX = 1, KK = 7, AXX = 8, GAMX = 14, ALPHA = 17, BETAX = 18, BX = 21 };

static int depth_of(uint32_t pos) { return (~pos) ? (int)(pos >> 27) : -1; }
static int is_active(uint32_t s, uint32_t d, uint32_t md) { return (s & ((1u << (md - d)) - 1u)) == 0u; }
static int S6(int i, int j) {
    const int a = i < j ? i : j, b = i < j ? j : i;
    return a == 0 ? b : (a == 1 ? 2 + b : 5);
}

/* ------------------------------------------------------------------ initial data */
static void initial_values(const orc_evo* e, const double* x, double* u) {
    if (e->physics != 0) {
        const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
        u[0] = e->id_kind == 3 ? exp(-r2 / ((double)e->width * e->width)) : 0.0;
        u[1] = 0.0;
        return;
    }
    for (int f = 0; f < NF_BSSN; f++) u[f] = 0.0;
    u[CHI] = 1; u[GXX] = u[GXX + 3] = u[GXX + 5] = 1; u[ALPHA] = 1;
    if (e->id_kind == 1) {   /* gauge wave at t = 0 */
        const double k = 6.283185307179586476925 / e->wavelength, A = e->amplitude;
        const double H = 1.0 - A * sin(k * x[0]), dH = -A * k * cos(k * x[0]);
        const double Kxx = -0.5 * A * k * cos(k * x[0]) / sqrt(H);
        const double chi = pow(H, -1.0 / 3.0), K = Kxx / H;
        u[CHI] = chi;
        u[GXX] = chi * H; u[GXX + 3] = u[GXX + 5] = chi;
        u[KK] = K;
        u[AXX] = chi * (Kxx - H * K / 3.0);
        u[AXX + 3] = u[AXX + 5] = -chi * K / 3.0;
        u[GAMX] = (2.0 / 3.0) * dH * pow(H, -5.0 / 3.0);
        u[ALPHA] = sqrt(H);
    } else if (e->id_kind == 2) {   /* Brill-Lindquist */
        double psi = 1.0;
        for (int a = 0; a < e->n_punctures; a++) {
            const double dx = x[0] - e->pos[a][0], dy = x[1] - e->pos[a][1], dz = x[2] - e->pos[a][2];
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r < 1e-6) r = 1e-6;
            psi += e->mass[a] / (2.0 * r);
        }
        u[CHI] = pow(psi, -4.0);
        u[ALPHA] = pow(psi, -2.0);
    }
}

static void centre_of(uint32_t pos, double* c) {
    const int d = depth_of(pos);
    uint32_t path = pos & 134217727u;
    double step = 0.25;
    c[0] = c[1] = c[2] = 0;
    for (int i = 0; i < d; i++, path >>= 3, step *= 0.5)
        for (int a = 0; a < 3; a++) c[a] += (path & (1u << a)) ? step : -step;
}

void orc_evo_initial_data(const orc_evo* e, double* const* fields, const uint32_t* positions, uint32_t used) {
    const uint32_t n = e->n, t = n + 2 * e->p;
    const int nf = e->physics == 0 ? NF_BSSN : NF_WAVE;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t sz = 0; sz < (int64_t)used * t; sz++) {
        const uint32_t slot = (uint32_t)(sz / t), z = (uint32_t)(sz % t);
        const int d = depth_of(positions[slot]);
        if (d == -1) continue;
        double c[3], u[NF_BSSN];
        centre_of(positions[slot], c);
        const double h = (double)e->outer_size / ((double)n * (double)(1u << d));
        for (uint32_t y = 0; y < t; y++)
            for (uint32_t xx = 0; xx < t; xx++) {
                const uint32_t idx[3] = {xx, y, z};
                double x[3];
                for (int k = 0; k < 3; k++) x[k] = c[k] * e->outer_size + ((double)idx[k] + 0.5 - 0.5 * t) * h;
                initial_values(e, x, u);
                const uint64_t o = (((uint64_t)slot * t + z) * t + y) * t + xx;
                for (int f = 0; f < nf; f++) fields[f][o] = u[f];
            }
    }
}

/* ------------------------------------------------------------------ derivatives at one cell */
typedef struct {
    double d1[NF_BSSN][3];    /* first derivatives of every field */
    double d2[NF_BSSN][3][3]; /* second derivatives (chi, gt, alpha, beta only) */
    double extra[NF_BSSN];    /* advection + Kreiss-Oliger */
} cell_derivs;

static void derivs_at(const orc_evo* e, double* const* f, uint64_t o, double h, int nf, cell_derivs* D) {
    const uint32_t t = e->n + 2 * e->p;
    const int64_t st[3] = {1, (int64_t)t, (int64_t)t * t};
    const double w1[4] = {1, -8, 8, -1};
    const int off[4] = {-2, -1, 1, 2};
    const int bssn = e->physics == 0;
    double beta[3] = {0, 0, 0};
    if (bssn)
        for (int k = 0; k < 3; k++) beta[k] = f[BETAX + k][o];
    for (int q = 0; q < nf; q++) {
        const double* u = f[q];
        double ko = 0;
        for (int a = 0; a < 3; a++) {
            const int64_t s = st[a];
            D->d1[q][a] = (u[o - 2 * s] - 8 * u[o - s] + 8 * u[o + s] - u[o + 2 * s]) / (12 * h);
            D->d2[q][a][a] = (-u[o - 2 * s] + 16 * u[o - s] - 30 * u[o] + 16 * u[o + s] - u[o + 2 * s]) / (12 * h * h);
            ko += u[o - 3 * s] - 6 * u[o - 2 * s] + 15 * u[o - s] - 20 * u[o] + 15 * u[o + s] - 6 * u[o + 2 * s] +
                  u[o + 3 * s];
        }
        for (int a = 0; a < 3; a++)
            for (int b = a + 1; b < 3; b++) {
                double acc = 0;
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) acc += w1[i] * w1[j] * u[o + off[i] * st[a] + off[j] * st[b]];
                D->d2[q][a][b] = D->d2[q][b][a] = acc / (144 * h * h);
            }
        double ex = e->ko_sigma / (64 * h) * ko;
        if (bssn) {
            ex += beta[0] * D->d1[q][0] + beta[1] * D->d1[q][1] + beta[2] * D->d1[q][2];
            if (!e->shift && q >= BETAX) ex = 0;
        }
        D->extra[q] = ex;
    }
}

/* ------------------------------------------------------------------ BSSN pieces */
typedef struct {
    double chi, ichi, g[3][3], gi[3][3], cl[3][3][3], cu[3][3][3], gd[3], R[3][3];
} geom;

static void geometry(const orc_evo* e, const double* u, const cell_derivs* D, geom* G) {
    G->chi = u[CHI];
    G->ichi = 1.0 / (u[CHI] > e->chi_floor ? u[CHI] : e->chi_floor);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) G->g[i][j] = u[GXX + S6(i, j)];
    double (*g)[3] = G->g;
    const double det = g[0][0] * (g[1][1] * g[2][2] - g[1][2] * g[2][1]) - g[0][1] * (g[1][0] * g[2][2] - g[1][2] * g[2][0]) +
                       g[0][2] * (g[1][0] * g[2][1] - g[1][1] * g[2][0]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const int i1 = (j + 1) % 3, i2 = (j + 2) % 3, j1 = (i + 1) % 3, j2 = (i + 2) % 3;
            G->gi[i][j] = (g[i1][j1] * g[i2][j2] - g[i1][j2] * g[i2][j1]) / det;
        }
    /* Gt_ijk = (d_j g_ik + d_k g_ij - d_i g_jk) / 2 */
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                G->cl[i][j][k] = 0.5 * (D->d1[GXX + S6(i, k)][j] + D->d1[GXX + S6(i, j)][k] - D->d1[GXX + S6(j, k)][i]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                double s = 0;
                for (int l = 0; l < 3; l++) s += G->gi[i][l] * G->cl[l][j][k];
                G->cu[i][j][k] = s;
            }
    for (int i = 0; i < 3; i++) {
        double s = 0;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) s += G->gi[j][k] * G->cu[i][j][k];
        G->gd[i] = s;
    }
    const double* dchi = D->d1[CHI];
    double ddchi[3][3], trdd = 0, dchi2 = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double v = D->d2[CHI][i][j];
            for (int k = 0; k < 3; k++) v -= G->cu[k][i][j] * dchi[k];
            ddchi[i][j] = v;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            trdd += G->gi[i][j] * ddchi[i][j];
            dchi2 += G->gi[i][j] * dchi[i] * dchi[j];
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double r = 0;
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++) r -= 0.5 * G->gi[l][m] * D->d2[GXX + S6(i, j)][l][m];
            for (int k = 0; k < 3; k++) r += 0.5 * (G->g[k][i] * D->d1[GAMX + k][j] + G->g[k][j] * D->d1[GAMX + k][i]);
            for (int k = 0; k < 3; k++) r += 0.5 * G->gd[k] * (G->cl[i][j][k] + G->cl[j][i][k]);
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++)
                    for (int k = 0; k < 3; k++)
                        r += G->gi[l][m] * (G->cu[k][l][i] * G->cl[j][k][m] + G->cu[k][l][j] * G->cl[i][k][m] +
                                            G->cu[k][i][m] * G->cl[k][l][j]);
            r += 0.5 * G->ichi * (ddchi[i][j] + G->g[i][j] * trdd) -
                 0.25 * G->ichi * G->ichi * (dchi[i] * dchi[j] + 3 * G->g[i][j] * dchi2);
            G->R[i][j] = r;
        }
}

static void bssn_rhs(const orc_evo* e, const double* u, const cell_derivs* D, double* rhs) {
    geom G;
    geometry(e, u, D, &G);
    const double K = u[KK], al = u[ALPHA];
    double A[3][3], Aud[3][3], Auu[3][3], AA = 0, db[3][3], divb = 0, dda[3][3], lap = 0, cd = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { A[i][j] = u[AXX + S6(i, j)]; db[i][j] = D->d1[BETAX + i][j]; }
    for (int k = 0; k < 3; k++) divb += db[k][k];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += G.gi[i][k] * A[k][j];
            Aud[i][j] = s;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += Aud[i][k] * G.gi[k][j];
            Auu[i][j] = s;
            AA += A[i][j] * s;
        }
    const double* dal = D->d1[ALPHA];
    const double* dchi = D->d1[CHI];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) cd += G.gi[k][l] * dchi[k] * dal[l];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double v = D->d2[ALPHA][i][j];
            for (int k = 0; k < 3; k++) v -= G.cu[k][i][j] * dal[k];
            v += 0.5 * G.ichi * (dchi[i] * dal[j] + dchi[j] * dal[i] - G.g[i][j] * cd);
            dda[i][j] = v;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) lap += G.gi[i][j] * dda[i][j];
    lap *= G.chi;
    rhs[CHI] = (2.0 / 3.0) * G.chi * (al * K - divb);
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            double v = -2 * al * A[i][j] - (2.0 / 3.0) * G.g[i][j] * divb;
            for (int k = 0; k < 3; k++) v += G.g[i][k] * db[k][j] + G.g[j][k] * db[k][i];
            rhs[GXX + S6(i, j)] = v;
        }
    rhs[KK] = -lap + al * (AA + K * K / 3.0);
    double X[3][3], trX = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) X[i][j] = -dda[i][j] + al * G.R[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) trX += G.gi[i][j] * X[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            double v = G.chi * (X[i][j] - G.g[i][j] * trX / 3.0);
            double aa = 0;
            for (int k = 0; k < 3; k++) aa += A[i][k] * Aud[k][j];
            v += al * (K * A[i][j] - 2 * aa) - (2.0 / 3.0) * A[i][j] * divb;
            for (int k = 0; k < 3; k++) v += A[i][k] * db[k][j] + A[j][k] * db[k][i];
            rhs[AXX + S6(i, j)] = v;
        }
    double core[3];
    for (int i = 0; i < 3; i++) {
        double v = (2.0 / 3.0) * u[GAMX + i] * divb, s1 = 0, s2 = 0, s3 = 0;
        for (int k = 0; k < 3; k++) v -= u[GAMX + k] * db[i][k];
        for (int j = 0; j < 3; j++) {
            double dd = 0;
            for (int k = 0; k < 3; k++) {
                v += G.gi[j][k] * D->d2[BETAX + i][j][k];
                dd += D->d2[BETAX + k][j][k];
                s1 += G.cu[i][j][k] * Auu[j][k];
            }
            v += G.gi[i][j] * dd / 3.0 - 2 * Auu[i][j] * dal[j];
            s2 += Auu[i][j] * dchi[j];
            s3 += G.gi[i][j] * D->d1[KK][j];
        }
        v += 2 * al * (s1 - 1.5 * s2 * G.ichi - (2.0 / 3.0) * s3);
        core[i] = v;
        rhs[GAMX + i] = v;
    }
    rhs[ALPHA] = e->slicing == 1 ? -al * al * K : -2 * al * K;
    for (int i = 0; i < 3; i++) {
        rhs[BETAX + i] = e->shift ? 0.75 * u[BX + i] : 0;
        rhs[BX + i] = e->shift ? core[i] - e->eta * u[BX + i] : 0;
    }
}

static void bssn_constraints(const orc_evo* e, const double* u, const cell_derivs* D, double* hm) {
    geom G;
    geometry(e, u, D, &G);
    double A[3][3], Aud[3][3], Auu[3][3], AA = 0, trR = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A[i][j] = u[AXX + S6(i, j)];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += G.gi[i][k] * A[k][j];
            Aud[i][j] = s;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += Aud[i][k] * G.gi[k][j];
            Auu[i][j] = s;
            AA += A[i][j] * s;
            trR += G.gi[i][j] * G.R[i][j];
        }
    hm[0] = G.chi * trR + (2.0 / 3.0) * u[KK] * u[KK] - AA;
    for (int i = 0; i < 3; i++) {
        double v = -(2.0 / 3.0) * D->d1[KK][i];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                v += G.gi[j][k] * D->d1[AXX + S6(k, i)][j];
                double s = 0;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) s += G.gi[j][a] * G.gi[k][b] * D->d1[GXX + S6(a, b)][j];
                v -= s * A[k][i];
                v -= 0.5 * Auu[j][k] * D->d1[GXX + S6(j, k)][i];
            }
        for (int l = 0; l < 3; l++) v -= 1.5 * Aud[l][i] * D->d1[CHI][l] * G.ichi;
        hm[1 + i] = v;
    }
}

/* ------------------------------------------------------------------ ghost fill of one axis pass */
static void ghost_pass(const orc_evo* e, double* const* X, double* const* oldf, double* const* newf, const uint64_t* bds,
                       const uint8_t* evolved, const uint32_t* items, uint32_t n_items, uint32_t s, uint32_t md, int d,
                       double c_stage, int nf) {
    const uint32_t n = e->n, p = e->p, t = n + 2 * p;
    const uint64_t cells = (uint64_t)t * t * t;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t it = 0; it < (int64_t)n_items * 2; it++) {
        const uint32_t slot = items[it / 2], side = (uint32_t)(it % 2), face = (uint32_t)d + 3u * side;
        const uint64_t bd = bds[(uint64_t)slot * 6 + face];
        const uint32_t w32 = (uint32_t)bd;
        const int32_t src = (int32_t)((w32 & 16777215u) | ((w32 & (1u << 23)) ? 4278190080u : 0u));
        const int cd = (w32 >> 28) == 15u ? -1 : (int)(w32 >> 28);
        if (src == -1 || cd <= 0) continue;
        const uint32_t dd = (w32 >> 24) & 15u;
        const int sd = cd - (int)dd;
        int mode;
        double frac = 0;
        if (!evolved[src]) mode = 0;
        else if (is_active(s, (uint32_t)sd, md)) { mode = dd == 0 ? 1 : 2; frac = 1.0 / (double)(1u << dd); }
        else {
            mode = 3;
            const uint32_t kp = (s >> (md - (uint32_t)cd)) & ((1u << dd) - 1u);
            frac = ((double)kp + c_stage) / (double)(1u << dd);
        }
        float relf[3];
        orc_cf3_decode((uint32_t)(bd >> 32), relf);
        const double rel_scale = 1.0 / (double)(1u << dd);
        uint32_t lo[3], ext[3];
        for (int a = 0; a < 3; a++) {
            if (a == d) { lo[a] = side == 0 ? p + n : 0; ext[a] = p; }
            else if (a < d) { lo[a] = 0; ext[a] = t; }
            else { lo[a] = p; ext[a] = n; }
        }
        for (uint32_t k = 0; k < ext[0] * ext[1] * ext[2]; k++) {
            const uint32_t w[3] = {lo[0] + k % ext[0], lo[1] + (k / ext[0]) % ext[1], lo[2] + k / (ext[0] * ext[1])};
            const uint64_t dst = slot * cells + ((uint64_t)w[2] * t + w[1]) * t + w[0];
            int64_t idx[3];
            double wgt[3][4];
            for (int a = 0; a < 3; a++) {
                double rp = (((double)w[a] - p) + 0.5) / n - 0.5;
                rp = rp * rel_scale + relf[a];
                const double ri = (rp + 0.5) * n + p - 0.5;
                if (dd == 0) { idx[a] = (int64_t)llround(ri); continue; }
                /* cubic Lagrange through cells b-1 .. b+2 (b = floor(ri)), kept inside the cells that are
                 * valid: the interior along the normal axis and the later axes, the whole padded range
                 * along the earlier axes (filled by earlier passes) and everywhere in the root (its
                 * frozen ghost layer is the outer boundary) */
                const int64_t lc = (src == 0 || a < d) ? 1 : (int64_t)p + 1;
                const int64_t hc = (src == 0 || a < d) ? (int64_t)t - 3 : (int64_t)(t - p) - 3;
                int64_t b = (int64_t)floor(ri);
                b = b < lc ? lc : (b > hc ? hc : b);
                const double x = ri - (double)b;
                idx[a] = b;
                wgt[a][0] = -x * (x - 1) * (x - 2) / 6;
                wgt[a][1] = (x + 1) * (x - 1) * (x - 2) / 2;
                wgt[a][2] = -(x + 1) * x * (x - 2) / 2;
                wgt[a][3] = (x + 1) * x * (x - 1) / 6;
            }
            const int64_t si = (int64_t)src * (int64_t)cells + (idx[2] * t + idx[1]) * t + idx[0];
            for (int f = 0; f < nf; f++) {
                const double* A0 = oldf[f];
                const double* A1 = mode == 3 ? newf[f] : X[f];
                double va = 0, vb = 0;
                if (dd == 0) { va = A0[si]; vb = A1[si]; }
                else
                    for (int k2 = 0; k2 < 4; k2++)
                        for (int k1 = 0; k1 < 4; k1++)
                            for (int k0 = 0; k0 < 4; k0++) {
                                const double wk = wgt[0][k0] * wgt[1][k1] * wgt[2][k2];
                                const int64_t q = si + ((int64_t)(k2 - 1) * t + (k1 - 1)) * t + (k0 - 1);
                                va += wk * A0[q];
                                if (mode != 0) vb += wk * A1[q];
                            }
                X[f][dst] = mode == 0 ? va : (mode == 1 ? vb : (1 - frac) * va + frac * vb);
            }
        }
    }
}

/* ------------------------------------------------------------------ restriction: old <- new; a cell covered by
 * a child <- the child's new field interpolated at the cell's centre (the corner shared by 2x2x2 child
 * cells) with the 4-point midpoint rule (-1, 9, 9, -1)/16 along each axis, which reads one child cell
 * beyond the 2x2x2 block on each side (the child's ghost layer at its faces).  The reference averages
 * the 2x2x2 block (AMR.h:961-996), a second-order rule whose error the coarse domain's second
 * derivatives amplify. */
static void restrict_all(const orc_evo* e, double* const* oldf, double* const* newf, const uint32_t* pos,
                         const int32_t* children, const uint32_t* items, uint32_t n_items, int nf) {
    const uint32_t n = e->n, p = e->p, t = n + 2 * p, h = n / 2;
    const uint64_t cells = (uint64_t)t * t * t;
    static const double w4[4] = {-1.0 / 16, 9.0 / 16, 9.0 / 16, -1.0 / 16};
    (void)pos;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t iz = 0; iz < (int64_t)n_items * t; iz++) {
        const uint32_t slot = items[iz / t], z = (uint32_t)(iz % t);
        for (uint32_t y = 0; y < t; y++)
            for (uint32_t x = 0; x < t; x++) {
                const uint32_t tx = (x - p) / h, ty = (y - p) / h, tz = (z - p) / h;
                const int32_t ch = (tx < 2u && ty < 2u && tz < 2u) ? children[tx + ty * 2u + tz * 4u + slot * 8u] : -1;
                const uint64_t o = slot * cells + ((uint64_t)z * t + y) * t + x;
                if (ch == -1) {
                    for (int f = 0; f < nf; f++) oldf[f][o] = newf[f][o];
                    continue;
                }
                /* child cells 2c-1 .. 2c+2 (c the coarse cell's index inside the child's half) */
                const uint32_t cx = ((x - p) * 2u) % n + p, cy = ((y - p) * 2u) % n + p, cz = ((z - p) * 2u) % n + p;
                const uint64_t base = (uint64_t)ch * cells + ((uint64_t)(cz - 1) * t + (cy - 1)) * t + (cx - 1);
                for (int f = 0; f < nf; f++) {
                    const double* v = newf[f];
                    double acc = 0;
                    for (int k2 = 0; k2 < 4; k2++)
                        for (int k1 = 0; k1 < 4; k1++)
                            for (int k0 = 0; k0 < 4; k0++)
                                acc += w4[k0] * w4[k1] * w4[k2] * v[base + ((uint64_t)k2 * t + k1) * t + k0];
                    oldf[f][o] = acc;
                }
            }
    }
}

/* ------------------------------------------------------------------ RK4 stage over the listed slots */
static void rk_stage(const orc_evo* e, double* const* in, double* const* out, double* const* oldf, double* const* acc,
                     const uint32_t* pos, const uint32_t* items, uint32_t n_items, int stage, int nf) {
    const uint32_t n = e->n, p = e->p, t = n + 2 * p;
    #pragma omp parallel for schedule(dynamic)
    for (int64_t iz = 0; iz < (int64_t)n_items * n; iz++) {
        const uint32_t slot = items[iz / n], z = (uint32_t)(iz % n);
        const int depth = depth_of(pos[slot]);
        const double h = (double)e->outer_size / ((double)n * (double)(1u << depth));
        const double dt = (double)e->cfl * e->outer_size / n / (double)(1u << depth);
        cell_derivs D;
        double u[NF_BSSN], rhs[NF_BSSN];
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t x = 0; x < n; x++) {
                const uint64_t o = (((uint64_t)slot * t + z + p) * t + y + p) * t + x + p;
                const uint64_t ii = (((uint64_t)slot * n + z) * n + y) * n + x;
                derivs_at(e, in, o, h, nf, &D);
                for (int f = 0; f < nf; f++) u[f] = in[f][o];
                if (e->physics == 0) bssn_rhs(e, u, &D, rhs);
                else { rhs[0] = u[1]; rhs[1] = D.d2[0][0][0] + D.d2[0][1][1] + D.d2[0][2][2]; }
                for (int f = 0; f < nf; f++) {
                    const double r = rhs[f] + D.extra[f];
                    const double uo = oldf[f][o];
                    switch (stage) {
                        case 1: acc[f][ii] = uo + dt / 6 * r; out[f][o] = uo + dt / 2 * r; break;
                        case 2: acc[f][ii] += dt / 3 * r; out[f][o] = uo + dt / 2 * r; break;
                        case 3: acc[f][ii] += dt / 3 * r; out[f][o] = uo + dt * r; break;
                        default: out[f][o] = acc[f][ii] + dt / 6 * r; break;
                    }
                    /* the conformal factor is kept at or above its floor (a NaN stays a NaN) */
                    if (e->physics == 0 && f == CHI && out[f][o] < e->chi_floor) out[f][o] = e->chi_floor;
                }
            }
    }
}

/* ------------------------------------------------------------------ one timestep (every substep until the
 * counter wraps), as the GPU's amr_sim_timestep on an evolution simulation */
void orc_evo_timestep(const orc_evo* e, double* const* oldf, double* const* newf, double* const* stagef,
                      double* const* acc, const uint32_t* pos, const int32_t* children, const uint64_t* bds,
                      uint32_t used, uint32_t max_depth, uint32_t* timer) {
    const int nf = e->physics == 0 ? NF_BSSN : NF_WAVE;
    uint8_t* evolved = (uint8_t*)calloc(used, 1);
    uint32_t* act = (uint32_t*)malloc(sizeof(uint32_t) * used);
    uint32_t* evo = (uint32_t*)malloc(sizeof(uint32_t) * used);
    /* every live domain is evolved, covered parents included: a leaf beside a covered parent of its
     * own depth takes its ghost values from it at every stage (the parent's values are replaced by
     * its children's at each restriction) */
    for (uint32_t i = 0; i < used; i++) evolved[i] = depth_of(pos[i]) != -1;
    do {
        const uint32_t s = *timer;
        uint32_t na = 0, ne = 0;
        for (uint32_t i = 0; i < used; i++) {
            const int d = depth_of(pos[i]);
            if (d == -1 || !is_active(s, (uint32_t)d, max_depth)) continue;
            act[na++] = i;
            if (evolved[i]) evo[ne++] = i;
        }
        restrict_all(e, oldf, newf, pos, children, act, na, nf);
        double* const* in[4] = {oldf, stagef, newf, stagef};
        double* const* out[4] = {stagef, newf, stagef, newf};
        const double cst[4] = {0.5, 0.5, 1.0, 1.0};
        for (int stage = 1; stage <= 4; stage++) {
            rk_stage(e, in[stage - 1], out[stage - 1], oldf, acc, pos, evo, ne, stage, nf);
            for (int d = 0; d < 3; d++)
                ghost_pass(e, out[stage - 1], oldf, newf, bds, evolved, evo, ne, s, max_depth, d, cst[stage - 1], nf);
        }
        *timer = (*timer + 1u) & ((1u << max_depth) - 1u);
    } while (*timer != 0u);
    free(evolved); free(act); free(evo);
}

/* Hamiltonian and momentum constraints of `fields` on every live slot; norms over the composite grid
 * (every interior cell that no child covers), leaving out cells closer than `excision` to a puncture:
 * out5 = rms H, max |H|, rms |M|, max |M|, cells.  cons4 (optional): H, M_x, M_y, M_z per inner cell. */
void orc_evo_constraints(const orc_evo* e, double* const* fields, const uint32_t* pos, const int32_t* children,
                         uint32_t used, double excision, double* const* cons4, double* out5) {
    const uint32_t n = e->n, p = e->p, t = n + 2 * p, hn = n / 2;
    double sh = 0, mh = 0, sm = 0, mm = 0, cells = 0;
    for (uint32_t slot = 0; slot < used; slot++) {
        const int depth = depth_of(pos[slot]);
        if (depth == -1) continue;
        const double h = (double)e->outer_size / ((double)n * (double)(1u << depth));
        double c[3];
        centre_of(pos[slot], c);
        #pragma omp parallel for reduction(+ : sh, sm, cells) reduction(max : mh, mm) schedule(dynamic)
        for (int64_t zz = 0; zz < (int64_t)n; zz++) {
            cell_derivs D;
            double u[NF_BSSN], hm[4];
            for (uint32_t y = 0; y < n; y++)
                for (uint32_t x = 0; x < n; x++) {
                    const uint64_t o = (((uint64_t)slot * t + zz + p) * t + y + p) * t + x + p;
                    const uint64_t ii = (((uint64_t)slot * n + zz) * n + y) * n + x;
                    derivs_at(e, fields, o, h, NF_BSSN, &D);
                    for (int f = 0; f < NF_BSSN; f++) u[f] = fields[f][o];
                    bssn_constraints(e, u, &D, hm);
                    if (cons4)
                        for (int k = 0; k < 4; k++) cons4[k][ii] = hm[k];
                    const uint32_t oct = (x / hn) | ((y / hn) << 1) | (((uint32_t)zz / hn) << 2);
                    if (children[slot * 8 + oct] != -1) continue;
                    const double X[3] = {c[0] * e->outer_size + (x + 0.5 - 0.5 * n) * h,
                                         c[1] * e->outer_size + (y + 0.5 - 0.5 * n) * h,
                                         c[2] * e->outer_size + (zz + 0.5 - 0.5 * n) * h};
                    int excised = 0;
                    for (int a = 0; a < e->n_punctures && excision > 0; a++) {
                        const double dx = X[0] - e->pos[a][0], dy = X[1] - e->pos[a][1], dz = X[2] - e->pos[a][2];
                        excised |= dx * dx + dy * dy + dz * dz < excision * excision;
                    }
                    if (excised) continue;
                    const double m2 = hm[1] * hm[1] + hm[2] * hm[2] + hm[3] * hm[3];
                    sh += hm[0] * hm[0];
                    sm += m2;
                    cells += 1;
                    if (fabs(hm[0]) > mh) mh = fabs(hm[0]);
                    if (sqrt(m2) > mm) mm = sqrt(m2);
                }
        }
    }
    out5[0] = cells ? sqrt(sh / cells) : 0;
    out5[1] = mh;
    out5[2] = cells ? sqrt(sm / cells) : 0;
    out5[3] = mm;
    out5[4] = cells;
}

/* ------------------------------------------------------------------ periodic face boundaries
 * Boundary words (AMR.h:56-100 layout: target | depth difference << 24 | depth << 28 | offset << 32)
 * of a periodic root: the neighbour one domain away along the face normal, coordinates taken modulo
 * the root, found by descending from the root to at most the domain's own depth (as AMR.h:255-263
 * does), with the offset of this domain's centre from the neighbour's (in neighbour edges) as if the
 * neighbour lay beside it.  Computed from integer cell coordinates, independently of the octree
 * code it checks. */
static void coords_of(uint32_t pos, uint32_t* ic) {
    const int d = depth_of(pos);
    uint32_t path = pos & 134217727u;
    ic[0] = ic[1] = ic[2] = 0;
    for (int i = 0; i < d; i++, path >>= 3)
        for (int a = 0; a < 3; a++) ic[a] = (ic[a] << 1) | ((path >> a) & 1u);
}
void orc_periodic_boundaries(const uint32_t* positions, const int32_t* children, uint32_t used, uint64_t* out) {
    for (uint32_t node = 0; node < used; node++) {
        for (int face = 0; face < 6; face++) out[(uint64_t)node * 6 + face] = 0xFFFFFFFFull;
        const int d = depth_of(positions[node]);
        if (d <= 0) continue;
        uint32_t ic[3];
        coords_of(positions[node], ic);
        for (int face = 0; face < 6; face++) {
            const int axis = face % 3, dir = face < 3 ? 1 : -1;
            int64_t jc[3] = {ic[0], ic[1], ic[2]};
            jc[axis] += dir;
            const int64_t side = (int64_t)1 << d;
            const int wrapped = jc[axis] < 0 || jc[axis] >= side;
            jc[axis] = (jc[axis] % side + side) % side;
            /* descend: at level i the child octant is made of bit (d-1-i) of each coordinate */
            uint32_t cur = 0;
            int od = 0;
            for (int i = 0; i < d; i++) {
                const uint32_t oct = (uint32_t)(((jc[0] >> (d - 1 - i)) & 1) | (((jc[1] >> (d - 1 - i)) & 1) << 1) |
                                                (((jc[2] >> (d - 1 - i)) & 1) << 2));
                const int32_t c = children[cur * 8 + oct];
                if (c == -1) break;
                cur = (uint32_t)c;
                od++;
            }
            /* centres in root edges, the neighbour's shifted by one root edge across a wrap */
            double ct[3], co[3];
            centre_of(positions[node], ct);
            centre_of(positions[cur], co);
            if (wrapped) co[axis] += dir;
            float r[3];
            for (int a = 0; a < 3; a++) r[a] = (float)((ct[a] - co[a]) * (double)(1u << od));
            const uint32_t nd = ((uint32_t)cur & 16777215u) | (((uint32_t)(d - od) & 15u) << 24) | (((uint32_t)d & 15u) << 28);
            out[(uint64_t)node * 6 + face] = (uint64_t)nd | ((uint64_t)orc_cf3_encode(r[0], r[1], r[2], NULL, 0) << 32);
        }
    }
}
