// evolve_physics.cuh -- pointwise physics of the evolution kernels: analytic initial data, the BSSN
// right-hand side (moving-puncture form: 1+log or harmonic slicing, Gamma-driver shift) and the
// Hamiltonian and momentum constraints.  The reference has none of these (its BSSN module stops at
// metric derivatives and Christoffel symbols, BSSN.h:38-102); the equations follow the standard
// conformal formulation (Baumgarte & Shapiro; Campanelli et al. and Baker et al. 2006 for the
// puncture gauge), with chi = det(gamma)^(-1/3):
//
//   d_t chi     = beta.d chi + 2/3 chi (alpha K - d_k beta^k)
//   d_t gt_ij   = beta.d gt_ij + gt_ik d_j beta^k + gt_jk d_i beta^k - 2/3 gt_ij d_k beta^k - 2 alpha At_ij
//   d_t K       = beta.d K - D^i D_i alpha + alpha (At_ij At^ij + K^2 / 3)
//   d_t At_ij   = beta.d At_ij + At_ik d_j beta^k + At_jk d_i beta^k - 2/3 At_ij d_k beta^k
//                 + alpha (K At_ij - 2 At_ik At^k_j) + chi [-D_i D_j alpha + alpha R_ij]^TF
//   d_t Gt^i    = beta.d Gt^i - Gt^k d_k beta^i + 2/3 Gt^i d_k beta^k + gt^jk d_j d_k beta^i
//                 + 1/3 gt^ij d_j d_k beta^k - 2 At^ij d_j alpha
//                 + 2 alpha (Gt^i_jk At^jk - 3/2 At^ij d_j chi / chi - 2/3 gt^ij d_j K)
//   d_t alpha   = beta.d alpha - 2 alpha K            (1+log)   or  - alpha^2 K  (harmonic)
//   d_t beta^i  = beta.d beta^i + 3/4 B^i ,   d_t B^i = beta.d B^i + (d_t - beta.d) Gt^i - eta B^i
//   R_ij = Rt_ij + Rchi_ij,
//   Rt_ij = -1/2 gt^lm d_l d_m gt_ij + gt_k(i d_j) Gt^k + Gt_d^k Gt_(ij)k
//           + gt^lm (2 Gt^k_l(i Gt_j)km + Gt^k_im Gt_klj)          (Gt_d^k = gt^ij Gt^k_ij)
//   Rchi_ij = (Dt_i Dt_j chi + gt_ij Dt^l Dt_l chi) / (2 chi) - (d_i chi d_j chi + 3 gt_ij d^l chi d_l chi) / (4 chi^2)
//   H   = chi gt^ij R_ij + 2/3 K^2 - At_ij At^ij
//   M_i = d_j At^j_i - 3/2 At^j_i d_j chi / chi - 1/2 At^jm d_i gt_jm - 2/3 d_i K
//         (d_j At^j_i = gt^jk d_j At_ki - gt^ja gt^kb d_j gt_ab At_ki: the physical momentum constraint)
// The advection terms beta.d u and the Kreiss-Oliger dissipation come from the derivative pass.
#pragma once

#include <cmath>

#include "amr_gb300.h"
#include "evolve.h"

namespace amr {

struct Mat3 {
    float m[3][3];
};

__device__ __forceinline__ int sidx(int i, int j) {        // xx xy xz yy yz zz
    const int a = i < j ? i : j, b = i < j ? j : i;
    return a == 0 ? b : (a == 1 ? 2 + b : 5);
}
__device__ __forceinline__ int didx(int i, int j) {        // xx yy zz xy xz yz
    return i == j ? i : (i + j == 1 ? 3 : (i + j == 2 ? 4 : 5));
}

// Inverse of a symmetric 3x3 matrix given as 6 components (cofactors over the determinant).
__device__ __forceinline__ void inverse_sym(const float* g, float gi[3][3]) {
    const float c00 = g[3] * g[5] - g[4] * g[4], c01 = g[2] * g[4] - g[1] * g[5], c02 = g[1] * g[4] - g[2] * g[3];
    const float det = g[0] * c00 + g[1] * c01 + g[2] * c02;
    const float id = 1.f / det;
    gi[0][0] = c00 * id;
    gi[0][1] = gi[1][0] = c01 * id;
    gi[0][2] = gi[2][0] = c02 * id;
    gi[1][1] = (g[0] * g[5] - g[2] * g[2]) * id;
    gi[1][2] = gi[2][1] = (g[1] * g[2] - g[0] * g[4]) * id;
    gi[2][2] = (g[0] * g[3] - g[1] * g[1]) * id;
}

// ------------------------------------------------------------------ initial data at a point
// In double precision (a one-off cost): the stored deviations from flat space (evolve.h) are then
// rounded once, instead of carrying the float rounding of the values near 1.
__device__ __forceinline__ void evo_initial_values(const InitData& id, int physics, const double* x, double* u) {
    if (physics != 0) {   // scalar wave: Gaussian pulse at rest
        const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
        u[W_U] = id.kind == AMR_ID_GAUSSIAN_PULSE ? exp(-r2 / ((double)id.width * id.width)) : 0.0;
        u[W_V] = 0.0;
        return;
    }
    for (int f = 0; f < BSSN_NF; f++) u[f] = 0.0;
    u[F_CHI] = 1.0;
    u[F_GXX] = u[F_GYY] = u[F_GZZ] = 1.0;
    u[F_ALPHA] = 1.0;
    if (id.kind == AMR_ID_GAUGE_WAVE) {
        // ds^2 = -H dt^2 + H dx^2 + dy^2 + dz^2, H = 1 - A sin(2 pi (x - t) / d), at t = 0
        const double A = id.amplitude, k = 6.283185307179586476925 / id.wavelength;
        const double sn = sin(k * x[0]), cs = cos(k * x[0]);
        const double H = 1.0 - A * sn;
        const double dH = -A * k * cs;                       // d_x H
        const double sq = sqrt(H);
        const double Kxx = -0.5 * A * k * cs / sq;           // -d_t gamma_xx / (2 alpha)
        const double chi = 1.0 / cbrt(H);
        const double K = Kxx / H;
        u[F_CHI] = chi;
        u[F_GXX] = chi * H;
        u[F_GYY] = u[F_GZZ] = chi;
        u[F_K] = K;
        u[F_AXX] = chi * (Kxx - H * K / 3.0);
        u[F_AYY] = u[F_AZZ] = -chi * K / 3.0;
        u[F_GAMX] = (2.0 / 3.0) * dH / (H * cbrt(H * H));    // -d_x (H^(-2/3))
        u[F_ALPHA] = sq;
    } else if (id.kind == AMR_ID_BRILL_LINDQUIST) {
        // psi = 1 + sum m_a / (2 r_a); chi = psi^-4, conformally flat, K_ij = 0, lapse psi^-2
        double psi = 1.0;
        for (int a = 0; a < id.n_punctures && a < 4; a++) {
            const double dx = x[0] - id.pos[a][0], dy = x[1] - id.pos[a][1], dz = x[2] - id.pos[a][2];
            const double r = fmax(sqrt(dx * dx + dy * dy + dz * dz), 1e-6);
            psi += id.mass[a] / (2.0 * r);
        }
        const double p2 = psi * psi;
        u[F_CHI] = 1.0 / (p2 * p2);
        u[F_ALPHA] = 1.0 / p2;
    }
}

// ------------------------------------------------------------------ the pieces both the right-hand
// side and the constraints use
struct Geometry {
    float chi, ichi;              // chi, 1 / max(chi, floor)
    float g[6], gi[3][3];         // conformal metric and its inverse
    float cl[3][6];               // Gt_ijk with the first index lowered, jk symmetric
    float cu[3][6];               // Gt^i_jk
    float gd[3];                  // Gt_d^i = gt^jk Gt^i_jk
    float dchi[3];
    float R[6];                   // R_ij
};

template <class DV>
__device__ __forceinline__ void geometry(const float* u, const DV& dv, const EvoParams& prm, Geometry& G) {
    G.chi = u[F_CHI];
    G.ichi = 1.f / fmaxf(G.chi, prm.chi_floor);
    for (int c = 0; c < 6; c++) G.g[c] = u[F_GXX + c];
    inverse_sym(G.g, G.gi);
    for (int k = 0; k < 3; k++) G.dchi[k] = dv(D_CHI1 + k);
    // lowered Christoffels: Gt_ijk = (d_j gt_ik + d_k gt_ij - d_i gt_jk) / 2
    auto dg = [&](int a, int b, int k) { return dv(D_G1 + 3 * sidx(a, b) + k); };
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k = j; k < 3; k++) G.cl[i][sidx(j, k)] = .5f * (dg(i, k, j) + dg(i, j, k) - dg(j, k, i));
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int c = 0; c < 6; c++) G.cu[i][c] = G.gi[i][0] * G.cl[0][c] + G.gi[i][1] * G.cl[1][c] + G.gi[i][2] * G.cl[2][c];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k = 0; k < 3; k++) s += G.gi[j][k] * G.cu[i][sidx(j, k)];
        G.gd[i] = s;
    }
    // Dt_i Dt_j chi and its trace, |d chi|^2
    float ddchi[6], tr_dd = 0.f, dchi2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            float v = dv(D_CHI2 + didx(i, j));
#pragma unroll
            for (int k = 0; k < 3; k++) v -= G.cu[k][sidx(i, j)] * G.dchi[k];
            ddchi[sidx(i, j)] = v;
        }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            tr_dd += G.gi[i][j] * ddchi[sidx(i, j)];
            dchi2 += G.gi[i][j] * G.dchi[i] * G.dchi[j];
        }
    // Ricci tensor (unrolled: every index is a constant, so the geometry stays in registers)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const int ij = sidx(i, j);
            float r = 0.f;
            // -1/2 gt^lm d_l d_m gt_ij (contracted by the derivative pass)
            r -= .5f * dv(D_GLAP + ij);
            // gt_k(i d_j) Gt^k
            for (int k = 0; k < 3; k++)
                r += .5f * (G.g[sidx(k, i)] * dv(D_GAM1 + 3 * k + j) + G.g[sidx(k, j)] * dv(D_GAM1 + 3 * k + i));
            // Gt_d^k Gt_(ij)k
            for (int k = 0; k < 3; k++) r += .5f * G.gd[k] * (G.cl[i][sidx(j, k)] + G.cl[j][sidx(i, k)]);
            // gt^lm (Gt^k_li Gt_jkm + Gt^k_lj Gt_ikm + Gt^k_im Gt_klj)
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++) {
                    float s = 0.f;
                    for (int k = 0; k < 3; k++)
                        s += G.cu[k][sidx(l, i)] * G.cl[j][sidx(k, m)] + G.cu[k][sidx(l, j)] * G.cl[i][sidx(k, m)] +
                             G.cu[k][sidx(i, m)] * G.cl[k][sidx(l, j)];
                    r += G.gi[l][m] * s;
                }
            // conformal-factor part
            r += .5f * G.ichi * (ddchi[ij] + G.g[ij] * tr_dd) -
                 .25f * G.ichi * G.ichi * (G.dchi[i] * G.dchi[j] + 3.f * G.g[ij] * dchi2);
            G.R[ij] = r;
        }
}

// ------------------------------------------------------------------ BSSN right-hand side (without the
// advection and dissipation terms, which the derivative pass supplies)
template <class DV>
__device__ __forceinline__ void bssn_rhs(const float* u, const DV& dv, const EvoParams& prm, float* rhs) {
    Geometry G;
    geometry(u, dv, prm, G);
    const float K = u[F_K], alpha = u[F_ALPHA];
    float A[6];
    for (int c = 0; c < 6; c++) A[c] = u[F_AXX + c];
    float dal[3], dK[3], db[3][3];
    for (int k = 0; k < 3; k++) { dal[k] = dv(D_AL1 + k); dK[k] = dv(D_K1 + k); }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) db[i][j] = dv(D_BE1 + 3 * i + j);   // d_j beta^i
    const float divb = db[0][0] + db[1][1] + db[2][2];
    // At^i_j and At^ij
    float Aud[3][3], Auu[3][3], AA = 0.f;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            Aud[i][j] = G.gi[i][0] * A[sidx(0, j)] + G.gi[i][1] * A[sidx(1, j)] + G.gi[i][2] * A[sidx(2, j)];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Auu[i][j] = Aud[i][0] * G.gi[0][j] + Aud[i][1] * G.gi[1][j] + Aud[i][2] * G.gi[2][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) AA += A[sidx(i, j)] * Auu[i][j];
    // D_i D_j alpha (physical) and its trace
    float dda[6], lap_a = 0.f;
    float dchi_dal = 0.f;
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) dchi_dal += G.gi[k][l] * G.dchi[k] * dal[l];
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            float v = dv(D_AL2 + didx(i, j));
            for (int k = 0; k < 3; k++) v -= G.cu[k][sidx(i, j)] * dal[k];
            v += .5f * G.ichi * (G.dchi[i] * dal[j] + G.dchi[j] * dal[i] - G.g[sidx(i, j)] * dchi_dal);
            dda[sidx(i, j)] = v;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) lap_a += G.gi[i][j] * dda[sidx(i, j)];
    lap_a *= G.chi;
    // chi
    rhs[F_CHI] = (2.f / 3.f) * G.chi * (alpha * K - divb);
    // conformal metric
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            float v = -2.f * alpha * A[sidx(i, j)] - (2.f / 3.f) * G.g[sidx(i, j)] * divb;
            for (int k = 0; k < 3; k++) v += G.g[sidx(i, k)] * db[k][j] + G.g[sidx(j, k)] * db[k][i];
            rhs[F_GXX + sidx(i, j)] = v;
        }
    // K
    rhs[F_K] = -lap_a + alpha * (AA + K * K * (1.f / 3.f));
    // trace-free part of -D_i D_j alpha + alpha R_ij
    float X[6], trX = 0.f;
    for (int c = 0; c < 6; c++) X[c] = -dda[c] + alpha * G.R[c];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) trX += G.gi[i][j] * X[sidx(i, j)];
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            const int ij = sidx(i, j);
            float v = G.chi * (X[ij] - G.g[ij] * trX * (1.f / 3.f));
            v += alpha * (K * A[ij] - 2.f * (A[sidx(i, 0)] * Aud[0][j] + A[sidx(i, 1)] * Aud[1][j] + A[sidx(i, 2)] * Aud[2][j]));
            v -= (2.f / 3.f) * A[ij] * divb;
            for (int k = 0; k < 3; k++) v += A[sidx(i, k)] * db[k][j] + A[sidx(j, k)] * db[k][i];
            rhs[F_AXX + ij] = v;
        }
    // conformal connection functions (core: without advection)
    float ddivb[3];   // d_j (d_k beta^k)
    for (int j = 0; j < 3; j++) ddivb[j] = dv(D_DDIVB + j);
    float gcore[3];
    for (int i = 0; i < 3; i++) {
        float v = (2.f / 3.f) * u[F_GAMX + i] * divb;
        for (int k = 0; k < 3; k++) v -= u[F_GAMX + k] * db[i][k];
        v += dv(D_BELAP + i);   // gt^jk d_j d_k beta^i
        float s1 = 0.f, s2 = 0.f, s3 = 0.f;
        for (int j = 0; j < 3; j++) {
            v += (1.f / 3.f) * G.gi[i][j] * ddivb[j] - 2.f * Auu[i][j] * dal[j];
            s2 += Auu[i][j] * G.dchi[j];
            s3 += G.gi[i][j] * dK[j];
            for (int k = 0; k < 3; k++) s1 += G.cu[i][sidx(j, k)] * Auu[j][k];
        }
        v += 2.f * alpha * (s1 - 1.5f * s2 * G.ichi - (2.f / 3.f) * s3);
        gcore[i] = v;
        rhs[F_GAMX + i] = v;
    }
    // lapse
    rhs[F_ALPHA] = prm.slicing == AMR_SLICING_HARMONIC ? -alpha * alpha * K : -2.f * alpha * K;
    // shift and its driver
    for (int i = 0; i < 3; i++) {
        if (prm.shift) {
            rhs[F_BETAX + i] = .75f * u[F_BX + i];
            rhs[F_BX + i] = gcore[i] - prm.eta * u[F_BX + i];
        } else {
            rhs[F_BETAX + i] = 0.f;
            rhs[F_BX + i] = 0.f;
        }
    }
}

// Hamiltonian constraint and the three components of the momentum constraint.
template <class DV>
__device__ __forceinline__ void bssn_constraints(const float* u, const DV& dv, const EvoParams& prm, float* hm) {
    Geometry G;
    geometry(u, dv, prm, G);
    const float K = u[F_K];
    float A[6];
    for (int c = 0; c < 6; c++) A[c] = u[F_AXX + c];
    float Aud[3][3], Auu[3][3], AA = 0.f, trR = 0.f;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            Aud[i][j] = G.gi[i][0] * A[sidx(0, j)] + G.gi[i][1] * A[sidx(1, j)] + G.gi[i][2] * A[sidx(2, j)];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Auu[i][j] = Aud[i][0] * G.gi[0][j] + Aud[i][1] * G.gi[1][j] + Aud[i][2] * G.gi[2][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            AA += A[sidx(i, j)] * Auu[i][j];
            trR += G.gi[i][j] * G.R[sidx(i, j)];
        }
    hm[0] = G.chi * trR + (2.f / 3.f) * K * K - AA;
    for (int i = 0; i < 3; i++) {
        float v = -(2.f / 3.f) * dv(D_K1 + i);
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                v += G.gi[j][k] * dv(D_AT1 + 3 * sidx(k, i) + j);
                float s = 0.f;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) s += G.gi[j][a] * G.gi[k][b] * dv(D_G1 + 3 * sidx(a, b) + j);
                v -= s * A[sidx(k, i)];
                v -= .5f * Auu[j][k] * dv(D_G1 + 3 * sidx(j, k) + i);
            }
        for (int l = 0; l < 3; l++) v -= 1.5f * Aud[l][i] * G.dchi[l] * G.ichi;
        hm[1 + i] = v;
    }
}

}  // namespace amr
