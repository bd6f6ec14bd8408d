/* Test infrastructure: a straightforward FP64 CPU adjoint of the implicit step, which
 * the GPU adjoint is compared against.  Only tests/ and bench-side gradient checks use it.
 *
 * Forward: ocr_step_f64 one step at a time (the reference step in FP64, with the pin
 * filter); every state is kept.  Backward, per step (REFERENCE Jacobian mode, vertex i
 * uses spring i's Jacobians, OpenCloth_Implicit/.../main.cpp IMP:737-798):
 *   X' = X + dt V' (y clamped at 0), V' = V + dt dV, A dV = b,
 *   A_i = m_i I - h Jv_i - h^2 J_i, b_i = h F_i + h^2 J_i V_i,
 *   J = Ks n n^T - (Ks C + Kd Cdot) D, D = C diag(1 - dP*dP), Jv = -Kd n n^T,
 *   f_s = (-Ks C + Kd (dV.dP)/L) n,  F_i = m g + damping V_i + ext_i + sum_s +-f_s.
 * The linear solve is differentiated as an exact solve: lambda = A^-1 g_dV (A is
 * symmetric), g_b = lambda, g_A = -lambda dV^T; each 3x3 block is solved directly. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oc_oracle.h"

static int is_pinned(const ocr_params* p, int32_t i) {
    return p->pinned ? p->pinned[i] != 0 : (i == 0 || i == p->num_x);
}

static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Adjoint of f = (-Ks C + Kd u) n for one spring; g is dL/df.  Adds to gdP, gdV. */
static void spring_force_adj(const double* dP, const double* dV, double rest, double ks, double kd, const double* g,
                             double* gdP, double* gdV, double* gks, double* gkd) {
    const double L = sqrt(dot3(dP, dP));
    double n[3] = {dP[0] / L, dP[1] / L, dP[2] / L};
    const double C = L - rest;
    const double u = dot3(dV, dP) / L;
    const double m = -ks * C + kd * u;
    const double gm = dot3(g, n);
    double gn[3] = {m * g[0], m * g[1], m * g[2]};
    /* dm/ddP = -Ks n + Kd (dV - u n)/L ; dm/ddV = Kd n */
    for (int k = 0; k < 3; ++k) gdP[k] += gm * (-ks * n[k] + kd * (dV[k] - u * n[k]) / L);
    for (int k = 0; k < 3; ++k) gdV[k] += gm * kd * n[k];
    /* n = dP / L: (I - n n^T) gn / L */
    const double ng = dot3(n, gn);
    for (int k = 0; k < 3; ++k) gdP[k] += (gn[k] - n[k] * ng) / L;
    *gks += -C * gm;
    *gkd += u * gm;
}

/* Jacobians of one spring: J (3x3 row-major J[r][c]) and Jv. */
static void spring_jac(const double* dP, const double* dV, double rest, double ks, double kd, double J[3][3],
                       double Jv[3][3]) {
    const double L = sqrt(dot3(dP, dP));
    double n[3] = {dP[0] / L, dP[1] / L, dP[2] / L};
    const double C = L - rest;
    const double Cd = -dot3(n, dV);
    const double w = ks * C + kd * Cd;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const double S = n[r] * n[c];
            const double D = (r == c) ? C * (1.0 - dP[r] * dP[r]) : 0.0;
            J[r][c] = ks * S - w * D;
            Jv[r][c] = -kd * S;
        }
}

/* Adjoint of (J, Jv) of one spring given G = dL/dJ, H = dL/dJv (full 3x3). */
static void spring_jac_adj(const double* dP, const double* dV, double rest, double ks, double kd, double G[3][3],
                           double H[3][3], double* gdP, double* gdV, double* gks, double* gkd) {
    const double L = sqrt(dot3(dP, dP));
    double n[3] = {dP[0] / L, dP[1] / L, dP[2] / L};
    const double C = L - rest;
    const double Cd = -dot3(n, dV);
    const double w = ks * C + kd * Cd;
    double gS[3][3];
    double gw = 0.0, gC = 0.0, gCd = 0.0, gq[3] = {0, 0, 0};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const double S = n[r] * n[c];
            gS[r][c] = ks * G[r][c] - kd * H[r][c];
            *gks += G[r][c] * S;
            *gkd += -H[r][c] * S;
        }
    for (int k = 0; k < 3; ++k) {
        const double D = C * (1.0 - dP[k] * dP[k]);
        gw += -G[k][k] * D;
        const double gD = -w * G[k][k];
        gC += gD * (1.0 - dP[k] * dP[k]);
        gq[k] = -C * gD;
    }
    gC += ks * gw;
    gCd = kd * gw;
    *gks += C * gw;
    *gkd += Cd * gw;
    double gn[3];
    for (int r = 0; r < 3; ++r) gn[r] = (gS[r][0] + gS[0][r]) * n[0] + (gS[r][1] + gS[1][r]) * n[1] + (gS[r][2] + gS[2][r]) * n[2];
    for (int k = 0; k < 3; ++k) {
        gn[k] += -gCd * dV[k];
        gdV[k] += -gCd * n[k];
        gdP[k] += 2.0 * dP[k] * gq[k] + gC * n[k];
    }
    const double ng = dot3(n, gn);
    for (int k = 0; k < 3; ++k) gdP[k] += (gn[k] - n[k] * ng) / L;
}

static void solve3(const double A[3][3], const double* b, double* x) {
    const double a = A[0][0], bb = A[0][1], c = A[0][2], d = A[1][0], e = A[1][1], f = A[1][2], g = A[2][0],
                 h = A[2][1], i = A[2][2];
    const double det = a * (e * i - f * h) - bb * (d * i - f * g) + c * (d * h - e * g);
    const double inv[3][3] = {{(e * i - f * h) / det, (c * h - bb * i) / det, (bb * f - c * e) / det},
                              {(f * g - d * i) / det, (a * i - c * g) / det, (c * d - a * f) / det},
                              {(d * h - e * g) / det, (bb * g - a * h) / det, (a * e - bb * d) / det}};
    for (int r = 0; r < 3; ++r) x[r] = inv[r][0] * b[0] + inv[r][1] * b[1] + inv[r][2] * b[2];
}

int ocr_adjoint_f64(const ocr_params* p, double dt, int32_t n_steps, const double* X0, const double* V0,
                    const double* gX_T, const double* gV_T, double* X_T, double* V_T, double* gX0, double* gV0,
                    double* gKs, double* gKd, double* gExt) {
    const int32_t N = p->n_vertices, S = p->n_springs;
    const size_t n3 = 3 * (size_t)N;
    double* Xs = (double*)malloc(sizeof(double) * n3 * (size_t)(n_steps + 1));
    double* Vs = (double*)malloc(sizeof(double) * n3 * (size_t)(n_steps + 1));
    double* dVs = (double*)malloc(sizeof(double) * n3 * (size_t)(n_steps + 1));
    double* gX = (double*)calloc(n3, sizeof(double));
    double* gV = (double*)calloc(n3, sizeof(double));
    double* gF = (double*)calloc(n3, sizeof(double));
    if (!Xs || !Vs || !dVs || !gX || !gV || !gF) {
        free(Xs); free(Vs); free(dVs); free(gX); free(gV); free(gF);
        return -1;
    }
    memcpy(Xs, X0, sizeof(double) * n3);
    memcpy(Vs, V0, sizeof(double) * n3);
    memset(dVs, 0, sizeof(double) * n3);
    for (int32_t t = 0; t < n_steps; ++t) {
        double* X = Xs + n3 * (size_t)(t + 1);
        double* V = Vs + n3 * (size_t)(t + 1);
        double* dV = dVs + n3 * (size_t)(t + 1);
        memcpy(X, Xs + n3 * (size_t)t, sizeof(double) * n3);
        memcpy(V, Vs + n3 * (size_t)t, sizeof(double) * n3);
        memcpy(dV, dVs + n3 * (size_t)t, sizeof(double) * n3);
        ocr_step_f64(p, dt, 1, X, V, dV, NULL, NULL);
    }
    memcpy(X_T, Xs + n3 * (size_t)n_steps, sizeof(double) * n3);
    memcpy(V_T, Vs + n3 * (size_t)n_steps, sizeof(double) * n3);
    memcpy(gX, gX_T, sizeof(double) * n3);
    if (gV_T) memcpy(gV, gV_T, sizeof(double) * n3);
    for (int32_t s = 0; s < S; ++s) gKs[s] = gKd[s] = 0.0;
    memset(gExt, 0, sizeof(double) * n3);
    const double h = dt;

    double* F = (double*)malloc(sizeof(double) * n3);
    double* A9 = (double*)malloc(sizeof(double) * 9 * (size_t)N);
    double* bb = (double*)malloc(sizeof(double) * n3);
    for (int32_t t = n_steps - 1; t >= 0; --t) {
        const double* X = Xs + n3 * (size_t)t;
        const double* V = Vs + n3 * (size_t)t;
        const double* dVn = dVs + n3 * (size_t)(t + 1); /* the step's solution */
        /* X' = X + dt V', V' = V + dt dV, clamp */
        for (int32_t i = 0; i < N; ++i) {
            const double vy = V[3 * (size_t)i + 1] + dt * dVn[3 * (size_t)i + 1];
            const double ypre = X[3 * (size_t)i + 1] + dt * vy;
            if (ypre < 0.0) gX[3 * (size_t)i + 1] = 0.0;
        }
        double* gdV = (double*)malloc(sizeof(double) * n3);
        for (size_t k = 0; k < n3; ++k) {
            gV[k] = gV[k] + dt * gX[k];
            gdV[k] = dt * gV[k];
        }
        ocr_compute_forces_f64(p, X, V, F);
        ocr_assemble_f64(p, h, X, V, F, A9, bb);
        for (int32_t i = 0; i < N; ++i) {
            double lam[3] = {0, 0, 0};
            if (!is_pinned(p, i)) {
                double A[3][3];
                for (int c = 0; c < 3; ++c)
                    for (int r = 0; r < 3; ++r) A[r][c] = A9[9 * (size_t)i + 3 * c + r];
                solve3(A, gdV + 3 * (size_t)i, lam);
            }
            const double* dv = dVn + 3 * (size_t)i;
            const double* v = V + 3 * (size_t)i;
            for (int k = 0; k < 3; ++k) gF[3 * (size_t)i + k] = h * lam[k];
            if (i < S) {
                const ocr_spring* sp = p->springs + i;
                double dP[3], dVv[3];
                for (int k = 0; k < 3; ++k) {
                    dP[k] = X[3 * (size_t)sp->p1 + k] - X[3 * (size_t)sp->p2 + k];
                    dVv[k] = V[3 * (size_t)sp->p1 + k] - V[3 * (size_t)sp->p2 + k];
                }
                double J[3][3], Jv[3][3], G[3][3], H[3][3];
                spring_jac(dP, dVv, sp->rest, sp->ks, sp->kd, J, Jv);
                for (int r = 0; r < 3; ++r) {
                    for (int c = 0; c < 3; ++c) {
                        G[r][c] = h * h * lam[r] * (v[c] + dv[c]);
                        H[r][c] = h * lam[r] * dv[c];
                    }
                    gV[3 * (size_t)i + r] += h * h * (J[0][r] * lam[0] + J[1][r] * lam[1] + J[2][r] * lam[2]);
                }
                double gdP[3] = {0, 0, 0}, gdVs[3] = {0, 0, 0};
                spring_jac_adj(dP, dVv, sp->rest, sp->ks, sp->kd, G, H, gdP, gdVs, gKs + i, gKd + i);
                for (int k = 0; k < 3; ++k) {
                    gX[3 * (size_t)sp->p1 + k] += gdP[k];
                    gX[3 * (size_t)sp->p2 + k] -= gdP[k];
                    gV[3 * (size_t)sp->p1 + k] += gdVs[k];
                    gV[3 * (size_t)sp->p2 + k] -= gdVs[k];
                }
            }
        }
        for (int32_t i = 0; i < N; ++i) {
            for (int k = 0; k < 3; ++k) gV[3 * (size_t)i + k] += p->damping * gF[3 * (size_t)i + k];
            if (!is_pinned(p, i))
                for (int k = 0; k < 3; ++k) gExt[3 * (size_t)i + k] += gF[3 * (size_t)i + k];
        }
        for (int32_t s = 0; s < S; ++s) {
            const ocr_spring* sp = p->springs + s;
            double g[3] = {0, 0, 0};
            for (int k = 0; k < 3; ++k) {
                if (!is_pinned(p, sp->p1)) g[k] += gF[3 * (size_t)sp->p1 + k];
                if (!is_pinned(p, sp->p2)) g[k] -= gF[3 * (size_t)sp->p2 + k];
            }
            double dP[3], dVv[3], gdP[3] = {0, 0, 0}, gdVs[3] = {0, 0, 0};
            for (int k = 0; k < 3; ++k) {
                dP[k] = X[3 * (size_t)sp->p1 + k] - X[3 * (size_t)sp->p2 + k];
                dVv[k] = V[3 * (size_t)sp->p1 + k] - V[3 * (size_t)sp->p2 + k];
            }
            spring_force_adj(dP, dVv, sp->rest, sp->ks, sp->kd, g, gdP, gdVs, gKs + s, gKd + s);
            for (int k = 0; k < 3; ++k) {
                gX[3 * (size_t)sp->p1 + k] += gdP[k];
                gX[3 * (size_t)sp->p2 + k] -= gdP[k];
                gV[3 * (size_t)sp->p1 + k] += gdVs[k];
                gV[3 * (size_t)sp->p2 + k] -= gdVs[k];
            }
        }
        free(gdV);
    }
    memcpy(gX0, gX, sizeof(double) * n3);
    memcpy(gV0, gV, sizeof(double) * n3);
    free(F); free(A9); free(bb);
    free(Xs); free(Vs); free(dVs); free(gX); free(gV); free(gF);
    return 0;
}
