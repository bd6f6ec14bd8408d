/* Test infrastructure: CPU restatement of the COUPLED Jacobian mode, included by
 * oc_oracle.c after oc_oracle_impl.h with REAL = float (_f32) and REAL = double (_f64).
 *
 * The reference has no coupled system (its vertex i takes spring i's blocks alone,
 * IMP:782), so this restatement defines the mode rather than following the reference.
 * It is Baraff-Witkin implicit Euler on the reference's own force model (IMP:698-735):
 *
 *   (M' + sum_s [B_s, -B_s; -B_s, B_s]) dV = h (F - h sum_s Kt_s (v_i - v_j))
 *   V += dV;  X += h V;  ground clamp;  the cloth's passes
 *
 * per spring s = (p1, p2, L, ks, kd) with n = (x1 - x2) / l, l = |x1 - x2|:
 *   Kt_s = ksn [n n^T + max(1 - L/l, 0) (I - n n^T)],  ksn = max(ks, 0)
 *        = kst I + (ksn - kst) n n^T,                   kst = ksn max(1 - L/l, 0)
 *   B_s  = h kdn n n^T + h^2 Kt_s = beta I + gamma n n^T, kdn = max(-kd, 0),
 *          beta = h^2 kst, gamma = (h kdn + h^2 ksn) - beta
 *   M'   = (m + h max(-c, 0)) I, c the velocity damping (the damping force c V).
 *
 * The clamps make every B_s positive semi-definite, so the system is SPD for any
 * input (the transverse term is dropped for compressed springs).  Pinned vertices are
 * Dirichlet rows: dV = 0, filtered out of the CG.  The PCG is standard, with the
 * inverse of each vertex's diagonal 3x3 block as preconditioner.
 *
 * Every vertex's sums run over its incident springs in spring-id order, and every
 * expression has a fixed operand order: the GPU kernels (oc_coupled.cu) evaluate the
 * same expressions, so the FP32 flavour is the bit-level specification of the GPU
 * step (its dot products sum per-vertex REAL terms in FP64). */

typedef struct SFX(cpl_coef) {
    REAL n[3];
    REAL beta, gamma; /* B_s = beta I + gamma n n^T */
    REAL ksn, kst;    /* Kt_s = kst I + (ksn - kst) n n^T */
} SFX(cpl_coef);

static void SFX(cpl_spring)(const ocr_spring* s, const REAL* X, REAL h, REAL hh, SFX(cpl_coef) * c) {
    const REAL* p1 = X + 3 * (size_t)s->p1;
    const REAL* p2 = X + 3 * (size_t)s->p2;
    const REAL dx = p1[0] - p2[0], dy = p1[1] - p2[1], dz = p1[2] - p2[2];
    const REAL l = SQRT(dx * dx + dy * dy + dz * dz);
    c->n[0] = dx / l;
    c->n[1] = dy / l;
    c->n[2] = dz / l;
    const REAL ks = (REAL)s->ks, kd = (REAL)s->kd, rest = (REAL)s->rest;
    const REAL zero = 0, one = 1;
    const REAL ksn = ks > zero ? ks : zero;
    const REAL kdn = -kd > zero ? -kd : zero;
    const REAL t = one - rest / l;
    const REAL kst = ksn * (t > zero ? t : zero);
    const REAL alpha = h * kdn + hh * ksn;
    c->beta = hh * kst;
    c->gamma = alpha - c->beta;
    c->ksn = ksn;
    c->kst = kst;
}

/* B_s e accumulated into acc: acc += beta e + (gamma (n.e)) n. */
static void SFX(cpl_apply)(const SFX(cpl_coef) * c, const REAL e[3], REAL acc[3]) {
    const REAL ne = c->n[0] * e[0] + c->n[1] * e[1] + c->n[2] * e[2];
    const REAL g = c->gamma * ne;
    acc[0] = acc[0] + (c->beta * e[0] + g * c->n[0]);
    acc[1] = acc[1] + (c->beta * e[1] + g * c->n[1]);
    acc[2] = acc[2] + (c->beta * e[2] + g * c->n[2]);
}

/* Incidence lists: for each vertex, its springs in spring-id order. */
typedef struct SFX(cpl_graph) {
    int32_t* rowptr; /* n_vertices + 1 */
    int32_t* sid;    /* 2 * n_springs */
} SFX(cpl_graph);

static int SFX(cpl_graph_build)(const ocr_params* p, SFX(cpl_graph) * g) {
    const int32_t N = p->n_vertices, S = p->n_springs;
    g->rowptr = (int32_t*)calloc((size_t)N + 1, sizeof(int32_t));
    g->sid = (int32_t*)malloc(sizeof(int32_t) * (2 * (size_t)S + 1));
    int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * ((size_t)N + 1));
    if (!g->rowptr || !g->sid || !cur) {
        free(g->rowptr); free(g->sid); free(cur);
        return -1;
    }
    for (int32_t s = 0; s < S; ++s) {
        ++g->rowptr[p->springs[s].p1 + 1];
        ++g->rowptr[p->springs[s].p2 + 1];
    }
    for (int32_t i = 0; i < N; ++i) g->rowptr[i + 1] += g->rowptr[i];
    for (int32_t i = 0; i < N; ++i) cur[i] = g->rowptr[i];
    for (int32_t s = 0; s < S; ++s) {
        g->sid[cur[p->springs[s].p1]++] = s;
        g->sid[cur[p->springs[s].p2]++] = s;
    }
    free(cur);
    return 0;
}

static int32_t SFX(cpl_other)(const ocr_spring* s, int32_t i) { return s->p1 == i ? s->p2 : s->p1; }

/* m' of vertex i. */
static REAL SFX(cpl_mass)(const ocr_params* p, int32_t i, REAL h) {
    const REAL m = p->mass ? (REAL)p->mass[i] : (REAL)1;
    const REAL nc = -(REAL)p->damping;
    return m + h * (nc > (REAL)0 ? nc : (REAL)0);
}

/* y = A w for the whole cloth (no pin filter): y_i = m'_i w_i + sum_s B_s (w_i - w_j). */
void SFX(ocr_coupled_matvec)(const ocr_params* p, REAL h, const REAL* X, const REAL* w, REAL* y) {
    SFX(cpl_graph) g;
    if (SFX(cpl_graph_build)(p, &g) != 0) return;
    const REAL hh = h * h;
    for (int32_t i = 0; i < p->n_vertices; ++i) {
        const REAL mp = SFX(cpl_mass)(p, i, h);
        const REAL* wi = w + 3 * (size_t)i;
        REAL acc[3] = {mp * wi[0], mp * wi[1], mp * wi[2]};
        for (int32_t k = g.rowptr[i]; k < g.rowptr[i + 1]; ++k) {
            const ocr_spring* s = p->springs + g.sid[k];
            SFX(cpl_coef) c;
            SFX(cpl_spring)(s, X, h, hh, &c);
            const REAL* wj = w + 3 * (size_t)SFX(cpl_other)(s, i);
            const REAL e[3] = {wi[0] - wj[0], wi[1] - wj[1], wi[2] - wj[2]};
            SFX(cpl_apply)(&c, e, acc);
        }
        y[3 * (size_t)i] = acc[0];
        y[3 * (size_t)i + 1] = acc[1];
        y[3 * (size_t)i + 2] = acc[2];
    }
    free(g.rowptr);
    free(g.sid);
}

/* The vertex system without the pin filter: D (diagonal 3x3 block, a00 a01 a02 a11 a12
 * a22), its inverse Pinv (same layout, cofactors over the determinant) and b. */
void SFX(ocr_coupled_system)(const ocr_params* p, REAL h, const REAL* X, const REAL* V, const REAL* F, REAL* D6,
                             REAL* P6, REAL* b) {
    SFX(cpl_graph) g;
    if (SFX(cpl_graph_build)(p, &g) != 0) return;
    const REAL hh = h * h;
    for (int32_t i = 0; i < p->n_vertices; ++i) {
        const REAL mp = SFX(cpl_mass)(p, i, h);
        REAL a[6] = {mp, 0, 0, mp, 0, mp};
        REAL w[3] = {0, 0, 0};
        const REAL* vi = V + 3 * (size_t)i;
        for (int32_t k = g.rowptr[i]; k < g.rowptr[i + 1]; ++k) {
            const ocr_spring* s = p->springs + g.sid[k];
            SFX(cpl_coef) c;
            SFX(cpl_spring)(s, X, h, hh, &c);
            const REAL g0 = c.gamma * c.n[0], g1 = c.gamma * c.n[1], g2 = c.gamma * c.n[2];
            a[0] = a[0] + (c.beta + g0 * c.n[0]);
            a[1] = a[1] + g0 * c.n[1];
            a[2] = a[2] + g0 * c.n[2];
            a[3] = a[3] + (c.beta + g1 * c.n[1]);
            a[4] = a[4] + g1 * c.n[2];
            a[5] = a[5] + (c.beta + g2 * c.n[2]);
            const REAL* vj = V + 3 * (size_t)SFX(cpl_other)(s, i);
            const REAL u[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
            const REAL nu = c.n[0] * u[0] + c.n[1] * u[1] + c.n[2] * u[2];
            const REAL kk = (c.ksn - c.kst) * nu;
            w[0] = w[0] + (c.kst * u[0] + kk * c.n[0]);
            w[1] = w[1] + (c.kst * u[1] + kk * c.n[1]);
            w[2] = w[2] + (c.kst * u[2] + kk * c.n[2]);
        }
        const REAL c00 = a[3] * a[5] - a[4] * a[4], c01 = a[2] * a[4] - a[1] * a[5], c02 = a[1] * a[4] - a[2] * a[3];
        const REAL c11 = a[0] * a[5] - a[2] * a[2], c12 = a[1] * a[2] - a[0] * a[4], c22 = a[0] * a[3] - a[1] * a[1];
        const REAL det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        const REAL inv = (REAL)1 / det;
        const REAL pinv[6] = {c00 * inv, c01 * inv, c02 * inv, c11 * inv, c12 * inv, c22 * inv};
        for (int k = 0; k < 6; ++k) {
            if (D6) D6[6 * (size_t)i + k] = a[k];
            if (P6) P6[6 * (size_t)i + k] = pinv[k];
        }
        const REAL* f = F + 3 * (size_t)i;
        if (b) {
            b[3 * (size_t)i] = h * (f[0] - h * w[0]);
            b[3 * (size_t)i + 1] = h * (f[1] - h * w[1]);
            b[3 * (size_t)i + 2] = h * (f[2] - h * w[2]);
        }
    }
    free(g.rowptr);
    free(g.sid);
}

/* Symmetric 3x3 (a00 a01 a02 a11 a12 a22) times a vector, row by row. */
static void SFX(cpl_symv)(const REAL* a, const REAL* x, REAL* y) {
    y[0] = (a[0] * x[0] + a[1] * x[1]) + a[2] * x[2];
    y[1] = (a[1] * x[0] + a[3] * x[1]) + a[4] * x[2];
    y[2] = (a[2] * x[0] + a[4] * x[1]) + a[5] * x[2];
}

static double SFX(cpl_dot)(const REAL* a, const REAL* b, int32_t N) {
    double sum = 0;
    for (int32_t i = 0; i < N; ++i) {
        const REAL t = a[3 * (size_t)i] * b[3 * (size_t)i] + a[3 * (size_t)i + 1] * b[3 * (size_t)i + 1] +
                       a[3 * (size_t)i + 2] * b[3 * (size_t)i + 2];
        sum += (double)t;
    }
    return sum;
}

/* n_steps coupled steps; dV is the warm start in and the last solution out.  iters /
 * rel_residual / flags (OC_FLAG_* bits) per step, each may be NULL. */
int SFX(ocr_coupled_step)(const ocr_params* p, REAL dt, int32_t n_steps, REAL* X, REAL* V, REAL* dV, int32_t* iters,
                          double* rel_residual, uint32_t* flags) {
    const int32_t N = p->n_vertices;
    const size_t n3 = 3 * (size_t)N;
    SFX(cpl_graph) g;
    if (SFX(cpl_graph_build)(p, &g) != 0) return -1;
    REAL* F = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* b = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* P6 = (REAL*)malloc(sizeof(REAL) * 6 * (size_t)N);
    REAL* r = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* z = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* d = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* dn = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* q = (REAL*)malloc(sizeof(REAL) * n3);
    uint8_t* pin = (uint8_t*)malloc((size_t)N + 1);
    if (!F || !b || !P6 || !r || !z || !d || !dn || !q || !pin) {
        free(F); free(b); free(P6); free(r); free(z); free(d); free(dn); free(q); free(pin);
        free(g.rowptr); free(g.sid);
        return -1;
    }
    for (int32_t i = 0; i < N; ++i) pin[i] = (uint8_t)SFX(is_pinned)(p, i);
    const REAL h = dt;
    const REAL eps = (REAL)p->eps;
    const REAL eps2 = eps * eps;
    for (int32_t step = 0; step < n_steps; ++step) {
        SFX(ocr_compute_forces)(p, X, V, F);
        SFX(ocr_coupled_system)(p, h, X, V, F, NULL, P6, b);
        for (int32_t i = 0; i < N; ++i)
            if (pin[i]) dV[3 * (size_t)i] = dV[3 * (size_t)i + 1] = dV[3 * (size_t)i + 2] = 0;
        SFX(ocr_coupled_matvec)(p, h, X, dV, q); /* A x with x filtered */
        for (int32_t i = 0; i < N; ++i) {
            REAL* ri = r + 3 * (size_t)i;
            for (int k = 0; k < 3; ++k) ri[k] = pin[i] ? (REAL)0 : b[3 * (size_t)i + k] - q[3 * (size_t)i + k];
            SFX(cpl_symv)(P6 + 6 * (size_t)i, ri, z + 3 * (size_t)i);
            if (pin[i]) z[3 * (size_t)i] = z[3 * (size_t)i + 1] = z[3 * (size_t)i + 2] = 0;
        }
        for (size_t k = 0; k < n3; ++k) d[k] = 0;
        double delta = SFX(cpl_dot)(r, z, N);
        const double delta0 = delta;
        uint32_t fl = 0;
        int32_t it = 0;
        REAL beta = 0;
        int run = p->i_max > 0 && delta > (double)eps2 * delta;
        if (!isfinite(delta)) {
            fl |= 4u;
            run = 0;
        }
        while (run) {
            for (size_t k = 0; k < n3; ++k) dn[k] = it == 0 ? z[k] : z[k] + d[k] * beta;
            SFX(ocr_coupled_matvec)(p, h, X, dn, q);
            for (int32_t i = 0; i < N; ++i)
                if (pin[i]) q[3 * (size_t)i] = q[3 * (size_t)i + 1] = q[3 * (size_t)i + 2] = 0;
            const double dq = SFX(cpl_dot)(dn, q, N);
            if (!(dq > 0.0) || !isfinite(dq)) {
                fl |= isfinite(dq) ? 2u : 4u;
                break;
            }
            const REAL alpha = (REAL)(delta / dq);
            for (int32_t i = 0; i < N; ++i) {
                for (int k = 0; k < 3; ++k) {
                    const size_t e = 3 * (size_t)i + k;
                    dV[e] = dV[e] + dn[e] * alpha;
                    r[e] = r[e] - q[e] * alpha;
                    d[e] = dn[e];
                }
                SFX(cpl_symv)(P6 + 6 * (size_t)i, r + 3 * (size_t)i, z + 3 * (size_t)i);
            }
            const double old = delta;
            delta = SFX(cpl_dot)(r, z, N);
            beta = (REAL)(delta / old);
            ++it;
            if (!isfinite(delta)) {
                fl |= 4u;
                break;
            }
            if (!(it < p->i_max && delta > (double)eps2 * delta0)) {
                if (delta > (double)eps2 * delta0) fl |= 1u;
                break;
            }
        }
        if (iters) iters[step] = it;
        if (rel_residual) rel_residual[step] = delta0 > 0 ? sqrt(delta / delta0) : 0.0;
        if (flags) flags[step] = fl;
        for (int32_t i = 0; i < N; ++i) {
            for (int k = 0; k < 3; ++k) V[3 * (size_t)i + k] += dV[3 * (size_t)i + k];
            for (int k = 0; k < 3; ++k) X[3 * (size_t)i + k] += h * V[3 * (size_t)i + k];
            if (X[3 * (size_t)i + 1] < 0) X[3 * (size_t)i + 1] = 0;
        }
        if (p->passes & 1) SFX(ellipsoid_pass)(p, X, V);
        if (p->passes & 2) SFX(provot_pass)(p, X, V);
    }
    free(F); free(b); free(P6); free(r); free(z); free(d); free(dn); free(q); free(pin);
    free(g.rowptr); free(g.sid);
    return 0;
}
