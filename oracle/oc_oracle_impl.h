/* Test infrastructure: body of the CPU restatement, included twice by oc_oracle.c
 * with REAL = float (suffix _f32) and REAL = double (suffix _f64).  Every expression
 * keeps the reference's operand order; citations are to
 * OpenCloth_Implicit/OpenCloth_Implicit/main.cpp (IMP) and dep/glm/glm/core (GLM). */

typedef struct SFX(spring_eval) {
    REAL C, Cdot;
    REAL n[3];   /* dc_dp = deltaP / dist                      IMP:722 */
    REAL dp2[3]; /* deltaP2 = componentwise deltaP * deltaP     IMP:724 */
    REAL f[3];   /* spring force on p1                          IMP:726-728 */
} SFX(spring_eval);

static int SFX(is_pinned)(const ocr_params* p, int32_t i) {
    /* IMP:705, :730, :732 hard-code the pins to vertices 0 and numX. */
    return p->pinned ? p->pinned[i] != 0 : (i == 0 || i == p->num_x);
}

/* One spring, IMP:713-728.  length() and normalize() are GLM/core/func_geometric.inl
 * :41-51 and :221-230: both square the components as ((x*x + y*y) + z*z); normalize
 * multiplies by inversesqrt = 1/sqrt (GLM/core/func_exponential.inl:309-318). */
static void SFX(eval_spring)(const ocr_spring* s, const REAL* X, const REAL* V, SFX(spring_eval) * e) {
    const REAL* p1 = X + 3 * (size_t)s->p1;
    const REAL* p2 = X + 3 * (size_t)s->p2;
    const REAL* v1 = V + 3 * (size_t)s->p1;
    const REAL* v2 = V + 3 * (size_t)s->p2;
    const REAL dPx = p1[0] - p2[0], dPy = p1[1] - p2[1], dPz = p1[2] - p2[2];
    const REAL dVx = v1[0] - v2[0], dVy = v1[1] - v2[1], dVz = v1[2] - v2[2];
    const REAL sqr = dPx * dPx + dPy * dPy + dPz * dPz;
    const REAL dist = SQRT(sqr);
    const REAL rest = (REAL)s->rest, ks = (REAL)s->ks, kd = (REAL)s->kd;
    e->C = dist - rest;
    e->n[0] = dPx / dist;
    e->n[1] = dPy / dist;
    e->n[2] = dPz / dist;
    e->Cdot = (v1[0] * (-e->n[0]) + v1[1] * (-e->n[1]) + v1[2] * (-e->n[2])) +
              (v2[0] * e->n[0] + v2[1] * e->n[1] + v2[2] * e->n[2]);
    e->dp2[0] = dPx * dPx;
    e->dp2[1] = dPy * dPy;
    e->dp2[2] = dPz * dPz;
    const REAL left = (-ks) * (dist - rest);
    const REAL right = kd * ((dVx * dPx + dVy * dPy + dVz * dPz) / dist);
    const REAL inv = (REAL)1 / SQRT(sqr);
    const REAL mag = left + right;
    e->f[0] = mag * (dPx * inv);
    e->f[1] = mag * (dPy * inv);
    e->f[2] = mag * (dPz * inv);
}

/* df_dx and df_dv of one spring, IMP:744-770.  Matrices are glm column-major:
 * element m[c][r] is stored at 3*c + r.  outerProduct(c, r) has m[i][j] = c[j]*r[i]
 * (GLM/core/func_matrix.inl:51-63). */
static void SFX(spring_jacobians)(const SFX(spring_eval) * e, REAL ks, REAL kd, REAL J[9], REAL Jv[9]) {
    const REAL c1 = e->C;
    REAL d00[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    REAL d01[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int k = 0; k < 3; ++k) {
        d00[4 * k] = (-c1) * e->dp2[k] + c1;
        d01[4 * k] = c1 * e->dp2[k] - c1;
    }
    for (int c = 0; c < 3; ++c) {
        for (int r = 0; r < 3; ++r) {
            const int k = 3 * c + r;
            const REAL dp1 = e->n[r] * e->n[c];
            const REAL dp2 = e->n[r] * (-e->n[c]);
            const REAL dp3 = (-e->n[r]) * (-e->n[c]);
            const REAL t1 = (-ks) * (dp1 + d00[k] * e->C) - kd * (d00[k] * e->Cdot);
            const REAL t2 = (-ks) * (dp2 + d01[k] * e->C) - kd * (d01[k] * e->Cdot);
            const REAL t3 = (-ks) * (dp2 + d00[k] * e->C) - kd * (d00[k] * e->Cdot);
            REAL j = 0;
            j += t1;
            j += t2;
            j += t3;
            J[k] = j;
            REAL jv = 0;
            jv += (-kd) * dp1;
            jv += (-kd) * dp2;
            jv += (-kd) * dp3;
            Jv[k] = jv;
        }
    }
}

/* ComputeForces, IMP:698-735 (plus the optional per-vertex mass and external force). */
void SFX(ocr_compute_forces)(const ocr_params* p, const REAL* X, const REAL* V, REAL* F) {
    const int32_t N = p->n_vertices;
    for (int32_t i = 0; i < N; ++i) {
        REAL* f = F + 3 * (size_t)i;
        f[0] = 0;
        f[1] = 0;
        f[2] = 0;
        const int pin = SFX(is_pinned)(p, i);
        if (!pin) {
            const REAL m = p->mass ? (REAL)p->mass[i] : (REAL)1;
            f[0] += m * (REAL)p->gravity[0];
            f[1] += m * (REAL)p->gravity[1];
            f[2] += m * (REAL)p->gravity[2];
        }
        const REAL damp = (REAL)p->damping;
        f[0] += damp * V[3 * (size_t)i];
        f[1] += damp * V[3 * (size_t)i + 1];
        f[2] += damp * V[3 * (size_t)i + 2];
        if (!pin && p->ext_force) {
            f[0] += (REAL)p->ext_force[3 * (size_t)i];
            f[1] += (REAL)p->ext_force[3 * (size_t)i + 1];
            f[2] += (REAL)p->ext_force[3 * (size_t)i + 2];
        }
    }
    for (int32_t s = 0; s < p->n_springs; ++s) {
        const ocr_spring* sp = p->springs + s;
        SFX(spring_eval) e;
        SFX(eval_spring)(sp, X, V, &e);
        if (!SFX(is_pinned)(p, sp->p1)) {
            REAL* f = F + 3 * (size_t)sp->p1;
            f[0] += e.f[0];
            f[1] += e.f[1];
            f[2] += e.f[2];
        }
        if (!SFX(is_pinned)(p, sp->p2)) {
            REAL* f = F + 3 * (size_t)sp->p2;
            f[0] -= e.f[0];
            f[1] -= e.f[1];
            f[2] -= e.f[2];
        }
    }
}

/* CalcForceDerivatives + the assembly loop of IntegrateImplicit, IMP:737-786.
 * Vertex i takes spring i's Jacobians (the reference indexes the per-spring arrays
 * by vertex); vertices with no spring of the same index get zero Jacobians.
 * A9 holds A_i column-major; b holds b_i. */
void SFX(ocr_assemble)(const ocr_params* p, REAL h, const REAL* X, const REAL* V, const REAL* F, REAL* A9, REAL* b) {
    const int32_t N = p->n_vertices;
    for (int32_t i = 0; i < N; ++i) {
        REAL J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Jv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (i < p->n_springs) {
            const ocr_spring* sp = p->springs + i;
            SFX(spring_eval) e;
            SFX(eval_spring)(sp, X, V, &e);
            SFX(spring_jacobians)(&e, (REAL)sp->ks, (REAL)sp->kd, J, Jv);
        }
        const REAL m = p->mass ? (REAL)p->mass[i] : (REAL)1;
        REAL* A = A9 + 9 * (size_t)i;
        REAL hJ[9];
        for (int k = 0; k < 9; ++k) {
            const REAL Mk = (k == 0 || k == 4 || k == 8) ? m : (REAL)0;
            A[k] = Mk - h * (Jv[k] + h * J[k]); /* IMP:782 */
            hJ[k] = h * J[k];
        }
        const REAL y = 0; /* IMP:779 */
        const REAL vx = V[3 * (size_t)i] + y, vy = V[3 * (size_t)i + 1] + y, vz = V[3 * (size_t)i + 2] + y;
        /* mat3 * vec3, GLM/core/type_mat3x3.inl:511-518 */
        const REAL wx = hJ[0] * vx + hJ[3] * vy + hJ[6] * vz;
        const REAL wy = hJ[1] * vx + hJ[4] * vy + hJ[7] * vz;
        const REAL wz = hJ[2] * vx + hJ[5] * vy + hJ[8] * vz;
        b[3 * (size_t)i] = h * (F[3 * (size_t)i] + wx); /* IMP:783 */
        b[3 * (size_t)i + 1] = h * (F[3 * (size_t)i + 1] + wy);
        b[3 * (size_t)i + 2] = h * (F[3 * (size_t)i + 2] + wz);
    }
}

static void SFX(matvec)(const REAL* A, const REAL* x, REAL* y) {
    y[0] = A[0] * x[0] + A[3] * x[1] + A[6] * x[2];
    y[1] = A[1] * x[0] + A[4] * x[1] + A[7] * x[2];
    y[2] = A[2] * x[0] + A[5] * x[1] + A[8] * x[2];
}

/* dot over LargeVector, IMP:273-279: per-vertex glm::dot in REAL, summed in REAL
 * (reference) or in double (dot_fp64). */
static double SFX(dot)(const ocr_params* p, const REAL* a, const REAL* b, int32_t N) {
    if (p->dot_fp64) {
        double sum = 0;
        for (int32_t i = 0; i < N; ++i) {
            const REAL t = a[3 * (size_t)i] * b[3 * (size_t)i] + a[3 * (size_t)i + 1] * b[3 * (size_t)i + 1] +
                           a[3 * (size_t)i + 2] * b[3 * (size_t)i + 2];
            sum += (double)t;
        }
        return sum;
    }
    REAL sum = 0;
    for (int32_t i = 0; i < N; ++i) {
        sum += a[3 * (size_t)i] * b[3 * (size_t)i] + a[3 * (size_t)i + 1] * b[3 * (size_t)i + 1] +
               a[3 * (size_t)i + 2] * b[3 * (size_t)i + 2];
    }
    return (double)sum;
}

/* EllipsoidCollision, IMP:824-848: a vertex inside the unit sphere of the ellipsoid's
 * object space (center 0, radius 1, IMP:136-137) is pushed to its surface and stopped.
 * Matrices are glm column-major (m[c][r] at 4c + r); mat4 * vec4 sums left to right
 * (GLM/core/type_mat4x4.inl:567-571). */
static void SFX(ellipsoid_pass)(const ocr_params* p, REAL* X, REAL* V) {
    const double* E = p->ellipsoid;
    const double* I = p->ellipsoid_inv;
    for (int32_t i = 0; i < p->n_vertices; ++i) {
        REAL* x = X + 3 * (size_t)i;
        const REAL one = 1;
        REAL d0x = (REAL)I[0] * x[0] + (REAL)I[4] * x[1] + (REAL)I[8] * x[2] + (REAL)I[12] * one;
        REAL d0y = (REAL)I[1] * x[0] + (REAL)I[5] * x[1] + (REAL)I[9] * x[2] + (REAL)I[13] * one;
        REAL d0z = (REAL)I[2] * x[0] + (REAL)I[6] * x[1] + (REAL)I[10] * x[2] + (REAL)I[14] * one;
        const REAL zero = 0;
        d0x = d0x - zero;
        d0y = d0y - zero;
        d0z = d0z - zero;
        const REAL dist = SQRT(d0x * d0x + d0y * d0y + d0z * d0z);
        if (dist < one) {
            const REAL k = one - dist;
            d0x = (k * d0x) / dist;
            d0y = (k * d0y) / dist;
            d0z = (k * d0z) / dist;
            REAL delta[3];
            for (int r = 0; r < 3; ++r) {
                REAL tx = (REAL)E[r], ty = (REAL)E[4 + r], tz = (REAL)E[8 + r];
                const REAL dd = tx * tx + ty * ty + tz * tz;
                tx = tx / dd;
                ty = ty / dd;
                tz = tz / dd;
                delta[r] = d0x * tx + d0y * ty + d0z * tz;
            }
            x[0] += delta[0];
            x[1] += delta[1];
            x[2] += delta[2];
            V[3 * (size_t)i] = V[3 * (size_t)i + 1] = V[3 * (size_t)i + 2] = 0;
        }
    }
}

/* ApplyProvotDynamicInverse, IMP:800-823: a spring stretched beyond ratio * rest moves
 * its endpoints' velocities by half the excess along the spring, pinned ends excepted. */
static void SFX(provot_pass)(const ocr_params* p, const REAL* X, REAL* V) {
    for (int32_t s = 0; s < p->n_springs; ++s) {
        const ocr_spring* sp = p->springs + s;
        const REAL* a = X + 3 * (size_t)sp->p1;
        const REAL* b = X + 3 * (size_t)sp->p2;
        REAL dP[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
        const REAL sqr = dP[0] * dP[0] + dP[1] * dP[1] + dP[2] * dP[2];
        REAL dist = SQRT(sqr);
        const REAL lim = (REAL)sp->rest * (REAL)p->provot_ratio;
        if (dist > lim) {
            dist -= lim;
            dist /= (REAL)2;
            const REAL inv = (REAL)1 / SQRT(sqr);
            for (int k = 0; k < 3; ++k) dP[k] = (dP[k] * inv) * dist;
            REAL* v1 = V + 3 * (size_t)sp->p1;
            REAL* v2 = V + 3 * (size_t)sp->p2;
            if (SFX(is_pinned)(p, sp->p1)) {
                for (int k = 0; k < 3; ++k) v2[k] += dP[k];
            } else if (SFX(is_pinned)(p, sp->p2)) {
                for (int k = 0; k < 3; ++k) v1[k] -= dP[k];
            } else {
                for (int k = 0; k < 3; ++k) v1[k] -= dP[k];
                for (int k = 0; k < 3; ++k) v2[k] += dP[k];
            }
        }
    }
}

void SFX(ocr_passes)(const ocr_params* p, REAL* X, REAL* V) {
    if (p->passes & 1) SFX(ellipsoid_pass)(p, X, V);
    if (p->passes & 2) SFX(provot_pass)(p, X, V);
}

/* ComputeForces(); IntegrateImplicit(dt); [EllipsoidCollision(); ApplyProvotDynamicInverse();]
 * repeated n_steps times (IMP:873-880).  dV is the persistent warm start (IMP:361). */
int SFX(ocr_step)(const ocr_params* p, REAL dt, int32_t n_steps, REAL* X, REAL* V, REAL* dV, int32_t* iters,
                  double* rel_residual) {
    const int32_t N = p->n_vertices;
    const size_t n3 = 3 * (size_t)N;
    REAL* F = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* A9 = (REAL*)malloc(sizeof(REAL) * 9 * (size_t)N);
    REAL* b = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* P = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* Pinv = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* r = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* d = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* q = (REAL*)malloc(sizeof(REAL) * n3);
    REAL* Pr = (REAL*)malloc(sizeof(REAL) * n3);
    if (!F || !A9 || !b || !P || !Pinv || !r || !d || !q || !Pr) {
        free(F); free(A9); free(b); free(P); free(Pinv); free(r); free(d); free(q); free(Pr);
        return -1;
    }
    const REAL h = dt;
    const REAL eps = (REAL)p->eps;
    const REAL eps2 = eps * eps; /* IMP:127 */
    for (int32_t step = 0; step < n_steps; ++step) {
        SFX(ocr_compute_forces)(p, X, V, F);
        SFX(ocr_assemble)(p, h, X, V, F, A9, b);
        for (int32_t i = 0; i < N; ++i) {
            const REAL* A = A9 + 9 * (size_t)i;
            P[3 * (size_t)i] = A[0]; /* IMP:784-785 */
            P[3 * (size_t)i + 1] = A[4];
            P[3 * (size_t)i + 2] = A[8];
            for (int k = 0; k < 3; ++k) Pinv[3 * (size_t)i + k] = (REAL)1 / P[3 * (size_t)i + k];
        }
        /* SolveConjugateGradientPreconditioned, IMP:308-330 */
        if (p->filter_pinned) {
            for (int32_t i = 0; i < N; ++i)
                if (SFX(is_pinned)(p, i)) dV[3 * (size_t)i] = dV[3 * (size_t)i + 1] = dV[3 * (size_t)i + 2] = 0;
        }
        for (int32_t i = 0; i < N; ++i) {
            REAL Ax[3];
            SFX(matvec)(A9 + 9 * (size_t)i, dV + 3 * (size_t)i, Ax);
            for (int k = 0; k < 3; ++k) r[3 * (size_t)i + k] = b[3 * (size_t)i + k] - Ax[k];
            if (p->filter_pinned && SFX(is_pinned)(p, i)) r[3 * (size_t)i] = r[3 * (size_t)i + 1] = r[3 * (size_t)i + 2] = 0;
        }
        for (size_t k = 0; k < n3; ++k) {
            d[k] = Pinv[k] * r[k];
            Pr[k] = P[k] * r[k];
        }
        double delta_new = SFX(dot)(p, r, Pr, N);
        const double delta0 = delta_new;
        const double thresh = p->dot_fp64 ? (double)eps2 * delta0 : (double)(REAL)(eps2 * (REAL)delta0);
        int32_t it = 0;
        while (it < p->i_max && delta_new > thresh) {
            for (int32_t i = 0; i < N; ++i) SFX(matvec)(A9 + 9 * (size_t)i, d + 3 * (size_t)i, q + 3 * (size_t)i);
            const double dq = SFX(dot)(p, d, q, N);
            const REAL alpha = p->dot_fp64 ? (REAL)(delta_new / dq) : (REAL)delta_new / (REAL)dq;
            for (size_t k = 0; k < n3; ++k) {
                dV[k] = dV[k] + d[k] * alpha;
                r[k] = r[k] - q[k] * alpha;
            }
            const double delta_old = delta_new;
            delta_new = SFX(dot)(p, r, r, N);
            const REAL beta = p->dot_fp64 ? (REAL)(delta_new / delta_old) : (REAL)delta_new / (REAL)delta_old;
            for (size_t k = 0; k < n3; ++k) d[k] = r[k] + d[k] * beta;
            ++it;
        }
        if (iters) iters[step] = it;
        if (rel_residual) rel_residual[step] = delta0 > 0 ? sqrt(delta_new / delta0) : 0.0;
        /* IMP:790-797 */
        for (int32_t i = 0; i < N; ++i) {
            for (int k = 0; k < 3; ++k) V[3 * (size_t)i + k] += dV[3 * (size_t)i + k] * dt;
            for (int k = 0; k < 3; ++k) X[3 * (size_t)i + k] += dt * V[3 * (size_t)i + k];
            if (X[3 * (size_t)i + 1] < 0) X[3 * (size_t)i + 1] = 0;
        }
        if (p->passes & 1) SFX(ellipsoid_pass)(p, X, V);
        if (p->passes & 2) SFX(provot_pass)(p, X, V);
    }
    free(F); free(A9); free(b); free(P); free(Pinv); free(r); free(d); free(q); free(Pr);
    return 0;
}
