/* Test infrastructure: CPU restatement of the FEM demo's block-sparse conjugate
 * gradient, ConjugateGradientSolver in
 * OpenCloth_CoRotated_Linear_FEM/OpenCloth_CoRotated_Linear_FEM/main.cpp (FEM:837-922).
 * Included by oc_oracle.c with REAL = float (_f32) and REAL = double (_f64).
 *
 * The reference's quirks are kept:
 *   - the unknown is V itself, warm-started from its current value (FEM:847-857);
 *   - fixed rows are skipped everywhere, but their `previous` entries (zero, never
 *     written) still enter the other rows' products (FEM:871-879);
 *   - d = r.r and d2 = p.(A p) are summed in the same pass (FEM:881-882) and clamped to
 *     `tiny` in magnitude before division (FEM:885-886, 908-909);
 *   - the early exit `i >= i_max && d1 < tolerence` (FEM:905) can never fire inside
 *     the loop, so exactly i_max iterations run;
 *   - the block product is prod.x = m[0][0] x + m[0][1] y + m[0][2] z, ... (FEM:873-875),
 *     i.e. block element m[c][r] (stored at 3c + r) multiplies component r of the
 *     vector into component c, summed left to right; a row's products are added in
 *     ascending column order (std::map iteration, FEM:120, FEM:868-878).
 * dot_fp64 = 0 sums the dot products in REAL sequentially, as the reference does; 1
 * sums each row's REAL dot term in double (the GPU's arithmetic), and the scalars
 * d3 = d / d2 and d4 = d1 / d are double quotients rounded to REAL. */

static void SFX(bsr_mv)(const float* m, const REAL* v, REAL* out) {
    out[0] = (REAL)m[0] * v[0] + (REAL)m[1] * v[1] + (REAL)m[2] * v[2];
    out[1] = (REAL)m[3] * v[0] + (REAL)m[4] * v[1] + (REAL)m[5] * v[2];
    out[2] = (REAL)m[6] * v[0] + (REAL)m[7] * v[1] + (REAL)m[8] * v[2];
}

static REAL SFX(bsr_dot)(const REAL* a, const REAL* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

int SFX(ocr_bsr_cg)(int32_t n, const int32_t* row_ptr, const int32_t* col, const float* blocks, const REAL* b,
                    REAL* x, const uint8_t* fixed, int32_t i_max, float tiny_f, int32_t dot_fp64, REAL* residual_out) {
    const size_t n3 = 3 * (size_t)n;
    REAL* r = (REAL*)calloc(n3 + 1, sizeof(REAL));
    REAL* p = (REAL*)calloc(n3 + 1, sizeof(REAL));
    REAL* q = (REAL*)calloc(n3 + 1, sizeof(REAL));
    if (!r || !p || !q) {
        free(r); free(p); free(q);
        return -1;
    }
    const REAL tiny = (REAL)tiny_f;
    /* r = b - A V, p = r (FEM:841-859) */
    for (int32_t k = 0; k < n; ++k) {
        if (fixed && fixed[k]) continue;
        REAL* rk = r + 3 * (size_t)k;
        rk[0] = b[3 * (size_t)k];
        rk[1] = b[3 * (size_t)k + 1];
        rk[2] = b[3 * (size_t)k + 2];
        for (int32_t e = row_ptr[k]; e < row_ptr[k + 1]; ++e) {
            REAL prod[3];
            SFX(bsr_mv)(blocks + 9 * (size_t)e, x + 3 * (size_t)col[e], prod);
            rk[0] -= prod[0];
            rk[1] -= prod[1];
            rk[2] -= prod[2];
        }
        p[3 * (size_t)k] = rk[0];
        p[3 * (size_t)k + 1] = rk[1];
        p[3 * (size_t)k + 2] = rk[2];
    }
    for (int32_t i = 0; i < i_max; ++i) {
        REAL d = 0, d2 = 0;
        double dd = 0, dd2 = 0;
        for (int32_t k = 0; k < n; ++k) { /* FEM:865-883 */
            if (fixed && fixed[k]) continue;
            REAL* qk = q + 3 * (size_t)k;
            qk[0] = qk[1] = qk[2] = 0;
            for (int32_t e = row_ptr[k]; e < row_ptr[k + 1]; ++e) {
                REAL prod[3];
                SFX(bsr_mv)(blocks + 9 * (size_t)e, p + 3 * (size_t)col[e], prod);
                qk[0] += prod[0];
                qk[1] += prod[1];
                qk[2] += prod[2];
            }
            const REAL t = SFX(bsr_dot)(r + 3 * (size_t)k, r + 3 * (size_t)k);
            const REAL t2 = SFX(bsr_dot)(p + 3 * (size_t)k, qk);
            if (dot_fp64) {
                dd += (double)t;
                dd2 += (double)t2;
            } else {
                d += t;
                d2 += t2;
            }
        }
        REAL d3;
        if (dot_fp64) {
            if (fabs(dd2) < (double)tiny) dd2 = (double)tiny;
            d3 = (REAL)(dd / dd2);
        } else {
            if (fabs(d2) < tiny) d2 = tiny; /* FEM:885-886 */
            d3 = d / d2;
        }
        REAL d1 = 0;
        double dd1 = 0;
        for (int32_t k = 0; k < n; ++k) { /* FEM:891-901 */
            if (fixed && fixed[k]) continue;
            for (int c = 0; c < 3; ++c) {
                const size_t e = 3 * (size_t)k + c;
                x[e] += p[e] * d3;
                r[e] -= q[e] * d3;
            }
            const REAL t = SFX(bsr_dot)(r + 3 * (size_t)k, r + 3 * (size_t)k);
            if (dot_fp64)
                dd1 += (double)t;
            else
                d1 += t;
        }
        REAL d4; /* FEM:905-911; the exit test cannot fire for i < i_max */
        if (dot_fp64) {
            if (fabs(dd) < (double)tiny) dd = (double)tiny;
            d4 = (REAL)(dd1 / dd);
        } else {
            if (fabs(d) < tiny) d = tiny;
            d4 = d1 / d;
        }
        for (int32_t k = 0; k < n; ++k) { /* FEM:913-917 */
            if (fixed && fixed[k]) continue;
            for (int c = 0; c < 3; ++c) {
                const size_t e = 3 * (size_t)k + c;
                p[e] = r[e] + p[e] * d4;
            }
        }
    }
    if (residual_out)
        for (size_t e = 0; e < n3; ++e) residual_out[e] = r[e];
    free(r);
    free(p);
    free(q);
    return 0;
}
