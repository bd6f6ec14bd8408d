/* Test infrastructure: the reference's cloth lattice and spring list (InitGL,
 * OpenCloth_Implicit/OpenCloth_Implicit/main.cpp:497-565, AddSpring main.cpp:370-380),
 * restated for the CPU arms of the benchmark so that they build their inputs without
 * the GPU library.
 *
 * The lattice is laid in the x-y plane with row 0 on top (the workloads' convention):
 *   x = ((i / (cols-1)) * 2 - 1) * size/2,  y = (size + 1) - (j / (rows-1)) * size,  z = 0
 * for vertex j * cols + i.  Springs follow InitGL's loops in order (horizontal
 * structural, vertical structural, two shear springs per quad, bend along rows plus one
 * repeat of the last per row, bend along columns plus one repeat per column), each with
 * its rest length taken from the exact lattice (main.cpp:377-378).  Afterwards every
 * coordinate gets i.i.d. N(0, (jitter * size / (cols-1))^2) noise from a splitmix64
 * stream (Steele, Lea and Flood, 2014) through the Box-Muller transform, two normals per
 * pair of uniforms, in coordinate order.  The same seed gives the same floats as the
 * library's own builder (tests/test_oracle.py compares the two). */
#include <math.h>
#include <stdint.h>

#include "oc_oracle.h"

static uint64_t next_u64(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* A uniform double in (0, 1): the top 53 bits, offset by half a step. */
static double open_unit(uint64_t* s) { return ((double)(next_u64(s) >> 11) + 0.5) / 9007199254740992.0; }

int64_t ocr_grid_spring_count(int32_t cols, int32_t rows) {
    if (cols < 3 || rows < 3) return -1;
    const int64_t u = cols, v = rows;
    return 2 * v * (u - 1) + 2 * u * (v - 1) + 2 * (v - 1) * (u - 1);
}

int ocr_grid_build(int32_t cols, int32_t rows, float size, const float ks[3], const float kd[3], float jitter,
                   uint64_t seed, float* X, ocr_spring* springs) {
    const int64_t ns = ocr_grid_spring_count(cols, rows);
    if (ns < 0 || !(size > 0.0f) || !(jitter >= 0.0f)) return 1;
    const int32_t u = cols, v = rows;
    const float half = size / 2.0f;
    for (int32_t j = 0; j < v; ++j)
        for (int32_t i = 0; i < u; ++i) {
            float* p = X + 3 * ((int64_t)j * u + i);
            p[0] = (((float)i / (float)(u - 1)) * 2.0f - 1.0f) * half;
            p[1] = (size + 1.0f) - ((float)j / (float)(v - 1)) * size;
            p[2] = 0.0f;
        }
    int64_t n = 0;
#define OCR_SPRING(A, B, T)                                                        \
    do {                                                                            \
        ocr_spring* s_ = springs + n++;                                             \
        const int32_t a_ = (A), b_ = (B);                                           \
        const float dx = X[3 * (int64_t)a_] - X[3 * (int64_t)b_];                   \
        const float dy = X[3 * (int64_t)a_ + 1] - X[3 * (int64_t)b_ + 1];           \
        const float dz = X[3 * (int64_t)a_ + 2] - X[3 * (int64_t)b_ + 2];           \
        s_->p1 = a_;                                                                \
        s_->p2 = b_;                                                                \
        s_->rest = sqrtf(dx * dx + dy * dy + dz * dz);                              \
        s_->ks = ks[T];                                                             \
        s_->kd = kd[T];                                                             \
        s_->type = (T);                                                             \
    } while (0)
    for (int32_t r = 0; r < v; ++r) /* horizontal structural, main.cpp:531-535 */
        for (int32_t c = 0; c < u - 1; ++c) OCR_SPRING(r * u + c, r * u + c + 1, 0);
    for (int32_t c = 0; c < u; ++c) /* vertical structural, main.cpp:538-541 */
        for (int32_t r = 0; r < v - 1; ++r) OCR_SPRING(r * u + c, (r + 1) * u + c, 0);
    for (int32_t r = 0; r < v - 1; ++r) /* shear, main.cpp:545-549 */
        for (int32_t c = 0; c < u - 1; ++c) {
            OCR_SPRING(r * u + c, (r + 1) * u + c + 1, 1);
            OCR_SPRING((r + 1) * u + c, r * u + c + 1, 1);
        }
    for (int32_t r = 0; r < v; ++r) { /* bend along rows, main.cpp:553-558 */
        for (int32_t c = 0; c < u - 2; ++c) OCR_SPRING(r * u + c, r * u + c + 2, 2);
        OCR_SPRING(r * u + u - 3, r * u + u - 1, 2);
    }
    for (int32_t c = 0; c < u; ++c) { /* bend along columns, main.cpp:559-564 */
        for (int32_t r = 0; r < v - 2; ++r) OCR_SPRING(r * u + c, (r + 2) * u + c, 2);
        OCR_SPRING((v - 3) * u + c, (v - 1) * u + c, 2);
    }
#undef OCR_SPRING
    if (jitter > 0.0f) {
        const double sigma = (double)jitter * (double)size / (double)(u - 1);
        const int64_t n3 = 3 * (int64_t)u * v;
        uint64_t state = seed;
        for (int64_t k = 0; k < n3; k += 2) {
            const double rad = sqrt(-2.0 * log(open_unit(&state)));
            const double ang = 6.283185307179586 * open_unit(&state);
            X[k] += (float)(sigma * rad * cos(ang));
            if (k + 1 < n3) X[k + 1] += (float)(sigma * rad * sin(ang));
        }
    }
    return n == ns ? 0 : 1;
}
