/* Test infrastructure: CPU restatement of the reference's implicit mass-spring step.
 *
 * Only tests/, bench.py's cpu_baseline / reference arm and __graft_entry__.smoke()
 * use this, and only as the reference results are compared against.  The library
 * (opencloth_gb300/) never links it.
 *
 * It restates, operation for operation and in the same rounding order (compile with
 * -ffp-contract=off), the reference's
 *   ComputeForces                          OpenCloth_Implicit/.../main.cpp:698-735
 *   CalcForceDerivatives                   main.cpp:737-772
 *   IntegrateImplicit (assembly + update)  main.cpp:775-798
 *   SolveConjugateGradientPreconditioned   main.cpp:308-330
 * with the glm 0.9.0 primitives those use (length, normalize = x * (1/sqrt(x.x)),
 * outerProduct, column-major mat3 * vec3).  Parity is pinned by tests that compare it
 * bit for bit with the reference itself built headless (oracle/build_ref.sh).
 *
 * Generalisations (each reduces to the reference when left at its default):
 *   pinned mask      NULL -> the reference's hard-coded pins {0, num_x}
 *   mass             NULL -> 1 (the reference's M = I, gravity added as a force)
 *   ext_force        NULL -> none (added after damping)
 *   dot_fp64         0 -> FP32 sequential dots as the reference; 1 -> per-vertex FP32
 *                    dot terms summed in FP64 (what the GPU solver does)
 *   filter_pinned    0 -> no filter (the reference); 1 -> pinned rows of the warm start
 *                    and of the residual are zeroed before the CG (the GPU solver)
 *   passes           0 -> ComputeForces + IntegrateImplicit only; bits add the ellipsoid
 *                    collision and the Provot correction of StepPhysics
 */
#ifndef OC_ORACLE_H
#define OC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ocr_spring {
    int32_t p1, p2;
    float rest, ks, kd;
    int32_t type;
} ocr_spring;

typedef struct ocr_params {
    int32_t n_vertices, n_springs;
    const ocr_spring* springs;
    const uint8_t* pinned; /* n_vertices flags, or NULL for {0, num_x} */
    int32_t num_x;
    const float* mass;      /* n_vertices, or NULL */
    const float* ext_force; /* 3 * n_vertices, or NULL */
    float gravity[3];
    float damping;
    int32_t i_max;
    float eps;
    int32_t dot_fp64;
    int32_t filter_pinned;
    /* Passes after the update, in StepPhysics' order (IMP:873-880): bit 1
     * EllipsoidCollision (IMP:824-848), bit 2 ApplyProvotDynamicInverse (IMP:800-823). */
    int32_t passes;
    /* Held in double so the FP64 flavour gets the FP64 reference's dmat4 values; the
     * FP32 flavour rounds them to float (exact for matrices that came from floats). */
    double ellipsoid[16];     /* object -> world, glm column-major (IMP:583-585) */
    double ellipsoid_inv[16]; /* its inverse (IMP:586) */
    double provot_ratio;      /* 1.01 in the reference (IMP:808) */
} ocr_params;

/* FP32 flavour: state arrays are 3 * n_vertices floats, AoS (x, y, z). */
void ocr_compute_forces_f32(const ocr_params* p, const float* X, const float* V, float* F);
void ocr_assemble_f32(const ocr_params* p, float dt, const float* X, const float* V, const float* F, float* A9,
                      float* b);
int ocr_step_f32(const ocr_params* p, float dt, int32_t n_steps, float* X, float* V, float* dV, int32_t* iters,
                 double* rel_residual);
/* The passes of p->passes alone, on (X, V) in place: EllipsoidCollision then
 * ApplyProvotDynamicInverse (IMP:877-880). */
void ocr_passes_f32(const ocr_params* p, float* X, float* V);

/* FP64 flavour of the same method (the reference built with double everywhere). */
void ocr_compute_forces_f64(const ocr_params* p, const double* X, const double* V, double* F);
void ocr_assemble_f64(const ocr_params* p, double dt, const double* X, const double* V, const double* F,
                      double* A9, double* b);
int ocr_step_f64(const ocr_params* p, double dt, int32_t n_steps, double* X, double* V, double* dV,
                 int32_t* iters, double* rel_residual);
void ocr_passes_f64(const ocr_params* p, double* X, double* V);

/* COUPLED Jacobian mode (oc_coupled_impl.h; no counterpart in the reference):
 * Baraff-Witkin coupling of the per-spring blocks into one SPD block-sparse system,
 * block-Jacobi PCG, V += dV.  Pins are p->pinned or {0, num_x}, always filtered; dot
 * products sum REAL per-vertex terms in double; p->dot_fp64 / filter_pinned unused.
 * matvec: y = A w (no pin filter).  system: diagonal blocks D6, their inverses P6 (6
 * per vertex: a00 a01 a02 a11 a12 a22; either may be NULL) and b, from F. */
void ocr_coupled_matvec_f32(const ocr_params* p, float h, const float* X, const float* w, float* y);
void ocr_coupled_system_f32(const ocr_params* p, float h, const float* X, const float* V, const float* F, float* D6,
                            float* P6, float* b);
int ocr_coupled_step_f32(const ocr_params* p, float dt, int32_t n_steps, float* X, float* V, float* dV,
                         int32_t* iters, double* rel_residual, uint32_t* flags);
void ocr_coupled_matvec_f64(const ocr_params* p, double h, const double* X, const double* w, double* y);
void ocr_coupled_system_f64(const ocr_params* p, double h, const double* X, const double* V, const double* F,
                            double* D6, double* P6, double* b);
int ocr_coupled_step_f64(const ocr_params* p, double dt, int32_t n_steps, double* X, double* V, double* dV,
                         int32_t* iters, double* rel_residual, uint32_t* flags);

/* The FEM demo's block-sparse CG, FEM:837-922 (oc_bsr_impl.h): block rows in CSR with
 * ascending columns, blocks of 9 floats (m[c][r] at 3c + r), fixed rows skipped; x (the
 * unknown V) is the warm start in and the solution out; residual_out (3n, may be NULL)
 * receives the final residual.  Exactly i_max iterations. */
int ocr_bsr_cg_f32(int32_t n, const int32_t* row_ptr, const int32_t* col, const float* blocks, const float* b,
                   float* x, const uint8_t* fixed, int32_t i_max, float tiny, int32_t dot_fp64, float* residual_out);
int ocr_bsr_cg_f64(int32_t n, const int32_t* row_ptr, const int32_t* col, const float* blocks, const double* b,
                   double* x, const uint8_t* fixed, int32_t i_max, float tiny, int32_t dot_fp64,
                   double* residual_out);

/* FP64 adjoint of n_steps steps from (X0, V0) with a zero warm start (oc_adjoint.c):
 * given dL/dX_T, dL/dV_T (NULL = 0), returns the final state and dL/dX0, dL/dV0,
 * dL/dKs, dL/dKd (per spring) and dL/d(external force) (per vertex, constant in time).
 * The linear solve is differentiated as an exact solve. */
int ocr_adjoint_f64(const ocr_params* p, double dt, int32_t n_steps, const double* X0, const double* V0,
                    const double* gX_T, const double* gV_T, double* X_T, double* V_T, double* gX0, double* gV0,
                    double* gKs, double* gKd, double* gExt);

/* InitGL's lattice and spring list (oc_grid.c): cols x rows vertices in the x-y plane,
 * springs in creation order with rest lengths from the exact lattice, then seeded
 * position jitter of sigma = jitter * spacing.  ocr_grid_spring_count gives the spring
 * count (-1 below 3 x 3); ocr_grid_build returns 0 on success. */
int64_t ocr_grid_spring_count(int32_t cols, int32_t rows);
int ocr_grid_build(int32_t cols, int32_t rows, float size, const float ks[3], const float kd[3], float jitter,
                   uint64_t seed, float* X, ocr_spring* springs);

#ifdef __cplusplus
}
#endif
#endif
