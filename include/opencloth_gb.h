/*
 * opencloth_gb.h — C ABI of the GB300 implicit mass-spring cloth step.
 *
 * Drop-in for the step of OpenCloth_Implicit (OpenCloth_Implicit/OpenCloth_Implicit/
 * main.cpp, cited below as IMP).  The reference step is a set of free functions on
 * globals:
 *
 *   ComputeForces()            IMP:698   -> oc_step (force gather) / oc_compute_forces
 *   CalcForceDerivatives()     IMP:737   -> oc_step (Jacobians)    / oc_assemble
 *   IntegrateImplicit(dt)      IMP:775   -> oc_step (assembly, PCG, update)
 *   StepPhysics(dt)            IMP:873   -> oc_step (ComputeForces + IntegrateImplicit)
 *   AddSpring(a,b,ks,kd,type)  IMP:370   -> oc_spring records in oc_cloth_desc
 *   globals X, V, dV           IMP:80-81, IMP:361 -> oc_set_state / oc_get_state
 *
 * Conventions
 *   - Every entry point returns an oc_status (0 = OC_OK); no C++ exception crosses the
 *     ABI.  oc_last_error() gives a message for the last failing call on a handle.
 *   - Host buffers passed in are copied; the library owns all device memory.
 *   - One CUDA stream per handle (library-owned unless the caller supplies one).  A
 *     handle is not thread-safe; different handles are independent.
 *   - Vectors are packed AoS float triples (x, y, z) over all instances of a handle,
 *     instance k occupying vertices [vertex_offset(k), vertex_offset(k) + n_vertices).
 *   - Device-side waits are bounded; a wait that gives up surfaces as
 *     OC_ERR_DEVICE_TIMEOUT.
 */
#ifndef OPENCLOTH_GB_H
#define OPENCLOTH_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
typedef int32_t oc_status;
#define OC_OK 0
#define OC_ERR_INVALID_ARGUMENT 1 /* NULL handle/pointer, non-positive size, bad enum */
#define OC_ERR_BAD_INDEX 2        /* spring endpoint or pinned index outside [0, n_vertices) */
#define OC_ERR_NON_FINITE 3       /* NaN or Inf in positions, velocities or parameters */
#define OC_ERR_DEGENERATE 4       /* zero-length spring (the reference divides by it, IMP:720-727) */
#define OC_ERR_CUDA 5             /* a CUDA runtime call failed; see oc_last_error */
#define OC_ERR_OUT_OF_MEMORY 6
#define OC_ERR_UNSUPPORTED 7      /* option not available for this configuration */
#define OC_ERR_DEVICE_TIMEOUT 8   /* a bounded device-side wait gave up */

/* ---- per-instance result flags (oc_get_stats) -------------------------------------- */
#define OC_FLAG_NOT_CONVERGED 1u /* CG stopped at cg_max_iter (normal for the reference's i_max=10) */
#define OC_FLAG_BREAKDOWN 2u     /* CG direction with d.(A d) <= 0 or non-finite: system not SPD */
#define OC_FLAG_NON_FINITE 4u    /* a non-finite value appeared in the step */

/* ---- spring: mirrors `struct Spring` IMP:70-75 ------------------------------------ */
#define OC_STRUCTURAL_SPRING 0 /* IMP:98 */
#define OC_SHEAR_SPRING 1      /* IMP:99 */
#define OC_BEND_SPRING 2       /* IMP:100 */

typedef struct oc_spring {
    int32_t p1, p2;    /* vertex indices within the instance */
    float rest_length; /* IMP:378: length at creation */
    float ks, kd;      /* stiffness and damping (kd negative by the reference's convention) */
    int32_t type;      /* OC_*_SPRING, informational */
} oc_spring;

/* ---- Jacobian modes -------------------------------------------------------------- */
/* REFERENCE: vertex i takes spring i's df/dx, df/dv (IMP:782-783 index the per-spring
 * arrays by vertex), giving a block-diagonal system solved by the reference's PCG. */
#define OC_JAC_REFERENCE 0
/* COUPLED: Baraff-Witkin coupling on the reference's force model (no counterpart in the
 * reference).  Every spring adds B = h kdn nn^T + h^2 Kt at (p1,p1), (p2,p2) and -B at
 * (p1,p2), (p2,p1), with Kt = ksn [nn^T + max(1 - L/l, 0)(I - nn^T)], ksn = max(ks, 0),
 * kdn = max(-kd, 0): positive semi-definite by construction, so the system
 * (m + h max(-c, 0)) I + sum B is SPD.  b = h (F - h sum Kt (v_i - v_j)); block-Jacobi
 * PCG to cg_tol; V += dV.  Streamed executor only; no adjoint, no oc_assemble. */
#define OC_JAC_COUPLED 1

/* Upper bound on cg_max_iter: the device-driven CG loop of a step runs at most this
 * many passes, so every step ends. */
#define OC_MAX_CG_ITER 100000

/* ---- one cloth (one instance) ----------------------------------------------------- */
typedef struct oc_cloth_desc {
    int32_t n_vertices;
    int32_t n_springs;
    const oc_spring* springs;  /* n_springs records, in the reference's creation order */
    const float* mass;         /* n_vertices, or NULL for 1.0 (the reference: M = I, IMP:363) */
    const int32_t* pinned;     /* indices of pinned vertices (the reference pins 0 and numX) */
    int32_t n_pinned;
    const float* ext_force;    /* 3*n_vertices constant external force, or NULL */
    float gravity[3];          /* IMP:108, added as m*g to unpinned vertices */
    float velocity_damping;    /* DEFAULT_DAMPING, IMP:104 (-0.125) */
    int32_t cg_max_iter;       /* i_max, IMP:128; at most OC_MAX_CG_ITER */
    float cg_tol;              /* EPS, IMP:126; the CG stops when r.r <= EPS^2 * delta0 */
    int32_t jacobian_mode;     /* OC_JAC_* */
    /* Passes after the update, in StepPhysics' order (IMP:873-880); 0 = none, i.e.
     * ComputeForces + IntegrateImplicit only.  Stepping only: oc_tape_forward refuses them. */
    int32_t passes;            /* OC_PASS_* bits */
    float ellipsoid[16];       /* OC_PASS_ELLIPSOID: object -> world, column-major (IMP:583-585) */
    float ellipsoid_inv[16];   /* its inverse as the caller computed it (IMP:586) */
    float provot_ratio;        /* OC_PASS_PROVOT: stretch limit over rest length; 0 -> 1.01 (IMP:808) */
} oc_cloth_desc;

/* ---- passes after the update ------------------------------------------------------- */
/* EllipsoidCollision (IMP:824-848): a vertex inside the unit sphere of the ellipsoid's
 * object space is moved to its surface and its velocity zeroed (pinned vertices too). */
#define OC_PASS_ELLIPSOID 1
/* ApplyProvotDynamicInverse (IMP:800-823): a spring longer than provot_ratio x rest moves
 * its endpoints' velocities together by half the excess; a pinned p1 leaves the whole
 * correction to p2, else a pinned p2 leaves it to p1. */
#define OC_PASS_PROVOT 2

/* ---- executors ---------------------------------------------------------------------- */
#define OC_EXEC_AUTO 0     /* resident kernels for instances that fit on chip, streamed otherwise */
#define OC_EXEC_STREAMED 1 /* multi-kernel step, CG loop in a CUDA-graph WHILE node */
#define OC_EXEC_RESIDENT 2 /* one cluster of CTAs per instance, the whole step on chip */
#define OC_EXEC_PLAIN 3    /* one launch sequence per cloth, CG loop driven from the host */

typedef struct oc_options {
    int32_t executor;        /* OC_EXEC_* */
    int32_t device;          /* CUDA device ordinal */
    void* stream;            /* cudaStream_t to use, or NULL for a library-owned stream */
    int32_t use_graph;       /* 1: replay the step as a CUDA graph (default) */
    int32_t block_threads;   /* 0: tuned default */
    int32_t vertices_per_thread; /* 0: tuned default (streamed executor) */
    int32_t resident_max_vertices; /* 0: tuned default; larger instances are streamed */
} oc_options;

typedef struct oc_solver oc_solver;

void oc_default_options(oc_options* opts);

/* Validate, pack and upload n_instances cloths.  Positions and velocities start at 0;
 * set them with oc_set_state.  Fails with OC_ERR_BAD_INDEX / OC_ERR_NON_FINITE /
 * OC_ERR_DEGENERATE on bad input, without allocating device memory. */
oc_status oc_create(const oc_cloth_desc* descs, int32_t n_instances, const oc_options* opts, oc_solver** out);
void oc_destroy(oc_solver* s);
const char* oc_last_error(const oc_solver* s);
const char* oc_status_string(oc_status status);

/* Sizes of a handle. */
oc_status oc_get_counts(const oc_solver* s, int64_t* total_vertices, int64_t* total_springs, int32_t* n_instances);
oc_status oc_get_vertex_offsets(const oc_solver* s, int64_t* offsets /* n_instances + 1 */);

/* State = X, V and the CG warm start dV (IMP:361, reused as the initial guess at
 * IMP:788).  Host pointers; any may be NULL to leave that array unchanged/unread.
 * Synchronous with respect to the handle's stream.  oc_set_state stages the arrays and
 * checks them on the device first: a NaN or Inf fails with OC_ERR_NON_FINITE and leaves
 * the state unchanged. */
oc_status oc_set_state(oc_solver* s, const float* X, const float* V, const float* dV);
oc_status oc_get_state(oc_solver* s, float* X, float* V, float* dV);
/* Same with device pointers (packed float triples); enqueued on the handle's stream,
 * with no wait and no check of the values. */
oc_status oc_set_state_device(oc_solver* s, const float* X, const float* V, const float* dV);
oc_status oc_get_state_device(oc_solver* s, float* X, float* V, float* dV);

/* n_steps x { ComputeForces(); IntegrateImplicit(dt); [passes] } for every instance.
 * Asynchronous: enqueued on the handle's stream. */
oc_status oc_step(oc_solver* s, float dt, int32_t n_steps);
oc_status oc_synchronize(oc_solver* s);
/* The reference's StepPhysics on host arrays (IMP:873-880 over the globals X, V of
 * IMP:80-81): X and V (packed float triples, either may be NULL) are copied in, n_steps
 * steps run, and X and V are copied back out.  The input is staged and checked on the
 * device before it is committed (one wait), then the step and the copy back out end
 * with a second wait.  A NaN or Inf in the input fails with OC_ERR_NON_FINITE and leaves
 * both the device state and the caller's arrays unchanged. */
oc_status oc_step_host(oc_solver* s, float dt, int32_t n_steps, float* X, float* V);
/* Set the passes after the update (OC_PASS_* bits) of one cloth (instance >= 0) or of
 * every cloth (-1); the matrices and ratio stay those given at oc_create.  Waits for the
 * handle's stream; the next oc_step rebuilds its graph. */
oc_status oc_set_passes(oc_solver* s, int32_t instance, int32_t passes);
/* Run the given passes once on the current state of every cloth, ellipsoid first, with
 * no step: the reference's EllipsoidCollision (IMP:824) and ApplyProvotDynamicInverse
 * (IMP:800) called on their own.  Asynchronous on the handle's stream. */
oc_status oc_apply_passes(oc_solver* s, int32_t passes);

/* ---- interaction and constraints (device state, on the handle's stream) --------------- */
/* The reference's picking loop (IMP:399-405): the lowest vertex index of cloth `instance`
 * (instance-local) whose distance to `point` is below `radius` (the reference uses 0.1),
 * or -1.  Waits for the handle's stream. */
oc_status oc_pick_vertex(oc_solver* s, int32_t instance, const float point[3], double radius, int32_t* index);
/* The reference's drag of a picked vertex (IMP:433-438): V = 0; X.x += delta[0];
 * X.y += delta[1] only if the result stays > 0; X.z += delta[2].  `index` is
 * instance-local.  (The reference's delta is Right[0] valX, Up[1] valY and
 * Right[2] valX + Up[2] valY from the view, IMP:424-438.) */
oc_status oc_drag_vertex(oc_solver* s, int32_t instance, int32_t index, const float delta[3]);
/* Overwrite the positions and/or velocities (either may be NULL) of n distinct vertices,
 * given by handle-global index, from host float triples: per-step position/velocity
 * constraints.  Masses and pin flags are kept. */
oc_status oc_set_vertices(oc_solver* s, int32_t n, const int64_t* indices, const float* X, const float* V);
/* Replace the pin set of one cloth (instance-local indices; n_pins may be 0).  Takes effect
 * from the next step; invalidates the tape of oc_tape_forward. */
oc_status oc_set_pins(oc_solver* s, int32_t instance, const int32_t* pins, int32_t n_pins);

/* Per-instance results of the last step: CG iterations, relative residual
 * sqrt(delta_new / delta0), OC_FLAG_* bits.  Any pointer may be NULL. */
oc_status oc_get_stats(oc_solver* s, int32_t* cg_iters, double* rel_residual, uint32_t* flags);

/* Kernels of the step (force/assembly, CG direction, CG update, integration)
 * launched by this handle so far, counted on the device for the graph's CG loop. */
oc_status oc_get_launch_count(oc_solver* s, int64_t* kernels_launched);

/* ComputeForces alone on the current state (IMP:698-735): F, packed float triples. */
oc_status oc_compute_forces(oc_solver* s, float* F);
/* ComputeForces + CalcForceDerivatives + assembly on the current state (IMP:737-786):
 * A as 9 floats per vertex (glm column-major) and b as float triples. */
oc_status oc_assemble(oc_solver* s, float dt, float* A9, float* b);

/* Per-kernel timing of n_steps un-graphed steps (CUDA events around every launch on the
 * handle's stream; the CG loop is driven from the host).  Per kernel: its name in a
 * 32-byte slot of names (up to max_kernels), total ms, launches, and the algorithmic
 * bytes it moved — each array element it must read or write counted once, for the
 * instances still iterating: per vertex k_assemble 120 B + 32 B per spring, k_cg_dir
 * 36 B on the first pass of a step and 60 B after, k_cg_update 84 B, k_integrate 76 B,
 * k_resident (the whole CG of a cloth in shared memory, plus the update) 136 B.
 * *n_kernels receives the number of kernels reported. */
oc_status oc_profile_steps(oc_solver* s, float dt, int32_t n_steps, int32_t max_kernels, char* names,
                           double* ms_total, int64_t* launches, double* algorithmic_bytes, int32_t* n_kernels);

/* ---- differentiation (no counterpart in the reference) ------------------------------ */
/* Per-spring Ks / Kd of the handle (host arrays over all springs, instance by instance
 * in creation order; either may be NULL to keep it). */
oc_status oc_set_spring_params(oc_solver* s, const float* ks, const float* kd);
/* A constant per-vertex external force added to every unpinned vertex (host, 3 floats
 * per vertex), for cloths created without one too. */
oc_status oc_set_ext_force(oc_solver* s, const float* ext);
/* Run n_steps steps from the current state, taped for oc_tape_backward.  Two tapes:
 *   OC_TAPE_REPLAY     the solution dV of every step (12 bytes per vertex and step) and,
 *                      per cloth, its state (X, V) every `every` steps, the interval chosen
 *                      per cloth.  Given dV the update is elementwise, so the reverse pass
 *                      rebuilds every state by replaying it from the checkpoint before,
 *                      bit for bit, without re-running the step's assembly and CG.
 *   OC_TAPE_RECOMPUTE  every cloth's state every checkpoint_every steps; the reverse pass
 *                      re-runs the steps of each segment from its checkpoint, except the
 *                      last segments, which the budget's room keeps from the forward.
 * Every cloth's interval is checkpoint_every (0: ceil(sqrt(n_steps)), which minimises a
 * cloth's checkpoints plus segment buffer; the replay costs the same at any interval, so
 * that is also the fastest); oc_tape_forward_intervals sets them cloth by cloth.  With
 * budget_bytes > 0 the replay tape is used when it fits the budget, otherwise the
 * recompute tape, or OC_ERR_OUT_OF_MEMORY when even its checkpoints would exceed the
 * budget.  With budget_bytes <= 0: the replay tape, or the recompute tape (one segment
 * buffer) when the replay tape's buffers cannot be allocated.  Both tapes give the same
 * gradients bit for bit.  Fails with OC_ERR_UNSUPPORTED when a cloth has passes after the
 * update (the adjoint covers the implicit step only). */
#define OC_TAPE_REPLAY 0
#define OC_TAPE_RECOMPUTE 1
oc_status oc_tape_forward(oc_solver* s, float dt, int32_t n_steps, int32_t checkpoint_every, int64_t budget_bytes);
/* oc_tape_forward on the replay tape with the given interval of every cloth (every[i] >= 1,
 * instance order; an interval above n_steps is taken as n_steps), no budget. */
oc_status oc_tape_forward_intervals(oc_solver* s, float dt, int32_t n_steps, const int32_t* every);
/* The last tape's kind (OC_TAPE_*) and every cloth's interval (instance order); either
 * may be NULL.  OC_ERR_INVALID_ARGUMENT without a tape. */
oc_status oc_tape_layout(const oc_solver* s, int32_t* kind, int32_t* every);
/* Reverse pass of the last oc_tape_forward: given dL/dX and dL/dV (NULL = 0) of its final
 * state, returns dL/dX0, dL/dV0 (initial state), dL/dKs, dL/dKd (per spring) and dL/dext
 * (the constant external force); any output may be NULL.  Each step's state comes from the
 * tape (replayed or recomputed), its system's diagonal blocks are rebuilt from spring i
 * as the step formed them, and its linear solve is back-propagated by one CG on the same
 * symmetric system (exact-solve adjoint).  The handle's state is left at the final state. */
oc_status oc_tape_backward(oc_solver* s, const float* dL_dX, const float* dL_dV, float* dL_dX0, float* dL_dV0,
                           float* dL_dKs, float* dL_dKd, float* dL_dext);
/* The default interval of the last tape and its device bytes (checkpoints, segment
 * buffers, the replay tape's dV and the final state). */
oc_status oc_tape_info(const oc_solver* s, int32_t* checkpoint_every, int64_t* tape_bytes);
/* How the taped forward holds positions.  OC_TAPE_POSITIONS: as the step does (FP32
 * positions; the forward is the step itself).  OC_TAPE_DISPLACEMENT: as the start
 * positions plus an FP32 displacement, with each spring's elongation formed from its
 * start constants rounded from FP64, so that a cloth that moves little keeps the digits
 * of its motion (an FP32 position near 5 resolves about 5e-7; a gradient of a loss whose
 * residual is a few 1e-6 needs about 1e-9).  The displacement forward otherwise follows
 * the step's arithmetic; it needs the handle to run its adjoint solves through the
 * cooperative CG (no COUPLED cloth, a device with cooperative launch, persistence not
 * switched off; OC_ERR_UNSUPPORTED otherwise).  Setting the mode invalidates the tape. */
#define OC_TAPE_POSITIONS 0
#define OC_TAPE_DISPLACEMENT 1
oc_status oc_set_tape_mode(oc_solver* s, int32_t mode);
/* After a displacement-mode oc_tape_forward: the final displacement from the positions
 * the forward started from (host float triples).  A caller forms its loss residual from
 * it in FP64 (start positions + displacement - target). */
oc_status oc_tape_displacement(oc_solver* s, float* u);

/* ---- launch configuration and its autotuner ------------------------------------------ */
/* How a handle launches its step: which cloths run resident and in what CTA shape, whether
 * the resident kernel also assembles, whether up to 16 streamed cloths run their CG as one
 * cooperative launch, the force-gather variant, and the strip sweep of grid cloths.  None
 * of these changes the method; the resident kernel's reductions follow its CTA shape, so
 * results of different resident shapes can differ in the last bits (each shape is
 * deterministic).  No counterpart in the reference (its step has one serial code path). */
typedef struct oc_launch_config {
    int32_t resident_max_vertices; /* OC_EXEC_AUTO: cloths up to this many vertices run resident; 0: none */
    int32_t resident_vcta;         /* vertices per resident CTA: 256, 512, 1024 or 2048 */
    int32_t resident_threads;      /* threads per resident CTA: 128, 256 or 512, with vcta <= 4 x threads */
    int32_t resident_fused;        /* 1: resident cloths assemble inside the resident kernel */
    int32_t persist;               /* 1: the CG of the streamed cloths as one cooperative launch */
    int32_t gather_variant;        /* incidence-record force gather: 0 block-cooperative, 1..6 per vertex */
    int32_t strip;                 /* 1: grid cloths in the reference's spring order take the strip sweep */
    int32_t strip_rows;            /* rows per strip band (1 ... 64); 0: chosen from the work size */
    int32_t strip_variant;         /* strip CTAs per SM the registers are capped for: 2 or 3 */
} oc_launch_config;

oc_status oc_get_launch_config(const oc_solver* s, oc_launch_config* cfg);
/* Re-plan the handle's launches (tables, resident buckets, graphs are rebuilt; the state is
 * kept; the adjoint tape is invalidated).  OC_ERR_INVALID_ARGUMENT for a value outside the
 * ranges above, OC_ERR_UNSUPPORTED when the executor cannot honour it (OC_EXEC_RESIDENT
 * with a cloth above resident_max_vertices); the earlier configuration then stays. */
oc_status oc_set_launch_config(oc_solver* s, const oc_launch_config* cfg);

/* Times candidate configurations on the handle's own cloths and current state and keeps
 * the fastest: one knob at a time from the current configuration (strip sweep on/off, band
 * rows and register cap; resident size cut-off, CTA shape and fused assembly; persistent
 * or WHILE-loop CG; gather variant), each candidate replaying the step graph for about
 * 20 ms after two warm-up steps (CUDA events on the handle's stream); a candidate must be
 * 1% faster to replace the current one.  The state is saved first and restored after every
 * candidate, so tuning does not advance the simulation.  With cache_path (may be NULL) the
 * choice is looked up first by oc_tune_key's key and stored after tuning (flags:
 * OC_TUNE_USE_CACHE, OC_TUNE_STORE).  *chosen and *ms_per_step (either may be NULL) receive
 * the configuration in use and its measured time per step (0 when taken from the cache). */
#define OC_TUNE_USE_CACHE 1
#define OC_TUNE_STORE 2
oc_status oc_autotune(oc_solver* s, float dt, const char* cache_path, int32_t flags, oc_launch_config* chosen,
                      double* ms_per_step);

/* Host only.  The tuning cache key of a set of cloths on a GPU: the GPU's name and SM
 * count, and a 64-bit FNV-1a hash of the sorted per-cloth signatures (vertices, grid
 * shape, Jacobian mode, passes), written as text into key (key_size >= 96). */
oc_status oc_tune_key(const oc_cloth_desc* descs, int32_t n_instances, const char* gpu_name, int32_t sm_count,
                      char* key, int32_t key_size);
/* The handle's own key (its device's name and SM count). */
oc_status oc_tune_key_of(const oc_solver* s, char* key, int32_t key_size);
/* Host only.  The cache is a text file, one line per key: the key, the nine configuration
 * fields and the measured ms per step; a later line for a key replaces an earlier one.
 * *found is 1 when the key is present. */
oc_status oc_tune_cache_lookup(const char* path, const char* key, oc_launch_config* cfg, int32_t* found);
oc_status oc_tune_cache_store(const char* path, const char* key, const oc_launch_config* cfg, double ms_per_step);

/* ---- testing aid: the bounded waits of the persistent CG -------------------------- */
/* The persistent CG (one cooperative launch per step for the streamed cloths, and for
 * the adjoint solves) waits, before each pass over a cloth's vertices, for that cloth's
 * previous pass to complete on every block; each wait gives up after a bounded number of
 * polls and the step then fails with OC_ERR_DEVICE_TIMEOUT at the next oc_synchronize /
 * oc_get_state / oc_get_stats, after which the handle steps on (a cloth whose solve had
 * not ended got no update).  For tests of that path: from the next step on, block
 * `withhold_block` of those launches returns before its first arrival (-1: none), and a
 * wait gives up after `max_polls` polls (0: the default, about half a second).  Nothing
 * waits longer than that bound.  Fails with OC_ERR_UNSUPPORTED when the handle runs no
 * persistent CG. */
oc_status oc_test_barrier_timeout(oc_solver* s, int32_t withhold_block, uint32_t max_polls);

/* No counterpart in the reference.  For tests: the step computes spring lengths, their
 * reciprocals, the quotients of ComputeForces / CalcForceDerivatives (IMP:720-727) and the
 * preconditioner's reciprocals (IMP:312-314) with branch-free correctly rounded sequences
 * when the arguments lie in [2^-60, 2^60], and with the IEEE intrinsics otherwise.  This
 * checks the sequences against the intrinsics on `device`: the reciprocal of every float
 * of that range and its negation, the square root of every float of that range, and
 * n_pairs random quotients (and their negations) from `seed`.  mismatches[3] receives the
 * number of results whose bits differ (reciprocal, square root, quotient). */
oc_status oc_test_cr_arith(int32_t device, uint64_t n_pairs, uint64_t seed, uint64_t* mismatches);

/* ---- allocation-free solve -------------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device memory
 * around a solve — an engine that manages a fixed device-memory budget itself, or a
 * real-time frame loop where a cudaMalloc/cudaFree (which may synchronise the device)
 * is not acceptable.  Runs the step's preconditioned CG (first iteration
 * preconditioned, FP64 dot accumulation, pinned rows filtered out) on a block-diagonal
 * system the caller assembled, such as the A and b that oc_assemble returns.
 *   A9      device, 9 floats per vertex (glm column-major, symmetric)
 *   b, x    device float triples; x holds the warm start on entry, the solution on return
 *   pinned  device, one byte per vertex (non-zero = pinned), or NULL; a pinned row's
 *           solution is 0 and its A and b are not used
 *   stream  cudaStream_t, or NULL for the default stream; the call is synchronous: it
 *           waits on the stream between iterations and before it returns
 * Scratch is a fixed static device array sized for OC_NOALLOC_MAX_VERTICES vertices
 * (about 3.8 MB, held by every GPU that loads the library until exit); larger systems
 * return OC_ERR_UNSUPPORTED.  All calls on a device share that array, which keeps the
 * last call's contents (each call clears what must start at zero): calls whose GPU work
 * overlaps race.  The first call on a device looks up the array's address; make that
 * call before any stream capture. */
#define OC_NOALLOC_MAX_VERTICES 65536
oc_status oc_pcg_solve_noalloc(const float* A9, const float* b, float* x, const uint8_t* pinned, int32_t n_vertices,
                               int32_t cg_max_iter, float cg_tol, int32_t* cg_iters, uint32_t* flags, void* stream);

/* ---- block-sparse CG of the FEM demo (FEM:837-922) --------------------------------- */
/* ConjugateGradientSolver of OpenCloth_CoRotated_Linear_FEM (FEM), batched: each system
 * is a block-row matrix (the reference's vector<map<int, mat3>> A_row, FEM:123) in CSR
 * with strictly ascending columns per row (std::map order), 3x3 float blocks stored as
 * glm keeps them (m[c][r] at 3c + r; the product's component c is
 * m[c][0] x + m[c][1] y + m[c][2] z, FEM:873-875), a right-hand side b and the unknown V
 * (warm start in, solution out).  Fixed rows (IsFixed, FEM:117) are skipped; their
 * blocks and b may be non-finite, as the reference's FLT_MAX masses make them.  Exactly
 * cg_max_iter iterations run (the reference's exit test, FEM:905, cannot fire). */
typedef struct oc_bsr_desc {
    int32_t n_rows;
    int32_t nnzb;
    const int32_t* row_ptr; /* n_rows + 1, row_ptr[0] = 0, row_ptr[n_rows] = nnzb */
    const int32_t* col;     /* nnzb, strictly ascending within each row */
    const uint8_t* fixed;   /* n_rows flags, or NULL for none */
    int32_t cg_max_iter;    /* i_max, FEM:134 */
    float tolerance;        /* tolerence, FEM:133 (kept for the record; see above) */
    float tiny;             /* tiny, FEM:132: the d and d2 clamps, FEM:885-886, 908-909 */
} oc_bsr_desc;

typedef struct oc_bsr_solver oc_bsr_solver;

/* Validate and upload the sparsity of n_systems systems (options: device, stream,
 * use_graph, executor).  Executors: OC_EXEC_AUTO solves each system of up to 256 rows
 * whose blocks fit in one CTA's shared memory in one CTA (the whole CG on chip, the
 * streamed path's bits) and streams the others; OC_EXEC_STREAMED (and OC_EXEC_PLAIN)
 * stream every system; OC_EXEC_RESIDENT fails with OC_ERR_UNSUPPORTED unless every
 * system fits.  Fails with OC_ERR_BAD_INDEX / OC_ERR_INVALID_ARGUMENT on bad patterns. */
oc_status oc_bsr_create(const oc_bsr_desc* descs, int32_t n_systems, const oc_options* opts, oc_bsr_solver** out);
void oc_bsr_destroy(oc_bsr_solver* s);
const char* oc_bsr_last_error(const oc_bsr_solver* s);
oc_status oc_bsr_get_counts(const oc_bsr_solver* s, int64_t* rows, int64_t* nnzb, int32_t* n_systems);
/* Host arrays concatenated over the systems in creation order: blocks 9 x nnzb, b and x
 * 3 x rows; NULL keeps the current value.  A non-finite block or b in a free row, or a
 * non-finite x, fails with OC_ERR_NON_FINITE and changes nothing (the arrays are staged
 * and checked on the device, then committed).  Returns when the host arrays may be
 * reused; the commit is ordered before the next solve on the handle's stream. */
oc_status oc_bsr_set_system(oc_bsr_solver* s, const float* blocks, const float* b, const float* x);
/* The CG on every system (asynchronous on the handle's stream). */
oc_status oc_bsr_solve(oc_bsr_solver* s);
/* The solution V and the final residual (3 x rows each; either may be NULL). */
oc_status oc_bsr_get_solution(oc_bsr_solver* s, float* x, float* residual);
oc_status oc_bsr_get_launch_count(oc_bsr_solver* s, int64_t* kernels_launched);
/* n_solves solves without the graph, each launch timed with CUDA events: per kernel
 * (names, 32 chars each) the total ms, launches and algorithmic bytes, as
 * oc_profile_steps does for the cloth step. */
oc_status oc_bsr_profile(oc_bsr_solver* s, int32_t n_solves, int32_t max_kernels, char* names, double* ms_total,
                         int64_t* launches, double* algorithmic_bytes, int32_t* n_kernels);
oc_status oc_bsr_synchronize(oc_bsr_solver* s);

/* ---- reference topology builder (IMP:497-565) ------------------------------------ */
/* Host only (no device work): validate the descriptors as oc_create does and report, per
 * cloth, the grid (cols x rows) on which its incidences follow a stencil, or 0 x 0.  A
 * grid cloth (the reference's lattice and spring order, at most 16 distinct
 * rest/ks/kd) is assembled without reading incidence records. */
oc_status oc_describe_instances(const oc_cloth_desc* descs, int32_t n_instances, int32_t* grid_cols,
                                int32_t* grid_rows);
/* Number of springs InitGL() creates for a cols x rows vertex grid (cols, rows >= 3):
 * rows*(cols-1) + cols*(rows-1) + 2*(rows-1)*(cols-1) + rows*(cols-1) + cols*(rows-1),
 * which includes the reference's one duplicate bend spring per row and column. */
oc_status oc_grid_spring_count(int32_t cols, int32_t rows, int32_t* n_springs);
/* Springs in the reference's creation order with rest lengths from the exact lattice,
 * then positions with i.i.d. N(0, (jitter * spacing)^2) noise per coordinate (seeded).
 * Lattice: x = ((i/(cols-1))*2 - 1) * size/2, y = size + 1 - (j/(rows-1)) * size, z = 0,
 * vertex j*cols + i; row 0 at the top, so the reference's pins 0 and cols-1 are the two
 * top corners.  ks/kd are indexed by spring type. */
oc_status oc_grid_build(int32_t cols, int32_t rows, float size, const float ks[3], const float kd[3],
                        float jitter, uint64_t seed, float* X, oc_spring* springs);

#ifdef __cplusplus
}
#endif
#endif /* OPENCLOTH_GB_H */
