// Internal types shared by the C-ABI layer and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "opencloth_gb.h"

namespace oc {

// Per-instance constants, device resident, read by every kernel of a step.
struct InstParams {
    float gravity[3];
    float damping;  // DEFAULT_DAMPING, IMP:104
    float eps2;     // EPS*EPS rounded to float, IMP:127
    int32_t imax;   // i_max, IMP:128
    int32_t blk0;   // first streamed block of the instance
    int32_t nblk;   // streamed blocks of the instance
    int64_t v_off;  // first vertex (global index)
    int32_t nv;
    int32_t has_ext;
    int32_t resident;  // 1: this cloth's CG runs in the resident kernel, not the streamed loop
    int32_t passes;    // OC_PASS_* bits applied after the update
    int32_t coupled;   // 1: OC_JAC_COUPLED (block-sparse system, oc_coupled.cu)
    int32_t grid_cols;  // > 0: the cloth is a grid whose incidences follow a stencil (k_assemble_grid)
    int32_t grid_rows;
    int32_t st_off;     // its class table and entries in StepArgs::st_data
    int32_t st_par;     // its first parameter slot in StepArgs::st_param
    int32_t st_rest;    // 1: rest lengths vary; read them per incidence from StepArgs::rest_inc
    // The strip sweep (k_assemble_strip), for grid cloths whose incidences follow the
    // reference's spring order: strip_slot is the cloth's first word in StepArgs::strip_slot
    // (36 words, one per anchor position class, six 4-bit parameter slots each: H, bR, V,
    // shA, shB, bC), strip_rest its first rest length in StepArgs::strip_rest (six planes of
    // nv floats, by kind and anchor vertex) or -1 when the slots hold the rest lengths;
    // strip_ok 1 when the cloth may take the sweep (strip 1 when it does); strip_w0 and
    // strip_nw its range of StepArgs::strip_work (and of strip_part).
    int32_t strip;
    int32_t strip_ok;
    int32_t strip_slot;
    int32_t strip_w0;
    int32_t strip_nw;
    int64_t strip_rest;
    float provot_ratio;     // IMP:808
    float ellipsoid[16];    // object -> world, column-major (IMP:583-585)
    float ellipsoid_inv[16];
};

// Per-instance CG scalars, device resident, written by the last block of each
// instance (deterministic fixed-order reduction of per-block FP64 partials).
struct InstState {
    double delta_new;  // r.r (first: r.(P r)), IMP:317/325
    double delta0;
    double dq;         // d.(A d), IMP:321
    float alpha, beta;
    int32_t iter;
    int32_t active;    // 1 while the CG loop runs for this instance
    uint32_t flags;    // OC_FLAG_*
    uint32_t ticket;   // arrivals of this instance's blocks in the current kernel
};

// One streamed block: a contiguous vertex range of one instance.
struct BlockInfo {
    int32_t inst;
    int32_t gblk;     // index of this block in the handle's full block table (partials slot)
    int64_t v_begin;  // global vertex range [v_begin, v_end)
    int64_t v_end;
};

// One warp's share of the strip sweep: columns c0 - 2 ... c0 + 29 of rows [r0, r1) of a
// grid cloth (lanes 2 ... 29 own their vertex; the two lanes each side only supply their
// springs and positions to the owners).
struct StripWork {
    int32_t inst;
    int32_t c0;
    int32_t r0, r1;
};
constexpr int kStripOwned = 28;    // owned columns per warp
constexpr int kStripThreads = 256;  // 8 warps per CTA

// Everything a streamed kernel needs, passed by value.
struct StepArgs {
    float4* X;               // x, y, z, mass
    float4* V;               // x, y, z, pinned (0 or 1)
    const float4* fext;      // external force or nullptr
    const int32_t* rowptr;   // vertex -> incidence range (global), n_vertices + 1
    const int4* inc;         // {other | is_p2 << 31, rest, ks, kd} in spring order
    const int2* own_ends;    // vertex i -> endpoints of spring i (global), or -1
    const float4* own_par;   // vertex i -> rest, ks, kd of spring i
    float* A[6];             // symmetric A: a00 a01 a02 a11 a12 a22 planes
    float* x[3];             // CG solution = persistent warm start dV
    float* r[3];
    float* d[3];
    double* partials;        // one per streamed block
    double* partials_b;      // a second set (the persistent CG's phases of odd parity)
    const InstParams* inst;
    InstState* state;
    const BlockInfo* blocks;
    int32_t* unconverged;    // number of instances whose CG is running
    uint32_t* grid_ticket;   // arrivals of all blocks in the current kernel
    unsigned long long* loop_count;  // completed (k_cg_dir, k_cg_update) launch pairs
    float dt;
    int32_t blk_base;        // first block of this launch (per-cloth launches)
    int32_t vpt;             // vertices per thread
    int32_t use_cond;        // 1: set the graph WHILE condition
    unsigned long long cond; // cudaGraphConditionalHandle
    int32_t all_streamed;    // 1: every cloth's CG runs in the streamed loop (adjoint solves)
    int32_t cg_only;         // k_cg_persist: 1 = the CG alone, no update (adjoint solves)
    int32_t persist_d0;      // k_cg_persist: 1 = it forms its strip-swept cloths' delta0 (the step's launch)
    // k_cg_persist's waits: polls of a cloth's arrival count before a wait gives up,
    // and a block that never arrives (-1: none; set only by oc_test_barrier_timeout).
    uint32_t barrier_polls;
    int32_t withhold_block;
    // Kernel variants of this handle: the incidence-record gather of k_assemble (0 block
    // cooperative, 1-6 one thread per vertex, see oc_kernels.cu) and the strip sweep's
    // register cap (2 or 3 CTAs per SM).
    int32_t gather_variant;
    int32_t strip_variant;
    float* dbg_F;            // optional debug outputs (float triples) or nullptr
    float* dbg_A9;
    float* dbg_b;
    const uint8_t* pinflag;  // 1 for pinned vertices (read by k_provot)
    int32_t only_passes;     // k_ellipsoid / k_provot: nonzero = apply these OC_PASS_* bits to
                             // every cloth (a pass run on its own), 0 = each cloth's own bits
    // COUPLED cloths (allocated only when the handle has one).  Per incidence record:
    // the other vertex and the spring block B = beta I + gamma n n^T of this step; per
    // vertex: m' and the CG vectors z = P^-1 r, the direction d and q = A d.  P^-1 (the
    // inverse of the vertex's diagonal block) lives in the A planes.
    // Grid cloths (InstParams::grid_cols > 0): per cloth 37 class starts then the entries
    // (di + 2 | dj + 2 << 3 | is_p2 << 6 | slot << 7), and kStencilSlots parameter slots
    // {rest, ks, kd, 0}.
    const int32_t* st_data;
    const float4* st_param;
    const float* rest_inc;   // rest length of every incidence record (CSR order), or nullptr
    // The strip sweep: its work items (strip_item0: the first item's index in the handle's
    // list, for a launch over a part of it), parameter-slot words and rest planes (see
    // InstParams), one delta0 partial per item (a float pair in each 8-byte slot), and the
    // cloths on the sweep (k_assemble_finish: one CTA each).
    const StripWork* strip_work;
    int32_t n_strip_work;
    int32_t strip_item0;
    const uint32_t* strip_slot;
    const float* strip_rest;
    double* strip_part;
    const int32_t* strip_ids;
    int32_t n_strip_ids;
    // Displacement mode of the adjoint tape (oc_set_tape_mode): X holds the displacement u
    // from Xbase (the positions at the tape's start, mass in w); each spring's elongation is
    // formed from its start constants {c0 = |d0| - rest, L0 = |d0|}, d0 the spring vector at
    // the start, rounded from FP64: per incidence record (gm_inc) and for vertex i's own
    // spring (gm_own).
    int32_t gm;
    const float4* Xbase;
    const float2* gm_inc;
    const float2* gm_own;
    // COUPLED per-incidence data is slot-major over slices of 32 consecutive vertices:
    // incidence e of vertex g sits at cpl_slice[g >> 5] + 32 e + (g & 31), so a warp's
    // accesses to one slot are contiguous.
    const int64_t* cpl_slice;
    const int32_t* cpl_o;
    float* cpl_c[5];         // n0, n1, n2, beta, gamma
    float* cpl_m;
    float4* cpl_z;           // z = P^-1 r, 16-byte records (w unused): a neighbour's z and d are
    float4* cpl_d;           // two vector loads in k_cpl_dir
    float* q[3];
};

// Adjoint buffers (oc_adjoint.cu); planes have the handle's vertex stride.
struct AdjArgs {
    float* gX[3];
    float* gV[3];
    float* gF[3];
    float* gOwn[6];          // spring i's Jacobian adjoint (dP 3, dV 3) at vertex i
    float* gExt[3];
    const float* dV[3];      // the step's solution dV
    float* gKs;              // per spring (handle-global spring id)
    float* gKd;
    const int32_t* inc_sid;  // spring id of every incidence record
    const int32_t* own_sid;  // vertex i -> id of spring i, or -1
    const int32_t* own_rowptr;  // vertex -> vertices whose spring touches it
    const int32_t* own_ent;     // that vertex | (1 << 31 when the vertex is the spring's p2)
    int32_t springs_variant;    // k_adj_springs' launch variant (OC_ADJ_SPRINGS_VARIANT; 0 default)
    int32_t vertex_variant;     // k_adj_vertex's launch variant (OC_ADJ_VERTEX_VARIANT; 0 default)
};

// Adjoint kernels (oc_adjoint.cu) over the blocks a.blocks[blk_base, blk_base + nblocks):
//   0 the displacement mode's seed (spring i's blocks rebuilt, adj_seed_vertex);
//   1 the vertex terms (k_adj_vertex); 2 the spring terms (k_adj_springs).
cudaError_t launch_adjoint(int which, const StepArgs& a, const AdjArgs& j, int nblocks, cudaStream_t stream);

// The replay tape of one cloth (oc_tape_forward).  The forward keeps the solution dV of
// every step; the cloth's state (X then V, nv float4 each) is kept every `every` steps
// (checkpoint c at arena + ck + 2 nv c) and the reverse pass rebuilds the states in
// between by replaying the update, which given dV is elementwise and exact; segment
// slot s lives at arena + buf + 2 nv s (every > 1 only).
struct TapeCloth {
    int32_t every;
    int32_t pad;
    int64_t ck;
    int64_t buf;
};

// Replay tape kernels (oc_kernels.cu), over the full block table a.blocks[0, nblocks):
//   save  the state of step t (before it) into the checkpoints that fall on t;
//   view  the state of step t into a.X, a.V: from the checkpoint, the segment slot, or
//         (at a segment's last step) by replaying the segment from its checkpoint with
//         the taped dV (dvt + step * dv_stride, three planes of a.x's stride), filling
//         the slots; a.gm selects the displacement mode's update;
//   seed  the adjoint seed with the system's diagonal blocks rebuilt from spring i
//         (own_blocks, as every assembly forms them): A planes written, then
//         adj_seed_vertex and the assembly epilogue.
cudaError_t launch_tape_save(const StepArgs& a, const TapeCloth* tc, float4* arena, int32_t t, int nblocks,
                             cudaStream_t stream);
cudaError_t launch_tape_view(const StepArgs& a, const TapeCloth* tc, float4* arena, const float* dvt,
                             int64_t dv_stride, int32_t t, int32_t n_steps, int nblocks, cudaStream_t stream);
cudaError_t launch_adj_seed_own(const StepArgs& a, const AdjArgs& j, int nblocks, cudaStream_t stream);
const void* adjoint_seed_own_fn();
// Displacement mode kernels (oc_adjoint.cu).  Per vertex (n = the vertex count):
//   0 Xbase = X;  4 the spring constants gm_inc, gm_own from Xbase and X = (0, 0, 0, mass);
//   3 X = Xbase + u.  Over the blocks a.blocks[blk_base, blk_base + n):
//   1 assembly: forces, spring i's Jacobians, A, b and the CG set-up (incidence records);
//   2 update: V += dt dV, u += dt V, ground clamp on Xbase.y + u.y.
cudaError_t launch_gm(int which, const StepArgs& a, int n, cudaStream_t stream);
// Tape snapshots: X, V into dX, dV (nv float4 each, skipped when dX is null) and nx floats
// of x into dx (skipped when dx is null).
cudaError_t launch_snapshot(const float4* X, const float4* V, float4* dX, float4* dV, const float* x, float* dx,
                            int64_t nv, int64_t nx, cudaStream_t stream);
cudaError_t launch_set_spring_params(const StepArgs& a, const AdjArgs& j, const float* ks, const float* kd,
                                     int64_t n_rec, int64_t nv, cudaStream_t stream);

constexpr int kStencilClasses = 36;  // 6 row classes x 6 column classes
constexpr int kStencilSlots = 16;    // distinct (rest, ks, kd) per grid cloth

// The position class of vertex (r, c) of a rows x cols grid, per dimension: 0 and 1 for
// the first two rows (columns), 5, 4 and 3 for the last three (the third-last carries
// the reference's extra bend spring, IMP:557-558 and 563-564), 2 inside.
__host__ __device__ inline int stencil_class_1d(int32_t i, int32_t n) {
    return i == 0 ? 0 : (i == n - 1 ? 5 : (i == 1 ? 1 : (i == n - 2 ? 4 : (i == n - 3 ? 3 : 2))));
}

enum KernelKind { K_ASSEMBLE = 0, K_CG_DIR = 1, K_CG_UPDATE = 2, K_INTEGRATE = 3, K_FORCES = 4, K_RESIDENT = 5,
                  K_PROVOT = 6, K_ELLIPSOID = 7, K_CPL_ASSEMBLE = 8, K_CPL_DIR = 9, K_CPL_UPDATE = 10,
                  K_ASSEMBLE_GRID = 11, K_CG_PERSIST = 12, K_ASSEMBLE_STRIP = 13, K_ASSEMBLE_FINISH = 14,
                  K_COUNT = 15 };

// The whole CG loop of the cloths of block table a.blocks[0, n_entries) in one
// cooperative launch of `grid` blocks (oc_kernels.cu), any number of cloths; a block
// owns at most persist_max_entries_per_block() entries.  words: one arrival count per
// cloth of the handle, indexed by cloth, zeroed before each launch.  The per-block
// partials are double buffered (StepArgs::partials, partials_b).  err: bit 0 set if a
// wait gave up.
int persist_max_entries_per_block();
int persist_blocks_per_sm();
cudaError_t launch_test_cr_arith(unsigned long long* counts, uint64_t n_pairs, uint64_t seed, cudaStream_t stream);
cudaError_t launch_cg_persist(const StepArgs& a, int32_t n_entries, int grid, unsigned* words, int* err,
                              cudaStream_t stream);

// Interaction kernels (oc_interact.cu).
cudaError_t launch_pick(const float4* X, int64_t v0, int64_t nv, const float pt[3], double radius, int32_t* out,
                        cudaStream_t stream);
cudaError_t launch_drag(float4* X, float4* V, int64_t g, const float delta[3], cudaStream_t stream);
cudaError_t launch_set_vertices(float4* X, float4* V, const int64_t* idx, const float* X3, const float* V3,
                                int32_t n, cudaStream_t stream);
cudaError_t launch_set_pins(float4* V, uint8_t* pinflag, int64_t v0, int64_t nv, const int32_t* pins, int32_t n,
                            cudaStream_t stream);

// COUPLED kernels (oc_coupled.cu).
const void* coupled_fn(KernelKind k);
cudaError_t launch_coupled(KernelKind k, const StepArgs& a, int nblocks, cudaStream_t stream);

const char* kernel_name(KernelKind k);
const void* kernel_fn(KernelKind k, const StepArgs& a);  // the variant a selects
int kernel_block_threads();
size_t kernel_smem_bytes(KernelKind k, const StepArgs& a);  // dynamic shared memory of a launch
cudaError_t prepare_kernels();  // function attributes (once per device)

// Host-side launch of one kernel kind over [blk_base, blk_base + nblocks).
cudaError_t launch_kernel(KernelKind k, const StepArgs& a, int nblocks, cudaStream_t stream);

// Resident executor (oc_resident.cu): one launch runs whole steps for n_clusters cloths,
// cluster CTAs of `threads` threads per cloth, at most vcta vertices per CTA.
struct ResidentLaunch {
    const int32_t* inst_ids;  // the cloth of each cluster
    int32_t cluster;
    int32_t vcta;
    int32_t fused;  // 1: the kernel assembles its cloth's system itself (no k_assemble pass)
};
constexpr int kResidentMaxVcta = 2048;
constexpr int kResidentVpt = 4;  // vertices per thread of the resident kernel: vcta <= 4 x threads
constexpr int kResidentMaxCluster = 16;
size_t resident_smem_bytes(int vcta);
cudaError_t prepare_resident();  // function attributes (once per device)
cudaError_t launch_resident(const StepArgs& a, const ResidentLaunch& L, int threads, int n_clusters,
                            cudaStream_t stream);

cudaError_t launch_state_in(const StepArgs& a, const float* X3, const float* V3, const float* dV3, int64_t nv,
                            int32_t* err, cudaStream_t stream);
cudaError_t launch_state_out(const StepArgs& a, float* X3, float* V3, float* dV3, int64_t nv, cudaStream_t stream);
// Sets *err when a staged triple array (any may be NULL) holds a NaN or Inf; writes nothing else.
cudaError_t launch_state_check(const float* X3, const float* V3, const float* dV3, int64_t nv, int32_t* err,
                               cudaStream_t stream);

// Topology / validation helpers (oc_topology.cpp).
struct PackedHost {
    int32_t n_inst = 0;
    int64_t nv = 0, ns = 0;
    std::vector<int64_t> v_off, s_off;
    std::vector<InstParams> inst;
    std::vector<float4> X0, V0, fext;  // fext empty when no instance has one
    std::vector<int32_t> rowptr;
    std::vector<int4> inc;
    std::vector<int2> own_ends;
    std::vector<float4> own_par;
    std::vector<BlockInfo> blocks;
    int32_t vertices_per_block = 0;
    std::vector<int32_t> inc_sid;                     // spring id of every incidence record
    std::vector<int32_t> own_sid;                     // vertex i -> id of spring i, or -1
    std::vector<int32_t> own_rowptr, own_ent;         // vertex -> vertices whose spring touches it
    std::vector<int32_t> st_data;                     // stencils of the grid cloths (see StepArgs)
    std::vector<float4> st_param;
    bool any_st_rest = false;                         // a grid cloth reads rest lengths per incidence
    std::vector<uint32_t> strip_slot;                 // strip sweep tables (see InstParams)
    std::vector<float> strip_rest;
    bool any_provot = false;                          // some cloth has OC_PASS_PROVOT
    bool any_coupled = false;                         // some cloth is OC_JAC_COUPLED
};

oc_status pack_instances(const oc_cloth_desc* descs, int32_t n, int32_t vertices_per_block, PackedHost* out,
                         std::string* err);
// Marks the grid cloths whose incidences follow the reference's spring order with one
// parameter slot per spring kind and anchor class (InstParams::strip_ok) and builds their
// slot words and, where the rest lengths vary, their rest planes.
void build_strip_tables(PackedHost* P);

}  // namespace oc
