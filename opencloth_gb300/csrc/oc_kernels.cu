// Streamed executor: the implicit step's kernels over a ragged batch, and the passes
// after it.
//
//   k_assemble   ComputeForces (IMP:698-735) as a per-vertex gather over the
//                incidence CSR, CalcForceDerivatives for spring i (IMP:737-772),
//                the assembly of A_i, b_i, P_i (IMP:781-786) and the CG set-up
//                r = b - A x, d = P^-1 r, delta0 = r.(P r) (IMP:310-318).
//   k_assemble_grid  the same for grid cloths, with the neighbours from a stencil
//   k_cg_dir     [d = r + beta d]; alpha = delta_new / d.(A d)    (IMP:320-321, 327)
//   k_cg_update  x += alpha d; r -= alpha A d; delta_new = r.r     (IMP:322-326)
//   k_cg_persist the CG loop of any number of cloths and their update in one
//                cooperative launch (the two passes above, per-cloth arrival counts)
//   k_integrate  V += dV dt; X += dt V; ground clamp               (IMP:790-797)
//                [+ EllipsoidCollision, IMP:824-848]
//   k_provot     ApplyProvotDynamicInverse as a per-vertex gather   (IMP:800-823)
//   k_ellipsoid  EllipsoidCollision on its own                      (IMP:824-848)
//
// Compiled with --fmad=false and IEEE division / square root so every FP32 operation
// rounds exactly as the reference's scalar code does.  The CG dot products are summed
// in extended precision: per-vertex FP32 terms, error-free float pairs within a warp,
// FP64 above (see Acc in oc_device.cuh).
//
// Reductions are deterministic: each block writes one FP64 partial; the last block of
// an instance to finish (atomic ticket) sums that instance's partials in a fixed order
// and updates the instance's CG scalars.  The last block of the whole grid sets the
// CUDA-graph WHILE condition to "some instance still iterating".  k_cg_persist forms
// the same sums in the same order at its grid barriers.
#include <algorithm>
#include <cstdint>
#include <cstdlib>

#include <cuda_runtime.h>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kThreads = 256;

// Shared-memory staging of one chunk (blockDim consecutive vertices of a block) for
// the cooperative force gather.
constexpr int kIncCap = 3328;  // incidence records staged per round (13 per thread)

struct GatherSmem {
    float4 X[kThreads];
    float4 V[kThreads];
    float fx[kIncCap], fy[kIncCap], fz[kIncCap];
    uint8_t owner[kIncCap];  // chunk-local vertex of each staged record
};
constexpr size_t kGatherSmem = sizeof(GatherSmem);

// F_i for the chunk [c0, c1): zero, gravity (m g) unless pinned, damping on all,
// optional external force, then every incident spring in spring-id order — the
// reference's scatter order (IMP:701-734).  The records of the chunk are contiguous;
// lanes evaluate them in parallel (coalesced record loads, independent neighbour
// gathers) into shared memory, and each vertex then adds its own forces sequentially,
// so the FP32 sum is the reference's.  Every thread of the block must call this.
__device__ float3 chunk_gather(const StepArgs& a, const InstParams& ip, int64_t c0, int64_t c1, GatherSmem& sm,
                               float4& Xg, float4& Vg) {
    const int t = threadIdx.x;
    const int64_t g = c0 + t;
    const bool valid = g < c1;
    Xg = make_float4(0.f, 0.f, 0.f, 1.f);
    Vg = make_float4(0.f, 0.f, 0.f, 0.f);
    int32_t k0 = 0, k1 = 0;
    if (valid) {
        Xg = __ldg(a.X + g);
        Vg = __ldg(a.V + g);
        k0 = __ldg(a.rowptr + g);
        k1 = __ldg(a.rowptr + g + 1);
    }
    sm.X[t] = Xg;
    sm.V[t] = Vg;
    const bool pinned = Vg.w != 0.0f;
    float Fx = 0.0f, Fy = 0.0f, Fz = 0.0f;
    if (valid) {
        if (!pinned) {
            Fx += Xg.w * ip.gravity[0];
            Fy += Xg.w * ip.gravity[1];
            Fz += Xg.w * ip.gravity[2];
        }
        Fx += ip.damping * Vg.x;
        Fy += ip.damping * Vg.y;
        Fz += ip.damping * Vg.z;
        if (!pinned && ip.has_ext) {
            const float4 e = __ldg(a.fext + g);
            Fx += e.x;
            Fy += e.y;
            Fz += e.z;
        }
    }
    const int32_t kb = __ldg(a.rowptr + c0), ke = __ldg(a.rowptr + c1);
    for (int32_t rb = kb; rb < ke; rb += kIncCap) {
        const int32_t re = min(ke, rb + kIncCap);
        __syncthreads();
        for (int32_t k = max(k0, rb); k < min(k1, re); ++k) sm.owner[k - rb] = (uint8_t)t;
        __syncthreads();
#pragma unroll 4
        for (int32_t k = rb + t; k < re; k += blockDim.x) {
            const int4 rec = __ldg(a.inc + k);
            const int self = sm.owner[k - rb];
            const float4 Xs = sm.X[self], Vs = sm.V[self];
            float3 f = make_float3(0.f, 0.f, 0.f);
            if (Vs.w == 0.0f) {  // pinned vertices take no spring force (IMP:730-733)
                const bool as_p2 = rec.x < 0;
                const int32_t o = rec.x & 0x7fffffff;
                const float4 Xo = __ldg(a.X + o), Vo = __ldg(a.V + o);
                const float rest = __int_as_float(rec.y), ks = __int_as_float(rec.z), kd = __int_as_float(rec.w);
                if (as_p2) {  // F[p2] -= f, IMP:733
                    f = spring_force(Xo, Xs, Vo, Vs, rest, ks, kd);
                    f = make_float3(-f.x, -f.y, -f.z);
                } else {  // F[p1] += f, IMP:731
                    f = spring_force(Xs, Xo, Vs, Vo, rest, ks, kd);
                }
            }
            sm.fx[k - rb] = f.x;
            sm.fy[k - rb] = f.y;
            sm.fz[k - rb] = f.z;
        }
        __syncthreads();
        if (valid && !pinned) {
            for (int32_t k = max(k0, rb); k < min(k1, re); ++k) {
                Fx += sm.fx[k - rb];
                Fy += sm.fy[k - rb];
                Fz += sm.fz[k - rb];
            }
        }
    }
    return make_float3(Fx, Fy, Fz);
}

// Per-vertex part of the assembly after the force gather: the vertex's system and CG
// set-up (pinned rows filtered out), stored to the SoA planes.  Returns the vertex's
// term of delta0.
__device__ __forceinline__ float store_system(const StepArgs& a, int64_t g, const float4 Vg, const VertexSystem& sys) {
    const bool pinned = Vg.w != 0.0f;
    const CgInit c = cg_init(sys, a.x[0][g], a.x[1][g], a.x[2][g], pinned);
    if (pinned) {
        a.x[0][g] = 0.0f;
        a.x[1][g] = 0.0f;
        a.x[2][g] = 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) a.A[k][g] = sys.A[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a.r[k][g] = c.r[k];
        a.d[k][g] = c.d[k];
    }
    if (a.dbg_A9) {
        const float* A = sys.A;
        float* o = a.dbg_A9 + 9 * g;
        o[0] = A[0]; o[1] = A[1]; o[2] = A[2];
        o[3] = A[1]; o[4] = A[3]; o[5] = A[4];
        o[6] = A[2]; o[7] = A[4]; o[8] = A[5];
    }
    if (a.dbg_b) {
        a.dbg_b[3 * g] = sys.b[0];
        a.dbg_b[3 * g + 1] = sys.b[1];
        a.dbg_b[3 * g + 2] = sys.b[2];
    }
    return c.term;
}

__device__ __forceinline__ float assemble_vertex(const StepArgs& a, int64_t g, const float4 Xg, const float4 Vg,
                                                 const float3 F, const OwnSpring& os) {
    return store_system(a, g, Vg, vertex_system(a.dt, Xg, Vg, F, os));
}

// Assembly with one thread per vertex (MINB: minimum resident blocks per SM, which caps
// the registers).
template <int B, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_assemble_thread(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    Acc part = acc_zero();
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Xg = __ldg(a.X + g), Vg = __ldg(a.V + g);
        const OwnSpring os = load_own(a, g);
        const float3 F = thread_gather<B>(a, ip, g, Xg, Vg);
        acc_add(part, assemble_vertex(a, g, Xg, Vg, F, os));
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

// Assembly of grid cloths (one thread per vertex, no incidence records).  Spring i's
// record and end states are loaded after the force gather: held across it, they made the
// kernel spill (1.78 against 1.74 ms on the 4096-cloth batch).  Its ends are loaded before
// the gather and the record and end states prefetched into L1 (1.74 -> 1.69 ms).
template <int B, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_assemble_grid(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    Acc part = acc_zero();
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Xg = __ldg(a.X + g), Vg = __ldg(a.V + g);
        const int2 ends = __ldg(a.own_ends + g);
        prefetch_own(a, g, ends);  // into L1 while the forces are gathered
        const float3 F = B == 1 ? stencil_gather(a, ip, g, Xg, Vg) : stencil_gather_ahead<B>(a, ip, g, Xg, Vg);
        acc_add(part, assemble_vertex(a, g, Xg, Vg, F, load_own_at(a, g, ends)));
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

// Two incidences fetched ahead at four CTAs per SM (the default), or one at a time
// (OC_GRID_VARIANT=1).  Measured on GB300: 1.78 against 1.81 ms on the 4096-cloth batch and
// 88 against 91.5 us on the 1M-vertex cloth; two or three ahead at three CTAs per SM and four
// at two were 8-44% slower.  All give the same bits.
typedef void (*GridAsmFn)(StepArgs);
GridAsmFn grid_asm_fn() {
    const char* e = std::getenv("OC_GRID_VARIANT");
    return (e && std::atoi(e) == 1) ? k_assemble_grid<1, 4> : k_assemble_grid<2, 4>;
}

// ---- the strip sweep: every spring force of a grid cloth evaluated once ----------------
// k_assemble_grid evaluates each spring at both of its ends (12 forces per vertex).  Here a
// warp owns 28 columns of a band of rows and walks down the band one row per iteration,
// lane l on column c0 - 2 + l, holding rows r, r+1 and r+2 of its column in registers.  In
// row r each lane evaluates the six springs anchored at its vertex (r, c):
//   H  (r,c)-(r,c+1)    bR (r,c)-(r,c+2)    V  (r,c)-(r+1,c)
//   shA (r,c)-(r+1,c+1) shB (r+1,c)-(r,c+1) bC (r,c)-(r+2,c)
// with its neighbours' positions from the lanes to its right (__shfl_down_sync), each in
// its p1 -> p2 orientation, as the stencil gather evaluates it.  The owned vertex (r, c)
// then has all twelve of its springs: its own six, H, bR and shB of the lanes to its left
// this row (__shfl_up_sync), shA of the lane to its left and V and shB of its own lane one
// row up, bC two rows up (registers); the reference's repeated bend springs are the
// originals' values again.  It adds them in spring-id order with the p1 / p2 signs, so F is
// the stencil gather's bits, then forms its system and CG set-up as k_assemble_grid does.
// The two lanes on each side own nothing, and a band starts two rows early to form the
// springs that reach into it from above.  delta0: each warp sums its vertices' terms as
// a float pair into its item's slot of strip_part, and k_assemble_finish sums a cloth's
// items in item order and sets the CG scalars.  delta0 is then summed in the sweep's own
// order, not k_assemble_grid's; F, A, b and the CG set-up are the stencil gather's bits.

__device__ __forceinline__ float3 shfl_down3(const float4 v, int d) {
    return make_float3(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
                       __shfl_down_sync(0xffffffffu, v.z, d));
}

__device__ __forceinline__ float3 shfl_up3(const float3 v, int d) {
    return make_float3(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
                       __shfl_up_sync(0xffffffffu, v.z, d));
}

__device__ __forceinline__ float4 xyz0(const float3 v) { return make_float4(v.x, v.y, v.z, 0.0f); }

__device__ __forceinline__ void add3(float& Fx, float& Fy, float& Fz, const float3 f) {
    Fx += f.x;
    Fy += f.y;
    Fz += f.z;
}

__device__ __forceinline__ void sub3(float& Fx, float& Fy, float& Fz, const float3 f) {
    Fx -= f.x;
    Fy -= f.y;
    Fz -= f.z;
}

// A warp's copy of its cloth's parameter slots and slot words, in shared memory.
struct StripParams {
    float4 par[kStencilSlots];
    uint32_t slot[kStencilClasses];
};

// (rest, ks, kd) of the spring of `kind` (slot word w of the anchor's class); rest lengths
// that vary come from the anchor's rest planes (rs, fetched a row ahead).
__device__ __forceinline__ float4 strip_param(const StripParams& sp, bool has_rest, const float* rs, uint32_t w,
                                              int kind) {
    float4 p = sp.par[(w >> (4 * kind)) & 15u];
    if (has_rest) p.x = rs[kind];
    return p;
}

__device__ __forceinline__ Acc shfl_down_acc(Acc v, int o) {
    return make_acc(__shfl_down_sync(0xffffffffu, v.s, o), __shfl_down_sync(0xffffffffu, v.c, o));
}

template <int MINB>
__global__ void __launch_bounds__(kStripThreads, MINB) k_assemble_strip(const StepArgs a) {
    const int lane = threadIdx.x & 31;
    const int wid = blockIdx.x * (kStripThreads / 32) + (threadIdx.x >> 5);
    if (wid >= a.n_strip_work) return;  // whole warps leave together; no block barrier follows
    const StripWork w = a.strip_work[wid];
    const InstParams& ip = a.inst[w.inst];
    const int32_t cols = ip.grid_cols, rows = ip.grid_rows, nvk = ip.nv;
    const int64_t vo = ip.v_off;
    const int32_t c = w.c0 - 2 + lane;
    const bool colok = c >= 0 && c < cols;
    const bool owner = colok && lane >= 2 && lane < 2 + kStripOwned;
    const bool right1 = colok && c + 1 < cols && lane < 31, right2 = colok && c + 2 < cols && lane < 30;
    __shared__ StripParams smem_par[kStripThreads / 32];
    StripParams& sp = smem_par[threadIdx.x >> 5];
    if (lane < kStencilSlots) sp.par[lane] = __ldg(a.st_param + ip.st_par + lane);
    for (int q = lane; q < kStencilClasses; q += 32) sp.slot[q] = __ldg(a.strip_slot + ip.strip_slot + q);
    __syncwarp();
    const bool has_rest = ip.strip_rest >= 0;
    const float* rest = has_rest ? a.strip_rest + ip.strip_rest : nullptr;
    const int ccls = colok ? stencil_class_1d(c, cols) : 0;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 zero3 = make_float3(0.f, 0.f, 0.f);
    const float h = a.dt;

    // Rows r, r+1, r+2 of this lane's column; row r+3 is fetched one iteration ahead, and
    // so are the rest lengths of the springs anchored one row down.
    int32_t r = max(w.r0 - 2, 0);
    const float4* Xcol = a.X + vo + c;
    const float4* Vcol = a.V + vo + c;
    float4 Xa = zero4, Va = zero4, Xb = zero4, Vb = zero4, Xc = zero4, Vc = zero4;
    if (colok) {
        Xa = __ldg(Xcol + (int64_t)r * cols);
        Va = __ldg(Vcol + (int64_t)r * cols);
        if (r + 1 < rows) {
            Xb = __ldg(Xcol + (int64_t)(r + 1) * cols);
            Vb = __ldg(Vcol + (int64_t)(r + 1) * cols);
        }
        if (r + 2 < rows) {
            Xc = __ldg(Xcol + (int64_t)(r + 2) * cols);
            Vc = __ldg(Vcol + (int64_t)(r + 2) * cols);
        }
    }
    // Spring i's ends of this row's vertex (own_ends, fetched a row ahead); its record and
    // end states are prefetched into L1 at the start of the row and loaded after the forces.
    int2 ends = colok ? __ldg(a.own_ends + vo + (int64_t)r * cols + c) : make_int2(-1, -1);
    float rs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (has_rest && colok)
#pragma unroll
        for (int k = 0; k < 6; ++k) rs[k] = __ldg(rest + (size_t)k * nvk + r * cols + c);
    // Springs anchored one and two rows up (this lane's column).
    float3 fV1 = zero3, fA1 = zero3, fB1 = zero3, fC1 = zero3, fC2 = zero3;
    Acc part = acc_zero();
    for (; r < w.r1; ++r) {
        const bool band = r >= w.r0;
        const bool own = owner && band;
        const bool springs = own && Va.w == 0.0f;  // pinned vertices take no spring force
        const int64_t g = vo + (int64_t)r * cols + c;
        const uint32_t sw = colok ? sp.slot[stencil_class_1d(r, rows) * 6 + ccls] : 0u;
        float rn[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (has_rest && colok && r + 1 < w.r1)
#pragma unroll
            for (int k = 0; k < 6; ++k) rn[k] = __ldg(rest + (size_t)k * nvk + (r + 1) * cols + c);
        const int2 ends_next = (colok && r + 1 < w.r1) ? __ldg(a.own_ends + g + cols) : make_int2(-1, -1);
        if (own) prefetch_own(a, g, ends);
        float4 Xd = zero4, Vd = zero4;
        if (colok && r + 3 < rows && r + 1 < w.r1) {
            Xd = __ldg(Xcol + (int64_t)(r + 3) * cols);
            Vd = __ldg(Vcol + (int64_t)(r + 3) * cols);
        }
        float Fx = 0.0f, Fy = 0.0f, Fz = 0.0f;
        if (own) {
            if (Va.w == 0.0f) {
                Fx += Xa.w * ip.gravity[0];
                Fy += Xa.w * ip.gravity[1];
                Fz += Xa.w * ip.gravity[2];
            }
            Fx += ip.damping * Va.x;
            Fy += ip.damping * Va.y;
            Fz += ip.damping * Va.z;
            if (springs && ip.has_ext) {
                const float4 e = __ldg(a.fext + g);
                Fx += e.x;
                Fy += e.y;
                Fz += e.z;
            }
        }
        // The springs in spring-id order (InitGL, IMP:531-565): each evaluated where it is
        // anchored, added at both ends, p2 subtracting and p1 adding (IMP:731-733).
        const float4 XR1 = xyz0(shfl_down3(Xa, 1)), VR1 = xyz0(shfl_down3(Va, 1));
        float3 fH = zero3;
        if (band && right1) {
            const float4 p = strip_param(sp, has_rest, rs, sw, 0);
            fH = spring_force(Xa, XR1, Va, VR1, p.x, p.y, p.z);
        }
        const float3 hL = shfl_up3(fH, 1);
        if (springs && c >= 1) sub3(Fx, Fy, Fz, hL);
        if (springs && c + 1 < cols) add3(Fx, Fy, Fz, fH);
        float3 fV = zero3, fA = zero3, fB = zero3;
        const bool down1 = colok && r + 1 < rows && r >= w.r0 - 1;
        if (down1) {
            const float4 p = strip_param(sp, has_rest, rs, sw, 2);
            fV = spring_force(Xa, Xb, Va, Vb, p.x, p.y, p.z);
        }
        if (springs && r >= 1) sub3(Fx, Fy, Fz, fV1);
        if (springs && r + 1 < rows) add3(Fx, Fy, Fz, fV);
        const float3 aL = shfl_up3(fA1, 1);
        if (springs && r >= 1 && c >= 1) sub3(Fx, Fy, Fz, aL);
        if (springs && r >= 1 && c + 1 < cols) add3(Fx, Fy, Fz, fB1);
        if (down1 && right1) {
            const float4 p = strip_param(sp, has_rest, rs, sw, 4);
            fB = spring_force(Xb, XR1, Vb, VR1, p.x, p.y, p.z);
        }
        const float3 bL = shfl_up3(fB, 1);
        if (springs && r + 1 < rows && c >= 1) sub3(Fx, Fy, Fz, bL);
        {
            const float4 XS1 = xyz0(shfl_down3(Xb, 1)), VS1 = xyz0(shfl_down3(Vb, 1));
            if (down1 && right1) {
                const float4 p = strip_param(sp, has_rest, rs, sw, 3);
                fA = spring_force(Xa, XS1, Va, VS1, p.x, p.y, p.z);
            }
        }
        if (springs && r + 1 < rows && c + 1 < cols) add3(Fx, Fy, Fz, fA);
        float3 fR = zero3;
        {
            const float4 XR2 = xyz0(shfl_down3(Xa, 2)), VR2 = xyz0(shfl_down3(Va, 2));
            if (band && right2) {
                const float4 p = strip_param(sp, has_rest, rs, sw, 1);
                fR = spring_force(Xa, XR2, Va, VR2, p.x, p.y, p.z);
            }
        }
        const float3 rL = shfl_up3(fR, 2);
        if (springs && c >= 2) sub3(Fx, Fy, Fz, rL);
        if (springs && c + 2 < cols) add3(Fx, Fy, Fz, fR);
        if (springs && c == cols - 3) add3(Fx, Fy, Fz, fR);  // the repeated bend spring
        if (springs && c == cols - 1) sub3(Fx, Fy, Fz, rL);
        float3 fC = zero3;
        if (colok && r + 2 < rows) {
            const float4 p = strip_param(sp, has_rest, rs, sw, 5);
            fC = spring_force(Xa, Xc, Va, Vc, p.x, p.y, p.z);
        }
        if (springs && r >= 2) sub3(Fx, Fy, Fz, fC2);
        if (springs && r + 2 < rows) add3(Fx, Fy, Fz, fC);
        if (springs && r == rows - 3) add3(Fx, Fy, Fz, fC);
        if (springs && r == rows - 1) sub3(Fx, Fy, Fz, fC2);
        if (own)  // spring i's record and end states, loaded here: held across the forces they spill
            acc_add(part, store_system(a, g, Va,
                                       system_from(own_blocks(h, Xa.w, load_own_at(a, g, ends)), h, Va, make_float3(Fx, Fy, Fz))));
        fC2 = fC1;
        fC1 = fC;
        fV1 = fV;
        fA1 = fA;
        fB1 = fB;
        Xa = Xb;
        Va = Vb;
        Xb = Xc;
        Vb = Vc;
        Xc = Xd;
        Vc = Vd;
        ends = ends_next;
#pragma unroll
        for (int k = 0; k < 6; ++k) rs[k] = rn[k];
    }
    // delta0: this item's pair (k_assemble_finish sums the cloth's items).
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part = acc_merge(part, shfl_down_acc(part, o));
    if (lane == 0)
        reinterpret_cast<float2*>(a.strip_part)[a.strip_item0 + wid] = make_float2(part.s, part.c);
}

// delta0 of a cloth on the strip sweep: one CTA per cloth sums its items' pairs in item
// order (a fixed tree) and sets the CG scalars as finish<K_ASSEMBLE> does; the last CTA
// sets the graph's WHILE condition.
// A strip-swept cloth's delta0: its work items' pairs merged in item order, eight in
// flight per thread, then across the CTA in a fixed tree.  Every thread of the CTA must
// call it; the result is valid in thread 0.
__device__ double strip_delta0(const StepArgs& a, const InstParams& ip) {
    __shared__ Acc warp_part[kThreads / 32];
    const float2* item_part = reinterpret_cast<const float2*>(a.strip_part) + ip.strip_w0;
    Acc tot = acc_zero();
    for (int j0 = threadIdx.x; j0 < ip.strip_nw; j0 += 8 * blockDim.x) {
        float2 p[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int j = j0 + u * blockDim.x;
            p[u] = j < ip.strip_nw ? __ldcg(item_part + j) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (j0 + u * (int)blockDim.x < ip.strip_nw) tot = acc_merge(tot, make_acc(p[u].x, p[u].y));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot = acc_merge(tot, shfl_down_acc(tot, o));
    if (lane == 0) warp_part[w] = tot;
    __syncthreads();
    if (w == 0) {
        tot = lane < (int)(blockDim.x >> 5) ? warp_part[lane] : acc_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tot = acc_merge(tot, shfl_down_acc(tot, o));
    }
    __syncthreads();  // warp_part may be written again by a later call
    return (double)tot.s + (double)tot.c;
}

__global__ void __launch_bounds__(kThreads) k_assemble_finish(const StepArgs a) {
    const int32_t inst = a.strip_ids[blockIdx.x];
    const InstParams& ip = a.inst[inst];
    const double total = strip_delta0(a, ip);
    if (threadIdx.x == 0) {
        InstState& st = a.state[inst];
        st.ticket = 0;
        st.delta0 = total;
        st.delta_new = total;
        st.dq = 0.0;
        st.alpha = 0.0f;
        st.beta = 0.0f;
        st.iter = 0;
        st.flags = 0u;
        bool run = (0 < ip.imax) && (total > (double)ip.eps2 * total);
        if (!isfinite(total)) {
            st.flags |= OC_FLAG_NON_FINITE;
            run = false;
        }
        st.active = run ? 1 : 0;
        if (run && (a.all_streamed || !ip.resident)) atomicAdd(a.unconverged, 1);
        __threadfence();
        if (a.use_cond) {  // the last CTA sets the graph's WHILE condition
            const unsigned t = atomicAdd(a.grid_ticket, 1u);
            if (t == gridDim.x - 1) {
                *a.grid_ticket = 0u;
                __threadfence();
                const int u = atomicAdd(a.unconverged, 0);
                cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, u > 0 ? 1u : 0u);
            }
        }
    }
}

// Assembly with the block-cooperative gather (shared-memory staging).
__global__ void __launch_bounds__(kThreads) k_assemble_coop(const StepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GatherSmem& sm = *reinterpret_cast<GatherSmem*>(smem_raw);
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    Acc part = acc_zero();
    for (int64_t c0 = bi.v_begin; c0 < bi.v_end; c0 += blockDim.x) {
        const int64_t g = c0 + threadIdx.x;
        float4 Xg, Vg;
        const OwnSpring os = load_own(a, g < bi.v_end ? g : bi.v_begin);
        const float3 F = chunk_gather(a, ip, c0, min(c0 + (int64_t)blockDim.x, bi.v_end), sm, Xg, Vg);
        if (g >= bi.v_end) continue;
        acc_add(part, assemble_vertex(a, g, Xg, Vg, F, os));
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

// The update (IMP:790-797) over vertices [v0, v1) of one block, two vertices per thread:
// both vertices' loads are issued before either is updated and stored.
__device__ __forceinline__ void update_range(const StepArgs& a, const InstParams& ip, int64_t v0, int64_t v1) {
    float4* __restrict__ X = a.X;
    float4* __restrict__ V = a.V;
    const float* __restrict__ D0 = a.x[0];
    const float* __restrict__ D1 = a.x[1];
    const float* __restrict__ D2 = a.x[2];
    const int64_t T = blockDim.x;
    for (int64_t g = v0 + threadIdx.x; g < v1; g += 2 * T) {
        const int64_t h = g + T;
        const bool ok = h < v1;
        const int64_t hq = ok ? h : g;
        float4 Xg = X[g], Vg = V[g], Xh = X[hq], Vh = V[hq];
        const float g0 = D0[g], g1 = D1[g], g2 = D2[g];
        const float h0 = D0[hq], h1 = D1[hq], h2 = D2[hq];
        update_vertex(ip, a.dt, g0, g1, g2, Xg, Vg);
        X[g] = Xg;
        V[g] = Vg;
        if (ok) {
            update_vertex(ip, a.dt, h0, h1, h2, Xh, Vh);
            X[h] = Xh;
            V[h] = Vh;
        }
    }
}

// The CG passes stream fifteen FP32 planes.  Each thread keeps two vertices' loads in
// flight (g and g + blockDim) before computing; __restrict__ lets the loads of the
// next pair be issued ahead of this pair's stores.  The per-thread FP64 partial still
// adds vertices in the order g, g + blockDim, g + 2 blockDim, ...
//
// The direction pass of one block: [d = r + beta d]; q = A d; its d.(A d) terms.
__device__ __forceinline__ Acc cg_dir_block(const StepArgs& a, const BlockInfo& bi, bool first, float beta) {
    Acc part = acc_zero();
    const float* __restrict__ A0 = a.A[0];
    const float* __restrict__ A1 = a.A[1];
    const float* __restrict__ A2 = a.A[2];
    const float* __restrict__ A3 = a.A[3];
    const float* __restrict__ A4 = a.A[4];
    const float* __restrict__ A5 = a.A[5];
    const float* __restrict__ R0 = a.r[0];
    const float* __restrict__ R1 = a.r[1];
    const float* __restrict__ R2 = a.r[2];
    float* __restrict__ D0 = a.d[0];
    float* __restrict__ D1 = a.d[1];
    float* __restrict__ D2 = a.d[2];
    const int64_t T = blockDim.x;
    for (int64_t base = bi.v_begin + threadIdx.x; base < bi.v_end; base += 2 * T) {
        float A[2][6], d[2][3], r[2][3];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int64_t g = base + u * T;
            ok[u] = g < bi.v_end;
            const int64_t q = ok[u] ? g : base;
            A[u][0] = A0[q]; A[u][1] = A1[q]; A[u][2] = A2[q];
            A[u][3] = A3[q]; A[u][4] = A4[q]; A[u][5] = A5[q];
            d[u][0] = D0[q]; d[u][1] = D1[q]; d[u][2] = D2[q];
            r[u][0] = 0.f; r[u][1] = 0.f; r[u][2] = 0.f;
            if (!first) {
                r[u][0] = R0[q]; r[u][1] = R1[q]; r[u][2] = R2[q];
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (!ok[u]) continue;
            const int64_t g = base + u * T;
            float d0 = d[u][0], d1 = d[u][1], d2 = d[u][2];
            if (!first) {  // d = r + beta d, IMP:327
                d0 = r[u][0] + d0 * beta;
                d1 = r[u][1] + d1 * beta;
                d2 = r[u][2] + d2 * beta;
                D0[g] = d0;
                D1[g] = d1;
                D2[g] = d2;
            }
            float q0, q1, q2;
            matvec(A[u], d0, d1, d2, q0, q1, q2);
            acc_add(part, d0 * q0 + d1 * q1 + d2 * q2);
        }
    }
    return part;
}

// The update pass of one block: x += alpha d; r -= alpha A d; its r.r terms.
__device__ __forceinline__ Acc cg_update_block(const StepArgs& a, const BlockInfo& bi, float alpha) {
    Acc part = acc_zero();
    const float* __restrict__ A0 = a.A[0];
    const float* __restrict__ A1 = a.A[1];
    const float* __restrict__ A2 = a.A[2];
    const float* __restrict__ A3 = a.A[3];
    const float* __restrict__ A4 = a.A[4];
    const float* __restrict__ A5 = a.A[5];
    const float* __restrict__ D0 = a.d[0];
    const float* __restrict__ D1 = a.d[1];
    const float* __restrict__ D2 = a.d[2];
    float* __restrict__ X0 = a.x[0];
    float* __restrict__ X1 = a.x[1];
    float* __restrict__ X2 = a.x[2];
    float* __restrict__ R0 = a.r[0];
    float* __restrict__ R1 = a.r[1];
    float* __restrict__ R2 = a.r[2];
    const int64_t T = blockDim.x;
    for (int64_t base = bi.v_begin + threadIdx.x; base < bi.v_end; base += 2 * T) {
        float A[2][6], d[2][3], x[2][3], r[2][3];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int64_t g = base + u * T;
            ok[u] = g < bi.v_end;
            const int64_t q = ok[u] ? g : base;
            A[u][0] = A0[q]; A[u][1] = A1[q]; A[u][2] = A2[q];
            A[u][3] = A3[q]; A[u][4] = A4[q]; A[u][5] = A5[q];
            d[u][0] = D0[q]; d[u][1] = D1[q]; d[u][2] = D2[q];
            x[u][0] = X0[q]; x[u][1] = X1[q]; x[u][2] = X2[q];
            r[u][0] = R0[q]; r[u][1] = R1[q]; r[u][2] = R2[q];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (!ok[u]) continue;
            const int64_t g = base + u * T;
            float q0, q1, q2;
            matvec(A[u], d[u][0], d[u][1], d[u][2], q0, q1, q2);
            X0[g] = x[u][0] + d[u][0] * alpha;  // x = x + alpha d, IMP:322
            X1[g] = x[u][1] + d[u][1] * alpha;
            X2[g] = x[u][2] + d[u][2] * alpha;
            const float r0 = r[u][0] - q0 * alpha;  // r = r - alpha q, IMP:323
            const float r1 = r[u][1] - q1 * alpha;
            const float r2 = r[u][2] - q2 * alpha;
            R0[g] = r0;
            R1[g] = r1;
            R2[g] = r2;
            acc_add(part, r0 * r0 + r1 * r1 + r2 * r2);
        }
    }
    return part;
}

__global__ void __launch_bounds__(kThreads) k_cg_dir(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstState& st = a.state[bi.inst];
    const bool active = st.active != 0;
    const Acc part = active ? cg_dir_block(a, bi, st.iter == 0, st.beta) : acc_zero();
    finish<K_CG_DIR>(a, bi.gblk, bi.inst, active, part);
}

__global__ void __launch_bounds__(kThreads) k_cg_update(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstState& st = a.state[bi.inst];
    const bool active = st.active != 0;
    const Acc part = active ? cg_update_block(a, bi, st.alpha) : acc_zero();
    finish<K_CG_UPDATE>(a, bi.gblk, bi.inst, active, part);
}

// ---- the whole CG loop in one cooperative launch ----------------------------------------
// For streamed cloths the loop's cost is the kernel boundaries, not the bytes: each
// (k_cg_dir, k_cg_update) launch pays a launch, a tail and a serial epilogue of about
// 12 us even on a small cloth.  k_cg_persist runs every iteration of every cloth of its
// block table in one launch, all its blocks co-resident (cooperative launch).  Block b
// owns the table entries b, b + grid, b + 2 grid, ... and runs on them the same
// per-block passes as k_cg_dir / k_cg_update, writing the same per-block partials.
//
// The cloths are independent, so there is no grid barrier: each cloth has its own word,
// which counts the arrivals of its entries (it is never reset within the launch).  Phase
// q of a cloth is the direction pass (q even) or the update pass (q odd) of iteration
// q / 2.  Phase q - 1 of cloth c is complete once c's word reaches q nblk(c).  Then every
// block that owns entries of c sums c's partials of phase q - 1 itself, in the
// last-block epilogue's fixed order, and applies the epilogue's scalar rule to its own
// copy of c's scalars in shared memory: all blocks compute the same totals and take the
// same decisions, with no last block that has to publish them first.  The partials are
// double buffered by phase parity: a block writes phase q + 1's only after phase q is
// complete, that is after every block has read phase q - 1's.  The block owning c's first
// entry writes c's state for the host.  Totals, scalars and decisions are those of the
// two-kernel loop bit for bit.  Progress: a block waits at phase q only for cloths it
// still runs, every owner of a running cloth makes its phase q - 1 arrival (one release
// add per run of its consecutive entries of that cloth) before its phase-q wait, and all
// blocks are co-resident.  A wait gives up after a.barrier_polls polls (the default,
// 2^22 polls with a 32 ns back-off, is about half a second) or when another block has
// given up: it sets bit 0 of *err and the block returns without its update.  The block
// a.withhold_block (a testing aid; normally -1) returns before its first arrival, so the
// waits on its cloths run out.

constexpr int kPersistMaxOwn = kThreads;  // table entries one block owns (one waiting thread each)

__device__ __forceinline__ unsigned load_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int load_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned x) {
    unsigned v;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "r"(x) : "memory");
    return v;
}

__global__ void __launch_bounds__(kThreads, 4) k_cg_persist(const StepArgs a, int32_t n_entries, unsigned* words,
                                                            int* err) {
    __shared__ double s_part[kPersistMaxOwn];
    __shared__ double s_dn[kPersistMaxOwn], s_d0[kPersistMaxOwn];  // delta_new, delta0
    __shared__ float s_scal[kPersistMaxOwn];                        // beta or alpha for the next pass
    __shared__ int s_it[kPersistMaxOwn];
    __shared__ uint32_t s_fl[kPersistMaxOwn];
    __shared__ unsigned char s_run[kPersistMaxOwn];  // 0 stopped, 1 runs, 2 runs its first direction pass
    __shared__ unsigned char s_head[kPersistMaxOwn];  // first owned entry of a run of one cloth
    __shared__ int s_any, s_ok;
    const int own = ((int)n_entries - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if (threadIdx.x == 0) s_ok = 1;
    for (int j = threadIdx.x; j < own; j += blockDim.x) {
        const int inst = a.blocks[blockIdx.x + j * gridDim.x].inst;
        const InstState& st = a.state[inst];
        s_head[j] = (j == 0 || a.blocks[blockIdx.x + (j - 1) * gridDim.x].inst != inst) ? 1 : 0;
        s_run[j] = __ldcg(&st.active) ? 2 : 0;
        s_dn[j] = __ldcg(&st.delta_new);
        s_d0[j] = __ldcg(&st.delta0);
        s_it[j] = __ldcg(&st.iter);
        s_fl[j] = __ldcg(&st.flags);
        s_scal[j] = 0.0f;
    }
    __syncthreads();
    if (a.persist_d0) {
        // The strip-swept cloths' delta0 and the decision to iterate, formed here as
        // k_assemble_finish forms them (the step then launches that kernel only for the
        // strip-swept cloths this launch does not run).
        for (int j = 0; j < own; ++j) {
            if (!s_head[j]) continue;
            const BlockInfo bj = a.blocks[blockIdx.x + j * gridDim.x];
            const InstParams& ip = a.inst[bj.inst];
            if (!ip.strip) continue;
            const double total = strip_delta0(a, ip);
            if (threadIdx.x == 0) {
                uint32_t fl = 0u;
                bool run = (0 < ip.imax) && (total > (double)ip.eps2 * total);
                if (!isfinite(total)) {
                    fl |= OC_FLAG_NON_FINITE;
                    run = false;
                }
                for (int k = j; k < own && (k == j || !s_head[k]); ++k) {
                    s_run[k] = run ? 2 : 0;
                    s_dn[k] = total;
                    s_d0[k] = total;
                    s_it[k] = 0;
                    s_fl[k] = fl;
                    s_scal[k] = 0.0f;
                }
                if (bj.gblk == ip.blk0) {
                    InstState& st = a.state[bj.inst];
                    st.ticket = 0;
                    st.delta0 = total;
                    st.delta_new = total;
                    st.dq = 0.0;
                    st.alpha = 0.0f;
                    st.beta = 0.0f;
                    st.iter = 0;
                    st.flags = fl;
                    st.active = run ? 1 : 0;
                }
            }
            __syncthreads();
        }
    }
    for (unsigned q = 0;; ++q) {
        const bool dir = (q & 1u) == 0u;
        if (q > 0) {
            // Phase q - 1 of every running cloth: wait for its arrivals (one thread per run).
            for (int j = threadIdx.x; j < own; j += blockDim.x) {
                if (!s_run[j] || !s_head[j]) continue;
                const BlockInfo bi = a.blocks[blockIdx.x + j * gridDim.x];
                const unsigned need = q * (unsigned)a.inst[bi.inst].nblk;
                unsigned spins = 0;
                while ((int)(load_acquire(words + bi.inst) - need) < 0) {
                    if (++spins > a.barrier_polls || ((spins & 63u) == 0 && load_relaxed(err) != 0)) {
                        atomicOr(err, 1);
                        s_ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __syncthreads();
            if (!s_ok) break;
            // Totals and rule of phase q - 1, per run of one cloth, in every block.
            const double* prev = (q & 1u) ? a.partials : a.partials_b;
            for (int j = 0; j < own; ++j) {
                if (!s_run[j] || !s_head[j]) continue;
                const int inst = a.blocks[blockIdx.x + j * gridDim.x].inst;
                const InstParams& ip = a.inst[inst];
                double acc = 0.0;
#pragma unroll 8
                for (int k = threadIdx.x; k < ip.nblk; k += blockDim.x) acc += __ldcg(prev + ip.blk0 + k);
                const double total = block_sum_packed(acc);  // block_sum's bits (kThreads = 256)
                if (threadIdx.x == 0) {
                    uint32_t fl = s_fl[j];
                    int it = s_it[j];
                    double dn = s_dn[j];
                    float scal = 0.0f;
                    bool run = true;
                    if (!dir) {  // phase q - 1 was a direction pass: d.(A d) -> alpha
                        if (!(total > 0.0) || !isfinite(total)) {
                            fl |= isfinite(total) ? OC_FLAG_BREAKDOWN : OC_FLAG_NON_FINITE;
                            run = false;
                        } else {
                            scal = (float)(dn / total);
                        }
                    } else {  // an update pass: r.r -> beta, the stop test
                        it += 1;
                        scal = (float)(total / dn);
                        dn = total;
                        const bool more = it < ip.imax && total > (double)ip.eps2 * s_d0[j];
                        if (!isfinite(total)) fl |= OC_FLAG_NON_FINITE;
                        if (!more || !isfinite(total)) {
                            if (isfinite(total) && total > (double)ip.eps2 * s_d0[j]) fl |= OC_FLAG_NOT_CONVERGED;
                            run = false;
                        }
                    }
                    // The run's entries share the cloth's copy.
                    for (int k = j; k < own && (k == j || !s_head[k]); ++k) {
                        s_fl[k] = fl;
                        s_it[k] = it;
                        s_dn[k] = dn;
                        s_scal[k] = scal;
                        s_run[k] = run ? 1 : 0;
                    }
                    if (a.blocks[blockIdx.x + j * gridDim.x].gblk == ip.blk0) {  // the cloth's first entry
                        InstState& st = a.state[inst];
                        if (!dir) {
                            st.dq = total;
                            if (run) st.alpha = scal;
                        } else {
                            st.delta_new = dn;
                            st.beta = scal;
                            st.iter = it;
                        }
                        st.flags = fl;
                        if (!run) st.active = 0;
                        st.ticket = 0;
                    }
                }
                __syncthreads();
            }
        }
        if (threadIdx.x == 0) {
            int any = 0;
            for (int j = 0; j < own; ++j) any |= s_run[j];
            s_any = any;
        }
        __syncthreads();
        if (!s_any) break;
        // The passes of the owned entries that run, as k_cg_persist's.
        for (int j = 0; j < own; ++j) {
            if (!s_run[j]) continue;
            const BlockInfo bi = a.blocks[blockIdx.x + j * gridDim.x];
            const double bsum = block_sum_acc(dir ? cg_dir_block(a, bi, s_run[j] == 2, s_scal[j])
                                                  : cg_update_block(a, bi, s_scal[j]));
            if (threadIdx.x == 0) s_part[j] = bsum;
        }
        __syncthreads();
        if ((int)blockIdx.x == a.withhold_block) {
            s_ok = 0;
            break;
        }
        // Arrivals: the partials of phase q into the buffer of its parity, then one release
        // add per run of one cloth.
        double* cur = (q & 1u) ? a.partials_b : a.partials;
        for (int j = threadIdx.x; j < own; j += blockDim.x) {
            if (!s_run[j] || !s_head[j]) continue;
            const int inst = a.blocks[blockIdx.x + j * gridDim.x].inst;
            unsigned n = 0;
            for (int k = j; k < own; ++k) {
                const BlockInfo bk = a.blocks[blockIdx.x + k * gridDim.x];
                if (bk.inst != inst) break;
                cur[bk.gblk] = s_part[k];
                ++n;
            }
            atom_add_acq_rel(words + inst, n);
        }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int j = 0; j < own; ++j)
                if (s_run[j] == 2) s_run[j] = 1;
        __syncthreads();
    }
    if (s_ok && !a.cg_only) {
        for (int32_t e = blockIdx.x; e < n_entries; e += gridDim.x) {
            const BlockInfo bi = a.blocks[e];
            update_range(a, a.inst[bi.inst], bi.v_begin, bi.v_end);
        }
    }
}

// ---- the replay tape ---------------------------------------------------------------
// Given the step's solution dV, the update (IMP:790-797) is elementwise: the forward
// keeps dV of every step and a cloth's (X, V) every `every` steps, and the reverse pass
// rebuilds any step's state from the checkpoint before it with the same update function
// the step used, bit for bit, instead of re-running the step's assembly and CG.

__global__ void __launch_bounds__(kThreads) k_tape_save(const StepArgs a, const TapeCloth* tc, float4* arena,
                                                        int32_t t) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const TapeCloth c = tc[bi.inst];
    if (t % c.every != 0) return;
    const InstParams& ip = a.inst[bi.inst];
    float4* dst = arena + c.ck + (int64_t)(t / c.every) * 2 * ip.nv;
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const int64_t l = g - ip.v_off;
        dst[l] = a.X[g];
        dst[ip.nv + l] = a.V[g];
    }
}

template <bool GM>
__global__ void __launch_bounds__(kThreads) k_tape_view(const StepArgs a, const TapeCloth* tc, float4* arena,
                                                        const float* dvt, int64_t dv_stride, int32_t t,
                                                        int32_t n_steps) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const TapeCloth c = tc[bi.inst];
    const InstParams& ip = a.inst[bi.inst];
    const int64_t nv = ip.nv, ps = a.x[1] - a.x[0];  // plane stride
    const int32_t seg = t / c.every, q = t - seg * c.every;
    const int32_t len = min(n_steps, (seg + 1) * c.every) - seg * c.every;
    const float4* ck = arena + c.ck + (int64_t)seg * 2 * nv;
    float4* buf = arena + c.buf;
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const int64_t l = g - ip.v_off;
        float4 X, V;
        if (q == 0) {
            X = ck[l];
            V = ck[nv + l];
        } else if (q < len - 1) {
            X = buf[(int64_t)q * 2 * nv + l];
            V = buf[(int64_t)q * 2 * nv + nv + l];
        } else {  // the segment's last step: replay it from the checkpoint, filling the slots
            X = ck[l];
            V = ck[nv + l];
            const float by = GM ? __ldg(a.Xbase + g).y : 0.0f;
            for (int32_t k = 1; k <= q; ++k) {
                const float* d = dvt + (int64_t)(seg * c.every + k - 1) * dv_stride;
                if constexpr (GM)
                    gm_advance(a.dt, d[g], d[ps + g], d[2 * ps + g], by, X, V);
                else
                    update_vertex(ip, a.dt, d[g], d[ps + g], d[2 * ps + g], X, V);
                if (k < q) {
                    buf[(int64_t)k * 2 * nv + l] = X;
                    buf[(int64_t)k * 2 * nv + nv + l] = V;
                }
            }
        }
        a.X[g] = X;
        a.V[g] = V;
    }
}

__global__ void __launch_bounds__(kThreads) k_adj_seed_own(const StepArgs a, const AdjArgs j) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    Acc part = acc_zero();
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Xg = __ldg(a.X + g), Vg = __ldg(a.V + g);
        const OwnBlocks ob = own_blocks(a.dt, Xg.w, load_own<true>(a, g));
#pragma unroll
        for (int k = 0; k < 6; ++k) a.A[k][g] = ob.A[k];
        acc_add(part, adj_seed_vertex(a, j, g, Xg, Vg, ob.A[0], ob.A[3], ob.A[5]));
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

__global__ void k_snapshot(const float4* X, const float4* V, float4* dX, float4* dV, const float* x, float* dx,
                           int64_t nv, int64_t nx) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (dX)
        for (int64_t g = t0; g < nv; g += stride) {
            dX[g] = X[g];
            dV[g] = V[g];
        }
    if (dx)
        for (int64_t k = t0; k < nx; k += stride) dx[k] = x[k];
}

__global__ void __launch_bounds__(kThreads) k_integrate(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    update_range(a, a.inst[bi.inst], bi.v_begin, bi.v_end);
}

// ApplyProvotDynamicInverse (IMP:800-823) as a per-vertex gather.  The reference walks
// the springs in order and moves the velocities of both ends; its corrections depend on
// positions only, so vertex g's final velocity is its own plus the corrections of its
// incident springs added in spring order — the order of g's incidence records (or of
// its class's stencil template, for a grid cloth: no records read).  Each spring's
// correction is recomputed at both ends from p1 - p2, so both ends see the same rounded
// value.  Pin flags come from a separate byte array: V is written here.
__device__ __forceinline__ void provot_incidence(const StepArgs& a, float ratio, const float4 Xg, bool pin_self,
                                                 int32_t o, bool is_p2, float rest, float4& Vg) {
    const float4 Xo = __ldg(a.X + o);
    const float4 p1 = is_p2 ? Xo : Xg, p2 = is_p2 ? Xg : Xo;
    const float dx = p1.x - p2.x, dy = p1.y - p2.y, dz = p1.z - p2.z;
    const float sqr = dx * dx + dy * dy + dz * dz;
    float dist = sqrtf(sqr);
    const float lim = rest * ratio;
    if (!(dist > lim)) return;
    dist = dist - lim;
    dist = dist / 2.0f;
    const float inv = 1.0f / sqrtf(sqr);
    const float cx = (dx * inv) * dist, cy = (dy * inv) * dist, cz = (dz * inv) * dist;
    const bool pin_o = __ldg(a.pinflag + o) != 0;
    if (!is_p2) {
        if (!pin_self) {  // p1 moves unless pinned
            Vg.x = Vg.x - cx;
            Vg.y = Vg.y - cy;
            Vg.z = Vg.z - cz;
        }
    } else if (pin_o || !pin_self) {  // p2 moves when p1 is pinned or p2 is free
        Vg.x = Vg.x + cx;
        Vg.y = Vg.y + cy;
        Vg.z = Vg.z + cz;
    }
}

__global__ void __launch_bounds__(kThreads) k_provot(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    if (!((a.only_passes ? a.only_passes : ip.passes) & OC_PASS_PROVOT)) return;
    const float ratio = ip.provot_ratio;
    const int32_t cols = ip.grid_cols;
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Xg = __ldg(a.X + g);
        float4 Vg = a.V[g];
        const bool pin_self = a.pinflag[g] != 0;
        if (cols > 0) {  // grid cloth: the incidences from its class's stencil template
            const int32_t l = (int32_t)(g - ip.v_off), r = l / cols, c = l - r * cols;
            const int cl = stencil_class_1d(r, ip.grid_rows) * 6 + stencil_class_1d(c, cols);
            const int32_t* st = a.st_data + ip.st_off;
            const float4* par = a.st_param + ip.st_par;
            const int32_t e0 = __ldg(st + cl), e1 = __ldg(st + cl + 1);
            const float* rest_inc = ip.st_rest ? a.rest_inc + __ldg(a.rowptr + g) - e0 : nullptr;
            for (int32_t e = e0; e < e1; ++e) {
                const int32_t v = __ldg(st + e);
                const int32_t o = (int32_t)(g + (int64_t)((v & 7) - 2) * cols + (((v >> 3) & 7) - 2));
                const float rest = rest_inc ? __ldg(rest_inc + e) : __ldg(par + (v >> 7)).x;
                provot_incidence(a, ratio, Xg, pin_self, o, (v & 64) != 0, rest, Vg);
            }
        } else {
            const int32_t k1 = __ldg(a.rowptr + g + 1);
            for (int32_t k = __ldg(a.rowptr + g); k < k1; ++k) {
                const int4 rec = __ldg(a.inc + k);
                provot_incidence(a, ratio, Xg, pin_self, rec.x & 0x7fffffff, rec.x < 0, __int_as_float(rec.y), Vg);
            }
        }
        a.V[g] = Vg;
    }
}

// EllipsoidCollision on its own (the step fuses it into the update).
__global__ void __launch_bounds__(kThreads) k_ellipsoid(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    if (!((a.only_passes ? a.only_passes : ip.passes) & OC_PASS_ELLIPSOID)) return;
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        float4 Xg = a.X[g], Vg = a.V[g];
        ellipsoid_vertex(ip, Xg, Vg);
        a.X[g] = Xg;
        a.V[g] = Vg;
    }
}

__global__ void __launch_bounds__(kThreads) k_forces(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Xg = __ldg(a.X + g), Vg = __ldg(a.V + g);
        const float3 F = thread_gather<1>(a, ip, g, Xg, Vg);
        a.dbg_F[3 * g] = F.x;
        a.dbg_F[3 * g + 1] = F.y;
        a.dbg_F[3 * g + 2] = F.z;
    }
}

// Packed float triples <-> the device layout (X/V float4, dV planes).  Flags a
// non-finite input in *err.
__global__ void k_state_in(const StepArgs a, const float* X3, const float* V3, const float* dV3, int64_t nv,
                           int32_t* err) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nv; g += (int64_t)gridDim.x * blockDim.x) {
        bool bad = false;
        if (X3) {
            float4 v = a.X[g];
            v.x = X3[3 * g];
            v.y = X3[3 * g + 1];
            v.z = X3[3 * g + 2];
            bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z);
            a.X[g] = v;
        }
        if (V3) {
            float4 v = a.V[g];
            v.x = V3[3 * g];
            v.y = V3[3 * g + 1];
            v.z = V3[3 * g + 2];
            bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z);
            a.V[g] = v;
        }
        if (dV3) {
            const float x0 = dV3[3 * g], x1 = dV3[3 * g + 1], x2 = dV3[3 * g + 2];
            bad |= !isfinite(x0) || !isfinite(x1) || !isfinite(x2);
            a.x[0][g] = x0;
            a.x[1][g] = x1;
            a.x[2][g] = x2;
        }
        if (bad) atomicOr(err, 1);
    }
}

// Flags a non-finite value among staged float triples in *err, writing nothing else: the
// host commits the staged state with k_state_in only when the flag stays clear.
__global__ void k_state_check(const float* X3, const float* V3, const float* dV3, int64_t nv, int32_t* err) {
    bool bad = false;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < 3 * nv; g += (int64_t)gridDim.x * blockDim.x) {
        if (X3) bad |= !isfinite(X3[g]);
        if (V3) bad |= !isfinite(V3[g]);
        if (dV3) bad |= !isfinite(dV3[g]);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, 1);
}

__global__ void k_state_out(const StepArgs a, float* X3, float* V3, float* dV3, int64_t nv) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nv; g += (int64_t)gridDim.x * blockDim.x) {
        if (X3) {
            const float4 v = a.X[g];
            X3[3 * g] = v.x;
            X3[3 * g + 1] = v.y;
            X3[3 * g + 2] = v.z;
        }
        if (V3) {
            const float4 v = a.V[g];
            V3[3 * g] = v.x;
            V3[3 * g + 1] = v.y;
            V3[3 * g + 2] = v.z;
        }
        if (dV3) {
            dV3[3 * g] = a.x[0][g];
            dV3[3 * g + 1] = a.x[1][g];
            dV3[3 * g + 2] = a.x[2][g];
        }
    }
}

// k_state_check for 16-byte aligned arrays: float4 loads, the same finiteness test.
__device__ __forceinline__ bool finite4(const float4 v) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w);
}

__global__ void k_state_check4(const float4* X3, const float4* V3, const float4* dV3, int64_t nv, int32_t* err) {
    const int64_t n = 3 * nv, n4 = n >> 2, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool bad = false;
    for (int64_t i = t; i < n4; i += stride) {
        if (X3) bad |= !finite4(X3[i]);
        if (V3) bad |= !finite4(V3[i]);
        if (dV3) bad |= !finite4(dV3[i]);
    }
    for (int64_t i = 4 * n4 + t; i < n; i += stride) {
        if (X3) bad |= !isfinite(reinterpret_cast<const float*>(X3)[i]);
        if (V3) bad |= !isfinite(reinterpret_cast<const float*>(V3)[i]);
        if (dV3) bad |= !isfinite(reinterpret_cast<const float*>(dV3)[i]);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, 1);
}

// Force-gather variant of k_assemble (StepArgs::gather_variant): 0 block-cooperative,
// 1/2/3 one thread per vertex fetching 1/2/4 incidences ahead, 4/5/6 one incidence ahead
// with registers capped for 5/6/4 resident blocks per SM.  Measured on GB300 (1025 x 1025
// cloth and the 4096-cloth batch, 4/6/8 vertices per thread): variant 6 at 8 vertices per
// thread is fastest (64 registers; the uncapped kernel takes 75 and runs 1.5x slower,
// tighter caps spill; wider prefetch costs occupancy).
//
// The strip sweep's register cap (StepArgs::strip_variant): 2 resident CTAs per SM (128
// registers, no spill) or 3 (80 registers, with spills).
const void* strip_fn(int v) {
    return v == 3 ? (const void*)k_assemble_strip<3> : (const void*)k_assemble_strip<2>;
}

const void* assemble_fn(int v) {
    switch (v) {
        case 0: return (const void*)k_assemble_coop;
        case 1: return (const void*)k_assemble_thread<1, 1>;
        case 2: return (const void*)k_assemble_thread<2, 1>;
        case 3: return (const void*)k_assemble_thread<4, 1>;
        case 4: return (const void*)k_assemble_thread<1, 5>;
        case 5: return (const void*)k_assemble_thread<1, 6>;
        default: return (const void*)k_assemble_thread<1, 4>;
    }
}

// ---- check of the branch-free correctly rounded arithmetic (tests) --------------------
// counts[0]: reciprocals, counts[1]: square roots, counts[2]: quotients that differ from
// the IEEE intrinsics' bits.
__global__ void k_test_cr_unary(unsigned long long* counts, uint32_t lo, uint32_t hi) {
    unsigned long long br = 0, bs = 0;
    for (uint64_t u = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < hi; u += (uint64_t)gridDim.x * blockDim.x) {
        const float x = __uint_as_float((uint32_t)u);
        br += __float_as_uint(rcp_cr(x)) != __float_as_uint(__frcp_rn(x));
        br += __float_as_uint(rcp_cr(-x)) != __float_as_uint(__frcp_rn(-x));
        bs += __float_as_uint(sqrt_cr(x)) != __float_as_uint(__fsqrt_rn(x));
    }
    if (br) atomicAdd(counts, br);
    if (bs) atomicAdd(counts + 1, bs);
}

__device__ __forceinline__ uint32_t mix32(uint64_t x) {  // splitmix64's finaliser
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return (uint32_t)x;
}

// Random a in +-[2^-60, 2^60] (or 0), b in [2^-30, 2^30] (the quotients of the springs'
// arithmetic: dot / dist and dP / dist, dist the square root of an argument in range);
// every 8th pair has a significand of b near all ones or near a power of two.
__global__ void k_test_cr_div(unsigned long long* counts, uint64_t n, uint64_t seed) {
    unsigned long long bad = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t h1 = mix32(seed + 3 * i), h2 = mix32(seed + 3 * i + 1), h3 = mix32(seed + 3 * i + 2);
        uint32_t mb = h2 & 0x7fffffu;
        if ((h3 & 7u) == 1u) mb = 0x7fffffu - ((h3 >> 20) & 15u);
        if ((h3 & 7u) == 2u) mb = (h3 >> 20) & 15u;
        const uint32_t ea = 67u + (h1 >> 23) % 121u, eb = 97u + (h3 >> 8) % 61u;
        const float a = (h3 & 0x70u) == 0x70u ? 0.0f : __uint_as_float((h3 & 0x80000000u) | ea << 23 | (h1 & 0x7fffffu));
        const float b = __uint_as_float(eb << 23 | mb);
        bad += __float_as_uint(div_cr(a, b, __frcp_rn(b))) != __float_as_uint(__fdiv_rn(a, b));
        bad += __float_as_uint(div_cr(-a, b, __frcp_rn(b))) != __float_as_uint(__fdiv_rn(-a, b));
    }
    if (bad) atomicAdd(counts + 2, bad);
}

}  // namespace

const char* kernel_name(KernelKind k) {
    switch (k) {
        case K_ASSEMBLE: return "k_assemble";
        case K_CG_DIR: return "k_cg_dir";
        case K_CG_UPDATE: return "k_cg_update";
        case K_INTEGRATE: return "k_integrate";
        case K_FORCES: return "k_forces";
        case K_RESIDENT: return "k_resident";
        case K_PROVOT: return "k_provot";
        case K_ELLIPSOID: return "k_ellipsoid";
        case K_CPL_ASSEMBLE: return "k_cpl_assemble";
        case K_ASSEMBLE_GRID: return "k_assemble_grid";
        case K_CG_PERSIST: return "k_cg_persist";
        case K_ASSEMBLE_STRIP: return "k_assemble_strip";
        case K_ASSEMBLE_FINISH: return "k_assemble_finish";
        case K_CPL_DIR: return "k_cpl_dir";
        case K_CPL_UPDATE: return "k_cpl_update";
        default: return "?";
    }
}

const void* kernel_fn(KernelKind k, const StepArgs& a) {
    switch (k) {
        case K_ASSEMBLE: return assemble_fn(a.gather_variant);
        case K_CG_DIR: return (const void*)k_cg_dir;
        case K_CG_UPDATE: return (const void*)k_cg_update;
        case K_INTEGRATE: return (const void*)k_integrate;
        case K_FORCES: return (const void*)k_forces;
        case K_PROVOT: return (const void*)k_provot;
        case K_ELLIPSOID: return (const void*)k_ellipsoid;
        case K_CPL_ASSEMBLE:
        case K_CPL_DIR:
        case K_CPL_UPDATE: return coupled_fn(k);
        case K_ASSEMBLE_GRID: return (const void*)grid_asm_fn();
        case K_ASSEMBLE_STRIP: return strip_fn(a.strip_variant);
        case K_ASSEMBLE_FINISH: return (const void*)k_assemble_finish;
        default: return nullptr;
    }
}

int kernel_block_threads() { return kThreads; }

size_t kernel_smem_bytes(KernelKind k, const StepArgs& a) {
    return (k == K_ASSEMBLE && a.gather_variant == 0) ? kGatherSmem : 0;
}

cudaError_t prepare_kernels() {
    return cudaFuncSetAttribute(k_assemble_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGatherSmem);
}

static int state_blocks(int64_t nv) {
    const int64_t b = (nv + kThreads - 1) / kThreads;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

cudaError_t launch_state_in(const StepArgs& a, const float* X3, const float* V3, const float* dV3, int64_t nv,
                            int32_t* err, cudaStream_t stream) {
    k_state_in<<<state_blocks(nv), kThreads, 0, stream>>>(a, X3, V3, dV3, nv, err);
    return cudaGetLastError();
}

cudaError_t launch_state_check(const float* X3, const float* V3, const float* dV3, int64_t nv, int32_t* err,
                               cudaStream_t stream) {
    if (aligned16(X3) && aligned16(V3) && aligned16(dV3))
        k_state_check4<<<state_blocks(std::max<int64_t>(3 * nv / 4, 1)), kThreads, 0, stream>>>(
            reinterpret_cast<const float4*>(X3), reinterpret_cast<const float4*>(V3),
            reinterpret_cast<const float4*>(dV3), nv, err);
    else
        k_state_check<<<state_blocks(3 * nv), kThreads, 0, stream>>>(X3, V3, dV3, nv, err);
    return cudaGetLastError();
}

cudaError_t launch_state_out(const StepArgs& a, float* X3, float* V3, float* dV3, int64_t nv, cudaStream_t stream) {
    k_state_out<<<state_blocks(nv), kThreads, 0, stream>>>(a, X3, V3, dV3, nv);
    return cudaGetLastError();
}

cudaError_t launch_kernel(KernelKind k, const StepArgs& a, int nblocks, cudaStream_t stream) {
    if (nblocks <= 0) return cudaSuccess;
    switch (k) {
        case K_ASSEMBLE:
            if (a.gather_variant == 0)
                k_assemble_coop<<<nblocks, kThreads, kGatherSmem, stream>>>(a);
            else
                reinterpret_cast<void (*)(StepArgs)>(const_cast<void*>(assemble_fn(a.gather_variant)))
                    <<<nblocks, kThreads, 0, stream>>>(a);
            break;
        case K_CG_DIR: k_cg_dir<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_CG_UPDATE: k_cg_update<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_INTEGRATE: k_integrate<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_FORCES: k_forces<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_PROVOT: k_provot<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_ELLIPSOID: k_ellipsoid<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_CPL_ASSEMBLE:
        case K_CPL_DIR:
        case K_CPL_UPDATE: return launch_coupled(k, a, nblocks, stream);
        case K_ASSEMBLE_GRID: grid_asm_fn()<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_ASSEMBLE_STRIP:
            reinterpret_cast<void (*)(StepArgs)>(const_cast<void*>(strip_fn(a.strip_variant)))
                <<<nblocks, kStripThreads, 0, stream>>>(a);
            break;
        case K_ASSEMBLE_FINISH: k_assemble_finish<<<nblocks, kThreads, 0, stream>>>(a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int persist_max_entries_per_block() { return kPersistMaxOwn; }

int persist_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cg_persist, kThreads, 0) != cudaSuccess) return 0;
    return n;
}

cudaError_t launch_snapshot(const float4* X, const float4* V, float4* dX, float4* dV, const float* x, float* dx,
                            int64_t nv, int64_t nx, cudaStream_t stream) {
    const int64_t n = std::max(dX ? nv : 0, dx ? nx : 0);
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 8);
    k_snapshot<<<blocks, kThreads, 0, stream>>>(X, V, dX, dV, x, dx, nv, nx);
    return cudaGetLastError();
}

cudaError_t launch_tape_save(const StepArgs& a, const TapeCloth* tc, float4* arena, int32_t t, int nblocks,
                             cudaStream_t stream) {
    if (nblocks <= 0) return cudaSuccess;
    k_tape_save<<<nblocks, kThreads, 0, stream>>>(a, tc, arena, t);
    return cudaGetLastError();
}

cudaError_t launch_tape_view(const StepArgs& a, const TapeCloth* tc, float4* arena, const float* dvt,
                             int64_t dv_stride, int32_t t, int32_t n_steps, int nblocks, cudaStream_t stream) {
    if (nblocks <= 0) return cudaSuccess;
    if (a.gm)
        k_tape_view<true><<<nblocks, kThreads, 0, stream>>>(a, tc, arena, dvt, dv_stride, t, n_steps);
    else
        k_tape_view<false><<<nblocks, kThreads, 0, stream>>>(a, tc, arena, dvt, dv_stride, t, n_steps);
    return cudaGetLastError();
}

cudaError_t launch_adj_seed_own(const StepArgs& a, const AdjArgs& j, int nblocks, cudaStream_t stream) {
    if (nblocks <= 0) return cudaSuccess;
    k_adj_seed_own<<<nblocks, kThreads, 0, stream>>>(a, j);
    return cudaGetLastError();
}

const void* adjoint_seed_own_fn() { return (const void*)k_adj_seed_own; }

cudaError_t launch_cg_persist(const StepArgs& a, int32_t n_entries, int grid, unsigned* words, int* err,
                              cudaStream_t stream) {
    if (grid <= 0 || (int64_t)n_entries > (int64_t)kPersistMaxOwn * grid) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cg_persist, a, n_entries, words, err);
}

cudaError_t launch_test_cr_arith(unsigned long long* counts, uint64_t n_pairs, uint64_t seed, cudaStream_t stream) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_test_cr_unary<<<8 * std::max(sms, 1), kThreads, 0, stream>>>(counts, 0x21800000u /* 2^-60 */, 0x5d800001u /* past 2^60 */);
    if (n_pairs > 0) k_test_cr_div<<<8 * std::max(sms, 1), kThreads, 0, stream>>>(counts, n_pairs, seed);
    return cudaGetLastError();
}

}  // namespace oc
