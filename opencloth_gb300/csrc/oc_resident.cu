// Resident step: one cluster of CTAs per cloth holds that cloth's CG state (A, x, r, d:
// 60 B per vertex) in shared memory, runs the complete preconditioned CG to the cloth's
// own tolerance (IMP:308-330) on chip, and applies the update (IMP:790-797).  Fused (an
// option of the solver), the CTAs first assemble their vertices' systems themselves (ComputeForces
// and the Jacobians, IMP:701-783, with the same per-vertex functions as k_assemble /
// k_assemble_grid) straight into shared memory, so a small cloth's whole step is one
// kernel whose HBM traffic is the state in and out; unfused, they load the state
// k_assemble left in the planes.  The CG loop touches no HBM and needs no per-iteration
// launch.  Unfused with a.cg_only, the kernel is the adjoint solve of a resident cloth:
// the CG state k_adj_seed left in the planes in, the solution out, no update.
// Dot products reduce per CTA and then across the cluster through distributed shared
// memory after a hardware cluster barrier, as error-free float pairs (about 48 bits, the
// role FP64 plays in the streamed kernels), in the same fixed order in every CTA, so all
// of them take identical decisions; alpha and beta are the pairs' quotients rounded to
// float.  There are no spin-waits.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace cgx = cooperative_groups;

namespace oc {
namespace {

// Sum over the CTA, then over the cluster (C CTAs), carried as error-free float pairs
// (Acc: the running sum and its exact rounding errors, about 48 significant bits) up to
// the cluster total.  FP64 is slow on this GPU and these reductions and the scalars after
// them are the serial part of every CG iteration, so no level uses it.
// The CTA's warps merge in a fixed tree in warp 0.  Each CTA then pushes its pair into
// slot [rank] of every CTA of the cluster (lane r of warp 0 stores into CTA r's shared
// memory), one cluster barrier makes the pushes visible, and every CTA merges its C local
// slots in the same fixed tree (absent ranks are zero pairs), so all CTAs get identical
// totals.  slots[2][16] is double-buffered per call: a buffer is written again only two
// barriers after its last reads.  The result is valid in thread 0.
__device__ __forceinline__ Acc shfl_acc(Acc v, int o) {
    Acc u;
    u.s = __shfl_down_sync(0xffffffffu, v.s, o);
    u.c = __shfl_down_sync(0xffffffffu, v.c, o);
    return u;
}

__device__ Acc cluster_sum(Acc part, int C, Acc (*slots)[kResidentMaxCluster], int& phase) {
    __shared__ Acc warp_part[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part = acc_merge(part, shfl_acc(part, o));
    __syncthreads();  // warp_part's previous readers are done
    if (lane == 0) warp_part[w] = part;
    __syncthreads();
    Acc v = acc_zero();
    if (w == 0) {
        v = lane < nw ? warp_part[lane] : acc_zero();
        for (int o = nw >> 1; o > 0; o >>= 1) v = acc_merge(v, shfl_acc(v, o));
    }
    if (C > 1) {
        // Every thread of every CTA takes part in the cluster barrier.
        cgx::cluster_group cl = cgx::this_cluster();
        Acc* slot = slots[phase & 1];
        if (w == 0) {
            const unsigned me = cl.block_rank();
            const Acc mine = make_acc(__shfl_sync(0xffffffffu, v.s, 0), __shfl_sync(0xffffffffu, v.c, 0));
            if (lane < C) cl.map_shared_rank(slot, lane)[me] = mine;
        }
        cl.sync();
        if (w == 0) {
            v = lane < C ? slot[lane] : acc_zero();
#pragma unroll
            for (int o = kResidentMaxCluster >> 1; o > 0; o >>= 1) v = acc_merge(v, shfl_acc(v, o));
        }
    }
    ++phase;
    return v;
}

// The CG's scalar arithmetic on the pairs, with no FP64 (one FP64 division costs a
// resident CTA about a tenth of its time on this GPU).  norm: the pair's value as
// hi + lo with hi = fl(hi + lo) (TwoSum).  div: the quotient of two normalised pairs,
// rounded to float: q0 = fl(a.hi / b.hi), the exact remainder a - q0 b (an FMA for the
// head product, Sterbenz for the subtraction), then q0 + remainder / b.hi rounded once;
// it is the correctly rounded quotient unless the exact one lies within about 2^-46 of a
// rounding boundary.  gt: a > b for normalised pairs.
__device__ __forceinline__ Acc pair_norm(Acc a) {
    const float s = a.s + a.c;
    const float bp = s - a.s;
    return make_acc(s, (a.s - (s - bp)) + (a.c - bp));
}

__device__ __forceinline__ float pair_div(Acc a, Acc b) {
    const float q0 = __fdiv_rn(a.s, b.s);
    const float ph = __fmul_rn(q0, b.s);
    const float pl = __fmaf_rn(q0, b.s, -ph);
    const float r = (((a.s - ph) - pl) + a.c) - __fmul_rn(q0, b.c);
    return __fadd_rn(q0, __fdiv_rn(r, b.s));
}

__device__ __forceinline__ bool pair_gt(Acc a, Acc b) { return a.s > b.s || (a.s == b.s && a.c > b.c); }

__device__ __forceinline__ bool pair_finite(Acc a) { return isfinite(a.s) && isfinite(a.c); }

__device__ __forceinline__ Acc pair_from(double x) {
    const float h = (float)x;
    return make_acc(h, (float)(x - (double)h));
}

// Resident CTAs per SM the register budget is set for: 128-thread CTAs hold up to 512
// vertices, 256-thread CTAs 256 to 1024, 512-thread CTAs 2048 (shared memory holds only
// A, 24 bytes per vertex; x, r and d are in registers).
template <int T>
constexpr int resident_min_blocks() {
    return T == 128 ? 8 : (T == 256 ? 4 : 1);
}

template <int T, bool FUSED>
__global__ void __launch_bounds__(T, resident_min_blocks<T>()) k_resident(const StepArgs a, const ResidentLaunch L) {
    extern __shared__ __align__(16) float smem[];
    __shared__ Acc slots[2][kResidentMaxCluster];
    // The CG scalars live in thread 0 (one thread does the divisions and tests, on float
    // pairs); the other threads get alpha, beta and the go / stop decision.
    __shared__ float s_alpha, s_beta;
    __shared__ int s_go;
    // Thread 0's scalars, in shared memory rather than in every thread's registers:
    // delta0 (FP64, set once), the iteration's r.r and threshold as pairs, the flags.
    __shared__ double s_delta0;
    __shared__ Acc s_delta, s_thresh;
    __shared__ uint32_t s_flags;
    const int C = L.cluster;
    const int rank = (C > 1) ? (int)cgx::this_cluster().block_rank() : 0;
    const int inst = L.inst_ids[blockIdx.x / C];
    const InstParams& ip = a.inst[inst];
    const int chunk = (ip.nv + C - 1) / C;
    const int lb = rank * chunk;
    const int n_local = max(0, min(ip.nv, lb + chunk) - lb);
    const int64_t base = ip.v_off + lb;
    const int cap = L.vcta;
    float* sA[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) sA[k] = smem + k * cap;
    // Thread t owns vertices t, t + T, t + 2T, t + 3T of the CTA's range (every launch
    // shape has vcta <= 4T): their x, r, d live in its registers for the whole solve, and
    // A in shared memory.
    float x[kResidentVpt][3], r[kResidentVpt][3], d[kResidentVpt][3];
    bool own[kResidentVpt];
#pragma unroll
    for (int u = 0; u < kResidentVpt; ++u) own[u] = (int)threadIdx.x + u * T < n_local;

    int phase = 0;
    Acc part;
    if (threadIdx.x == 0) {
        s_delta0 = 0.0;
        s_flags = 0u;
    }
    if constexpr (FUSED) {
        // The assembly of these vertices (k_assemble / k_assemble_grid); X and V are
        // written at the end of this kernel, so they are read with plain loads.
        part = acc_zero();
#pragma unroll
        for (int u = 0; u < kResidentVpt; ++u) {
            if (!own[u]) continue;
            const int j = threadIdx.x + u * T;
            const int64_t g = base + j;
            const float4 Xg = a.X[g], Vg = a.V[g];
            const OwnSpring os = load_own<false>(a, g);
            const float3 F =
                ip.grid_cols > 0 ? stencil_gather<false>(a, ip, g, Xg, Vg) : thread_gather<1, false>(a, ip, g, Xg, Vg);
            const VertexSystem sys = vertex_system(a.dt, Xg, Vg, F, os);
            const CgInit c = cg_init(sys, a.x[0][g], a.x[1][g], a.x[2][g], Vg.w != 0.0f);
#pragma unroll
            for (int k = 0; k < 6; ++k) sA[k][j] = sys.A[k];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                x[u][k] = c.x[k];
                r[u][k] = c.r[k];
                d[u][k] = c.d[k];
            }
            acc_add(part, c.term);
        }
        // delta0 and the decision to iterate, as the assembly's last-block epilogue takes
        // them (finish<K_ASSEMBLE>).  The cluster reduction also orders every CTA's reads
        // of X and V before any CTA's writes below.
        const Acc tp = pair_norm(cluster_sum(part, C, slots, phase));
        if (threadIdx.x == 0) {
            const double total = (double)tp.s + (double)tp.c;
            s_delta0 = total;
            bool run = (0 < ip.imax) && (total > (double)ip.eps2 * total);
            if (!isfinite(total)) {
                s_flags |= OC_FLAG_NON_FINITE;
                run = false;
            }
            s_go = run ? 1 : 0;
        }
    } else {
        // The CG state k_assemble left in the planes: A -> shared memory, x, r, d ->
        // registers.
#pragma unroll
        for (int u = 0; u < kResidentVpt; ++u) {
            if (!own[u]) continue;
            const int j = threadIdx.x + u * T;
            const int64_t g = base + j;
#pragma unroll
            for (int k = 0; k < 6; ++k) sA[k][j] = a.A[k][g];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                x[u][k] = a.x[k][g];
                r[u][k] = a.r[k][g];
                d[u][k] = a.d[k][g];
            }
        }
        if (threadIdx.x == 0) {
            const InstState& st0 = a.state[inst];
            s_delta0 = st0.delta0;
            s_flags = st0.flags;
            s_go = st0.active != 0 ? 1 : 0;
        }
    }
    __syncthreads();
    bool run = s_go != 0;
    if (threadIdx.x == 0) {
        s_delta = pair_from(s_delta0);
        s_thresh = pair_from((double)ip.eps2 * s_delta0);
    }
    int it = 0;
    float beta = 0.0f;
    while (run) {
        // d = r + beta d (after the first iteration), d.(A d), IMP:320-321, 327.
        part = acc_zero();
#pragma unroll
        for (int u = 0; u < kResidentVpt; ++u) {
            if (!own[u]) continue;
            const int j = threadIdx.x + u * T;
            if (it > 0) {
                d[u][0] = r[u][0] + d[u][0] * beta;
                d[u][1] = r[u][1] + d[u][1] * beta;
                d[u][2] = r[u][2] + d[u][2] * beta;
            }
            const float A[6] = {sA[0][j], sA[1][j], sA[2][j], sA[3][j], sA[4][j], sA[5][j]};
            float q0, q1, q2;
            matvec(A, d[u][0], d[u][1], d[u][2], q0, q1, q2);
            acc_add(part, d[u][0] * q0 + d[u][1] * q1 + d[u][2] * q2);
        }
        const Acc dq = pair_norm(cluster_sum(part, C, slots, phase));
        if (threadIdx.x == 0) {
            if (!(dq.s > 0.0f) || !pair_finite(dq)) {
                s_flags |= pair_finite(dq) ? OC_FLAG_BREAKDOWN : OC_FLAG_NON_FINITE;
                s_go = 0;
            } else {
                s_alpha = pair_div(s_delta, dq);
                s_go = 1;
            }
        }
        __syncthreads();
        if (!s_go) break;
        const float alpha = s_alpha;
        // x += alpha d; r -= alpha A d; r.r, IMP:322-325.
        part = acc_zero();
#pragma unroll
        for (int u = 0; u < kResidentVpt; ++u) {
            if (!own[u]) continue;
            const int j = threadIdx.x + u * T;
            const float A[6] = {sA[0][j], sA[1][j], sA[2][j], sA[3][j], sA[4][j], sA[5][j]};
            float q[3];
            matvec(A, d[u][0], d[u][1], d[u][2], q[0], q[1], q[2]);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                x[u][k] = x[u][k] + d[u][k] * alpha;
                r[u][k] = r[u][k] - q[k] * alpha;
            }
            acc_add(part, r[u][0] * r[u][0] + r[u][1] * r[u][1] + r[u][2] * r[u][2]);
        }
        const Acc rr = pair_norm(cluster_sum(part, C, slots, phase));
        ++it;
        if (threadIdx.x == 0) {
            const Acc old = s_delta, thresh = s_thresh;
            const Acc delta = rr;
            s_delta = delta;
            s_beta = pair_div(delta, old);
            int go = 1;
            if (!pair_finite(delta)) {
                s_flags |= OC_FLAG_NON_FINITE;
                go = 0;
            } else if (!(it < ip.imax && pair_gt(delta, thresh))) {
                if (pair_gt(delta, thresh)) s_flags |= OC_FLAG_NOT_CONVERGED;
                go = 0;
            }
            s_go = go;
        }
        __syncthreads();
        beta = s_beta;
        if (!s_go) break;
    }
    // V += dV dt; X += dt V; ground clamp (IMP:790-797), then the ellipsoid pass when
    // enabled; dV stays as the warm start.  An adjoint solve (cg_only, unfused) stops at
    // the solution.
    const float dt = a.dt;
    const bool upd = !a.cg_only;
#pragma unroll
    for (int u = 0; u < kResidentVpt; ++u) {
        if (!own[u]) continue;
        const int64_t g = base + threadIdx.x + u * T;
        if (upd) {
            float4 Xg = a.X[g], Vg = a.V[g];
            update_vertex(ip, dt, x[u][0], x[u][1], x[u][2], Xg, Vg);
            a.X[g] = Xg;
            a.V[g] = Vg;
        }
        a.x[0][g] = x[u][0];
        a.x[1][g] = x[u][1];
        a.x[2][g] = x[u][2];
    }
    if (rank == 0 && threadIdx.x == 0) {
        InstState& st = a.state[inst];
        st.delta0 = s_delta0;
        st.delta_new = (double)s_delta.s + (double)s_delta.c;
        st.dq = 0.0;
        st.iter = it;
        st.flags = s_flags;
        st.active = 0;
        st.alpha = 0.0f;
        st.beta = beta;
    }
    // A CTA's shared memory must outlive the other CTAs' reads of it.
    if (C > 1) cgx::this_cluster().sync();
}

template <int T, bool FUSED>
cudaError_t prepare_k() {
    cudaError_t e = cudaFuncSetAttribute(k_resident<T, FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)resident_smem_bytes(kResidentMaxVcta));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_resident<T, FUSED>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

template <int T>
cudaError_t prepare_t() {
    cudaError_t e = prepare_k<T, false>();
    return e == cudaSuccess ? prepare_k<T, true>() : e;
}

template <int T>
cudaError_t launch_t(const StepArgs& a, const ResidentLaunch& L, int n_clusters, cudaStream_t stream) {
    const size_t smem = resident_smem_bytes(L.vcta);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(n_clusters * L.cluster));
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = L.cluster > 1 ? 1 : 0;
    return L.fused ? cudaLaunchKernelEx(&cfg, k_resident<T, true>, a, L) : cudaLaunchKernelEx(&cfg, k_resident<T, false>, a, L);
}

}  // namespace

size_t resident_smem_bytes(int vcta) { return (size_t)6 * vcta * sizeof(float); }  // A

cudaError_t prepare_resident() {
    cudaError_t e = prepare_t<128>();
    if (e == cudaSuccess) e = prepare_t<256>();
    if (e == cudaSuccess) e = prepare_t<512>();
    return e;
}

cudaError_t launch_resident(const StepArgs& a, const ResidentLaunch& L, int threads, int n_clusters,
                            cudaStream_t stream) {
    if (n_clusters <= 0) return cudaSuccess;
    if (L.vcta > kResidentVpt * threads) return cudaErrorInvalidValue;  // a thread holds at most kResidentVpt
    switch (threads) {
        case 128: return launch_t<128>(a, L, n_clusters, stream);
        case 256: return launch_t<256>(a, L, n_clusters, stream);
        case 512: return launch_t<512>(a, L, n_clusters, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace oc
