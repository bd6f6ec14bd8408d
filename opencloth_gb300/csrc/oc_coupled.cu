// COUPLED Jacobian mode: Baraff-Witkin coupling of the per-spring blocks into one
// symmetric positive-definite block-sparse system per cloth, solved by a block-Jacobi
// preconditioned CG.  The reference has no such system (its vertex i takes spring i's
// blocks alone, IMP:782); the mode is defined on the reference's own force model:
//
//   (M' + sum_s [B_s, -B_s; -B_s, B_s]) dV = h (F - h sum_s Kt_s (v_i - v_j)),  V += dV
//
// with, for spring s and n = (x1 - x2) / |x1 - x2|,
//   Kt_s = kst I + (ksn - kst) n n^T,   ksn = max(ks, 0),  kst = ksn max(1 - L/l, 0)
//   B_s  = beta I + gamma n n^T,        beta = h^2 kst,  gamma = (h kdn + h^2 ksn) - beta,
//                                       kdn = max(-kd, 0)
//   M'   = (m + h max(-c, 0)) I,        c the velocity damping.
// The clamps keep every B_s positive semi-definite (the transverse term is dropped for a
// compressed spring), so the CG always sees an SPD system.  Pinned vertices are
// Dirichlet rows filtered out of the CG.
//
//   k_cpl_assemble  F (the reference's forces, bit for bit), each incidence's B_s into
//                   slot-major per-incidence planes (StepArgs::cpl_slice), the diagonal block and its inverse P^-1, b, and
//                   the CG set-up r = b - A x, z = P^-1 r, delta0 = r.z
//   k_cpl_dir       dn = z + beta d (first pass: z); q = A dn with the neighbours' dn
//                   rebuilt from their z and d; d.q
//   k_cpl_update    dn again; x += alpha dn; r -= alpha q; d = dn; z = P^-1 r; r.z
//
// The direction is never written during the matrix-vector pass, so a vertex's
// neighbours read its previous d and z while it runs: no second buffer is needed.
// Every per-vertex sum runs over the vertex's incidence records in spring-id order with
// a fixed operand order, the same expressions as the CPU restatement
// (oracle/oc_coupled_impl.h), and the CG scalars go through the streamed executor's
// deterministic per-instance reductions (finish in oc_device.cuh).
#include <cuda_runtime.h>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kThreads = 256;

struct SpringBlock {
    float n0, n1, n2, beta, gamma, ksn, kst;
};

__device__ __forceinline__ SpringBlock spring_block(const float4 p1, const float4 p2, float rest, float ks, float kd,
                                                    float h, float hh) {
    SpringBlock c;
    const float dx = p1.x - p2.x, dy = p1.y - p2.y, dz = p1.z - p2.z;
    const float sqr = dx * dx + dy * dy + dz * dz;
    float l, rl;
    if (cr_arg(sqr) && cr_num(dx) && cr_num(dy) && cr_num(dz) && cr_num(rest)) {
        l = sqrt_cr(sqr);
        const float inv = rcp_cr(l);
        c.n0 = div_cr(dx, l, inv);
        c.n1 = div_cr(dy, l, inv);
        c.n2 = div_cr(dz, l, inv);
        rl = div_cr(rest, l, inv);
    } else {
        l = __fsqrt_rn(sqr);
        c.n0 = __fdiv_rn(dx, l);
        c.n1 = __fdiv_rn(dy, l);
        c.n2 = __fdiv_rn(dz, l);
        rl = __fdiv_rn(rest, l);
    }
    const float ksn = ks > 0.0f ? ks : 0.0f;
    const float kdn = -kd > 0.0f ? -kd : 0.0f;
    const float t = 1.0f - rl;
    const float kst = ksn * (t > 0.0f ? t : 0.0f);
    const float alpha = h * kdn + hh * ksn;
    c.beta = hh * kst;
    c.gamma = alpha - c.beta;
    c.ksn = ksn;
    c.kst = kst;
    return c;
}

// acc += beta e + (gamma (n.e)) n
__device__ __forceinline__ void block_apply(float n0, float n1, float n2, float beta, float gamma, float e0, float e1,
                                            float e2, float& a0, float& a1, float& a2) {
    const float ne = n0 * e0 + n1 * e1 + n2 * e2;
    const float g = gamma * ne;
    a0 = a0 + (beta * e0 + g * n0);
    a1 = a1 + (beta * e1 + g * n1);
    a2 = a2 + (beta * e2 + g * n2);
}

__global__ void __launch_bounds__(kThreads, 4) k_cpl_assemble(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    const float h = a.dt, hh = h * h;
    const float nc = -ip.damping;
    const float mdamp = h * (nc > 0.0f ? nc : 0.0f);
    Acc part = acc_zero();
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Xg = __ldg(a.X + g), Vg = __ldg(a.V + g);
        const bool pinned = Vg.w != 0.0f;
        const float mp = Xg.w + mdamp;
        float xi0 = a.x[0][g], xi1 = a.x[1][g], xi2 = a.x[2][g];
        if (pinned) xi0 = xi1 = xi2 = 0.0f;
        // Forces in the reference's order (IMP:701-734): gravity unless pinned, damping,
        // external force unless pinned, then the springs in spring-id order.
        float Fx = 0.0f, Fy = 0.0f, Fz = 0.0f;
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
        float D[6] = {mp, 0.0f, 0.0f, mp, 0.0f, mp};
        float w0 = 0.0f, w1 = 0.0f, w2 = 0.0f;
        float ax0 = mp * xi0, ax1 = mp * xi1, ax2 = mp * xi2;
        const int64_t slot0 = __ldg(a.cpl_slice + (g >> 5)) + (g & 31);
        // Incidence e of the vertex (spring-id order): neighbour o, the vertex's side, and
        // the spring's parameters.
        auto incidence = [&](int32_t e, int32_t o, bool as_p2, float rest, float ks, float kd) {
            const int64_t sk = slot0 + 32 * (int64_t)e;
            const float4 Xo = __ldg(a.X + o), Vo = __ldg(a.V + o);
            if (!pinned) {  // pinned vertices take no spring force (IMP:730-733)
                if (as_p2) {
                    const float3 f = spring_force(Xo, Xg, Vo, Vg, rest, ks, kd);
                    Fx -= f.x;
                    Fy -= f.y;
                    Fz -= f.z;
                } else {
                    const float3 f = spring_force(Xg, Xo, Vg, Vo, rest, ks, kd);
                    Fx += f.x;
                    Fy += f.y;
                    Fz += f.z;
                }
            }
            const SpringBlock c = as_p2 ? spring_block(Xo, Xg, rest, ks, kd, h, hh)
                                        : spring_block(Xg, Xo, rest, ks, kd, h, hh);
            a.cpl_c[0][sk] = c.n0;
            a.cpl_c[1][sk] = c.n1;
            a.cpl_c[2][sk] = c.n2;
            a.cpl_c[3][sk] = c.beta;
            a.cpl_c[4][sk] = c.gamma;
            const float g0 = c.gamma * c.n0, g1 = c.gamma * c.n1, g2 = c.gamma * c.n2;
            D[0] = D[0] + (c.beta + g0 * c.n0);
            D[1] = D[1] + g0 * c.n1;
            D[2] = D[2] + g0 * c.n2;
            D[3] = D[3] + (c.beta + g1 * c.n1);
            D[4] = D[4] + g1 * c.n2;
            D[5] = D[5] + (c.beta + g2 * c.n2);
            const float u0 = Vg.x - Vo.x, u1 = Vg.y - Vo.y, u2 = Vg.z - Vo.z;
            const float nu = c.n0 * u0 + c.n1 * u1 + c.n2 * u2;
            const float kk = (c.ksn - c.kst) * nu;
            w0 = w0 + (c.kst * u0 + kk * c.n0);
            w1 = w1 + (c.kst * u1 + kk * c.n1);
            w2 = w2 + (c.kst * u2 + kk * c.n2);
            // A x with the warm start filtered: a pinned neighbour's x is not read.
            float xo0 = 0.0f, xo1 = 0.0f, xo2 = 0.0f;
            if (!__ldg(a.pinflag + o)) {
                xo0 = a.x[0][o];
                xo1 = a.x[1][o];
                xo2 = a.x[2][o];
            }
            block_apply(c.n0, c.n1, c.n2, c.beta, c.gamma, xi0 - xo0, xi1 - xo1, xi2 - xo2, ax0, ax1, ax2);
        };
        if (ip.grid_cols > 0) {  // grid cloth: its class's stencil template, no records
            const int32_t cols = ip.grid_cols;
            const int32_t l = (int32_t)(g - ip.v_off), row = l / cols, col = l - row * cols;
            const int cl = stencil_class_1d(row, ip.grid_rows) * 6 + stencil_class_1d(col, cols);
            const int32_t* st = a.st_data + ip.st_off;
            const float4* par = a.st_param + ip.st_par;
            const int32_t e0 = __ldg(st + cl), e1 = __ldg(st + cl + 1);
            const float* rest_inc = ip.st_rest ? a.rest_inc + __ldg(a.rowptr + g) - e0 : nullptr;
            for (int32_t e = e0; e < e1; ++e) {
                const int32_t v = __ldg(st + e);
                const float4 p = __ldg(par + (v >> 7));
                const int32_t o = (int32_t)(g + (int64_t)((v & 7) - 2) * cols + (((v >> 3) & 7) - 2));
                incidence(e - e0, o, (v & 64) != 0, rest_inc ? __ldg(rest_inc + e) : p.x, p.y, p.z);
            }
        } else {
            const int32_t k0 = __ldg(a.rowptr + g), k1 = __ldg(a.rowptr + g + 1);
            for (int32_t k = k0; k < k1; ++k) {
                const int4 rec = __ldg(a.inc + k);
                incidence(k - k0, rec.x & 0x7fffffff, rec.x < 0, __int_as_float(rec.y), __int_as_float(rec.z),
                          __int_as_float(rec.w));
            }
        }
        const float c00 = D[3] * D[5] - D[4] * D[4], c01 = D[2] * D[4] - D[1] * D[5], c02 = D[1] * D[4] - D[2] * D[3];
        const float c11 = D[0] * D[5] - D[2] * D[2], c12 = D[1] * D[2] - D[0] * D[4], c22 = D[0] * D[3] - D[1] * D[1];
        const float det = D[0] * c00 + D[1] * c01 + D[2] * c02;
        const float inv = 1.0f / det;
        const float P[6] = {c00 * inv, c01 * inv, c02 * inv, c11 * inv, c12 * inv, c22 * inv};
        const float b0 = h * (Fx - h * w0), b1 = h * (Fy - h * w1), b2 = h * (Fz - h * w2);
        float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, z0 = 0.0f, z1 = 0.0f, z2 = 0.0f;
        if (!pinned) {
            r0 = b0 - ax0;
            r1 = b1 - ax1;
            r2 = b2 - ax2;
            matvec(P, r0, r1, r2, z0, z1, z2);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) a.A[k][g] = P[k];
        a.cpl_m[g] = mp;
        a.r[0][g] = r0;
        a.r[1][g] = r1;
        a.r[2][g] = r2;
        a.cpl_z[g] = make_float4(z0, z1, z2, 0.0f);
        a.cpl_d[g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (pinned) {
            a.x[0][g] = 0.0f;
            a.x[1][g] = 0.0f;
            a.x[2][g] = 0.0f;
        }
        acc_add(part, r0 * z0 + r1 * z1 + r2 * z2);
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

__global__ void __launch_bounds__(kThreads) k_cpl_dir(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstState& st = a.state[bi.inst];
    const bool active = st.active != 0;
    Acc part = acc_zero();
    if (active) {
        const bool first = st.iter == 0;
        const float beta = st.beta;
        const float4* __restrict__ Z = a.cpl_z;
        const float4* __restrict__ D = a.cpl_d;
        const float* __restrict__ C0 = a.cpl_c[0];
        const float* __restrict__ C1 = a.cpl_c[1];
        const float* __restrict__ C2 = a.cpl_c[2];
        const float* __restrict__ C3 = a.cpl_c[3];
        const float* __restrict__ C4 = a.cpl_c[4];
        for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
            float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f;
            if (!__ldg(a.pinflag + g)) {
                const float4 zg = Z[g];
                float n0 = zg.x, n1 = zg.y, n2 = zg.z;
                if (!first) {
                    const float4 dg = D[g];
                    n0 = n0 + dg.x * beta;
                    n1 = n1 + dg.y * beta;
                    n2 = n2 + dg.z * beta;
                }
                const float mp = __ldg(a.cpl_m + g);
                q0 = mp * n0;
                q1 = mp * n1;
                q2 = mp * n2;
                const int32_t deg = __ldg(a.rowptr + g + 1) - __ldg(a.rowptr + g);
                const int64_t slot0 = __ldg(a.cpl_slice + (g >> 5)) + (g & 31);
                // The per-incidence planes are read once per pass (evict-first, .cs), so
                // the gathered z and d records stay in L2.
                for (int32_t e = 0; e < deg; ++e) {
                    const int64_t k = slot0 + 32 * (int64_t)e;
                    const int32_t o = __ldcs(a.cpl_o + k);
                    const float4 zo = Z[o];
                    float m0 = zo.x, m1 = zo.y, m2 = zo.z;
                    if (!first) {
                        const float4 dd = D[o];
                        m0 = m0 + dd.x * beta;
                        m1 = m1 + dd.y * beta;
                        m2 = m2 + dd.z * beta;
                    }
                    block_apply(__ldcs(C0 + k), __ldcs(C1 + k), __ldcs(C2 + k), __ldcs(C3 + k), __ldcs(C4 + k),
                                n0 - m0, n1 - m1, n2 - m2, q0, q1, q2);
                }
                acc_add(part, n0 * q0 + n1 * q1 + n2 * q2);
            }
            a.q[0][g] = q0;
            a.q[1][g] = q1;
            a.q[2][g] = q2;
        }
    }
    finish<K_CG_DIR>(a, bi.gblk, bi.inst, active, part);
}

__global__ void __launch_bounds__(kThreads) k_cpl_update(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstState& st = a.state[bi.inst];
    const bool active = st.active != 0;
    Acc part = acc_zero();
    if (active) {
        const bool first = st.iter == 0;
        const float alpha = st.alpha, beta = st.beta;
        for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
            float dn[3], r[3];
            const float4 zg = a.cpl_z[g], dg = a.cpl_d[g];
            const float zv[3] = {zg.x, zg.y, zg.z}, dv[3] = {dg.x, dg.y, dg.z};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float v = zv[k];
                if (!first) v = v + dv[k] * beta;
                dn[k] = v;
                a.x[k][g] = a.x[k][g] + dn[k] * alpha;
                r[k] = a.r[k][g] - a.q[k][g] * alpha;
                a.r[k][g] = r[k];
            }
            a.cpl_d[g] = make_float4(dn[0], dn[1], dn[2], 0.0f);
            const float P[6] = {a.A[0][g], a.A[1][g], a.A[2][g], a.A[3][g], a.A[4][g], a.A[5][g]};
            float z0, z1, z2;
            matvec(P, r[0], r[1], r[2], z0, z1, z2);
            a.cpl_z[g] = make_float4(z0, z1, z2, 0.0f);
            acc_add(part, r[0] * z0 + r[1] * z1 + r[2] * z2);
        }
    }
    finish<K_CG_UPDATE>(a, bi.gblk, bi.inst, active, part);
}

}  // namespace

const void* coupled_fn(KernelKind k) {
    switch (k) {
        case K_CPL_ASSEMBLE: return (const void*)k_cpl_assemble;
        case K_CPL_DIR: return (const void*)k_cpl_dir;
        case K_CPL_UPDATE: return (const void*)k_cpl_update;
        default: return nullptr;
    }
}

cudaError_t launch_coupled(KernelKind k, const StepArgs& a, int nblocks, cudaStream_t stream) {
    if (nblocks <= 0) return cudaSuccess;
    switch (k) {
        case K_CPL_ASSEMBLE: k_cpl_assemble<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_CPL_DIR: k_cpl_dir<<<nblocks, kThreads, 0, stream>>>(a); break;
        case K_CPL_UPDATE: k_cpl_update<<<nblocks, kThreads, 0, stream>>>(a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace oc
