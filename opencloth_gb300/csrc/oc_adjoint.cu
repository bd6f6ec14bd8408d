// Adjoint of the implicit step (no counterpart in the reference): reverse-mode
// gradients of a trajectory with respect to per-spring Ks and Kd, the initial state and
// a per-vertex constant external force.
//
// Per step (REFERENCE Jacobian mode; vertex i takes spring i's Jacobians, IMP:737-798):
//   X' = X + dt V' (y clamped at 0), V' = V + dt dV, A dV = b,
//   A_i = m_i I - h Jv_i - h^2 J_i, b_i = h F_i + h^2 J_i V_i,
//   J = Ks n n^T - (Ks C + Kd Cdot) D, D = C diag(1 - dP*dP), Jv = -Kd n n^T,
//   f_s = (-Ks C + Kd (dV.dP)/L) n, F_i = m g + damping V_i + ext_i + sum_s +-f_s.
// The solve is differentiated as an exact solve: one extra CG on the same symmetric A
// gives lambda = A^-1 g_dV, then g_b = lambda and g_A = -lambda dV^T.  All sums are
// gathers in a fixed order (spring-ordered incidences, and per vertex the list of the
// vertices whose own spring touches it), so gradients are deterministic.  This unit is
// compiled with multiply-add contraction and approximate division and square root: the
// gradients are checked against finite differences and an FP64 adjoint, not against the
// reference's rounding sequence.
#include <cuda_runtime.h>

#include <algorithm>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kAdjThreads = 256;

__device__ __forceinline__ float dot3f(float ax, float ay, float az, float bx, float by, float bz) {
    return ax * bx + ay * by + az * bz;
}

// A spring's geometry: dP = x_p1 - x_p2, its length L, 1/L and the elongation C = L - rest.
struct Geo {
    float dP[3];
    float L, iL, C;
};

// From positions.
__device__ __forceinline__ Geo geo_plain(const float4 p1, const float4 p2, float rest) {
    Geo g;
    g.dP[0] = p1.x - p2.x;
    g.dP[1] = p1.y - p2.y;
    g.dP[2] = p1.z - p2.z;
    g.L = sqrtf(dot3f(g.dP[0], g.dP[1], g.dP[2], g.dP[0], g.dP[1], g.dP[2]));
    g.iL = 1.0f / g.L;
    g.C = g.L - rest;
    return g;
}

// Displacement mode: base positions b and displacements u of the two ends, and the
// spring's constants k = {c0, L0} (c0 = |d0| - rest, L0 = |d0|, d0 = b1 - b2, rounded
// from FP64).  dP = d0 + (u1 - u2); the elongation is c0 + (|dP|^2 - |d0|^2) / (|dP| + |d0|)
// with |dP|^2 - |d0|^2 = 2 d0.du + du.du, so it keeps its relative precision when the
// elongation is small against the length (an FP32 L - rest would not).
__device__ __forceinline__ Geo geo_disp(const float4 b1, const float4 b2, const float4 u1, const float4 u2,
                                        const float2 k) {
    const float d0[3] = {b1.x - b2.x, b1.y - b2.y, b1.z - b2.z};
    const float du[3] = {u1.x - u2.x, u1.y - u2.y, u1.z - u2.z};
    Geo g;
#pragma unroll
    for (int c = 0; c < 3; ++c) g.dP[c] = d0[c] + du[c];
    g.L = sqrtf(dot3f(g.dP[0], g.dP[1], g.dP[2], g.dP[0], g.dP[1], g.dP[2]));
    g.iL = 1.0f / g.L;
    const float grow =
        2.0f * dot3f(d0[0], d0[1], d0[2], du[0], du[1], du[2]) + dot3f(du[0], du[1], du[2], du[0], du[1], du[2]);
    g.C = k.x + grow / (g.L + k.y);
    return g;
}

// Spring (p1, p2) with ends at x1, x2 (positions, or displacements in the displacement
// mode, where consts[at] holds its start constants).
__device__ __forceinline__ Geo spring_geo(const StepArgs& a, int32_t p1, int32_t p2, const float4 x1, const float4 x2,
                                          float rest, const float2* consts, int64_t at) {
    if (!a.gm) return geo_plain(x1, x2, rest);
    return geo_disp(__ldg(a.Xbase + p1), __ldg(a.Xbase + p2), x1, x2, __ldg(consts + at));
}

// The per-spring quantities of CalcForceDerivatives (IMP:719-724) from a geometry.
__device__ __forceinline__ void spring_eval(const Geo& G, const float4 v1, const float4 v2, SpringEval& e) {
    e.C = G.C;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        e.n[c] = G.dP[c] * G.iL;
        e.q[c] = G.dP[c] * G.dP[c];
    }
    e.Cdot = (v1.x * (-e.n[0]) + v1.y * (-e.n[1]) + v1.z * (-e.n[2])) + (v2.x * e.n[0] + v2.y * e.n[1] + v2.z * e.n[2]);
}

// Adjoint of one spring force f = (-Ks C + Kd u) n for dL/df = g.
__device__ __forceinline__ void spring_force_adj(const Geo& G, const float4 v1, const float4 v2, float ks, float kd,
                                                 const float g[3], float gdP[3], float gdV[3], float& gks,
                                                 float& gkd) {
    const float* dP = G.dP;
    const float dV[3] = {v1.x - v2.x, v1.y - v2.y, v1.z - v2.z};
    const float iL = G.iL;
    const float n[3] = {dP[0] * iL, dP[1] * iL, dP[2] * iL};
    const float C = G.C;
    const float u = dot3f(dV[0], dV[1], dV[2], dP[0], dP[1], dP[2]) * iL;
    const float m = -ks * C + kd * u;
    const float gm = dot3f(g[0], g[1], g[2], n[0], n[1], n[2]);
    const float gn[3] = {m * g[0], m * g[1], m * g[2]};
    const float ng = dot3f(n[0], n[1], n[2], gn[0], gn[1], gn[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        gdP[k] = gm * (-ks * n[k] + kd * (dV[k] - u * n[k]) * iL) + (gn[k] - n[k] * ng) * iL;
        gdV[k] = gm * kd * n[k];
    }
    gks = -C * gm;
    gkd = u * gm;
}

// Adjoint of spring i's (J, Jv) for G = dL/dJ, H = dL/dJv (full 3x3, row-major).
__device__ __forceinline__ void spring_jac_adj(const Geo& Gm, const float4 v1, const float4 v2, float ks, float kd,
                                               const float G[3][3], const float H[3][3], float gdP[3], float gdV[3],
                                               float& gks, float& gkd) {
    const float* dP = Gm.dP;
    const float dV[3] = {v1.x - v2.x, v1.y - v2.y, v1.z - v2.z};
    const float iL = Gm.iL;
    const float n[3] = {dP[0] * iL, dP[1] * iL, dP[2] * iL};
    const float C = Gm.C;
    const float Cd = -dot3f(n[0], n[1], n[2], dV[0], dV[1], dV[2]);
    const float w = ks * C + kd * Cd;
    float gS[3][3];
    gks = 0.0f;
    gkd = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float S = n[r] * n[c];
            gS[r][c] = ks * G[r][c] - kd * H[r][c];
            gks += G[r][c] * S;
            gkd += -H[r][c] * S;
        }
    float gw = 0.0f, gC = 0.0f, gq[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float D = C * (1.0f - dP[k] * dP[k]);
        gw += -G[k][k] * D;
        const float gD = -w * G[k][k];
        gC += gD * (1.0f - dP[k] * dP[k]);
        gq[k] = -C * gD;
    }
    gC += ks * gw;
    const float gCd = kd * gw;
    gks += C * gw;
    gkd += Cd * gw;
    float gn[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        gn[r] = (gS[r][0] + gS[0][r]) * n[0] + (gS[r][1] + gS[1][r]) * n[1] + (gS[r][2] + gS[2][r]) * n[2] -
                gCd * dV[r];
    const float ng = dot3f(n[0], n[1], n[2], gn[0], gn[1], gn[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        gdV[k] = -gCd * n[k];
        gdP[k] = 2.0f * dP[k] * gq[k] + gC * n[k] + (gn[k] - n[k] * ng) * iL;
    }
}

// Per vertex i: lambda -> g_F = h lambda, the terms of A_i and b_i: g_J = h^2 lambda (V +
// dV)^T, g_Jv = h lambda dV^T, g_V += h^2 J lambda + damping g_F, g_ext += g_F; spring
// i's Jacobian adjoint goes to the vertex's own-spring slots and to Ks_i, Kd_i.
// Variants (AdjArgs::vertex_variant): VPT vertices per thread with every load of a stage
// in flight together (the vertex's own entries, then spring i's ends and old gradient
// entries, then the arithmetic), and CTAs per SM the register budget is set for.  The
// default, one vertex and three CTAs, measured 0.08 ms faster per reverse step on 12 M
// vertices than two vertices and two CTAs.
template <int VPT, int MINB>
__global__ void __launch_bounds__(kAdjThreads, MINB) k_adj_vertex(const StepArgs a, const AdjArgs j) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    const float h = a.dt;
    const int64_t T = blockDim.x;
    for (int64_t base = bi.v_begin + threadIdx.x; base < bi.v_end; base += VPT * T) {
        float4 Vg[VPT];
        float lam[VPT][3], dv[VPT][3], gv[VPT][3];
        OwnSpring os[VPT];
        int32_t sid[VPT];
        float gk_old[VPT], gd_old[VPT];
        bool ok[VPT];
#pragma unroll
        for (int u = 0; u < VPT; ++u) {
            const int64_t g = base + u * T;
            ok[u] = g < bi.v_end;
            const int64_t q = ok[u] ? g : base;
            Vg[u] = a.V[q];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                lam[u][k] = a.x[k][q];
                dv[u][k] = j.dV[k][q];
                gv[u][k] = j.gV[k][q];
            }
            os[u].ends = __ldg(a.own_ends + q);
            sid[u] = __ldg(j.own_sid + q);
            if (!ok[u]) os[u].ends.x = -1;
        }
#pragma unroll
        for (int u = 0; u < VPT; ++u) {
            os[u].par = make_float4(0.f, 0.f, 0.f, 0.f);
            os[u].E1 = os[u].E2 = os[u].W1 = os[u].W2 = make_float4(0.f, 0.f, 0.f, 0.f);
            gk_old[u] = gd_old[u] = 0.0f;
            if (os[u].ends.x >= 0 && Vg[u].w == 0.0f) {
                const int64_t g = base + u * T;
                os[u].par = __ldg(a.own_par + g);
                os[u].E1 = __ldg(a.X + os[u].ends.x);
                os[u].E2 = __ldg(a.X + os[u].ends.y);
                os[u].W1 = __ldg(a.V + os[u].ends.x);
                os[u].W2 = __ldg(a.V + os[u].ends.y);
                gk_old[u] = j.gKs[sid[u]];
                gd_old[u] = j.gKd[sid[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < VPT; ++u) {
            if (!ok[u]) continue;
            const int64_t g = base + u * T;
            const bool pinned = Vg[u].w != 0.0f;
            const float v[3] = {Vg[u].x, Vg[u].y, Vg[u].z};
            float gF[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) gF[k] = pinned ? 0.0f : h * lam[u][k];
            float gdP[3] = {0.f, 0.f, 0.f}, gdVs[3] = {0.f, 0.f, 0.f};
            if (os[u].ends.x >= 0 && !pinned) {
                const Geo geo = spring_geo(a, os[u].ends.x, os[u].ends.y, os[u].E1, os[u].E2, os[u].par.x, a.gm_own, g);
                SpringEval e;
                spring_eval(geo, os[u].W1, os[u].W2, e);
                float J[6], Jv[6];
                jac_element(e, os[u].par.y, os[u].par.z, 0, 0, J[0], Jv[0]);
                jac_element(e, os[u].par.y, os[u].par.z, 0, 1, J[1], Jv[1]);
                jac_element(e, os[u].par.y, os[u].par.z, 0, 2, J[2], Jv[2]);
                jac_element(e, os[u].par.y, os[u].par.z, 1, 1, J[3], Jv[3]);
                jac_element(e, os[u].par.y, os[u].par.z, 1, 2, J[4], Jv[4]);
                jac_element(e, os[u].par.y, os[u].par.z, 2, 2, J[5], Jv[5]);
                float jl0, jl1, jl2;
                matvec(J, lam[u][0], lam[u][1], lam[u][2], jl0, jl1, jl2);
                gv[u][0] += h * h * jl0;
                gv[u][1] += h * h * jl1;
                gv[u][2] += h * h * jl2;
                float G[3][3], H[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        G[r][c] = h * h * lam[u][r] * (v[c] + dv[u][c]);
                        H[r][c] = h * lam[u][r] * dv[u][c];
                    }
                float gks, gkd;
                spring_jac_adj(geo, os[u].W1, os[u].W2, os[u].par.y, os[u].par.z, G, H, gdP, gdVs, gks, gkd);
                j.gKs[sid[u]] = gk_old[u] + gks;
                j.gKd[sid[u]] = gd_old[u] + gkd;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                gv[u][k] += ip.damping * gF[k];
                j.gV[k][g] = gv[u][k];
                j.gF[k][g] = gF[k];
                j.gOwn[k][g] = gdP[k];
                j.gOwn[3 + k][g] = gdVs[k];
                if (!pinned) j.gExt[k][g] += gF[k];
            }
        }
    }
}

// Per vertex v: every incident spring's force adjoint, in spring-id order (the spring's
// p1 side also adds to Ks_s, Kd_s), then the own-spring Jacobian terms of the vertices
// whose spring touches v.  The incidences are taken kAdjAhead at a time: their
// neighbours' states and gradient entries are all in flight before the first is used.
// An incidence comes from the vertex's record (neighbour | p2 flag, rest, Ks, Kd), or,
// for a grid cloth whose parameters fit its stencil slots (the forward's stencil
// condition), from its class's template entry: the neighbour offset and the parameter
// slot, no record read (rest lengths that vary from rest_inc, as the forward reads them).
// Both give the same incidences in the same order, so the same bits.  A spring's Ks / Kd
// gradient is written only by its p1 vertex, so its old value can be fetched early.
struct AdjInc {
    int32_t o;      // the other end
    bool p2;        // this vertex is the spring's p2
    float rest, ks, kd;
};

template <bool STENCIL, int kAdjAhead>
__device__ __forceinline__ void adj_springs_vertex(const StepArgs& a, const AdjArgs& j, const InstParams& ip,
                                                   int64_t g) {
    const float4* __restrict__ X = a.X;
    const float4* __restrict__ V = a.V;
    const float* __restrict__ gF0 = j.gF[0];
    const float* __restrict__ gF1 = j.gF[1];
    const float* __restrict__ gF2 = j.gF[2];
    const float4 Xg = __ldg(X + g), Vg = __ldg(V + g);
    const float gFg[3] = {__ldg(gF0 + g), __ldg(gF1 + g), __ldg(gF2 + g)};
    float gx[3] = {j.gX[0][g], j.gX[1][g], j.gX[2][g]};
    float gv[3] = {j.gV[0][g], j.gV[1][g], j.gV[2][g]};
    const int32_t k0 = __ldg(a.rowptr + g), k1 = __ldg(a.rowptr + g + 1);
    const int32_t* st = nullptr;
    const float4* par = nullptr;
    int32_t ebase = 0;
    const int32_t cols = ip.grid_cols;
    if constexpr (STENCIL) {
        const int32_t l = (int32_t)(g - ip.v_off);
        const int32_t r = l / cols, c = l - r * cols;
        st = a.st_data + ip.st_off;
        par = a.st_param + ip.st_par;
        ebase = __ldg(st + stencil_class_1d(r, ip.grid_rows) * 6 + stencil_class_1d(c, cols)) - k0;
    }
    for (int32_t kb = k0; kb < k1; kb += kAdjAhead) {
        AdjInc in[kAdjAhead];
        int32_t sid[kAdjAhead];
#pragma unroll
        for (int u = 0; u < kAdjAhead; ++u) {
            const int32_t k = kb + u;
            if (k >= k1) {
                in[u] = AdjInc{(int32_t)g, true, 0.0f, 0.0f, 0.0f};
            } else if constexpr (STENCIL) {
                const int32_t v = __ldg(st + ebase + k);
                const int32_t di = (v & 7) - 2, dj = ((v >> 3) & 7) - 2;
                const float4 p = __ldg(par + (v >> 7));
                in[u] = AdjInc{(int32_t)(g + (int64_t)di * cols + dj), (v & 64) != 0,
                               ip.st_rest ? __ldg(a.rest_inc + k) : p.x, p.y, p.z};
            } else {
                const int4 rec = __ldg(a.inc + k);
                in[u] = AdjInc{rec.x & 0x7fffffff, rec.x < 0, __int_as_float(rec.y), __int_as_float(rec.z),
                               __int_as_float(rec.w)};
            }
            sid[u] = (k < k1 && !in[u].p2) ? __ldg(j.inc_sid + k) : 0;
        }
        float4 Xo[kAdjAhead], Vo[kAdjAhead];
        float gFo[kAdjAhead][3], gk_old[kAdjAhead], gd_old[kAdjAhead];
#pragma unroll
        for (int u = 0; u < kAdjAhead; ++u) {
            const int32_t o = in[u].o;
            Xo[u] = __ldg(X + o);
            Vo[u] = __ldg(V + o);
            gFo[u][0] = __ldg(gF0 + o);
            gFo[u][1] = __ldg(gF1 + o);
            gFo[u][2] = __ldg(gF2 + o);
            const bool p1 = kb + u < k1 && !in[u].p2;
            gk_old[u] = p1 ? j.gKs[sid[u]] : 0.0f;
            gd_old[u] = p1 ? j.gKd[sid[u]] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < kAdjAhead; ++u) {
            if (kb + u >= k1) break;
            const bool as_p2 = in[u].p2;
            // g_f = [p1 free] gF[p1] - [p2 free] gF[p2]; k_adj_vertex leaves gF = 0 at
            // pinned vertices.
            float gf[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) gf[c] = as_p2 ? gFo[u][c] - gFg[c] : gFg[c] - gFo[u][c];
            float gdP[3], gdV[3], gks, gkd;
            const int32_t o = in[u].o;
            if (as_p2)
                spring_force_adj(spring_geo(a, o, (int32_t)g, Xo[u], Xg, in[u].rest, a.gm_inc, kb + u), Vo[u], Vg,
                                 in[u].ks, in[u].kd, gf, gdP, gdV, gks, gkd);
            else
                spring_force_adj(spring_geo(a, (int32_t)g, o, Xg, Xo[u], in[u].rest, a.gm_inc, kb + u), Vg, Vo[u],
                                 in[u].ks, in[u].kd, gf, gdP, gdV, gks, gkd);
            const float sgn = as_p2 ? -1.0f : 1.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                gx[c] += sgn * gdP[c];
                gv[c] += sgn * gdV[c];
            }
            if (!as_p2) {
                j.gKs[sid[u]] = gk_old[u] + gks;
                j.gKd[sid[u]] = gd_old[u] + gkd;
            }
        }
    }
    const int32_t o0 = __ldg(j.own_rowptr + g), o1 = __ldg(j.own_rowptr + g + 1);
    for (int32_t k = o0; k < o1; ++k) {
        const int32_t e = __ldg(j.own_ent + k);
        const int32_t i = e & 0x7fffffff;
        const float sgn = e < 0 ? -1.0f : 1.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            gx[c] += sgn * j.gOwn[c][i];
            gv[c] += sgn * j.gOwn[3 + c][i];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        j.gX[c][g] = gx[c];
        j.gV[c][g] = gv[c];
    }
}

// Variants (AdjArgs::springs_variant): incidences in flight per batch and CTAs per SM
// the register budget is set for.  The default, two incidences and three CTAs (80
// registers), measured 0.3 ms faster per reverse step on 12M vertices than four and two.
template <int AHEAD, int MINB>
__global__ void __launch_bounds__(kAdjThreads, MINB) k_adj_springs(const StepArgs a, const AdjArgs j) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    if (ip.grid_cols > 0) {
        for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x)
            adj_springs_vertex<true, AHEAD>(a, j, ip, g);
    } else {
        for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x)
            adj_springs_vertex<false, AHEAD>(a, j, ip, g);
    }
}

// ---- displacement mode: the taped forward in X = Xbase + u --------------------------------
// An FP32 position near 5 resolves steps of about 5e-7, and an FP32 L - rest loses the
// bits of an elongation 1e-3 of the length, so an FP32 trajectory of a slow cloth drifts
// from the FP64 one by a good fraction of a small loss residual.  In this mode the state
// holds the displacement u from the tape's start and each spring's elongation is formed
// from its FP64-rounded start constants (geo_disp); the forward otherwise follows the
// step's arithmetic, the CG included.

// 0: Xbase = X.
__global__ void k_gm_base(const StepArgs a, int64_t nv) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nv; g += (int64_t)gridDim.x * blockDim.x)
        const_cast<float4*>(a.Xbase)[g] = a.X[g];
}

__device__ __forceinline__ float2 spring_consts(const float4 b1, const float4 b2, float rest) {
    const double dx = (double)b1.x - (double)b2.x, dy = (double)b1.y - (double)b2.y, dz = (double)b1.z - (double)b2.z;
    const double L0 = sqrt(dx * dx + dy * dy + dz * dz);
    return make_float2((float)(L0 - (double)rest), (float)L0);
}

// 4: the spring constants from Xbase, and u = 0 (mass kept in w).
__global__ void k_gm_consts(const StepArgs a, int64_t nv) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nv; g += (int64_t)gridDim.x * blockDim.x) {
        const float4 bg = __ldg(a.Xbase + g);
        const int32_t k0 = __ldg(a.rowptr + g), k1 = __ldg(a.rowptr + g + 1);
        for (int32_t k = k0; k < k1; ++k) {
            const int4 rec = __ldg(a.inc + k);
            const float4 bo = __ldg(a.Xbase + (rec.x & 0x7fffffff));
            const float rest = __int_as_float(rec.y);
            const_cast<float2*>(a.gm_inc)[k] = rec.x < 0 ? spring_consts(bo, bg, rest) : spring_consts(bg, bo, rest);
        }
        const int2 e = __ldg(a.own_ends + g);
        float2 own = make_float2(0.f, 0.f);
        if (e.x >= 0) own = spring_consts(__ldg(a.Xbase + e.x), __ldg(a.Xbase + e.y), __ldg(a.own_par + g).x);
        const_cast<float2*>(a.gm_own)[g] = own;
        a.X[g] = make_float4(0.f, 0.f, 0.f, bg.w);
    }
}

// 3: X = Xbase + u.
__global__ void k_gm_leave(const StepArgs a, int64_t nv) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nv; g += (int64_t)gridDim.x * blockDim.x) {
        const float4 b = __ldg(a.Xbase + g), u = a.X[g];
        a.X[g] = make_float4(b.x + u.x, b.y + u.y, b.z + u.z, u.w);
    }
}

// The spring force on p1 (IMP:717-728) from a geometry.
__device__ __forceinline__ float3 spring_force_geo(const Geo& G, const float4 v1, const float4 v2, float ks, float kd) {
    const float dVx = v1.x - v2.x, dVy = v1.y - v2.y, dVz = v1.z - v2.z;
    const float left = (-ks) * G.C;
    const float right = kd * (dot3f(dVx, dVy, dVz, G.dP[0], G.dP[1], G.dP[2]) * G.iL);
    const float mag = left + right;
    return make_float3(mag * (G.dP[0] * G.iL), mag * (G.dP[1] * G.iL), mag * (G.dP[2] * G.iL));
}

// 1: the step's assembly in displacement mode (incidence-record gather in spring order,
// spring i's Jacobians, A and b, the CG set-up), one thread per vertex.
// Spring i's blocks of vertex g in the displacement mode (IMP:744-770 on geo_disp):
// A = M - h (Jv + h J) and h J.  The assembly and the reverse pass's seed both form them
// here.
__device__ __forceinline__ void gm_own_blocks(const StepArgs& a, int64_t g, float mass, float h, float A[6],
                                              float hJ[6]) {
    const OwnSpring os = load_own(a, g);
    float J[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, Jv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (os.ends.x >= 0) {
        SpringEval e;
        spring_eval(spring_geo(a, os.ends.x, os.ends.y, os.E1, os.E2, 0.0f, a.gm_own, g), os.W1, os.W2, e);
        jac_element(e, os.par.y, os.par.z, 0, 0, J[0], Jv[0]);
        jac_element(e, os.par.y, os.par.z, 0, 1, J[1], Jv[1]);
        jac_element(e, os.par.y, os.par.z, 0, 2, J[2], Jv[2]);
        jac_element(e, os.par.y, os.par.z, 1, 1, J[3], Jv[3]);
        jac_element(e, os.par.y, os.par.z, 1, 2, J[4], Jv[4]);
        jac_element(e, os.par.y, os.par.z, 2, 2, J[5], Jv[5]);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float Mk = (k == 0 || k == 3 || k == 5) ? mass : 0.0f;
        A[k] = Mk - h * (Jv[k] + h * J[k]);
        hJ[k] = h * J[k];
    }
}

__global__ void __launch_bounds__(kAdjThreads) k_gm_assemble(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const InstParams& ip = a.inst[bi.inst];
    const float h = a.dt;
    Acc part = acc_zero();
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Ug = a.X[g], Vg = a.V[g];
        const bool pinned = Vg.w != 0.0f;
        float Fx = 0.0f, Fy = 0.0f, Fz = 0.0f;
        if (!pinned) {
            Fx += Ug.w * ip.gravity[0];
            Fy += Ug.w * ip.gravity[1];
            Fz += Ug.w * ip.gravity[2];
        }
        Fx += ip.damping * Vg.x;
        Fy += ip.damping * Vg.y;
        Fz += ip.damping * Vg.z;
        if (!pinned) {
            if (ip.has_ext) {
                const float4 e = __ldg(a.fext + g);
                Fx += e.x;
                Fy += e.y;
                Fz += e.z;
            }
            const int32_t k0 = __ldg(a.rowptr + g), k1 = __ldg(a.rowptr + g + 1);
            for (int32_t k = k0; k < k1; ++k) {
                const int4 rec = __ldg(a.inc + k);
                const int32_t o = rec.x & 0x7fffffff;
                const float4 Uo = a.X[o], Vo = a.V[o];
                const float ks = __int_as_float(rec.z), kd = __int_as_float(rec.w);
                if (rec.x < 0) {  // F[p2] -= f
                    const float3 f =
                        spring_force_geo(spring_geo(a, o, (int32_t)g, Uo, Ug, 0.0f, a.gm_inc, k), Vo, Vg, ks, kd);
                    Fx -= f.x;
                    Fy -= f.y;
                    Fz -= f.z;
                } else {  // F[p1] += f
                    const float3 f =
                        spring_force_geo(spring_geo(a, (int32_t)g, o, Ug, Uo, 0.0f, a.gm_inc, k), Vg, Vo, ks, kd);
                    Fx += f.x;
                    Fy += f.y;
                    Fz += f.z;
                }
            }
        }
        // Spring i's Jacobians (IMP:744-770) and the vertex's system.
        VertexSystem sys;
        float hJ[6];
        gm_own_blocks(a, g, Ug.w, h, sys.A, hJ);
        float wx, wy, wz;
        matvec(hJ, Vg.x, Vg.y, Vg.z, wx, wy, wz);
        sys.b[0] = h * (Fx + wx);
        sys.b[1] = h * (Fy + wy);
        sys.b[2] = h * (Fz + wz);
        const CgInit c = cg_init(sys, a.x[0][g], a.x[1][g], a.x[2][g], pinned);
#pragma unroll
        for (int k = 0; k < 6; ++k) a.A[k][g] = sys.A[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            a.x[k][g] = c.x[k];
            a.r[k][g] = c.r[k];
            a.d[k][g] = c.d[k];
        }
        acc_add(part, c.term);
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

// The reverse pass's seed in the displacement mode: spring i's blocks rebuilt as the
// assembly formed them (A planes written), then adj_seed_vertex and the epilogue.
__global__ void __launch_bounds__(kAdjThreads) k_gm_seed_own(const StepArgs a, const AdjArgs j) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    Acc part = acc_zero();
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const float4 Ug = a.X[g], Vg = a.V[g];
        float A[6], hJ[6];
        gm_own_blocks(a, g, Ug.w, a.dt, A, hJ);
#pragma unroll
        for (int k = 0; k < 6; ++k) a.A[k][g] = A[k];
        acc_add(part, adj_seed_vertex(a, j, g, Ug, Vg, A[0], A[3], A[5]));
    }
    finish<K_ASSEMBLE>(a, bi.gblk, bi.inst, true, part);
}

// 2: V += dV dt, u += dt V, ground clamp on the position (IMP:790-797).
__global__ void __launch_bounds__(kAdjThreads) k_gm_update(const StepArgs a) {
    const int blk = blockIdx.x + a.blk_base;
    const BlockInfo bi = a.blocks[blk];
    const float dt = a.dt;
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        float4 U = a.X[g], V = a.V[g];
        gm_advance(dt, a.x[0][g], a.x[1][g], a.x[2][g], __ldg(a.Xbase + g).y, U, V);
        a.X[g] = U;
        a.V[g] = V;
    }
}

// Per-spring Ks / Kd into the incidence records and spring i's parameters.
__global__ void k_set_spring_params(const StepArgs a, const AdjArgs j, const float* ks, const float* kd, int64_t n_rec,
                                    int64_t nv) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_rec; k += stride) {
        const int32_t s = j.inc_sid[k];
        int4 rec = a.inc[k];
        rec.z = __float_as_int(ks[s]);
        rec.w = __float_as_int(kd[s]);
        const_cast<int4*>(a.inc)[k] = rec;
    }
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nv; g += stride) {
        const int32_t s = j.own_sid[g];
        if (s >= 0) {
            float4 p = a.own_par[g];
            p.y = ks[s];
            p.z = kd[s];
            const_cast<float4*>(a.own_par)[g] = p;
        }
    }
}

}  // namespace

cudaError_t launch_adjoint(int which, const StepArgs& a, const AdjArgs& j, int nblocks, cudaStream_t stream) {
    if (nblocks <= 0) return cudaSuccess;
    switch (which) {
        case 0: k_gm_seed_own<<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
        case 1:
            switch (j.vertex_variant) {
                case 1: k_adj_vertex<2, 2><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
                case 2: k_adj_vertex<2, 3><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
                default: k_adj_vertex<1, 3><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
            }
            break;
        case 2:
            switch (j.springs_variant) {
                case 1: k_adj_springs<4, 2><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
                case 2: k_adj_springs<2, 2><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
                case 3: k_adj_springs<1, 4><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
                default: k_adj_springs<2, 3><<<nblocks, kAdjThreads, 0, stream>>>(a, j); break;
            }
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}


cudaError_t launch_gm(int which, const StepArgs& a, int n, cudaStream_t stream) {
    const int64_t nv = (int64_t)n;  // the per-vertex kernels (0, 3, 4) take the vertex count
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((nv + kAdjThreads - 1) / kAdjThreads, 152 * 8));
    switch (which) {
        case 0: k_gm_base<<<gs, kAdjThreads, 0, stream>>>(a, nv); break;
        case 1: if (n > 0) k_gm_assemble<<<n, kAdjThreads, 0, stream>>>(a); break;
        case 2: if (n > 0) k_gm_update<<<n, kAdjThreads, 0, stream>>>(a); break;
        case 3: k_gm_leave<<<gs, kAdjThreads, 0, stream>>>(a, nv); break;
        case 4: k_gm_consts<<<gs, kAdjThreads, 0, stream>>>(a, nv); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_set_spring_params(const StepArgs& a, const AdjArgs& j, const float* ks, const float* kd,
                                     int64_t n_rec, int64_t nv, cudaStream_t stream) {
    k_set_spring_params<<<152 * 8, 256, 0, stream>>>(a, j, ks, kd, n_rec, nv);
    return cudaGetLastError();
}

}  // namespace oc
