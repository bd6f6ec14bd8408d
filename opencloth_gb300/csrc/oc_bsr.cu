// Batched block-sparse conjugate gradient with the FEM demo's semantics:
// ConjugateGradientSolver of OpenCloth_CoRotated_Linear_FEM/.../main.cpp (FEM:837-922),
// on the same engine shape as the cloth step (fixed-order per-system reductions, a
// CUDA-graph WHILE loop, batches of independent systems).
//
// The reference keeps each block row as a std::map<int, mat3> and walks it in ascending
// column order.  Here the rows of a system are reordered by block count (within windows)
// and cut into slices of 32 rows (one warp) stored slot-major (sliced ELL with sorting):
// slot j of lane l of slice s holds the j-th block of that row as two float4 and a
// {component 8, column} pair, so every load of a warp is coalesced; the columns are a
// static table built at create time, and each solve first packs the caller's CSR blocks.
// Each lane sums its own row's products in slot order (the reference's order).
//
//   k_bsr_pack    CSR blocks -> sliced planes
//   k_bsr_init    r = b - A V, p = r               (FEM:841-859)
//   k_bsr_spmv    p = r + d4 p (not in the first pass, FEM:913-917, rebuilt for the
//                 neighbours from their r and p); q = A p; d = r.r, d2 = p.q  (FEM:865-883)
//   k_bsr_update  d3 = d / d2; V += d3 p; r -= d3 q; d1 = r.r  (FEM:885-901), d4 = d1 / d
//   k_bsr_resident  all of the above for a system of up to 256 rows whose blocks fit in
//                 shared memory, in one CTA: the blocks are read once, the iterations run
//                 on chip, with the streamed kernels' bits (the default executor's choice)
//
// FP32 vector arithmetic in the reference's order (--fmad=false); the dot products sum
// FP32 per-row terms in error-free float pairs within a warp and FP64 above, and
// d3 = d / d2, d4 = d1 / d are FP64 quotients rounded to FP32, after the reference's
// `tiny` clamps (FEM:885-886, 908-909).  Exactly i_max iterations run: the reference's
// exit test (FEM:905) cannot fire inside its loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerBlock = 256;  // one row per thread: enough warps to cover the gathers
constexpr int kSortWindow = 2048;   // rows reordered by block count within windows of this size
static_assert(kSortWindow >= kThreads, "a resident system's rows are sorted as one window");

struct BsrState {
    double d, d2, d1;
    float d3, d4;
    int32_t iter;
    int32_t active;
    uint32_t ticket;
    int32_t pad_;
};

struct BsrParams {
    int32_t imax;
    float tiny;
    int32_t blk0, nblk;  // the system's blocks in the streamed block table (none if resident)
    int64_t row0;         // first (global) row
    int64_t slice0;       // first slice
    int32_t n_rows;
    int32_t pad_;
};

struct BsrArgs {
    const BlockInfo* blocks;
    const BsrParams* sys;
    BsrState* state;
    const int64_t* slice_ptr;  // slot offset of each slice (units of 32 entries)
    const int32_t* sb2_col;    // the static column of each slot (-1 for padding), merged into sb2 by pack
    const int32_t* width;      // slots of each slice
    float4* sb0;               // sliced blocks: components 0-3 and 4-7 of each slot, and
    float4* sb1;               // {component 8, column (global row; -1 for padding)}
    float2* sb2;
    const int32_t* row_ptr;    // caller's CSR (global, over all systems, the caller's row order)
    const int32_t* iperm;      // internal row -> caller's row
    const int32_t* deg;        // blocks of each internal row
    const float* cblk;         // caller's CSR blocks (9 per block)
    const uint8_t* fixed;
    const float* b;            // 3 per row
    float* x[3];               // V (unknown) planes
    float4* r4;                // residual and direction, gathered by the neighbours: one
    float4* p4;                // 16-byte load each (w unused)
    float* q[3];
    double* partials;          // 2 per block
    int32_t* unfinished;
    uint32_t* grid_ticket;
    unsigned long long* loop_count;
    int32_t use_cond;
    unsigned long long cond;
};

__device__ __forceinline__ void block_mv(const float m[9], float v0, float v1, float v2, float& o0, float& o1,
                                         float& o2) {
    // prod.x = m[0][0] x + m[0][1] y + m[0][2] z (FEM:873-875)
    o0 = m[0] * v0 + m[1] * v1 + m[2] * v2;
    o1 = m[3] * v0 + m[4] * v1 + m[5] * v2;
    o2 = m[6] * v0 + m[7] * v1 + m[8] * v2;
}

// Slot j of row g's slice: (index, lane) -> position in the sliced arrays.
__device__ __forceinline__ int64_t slot_pos(const BsrArgs& a, const BsrParams& sp, int64_t g, int j) {
    const int64_t local = g - sp.row0;
    const int64_t s = sp.slice0 + (local >> 5);
    return (a.slice_ptr[s] + j) * 32 + (local & 31);
}

// One slot: the block and its column.  The sliced planes are read once per pass and are
// far larger than L2, so they are loaded evict-first (.cs): the direction and residual
// records the rows gather stay in L2.
__device__ __forceinline__ int32_t load_block(const BsrArgs& a, int64_t pos, float m[9]) {
    const float4 u = __ldcs(a.sb0 + pos), v = __ldcs(a.sb1 + pos);
    const float2 w = __ldcs(a.sb2 + pos);
    m[0] = u.x; m[1] = u.y; m[2] = u.z; m[3] = u.w;
    m[4] = v.x; m[5] = v.y; m[6] = v.z; m[7] = v.w;
    m[8] = w.x;
    return __float_as_int(w.y);
}

__global__ void __launch_bounds__(kThreads) k_bsr_pack(const BsrArgs a) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const BsrParams& sp = a.sys[bi.inst];
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const int64_t u = a.iperm[g];
        const int32_t e0 = a.row_ptr[u], e1 = a.row_ptr[u + 1];
        for (int32_t e = e0; e < e1; ++e) {
            const int64_t pos = slot_pos(a, sp, g, e - e0);
            const float* m = a.cblk + 9 * (size_t)e;
            a.sb0[pos] = make_float4(m[0], m[1], m[2], m[3]);
            a.sb1[pos] = make_float4(m[4], m[5], m[6], m[7]);
            a.sb2[pos] = make_float2(m[8], __int_as_float(__ldg(a.sb2_col + pos)));
        }
    }
}

// Two-value last-block epilogue (per system), and the grid-wide WHILE condition.
// The per-system scalars from the system's totals (thread 0 of the system's last block).
template <int KIND>
__device__ void bsr_scalars(const BsrArgs& a, int inst, double tot0, double tot1) {
    const BsrParams& sp = a.sys[inst];
    BsrState& st = a.state[inst];
    st.ticket = 0;
    const double tiny = (double)sp.tiny;
    if (KIND == 0) {  // after the matrix-vector pass: d, d2, d3
        st.d = tot0;
        double d2 = tot1;
        st.d2 = d2;
        if (fabs(d2) < tiny) d2 = tiny;  // FEM:885-886
        st.d3 = (float)(tot0 / d2);
    } else {  // after the update: d1, d4, next iteration
        st.d1 = tot0;
        double d = st.d;
        if (fabs(d) < tiny) d = tiny;  // FEM:908-909
        st.d4 = (float)(tot0 / d);
        st.iter += 1;
        if (st.iter >= sp.imax) {
            st.active = 0;
            atomicSub(a.unfinished, 1);
        }
    }
    __threadfence();
}

template <int KIND>
__device__ void bsr_finish(const BsrArgs& a, int blk, int inst, bool participates, Acc p0, Acc p1) {
    __shared__ int s_last;
    if (participates && a.sys[inst].nblk == 1) {
        // A one-block system: its block sums are the totals (the multi-block path would
        // add this one partial to zeros, which is exact).
        const double s0 = block_sum_acc(p0);
        const double s1 = KIND == 0 ? block_sum_acc(p1) : 0.0;
        if (threadIdx.x == 0) bsr_scalars<KIND>(a, inst, s0, s1);
    } else if (participates) {
        const double s0 = block_sum_acc(p0);
        const double s1 = KIND == 0 ? block_sum_acc(p1) : 0.0;
        if (threadIdx.x == 0) {
            a.partials[2 * blk] = s0;
            a.partials[2 * blk + 1] = s1;
            __threadfence();
            const unsigned t = atomicAdd(&a.state[inst].ticket, 1u);
            s_last = (t == (unsigned)(a.sys[inst].nblk - 1));
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            const BsrParams& sp = a.sys[inst];
            double t0 = 0.0, t1 = 0.0;
            for (int j = threadIdx.x; j < sp.nblk; j += blockDim.x) {
                t0 += __ldcg(a.partials + 2 * (sp.blk0 + j));
                t1 += __ldcg(a.partials + 2 * (sp.blk0 + j) + 1);
            }
            const double tot0 = block_sum(t0);
            const double tot1 = KIND == 0 ? block_sum(t1) : 0.0;
            if (threadIdx.x == 0) bsr_scalars<KIND>(a, inst, tot0, tot1);
        }
    }
    if (KIND == 1 && threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(a.grid_ticket, 1u);
        if (t == gridDim.x - 1) {
            *a.grid_ticket = 0u;
            atomicAdd(a.loop_count, 1ull);
            __threadfence();
            if (a.use_cond) {
                const int u = atomicAdd(a.unfinished, 0);
                cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, u > 0 ? 1u : 0u);
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_bsr_init(const BsrArgs a) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const BsrParams& sp = a.sys[bi.inst];
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
        if (!a.fixed[g]) {
            r0 = a.b[3 * g];
            r1 = a.b[3 * g + 1];
            r2 = a.b[3 * g + 2];
            const int n = a.deg[g];
            const int64_t base = slot_pos(a, sp, g, 0);
            for (int j = 0; j < n; ++j) {
                const int64_t pos = base + 32 * (int64_t)j;
                float m[9];
                const int32_t c = load_block(a, pos, m);
                float o0, o1, o2;
                block_mv(m, a.x[0][c], a.x[1][c], a.x[2][c], o0, o1, o2);
                r0 = r0 - o0;
                r1 = r1 - o1;
                r2 = r2 - o2;
            }
        }
        a.r4[g] = make_float4(r0, r1, r2, 0.0f);
        a.p4[g] = make_float4(r0, r1, r2, 0.0f);
    }
    if (threadIdx.x == 0 && bi.gblk == a.sys[bi.inst].blk0) {
        BsrState& st = a.state[bi.inst];
        st.iter = 0;
        st.d3 = st.d4 = 0.0f;
        st.d = st.d1 = st.d2 = 0.0;
        st.ticket = 0;
        const bool run = sp.imax > 0;
        st.active = run ? 1 : 0;
        if (run) atomicAdd(a.unfinished, 1);
    }
}

template <int UNROLL, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_bsr_spmv(const BsrArgs a) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const BsrParams& sp = a.sys[bi.inst];
    const BsrState& st = a.state[bi.inst];
    const bool active = st.active != 0;
    Acc pd = acc_zero(), pd2 = acc_zero();
    if (active) {
        const bool first = st.iter == 0;
        const float d4 = st.d4;
        for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
            if (a.fixed[g]) continue;
            const float4 rg = a.r4[g];
            const float r0 = rg.x, r1 = rg.y, r2 = rg.z;
            const float4 pg = a.p4[g];
            float n0 = pg.x, n1 = pg.y, n2 = pg.z;
            if (!first) {
                n0 = r0 + n0 * d4;
                n1 = r1 + n1 * d4;
                n2 = r2 + n2 * d4;
            }
            float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f;
            const int n = a.deg[g];
            const int64_t base = slot_pos(a, sp, g, 0);
#pragma unroll UNROLL
            for (int j = 0; j < n; ++j) {
                const int64_t pos = base + 32 * (int64_t)j;
                float m[9];
                const int32_t c = load_block(a, pos, m);
                const float4 pc = a.p4[c];
                float v0 = pc.x, v1 = pc.y, v2 = pc.z;
                if (!first) {
                    const float4 rc = a.r4[c];
                    v0 = rc.x + v0 * d4;
                    v1 = rc.y + v1 * d4;
                    v2 = rc.z + v2 * d4;
                }
                float o0, o1, o2;
                block_mv(m, v0, v1, v2, o0, o1, o2);
                q0 = q0 + o0;
                q1 = q1 + o1;
                q2 = q2 + o2;
            }
            a.q[0][g] = q0;
            a.q[1][g] = q1;
            a.q[2][g] = q2;
            acc_add(pd, r0 * r0 + r1 * r1 + r2 * r2);
            acc_add(pd2, n0 * q0 + n1 * q1 + n2 * q2);
        }
    }
    bsr_finish<0>(a, bi.gblk, bi.inst, active, pd, pd2);
}

__global__ void __launch_bounds__(kThreads) k_bsr_update(const BsrArgs a) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const BsrState& st = a.state[bi.inst];
    const bool active = st.active != 0;
    Acc pd1 = acc_zero();
    if (active) {
        const bool first = st.iter == 0;
        const float d3 = st.d3, d4 = st.d4;
        for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
            if (a.fixed[g]) continue;
            const float4 rg = a.r4[g], pg = a.p4[g];
            const float ro[3] = {rg.x, rg.y, rg.z}, po[3] = {pg.x, pg.y, pg.z};
            float r[3], pn[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float pk = po[k];
                if (!first) pk = ro[k] + pk * d4;
                pn[k] = pk;
                a.x[k][g] = a.x[k][g] + pk * d3;  // V += p d3, FEM:895
                r[k] = ro[k] - a.q[k][g] * d3;    // r -= q d3, FEM:896
            }
            a.r4[g] = make_float4(r[0], r[1], r[2], 0.0f);
            a.p4[g] = make_float4(pn[0], pn[1], pn[2], 0.0f);
            acc_add(pd1, r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        }
    }
    bsr_finish<1>(a, bi.gblk, bi.inst, active, pd1, acc_zero());
}

// Dynamic shared memory of the resident CG: each row's new direction r + d4 p (a 16-byte
// record the neighbours gather; x passes through it during init); the system's blocks
// without padding: two float4 planes, component 8 and an 8-bit local column (a resident
// system has at most 256 rows); each warp's offset of each slot (ints, `stride` of them
// per warp: the longest row's block count).
__host__ __device__ constexpr size_t resident_vec_bytes(int threads) { return 16 * (size_t)threads; }
__host__ __device__ constexpr size_t resident_smem_bytes(int threads, int64_t nnzb, int stride) {
    return resident_vec_bytes(threads) + ((size_t)nnzb * 37 + 15) / 16 * 16 + 4 * (size_t)(threads / 32) * stride;
}
constexpr int kResSlots = 4;    // slots of a row multiplied together in the resident loop
constexpr int kResMaxDeg = 64;  // blocks of a resident system's longest row (bounds the offset table)

// The first half of block_sum_acc: each warp's pair, reduced by the same shuffle tree,
// is stored in wacc[warp] (read after a barrier).
__device__ __forceinline__ void warp_partial(Acc v, Acc* wacc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Acc u;
        u.s = __shfl_down_sync(0xffffffffu, v.s, o);
        u.c = __shfl_down_sync(0xffffffffu, v.c, o);
        v = acc_merge(v, u);
    }
    if ((threadIdx.x & 31) == 0) wacc[threadIdx.x >> 5] = v;
}

// The second half, by warp 0 (every lane calls it; the result is valid in lane 0): lane i
// turns warp i's pair into s + c in FP64, then block_sum_acc's shuffle tree over at most 8
// warp values.  The tree's first two levels add zeros (lanes 8-31), which leaves each value
// unchanged (a warp value is never -0: its pair starts at +0), so its result is
// ((w0 + w4) + (w2 + w6)) + ((w1 + w5) + (w3 + w7)), formed here by three shuffle levels:
// the same bits, with one FP64 warp instruction per conversion or level rather than one
// per warp and a serial sum in one thread.
__device__ __forceinline__ double sum_warp_pairs(const Acc* wacc, int nw) {
    const int lane = threadIdx.x & 31;
    double v = lane < nw ? (double)wacc[lane].s + (double)wacc[lane].c : 0.0;
    v += __shfl_down_sync(0xffffffffu, v, 4);
    v += __shfl_down_sync(0xffffffffu, v, 2);
    v += __shfl_down_sync(0xffffffffu, v, 1);
    return v;
}

// The whole solve of one small system in one CTA: the system's blocks are read once
// from the caller's CSR into shared memory (the pack), then init and every iteration
// run on chip with the streamed kernels' arithmetic.  Thread t owns internal row
// row0 + t, as in the system's only block of the streamed path, and the dot products
// go through the same block sums, so the results are the streamed path's bits.
//
// Shared-memory layout of the blocks (jagged diagonals): a system's rows are sorted by
// decreasing block count, so in each warp the lanes whose row has more than j blocks
// are lanes 0 .. cnt_j - 1.  Slot j of the warp's rows is stored as those cnt_j entries,
// after the warp's slots 0 .. j-1; cnt_j is a ballot over the warp.
// map[e] places the caller's block e: its internal local row (bits 0-7), its slot in the
// row (bits 8-15) and its internal local column (bits 16-23), so the pack reads the
// caller's blocks in order, coalesced.
__global__ void __launch_bounds__(kThreads) k_bsr_resident(const BsrArgs a, const int32_t* ids, int64_t nnzb_max,
                                                           const uint32_t* map, int stride) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ float s_d3, s_d4;
    __shared__ int s_wcount[kThreads / 32];
    __shared__ Acc s_w0[kThreads / 32], s_w1[kThreads / 32], s_w2[kThreads / 32];
    static_assert(kThreads / 32 <= 8, "sum_warp_pairs takes at most 8 warps");
    float4* s_n4 = reinterpret_cast<float4*>(smem);
    float4* s_b0 = s_n4 + blockDim.x;
    float4* s_b1 = s_b0 + nnzb_max;
    float* s_b8 = reinterpret_cast<float*>(s_b1 + nnzb_max);
    uint8_t* s_col = reinterpret_cast<uint8_t*>(s_b8 + nnzb_max);
    int* s_pre = reinterpret_cast<int*>(smem + resident_smem_bytes(blockDim.x, nnzb_max, 0));
    constexpr unsigned kFull = 0xffffffffu;

    const int k = ids[blockIdx.x];
    const BsrParams& sp = a.sys[k];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const bool valid = t < sp.n_rows;
    const int64_t g = sp.row0 + t;
    bool fx = true;
    int n = 0;
    float x0 = 0.0f, x1 = 0.0f, x2 = 0.0f;
    if (valid) {
        fx = a.fixed[g] != 0;
        n = a.deg[g];
    }
    const int width = __reduce_max_sync(kFull, n);
    const int wsum = __reduce_add_sync(kFull, n);
    if (lane == 0) s_wcount[w] = wsum;
    __syncthreads();
    int base = 0;
    for (int u = 0; u < w; ++u) base += s_wcount[u];
    {  // each warp's slot offsets, then k_bsr_pack into shared memory
        int pre = base;
        for (int j = 0; j < width; ++j) {
            const int cnt = __popc(__ballot_sync(kFull, n > j));
            if (lane == 0) s_pre[w * stride + j] = pre;
            pre += cnt;
        }
        __syncthreads();
        const int64_t e1 = a.row_ptr[sp.row0 + sp.n_rows];
#pragma unroll 4
        for (int64_t e = a.row_ptr[sp.row0] + t; e < e1; e += blockDim.x) {
            const uint32_t mp = __ldg(map + e);
            const int i = mp & 255, j = (mp >> 8) & 255;
            const float* m = a.cblk + 9 * (size_t)e;
            const int pos = s_pre[(i >> 5) * stride + j] + (i & 31);
            s_b0[pos] = make_float4(m[0], m[1], m[2], m[3]);
            s_b1[pos] = make_float4(m[4], m[5], m[6], m[7]);
            s_b8[pos] = m[8];
            s_col[pos] = (uint8_t)(mp >> 16);
        }
    }
    if (valid) {
        x0 = a.x[0][g];
        x1 = a.x[1][g];
        x2 = a.x[2][g];
        s_n4[t] = make_float4(x0, x1, x2, 0.0f);  // x, for init's gathers
    }
    __syncthreads();
    // k_bsr_init: r = b - A V, p = r.
    const bool act = valid && !fx;
    float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
    if (act) {
        r0 = a.b[3 * g];
        r1 = a.b[3 * g + 1];
        r2 = a.b[3 * g + 2];
    }
    {
        int pre = base;
        for (int j = 0; j < width; ++j) {
            const int cnt = __popc(__ballot_sync(kFull, n > j));
            if (act && j < n) {
                const int pos = pre + lane;
                const float4 u = s_b0[pos], v = s_b1[pos];
                const float m[9] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w, s_b8[pos]};
                const float4 xc = s_n4[s_col[pos]];
                float o0, o1, o2;
                block_mv(m, xc.x, xc.y, xc.z, o0, o1, o2);
                r0 = r0 - o0;
                r1 = r1 - o1;
                r2 = r2 - o2;
            }
            pre += cnt;
        }
    }
    float p0 = r0, p1 = r1, p2 = r2;
    double d = 0.0, d1 = 0.0, d2 = 0.0;
    float d3 = 0.0f, d4 = 0.0f;
    const double tiny = (double)sp.tiny;
    const int nw = (int)(blockDim.x >> 5);
    // Five barriers an iteration: after the directions, the products (d2), d3, the
    // update (d1) and d4; the last also orders this iteration's reads of the directions
    // before the next iteration writes them.
    for (int it = 0; it < sp.imax; ++it) {
        const bool first = it == 0;
        // The new direction of every row, fixed rows included (r = p = 0 there), by the
        // expression the streamed pass evaluates for each neighbour and for its own row.
        float n0 = p0, n1 = p1, n2 = p2;
        if (!first) {
            n0 = r0 + n0 * d4;
            n1 = r1 + n1 * d4;
            n2 = r2 + n2 * d4;
        }
        if (first) __syncthreads();  // init's reads of x are done (later: the barrier after d4)
        if (valid) s_n4[t] = make_float4(n0, n1, n2, 0.0f);
        __syncthreads();
        // k_bsr_spmv
        Acc pd = acc_zero(), pd2 = acc_zero();
        float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f;
        // Four slots at a time: their loads and products are independent, so they are
        // issued together (a slot past the row's end reads entry 0, which every system
        // with blocks has, and is not added); the sums still run in slot order.
        int pre = base;
        for (int j = 0; j < width; j += kResSlots) {
            int pos[kResSlots];
            bool ok[kResSlots];
#pragma unroll
            for (int u = 0; u < kResSlots; ++u) {
                const int cnt = __popc(__ballot_sync(kFull, n > j + u));
                ok[u] = act && j + u < n;
                pos[u] = ok[u] ? pre + lane : 0;
                pre += cnt;
            }
            float o[kResSlots][3];
#pragma unroll
            for (int u = 0; u < kResSlots; ++u) {
                const float4 b0 = s_b0[pos[u]], b1 = s_b1[pos[u]];
                const float m[9] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w, s_b8[pos[u]]};
                const float4 nc = s_n4[s_col[pos[u]]];
                block_mv(m, nc.x, nc.y, nc.z, o[u][0], o[u][1], o[u][2]);
            }
#pragma unroll
            for (int u = 0; u < kResSlots; ++u) {
                if (ok[u]) {
                    q0 = q0 + o[u][0];
                    q1 = q1 + o[u][1];
                    q2 = q2 + o[u][2];
                }
            }
        }
        if (act) {
            acc_add(pd, r0 * r0 + r1 * r1 + r2 * r2);
            acc_add(pd2, n0 * q0 + n1 * q1 + n2 * q2);
        }
        // d = r.r is the previous update's d1: the same terms in the same order.
        if (first) warp_partial(pd, s_w0);
        warp_partial(pd2, s_w1);
        __syncthreads();
        if (w == 0) {  // bsr_scalars<0>, in thread 0
            const double t0 = first ? sum_warp_pairs(s_w0, nw) : d1;
            const double t1 = sum_warp_pairs(s_w1, nw);
            if (t == 0) {
                d = t0;
                d2 = t1;
                double dd2 = d2;
                if (fabs(dd2) < tiny) dd2 = tiny;  // FEM:885-886
                s_d3 = (float)(t0 / dd2);
            }
        }
        __syncthreads();  // d3, and every row's reads of r and p are done
        d3 = s_d3;
        // k_bsr_update
        Acc pd1 = acc_zero();
        if (act) {
            x0 = x0 + n0 * d3;  // V += p d3, FEM:895
            x1 = x1 + n1 * d3;
            x2 = x2 + n2 * d3;
            r0 = r0 - q0 * d3;  // r -= q d3, FEM:896
            r1 = r1 - q1 * d3;
            r2 = r2 - q2 * d3;
            p0 = n0;
            p1 = n1;
            p2 = n2;
            acc_add(pd1, r0 * r0 + r1 * r1 + r2 * r2);
        }
        warp_partial(pd1, s_w2);
        __syncthreads();
        if (w == 0) {  // bsr_scalars<1>, in thread 0
            const double t2 = sum_warp_pairs(s_w2, nw);
            if (t == 0) {
                d1 = t2;
                double dd = d;
                if (fabs(dd) < tiny) dd = tiny;  // FEM:908-909
                s_d4 = (float)(t2 / dd);
            }
        }
        __syncthreads();
        d4 = s_d4;
    }
    if (valid) {
        if (!fx) {
            a.x[0][g] = x0;
            a.x[1][g] = x1;
            a.x[2][g] = x2;
        }
        a.r4[g] = make_float4(r0, r1, r2, 0.0f);
        a.p4[g] = make_float4(p0, p1, p2, 0.0f);
    }
    if (t == 0) {
        BsrState& st = a.state[k];
        st.d = d;
        st.d1 = d1;
        st.d2 = d2;
        st.d3 = d3;
        st.d4 = d4;
        st.iter = sp.imax;
        st.active = 0;
        st.ticket = 0;
    }
}

// Host arrays arrive in the caller's order in staging buffers.  k_bsr_check flags a
// non-finite block or b in a free row, or a non-finite x (FEM:392-393 puts FLT_MAX in
// fixed rows); nothing is committed unless the flag stays clear.
__global__ void __launch_bounds__(kThreads) k_bsr_check(const float* blk, const float* b, const float* x,
                                                       const int32_t* row_ptr, const uint8_t* fixed_caller,
                                                       int64_t rows, int* flag) {
    int bad = 0;  // bit 0: a block, bit 1: b, bit 2: x
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        if (x)
            for (int c = 0; c < 3; ++c) bad |= isfinite(x[3 * r + c]) ? 0 : 4;
        if (fixed_caller[r]) continue;
        if (b)
            for (int c = 0; c < 3; ++c) bad |= isfinite(b[3 * r + c]) ? 0 : 2;
        if (blk)
            for (int64_t i = 9 * (int64_t)row_ptr[r]; i < 9 * (int64_t)row_ptr[r + 1]; ++i)
                bad |= isfinite(blk[i]) ? 0 : 1;
    }
    if (bad) atomicOr(flag, bad);
}

// b into the internal row order, x into planes in the internal order.
__global__ void __launch_bounds__(kThreads) k_bsr_commit(const BsrArgs a, float* bint, const float* b, const float* x,
                                                        const int32_t* perm, int64_t rows) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = perm[r];
        if (b)
            for (int c = 0; c < 3; ++c) bint[3 * i + c] = b[3 * r + c];
        if (x)
            for (int c = 0; c < 3; ++c) a.x[c][i] = x[3 * r + c];
    }
}

// The solution and the residual back in the caller's order (3 floats per row).
__global__ void __launch_bounds__(kThreads) k_bsr_gather_out(const BsrArgs a, const int32_t* perm, int64_t rows,
                                                            float* x, float* res) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = perm[r];
        if (x)
            for (int c = 0; c < 3; ++c) x[3 * r + c] = a.x[c][i];
        if (res) {
            const float4 v = a.r4[i];
            res[3 * r] = v.x;
            res[3 * r + 1] = v.y;
            res[3 * r + 2] = v.z;
        }
    }
}

// Launch shapes of the matrix-vector pass (unroll of the slot loop, minimum resident
// blocks per SM, which caps the registers).  OC_BSR_VARIANT picks one; the default was
// chosen by measurement on GB300.
typedef void (*SpmvFn)(BsrArgs);
SpmvFn spmv_variant() {
    int v = 0;
    if (const char* e = std::getenv("OC_BSR_VARIANT")) v = std::atoi(e);
    switch (v) {
        case 1: return k_bsr_spmv<4, 5>;
        case 2: return k_bsr_spmv<2, 6>;
        case 3: return k_bsr_spmv<4, 6>;
        case 5: return k_bsr_spmv<2, 4>;
        case 6: return k_bsr_spmv<4, 4>;
        case 7: return k_bsr_spmv<2, 1>;
        default: return k_bsr_spmv<1, 8>;  // fastest on the 386k-row mesh and on the streamed 4096-body batch
    }
}

}  // namespace
}  // namespace oc

using namespace oc;

struct oc_bsr_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool use_graph = true;
    int32_t n_sys = 0;
    int64_t n_rows = 0, nnzb = 0, n_slots = 0;
    int32_t n_blocks = 0;
    std::vector<int64_t> row_off, nnz_off;
    bool any_iter = false;  // some system has cg_max_iter > 0
    BsrArgs args{};
    std::vector<void*> allocs;
    uint8_t* d_fixed = nullptr;
    int32_t* d_row_ptr = nullptr;
    float* d_cblk = nullptr;  // the caller's CSR blocks (packed at each solve)
    float* d_b = nullptr;
    // set_system's staging (caller order) and the tables its kernels use
    float* d_stage_blk = nullptr;
    float* d_stage_b = nullptr;
    float* d_stage_x = nullptr;
    float* d_out = nullptr;  // get_solution: x and residual in the caller's order
    uint8_t* d_fixed_caller = nullptr;
    int32_t* d_perm = nullptr;
    int* d_flag = nullptr;
    int* h_flag = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
    unsigned long long* h_loop = nullptr;
    SpmvFn spmv = nullptr;
    // Systems solved by k_bsr_resident (one CTA each) and its launch shape.
    int32_t n_res = 0;
    int32_t* d_res_ids = nullptr;
    int32_t res_threads = 0;
    int64_t res_nnzb_max = 0;  // blocks of the largest resident system
    int32_t res_stride = 0;    // blocks of the longest row of a resident system
    uint32_t* d_res_map = nullptr;
    size_t res_smem = 0;
    int64_t st_rows = 0, st_nnzb = 0, res_rows = 0, res_nnzb = 0;  // streamed / resident sizes
    std::string err;
};

namespace {

oc_status bsr_fail(oc_bsr_solver* s, oc_status code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}

oc_status bsr_fail_cuda(oc_bsr_solver* s, cudaError_t e, const char* what) {
    const oc_status code = (e == cudaErrorMemoryAllocation) ? OC_ERR_OUT_OF_MEMORY : OC_ERR_CUDA;
    return bsr_fail(s, code, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define BSR_TRY(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return bsr_fail_cuda(s, e_, #call); \
    } while (0)

template <class T>
cudaError_t bsr_alloc(oc_bsr_solver* s, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) s->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return e;
}

template <class T>
cudaError_t bsr_upload(oc_bsr_solver* s, T** p, const std::vector<T>& v) {
    cudaError_t e = bsr_alloc(s, p, v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void bsr_release(oc_bsr_solver* s) {
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    for (void* p : s->allocs) cudaFree(p);
    s->allocs.clear();
    if (s->h_loop) cudaFreeHost(s->h_loop);
    if (s->h_flag) cudaFreeHost(s->h_flag);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
}

bool bsr_valid(const oc_bsr_solver* s) { return s != nullptr && s->n_sys > 0; }

// Grid of the row-parallel host-facing kernels (grid-stride over the rows).
int row_grid(int64_t rows) { return (int)std::max<int64_t>(1, std::min<int64_t>((rows + kThreads - 1) / kThreads, 152 * 8)); }

void launch(void (*k)(BsrArgs), const BsrArgs& a, int n, cudaStream_t stream) {
    if (n > 0) k<<<n, kThreads, 0, stream>>>(a);
}

void launch_resident(const oc_bsr_solver* s, const BsrArgs& a) {
    k_bsr_resident<<<s->n_res, s->res_threads, s->res_smem, s->stream>>>(a, s->d_res_ids, s->res_nnzb_max,
                                                                        s->d_res_map, s->res_stride);
}

oc_status bsr_build_graph(oc_bsr_solver* s) {
    cudaGraph_t g = nullptr;
    BSR_TRY(cudaGraphCreate(&g, 0));
    s->graph = g;
    BsrArgs a = s->args;
    a.use_cond = 0;
    void* params[] = {&a};
    auto kp = [&](void (*k)(BsrArgs)) {
        cudaKernelNodeParams p{};
        p.func = (void*)k;
        p.gridDim = dim3((unsigned)s->n_blocks);
        p.blockDim = dim3(kThreads);
        p.sharedMemBytes = 0;
        p.kernelParams = params;
        return p;
    };
    cudaGraphNode_t n_reset, n_pack, n_init, n_loop, n_spmv, n_upd, n_res;
    if (s->n_res > 0) {  // independent of the streamed systems' nodes
        const int32_t* ids = s->d_res_ids;
        int64_t nnzb_max = s->res_nnzb_max;
        const uint32_t* map = s->d_res_map;
        int stride = s->res_stride;
        void* rparams[] = {&a, &ids, &nnzb_max, &map, &stride};
        cudaKernelNodeParams p{};
        p.func = (void*)k_bsr_resident;
        p.gridDim = dim3((unsigned)s->n_res);
        p.blockDim = dim3((unsigned)s->res_threads);
        p.sharedMemBytes = (unsigned)s->res_smem;
        p.kernelParams = rparams;
        BSR_TRY(cudaGraphAddKernelNode(&n_res, g, nullptr, 0, &p));
    }
    if (s->n_blocks == 0) {  // every system resident: no loop (a conditional handle needs its node)
        BSR_TRY(cudaGraphInstantiate(&s->exec, g, 0));
        return OC_OK;
    }
    // The loop condition starts every launch at "some system iterates" (nothing before
    // the loop sets it); the last block of each update pass sets it from then on.
    cudaGraphConditionalHandle handle = 0;
    BSR_TRY(cudaGraphConditionalHandleCreate(&handle, g, s->any_iter ? 1u : 0u, cudaGraphCondAssignDefault));
    a.use_cond = 1;
    a.cond = (unsigned long long)handle;
    cudaMemsetParams mp{};
    mp.dst = a.unfinished;
    mp.value = 0;
    mp.elementSize = sizeof(int32_t);
    mp.width = 1;
    mp.height = 1;
    mp.pitch = sizeof(int32_t);
    BSR_TRY(cudaGraphAddMemsetNode(&n_reset, g, nullptr, 0, &mp));
    cudaKernelNodeParams p = kp(k_bsr_pack);
    BSR_TRY(cudaGraphAddKernelNode(&n_pack, g, &n_reset, 1, &p));
    p = kp(k_bsr_init);
    BSR_TRY(cudaGraphAddKernelNode(&n_init, g, &n_pack, 1, &p));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    BSR_TRY(cudaGraphAddNode(&n_loop, g, &n_init, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    p = kp(s->spmv);
    BSR_TRY(cudaGraphAddKernelNode(&n_spmv, body, nullptr, 0, &p));
    p = kp(k_bsr_update);
    BSR_TRY(cudaGraphAddKernelNode(&n_upd, body, &n_spmv, 1, &p));
    BSR_TRY(cudaGraphInstantiate(&s->exec, g, 0));
    return OC_OK;
}

}  // namespace

extern "C" {

oc_status oc_bsr_create(const oc_bsr_desc* descs, int32_t n_systems, const oc_options* opts, oc_bsr_solver** out) {
    if (!descs || n_systems < 1 || !out) return OC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    oc_options o;
    oc_default_options(&o);
    if (opts) o = *opts;
    if (o.executor < OC_EXEC_AUTO || o.executor > OC_EXEC_PLAIN) return OC_ERR_INVALID_ARGUMENT;
    std::string err;
    int64_t rows = 0, nnzb = 0;
    for (int32_t k = 0; k < n_systems; ++k) {
        const oc_bsr_desc& d = descs[k];
        const std::string who = "system " + std::to_string(k) + ": ";
        if (d.n_rows < 1 || d.nnzb < 0 || !d.row_ptr || (d.nnzb > 0 && !d.col) || d.cg_max_iter < 0 ||
            d.cg_max_iter > OC_MAX_CG_ITER || !std::isfinite(d.tiny) || d.tiny < 0.0f || !std::isfinite(d.tolerance))
            return OC_ERR_INVALID_ARGUMENT;
        if (d.row_ptr[0] != 0 || d.row_ptr[d.n_rows] != d.nnzb) return OC_ERR_INVALID_ARGUMENT;
        for (int32_t r = 0; r < d.n_rows; ++r) {
            if (d.row_ptr[r + 1] < d.row_ptr[r]) return OC_ERR_INVALID_ARGUMENT;
            for (int32_t e = d.row_ptr[r]; e < d.row_ptr[r + 1]; ++e) {
                if (d.col[e] < 0 || d.col[e] >= d.n_rows) return OC_ERR_BAD_INDEX;
                if (e > d.row_ptr[r] && d.col[e] <= d.col[e - 1]) return OC_ERR_INVALID_ARGUMENT;  // std::map order
            }
        }
        rows += d.n_rows;
        nnzb += d.nnzb;
    }
    if (rows >= (int64_t)1 << 31 || nnzb >= (int64_t)1 << 31) return OC_ERR_UNSUPPORTED;

    oc_bsr_solver* s = new (std::nothrow) oc_bsr_solver();
    if (!s) return OC_ERR_OUT_OF_MEMORY;
    auto bail = [&](oc_status st) {
        bsr_release(s);
        delete s;
        return st;
    };
#define BSR_CREATE_TRY(call)                    \
    do {                                        \
        cudaError_t e_ = (call);                \
        if (e_ != cudaSuccess) {                \
            bsr_fail_cuda(s, e_, #call);        \
            return bail(e_ == cudaErrorMemoryAllocation ? OC_ERR_OUT_OF_MEMORY : OC_ERR_CUDA); \
        }                                       \
    } while (0)
    s->device = o.device;
    s->use_graph = o.use_graph != 0;
    s->spmv = spmv_variant();
    s->n_sys = n_systems;
    s->n_rows = rows;
    s->nnzb = nnzb;
    BSR_CREATE_TRY(cudaSetDevice(s->device));
    if (o.stream) {
        s->stream = (cudaStream_t)o.stream;
    } else {
        BSR_CREATE_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }

    // Global CSR (the caller's order), systems, blocks of rows and slices (internal order).
    // Within each system the rows are reordered, window by window (kSortWindow rows), by
    // decreasing number of blocks, so that the 32 rows of a slice have nearly the same
    // count and the sliced layout carries little padding (sliced ELL with sorting,
    // "SELL-C-sigma").  Each row still sums its own blocks in column order.
    std::vector<int32_t> row_ptr(1, 0), perm(rows), iperm(rows), deg_int(rows);
    std::vector<uint8_t> fixed(rows), fixed_int(rows);
    std::vector<BsrParams> sys(n_systems);
    std::vector<BlockInfo> blocks;
    std::vector<int64_t> slice_ptr;
    std::vector<int32_t> width;
    std::vector<int32_t> res_ids;
    int smem_optin = 0;
    BSR_CREATE_TRY(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
    // Room for the kernel's static shared memory (block sums and the two broadcast scalars).
    const size_t smem_cap = smem_optin > 1024 ? (size_t)smem_optin - 1024 : 0;
    auto who_of = [](int32_t k) { return "system " + std::to_string(k) + ": "; };
    s->row_off.assign(n_systems + 1, 0);
    s->nnz_off.assign(n_systems + 1, 0);
    int64_t slots = 0;
    for (int32_t k = 0; k < n_systems; ++k) {
        const oc_bsr_desc& d = descs[k];
        const int64_t r0 = s->row_off[k], e0 = s->nnz_off[k];
        s->row_off[k + 1] = r0 + d.n_rows;
        s->nnz_off[k + 1] = e0 + d.nnzb;
        BsrParams& sp = sys[k];
        sp.imax = d.cg_max_iter;
        sp.tiny = d.tiny;
        sp.row0 = r0;
        sp.n_rows = d.n_rows;
        sp.slice0 = (int64_t)slice_ptr.size();
        std::vector<int32_t> order(d.n_rows);
        for (int32_t r = 0; r < d.n_rows; ++r) {
            row_ptr.push_back((int32_t)(e0 + d.row_ptr[r + 1]));
            fixed[r0 + r] = d.fixed ? (d.fixed[r] ? 1 : 0) : 0;
            order[r] = r;
        }
        auto degree = [&](int32_t r) { return d.row_ptr[r + 1] - d.row_ptr[r]; };
        for (int32_t w0 = 0; w0 < d.n_rows; w0 += kSortWindow) {
            const int32_t w1 = std::min(d.n_rows, w0 + kSortWindow);
            std::stable_sort(order.begin() + w0, order.begin() + w1,
                             [&](int32_t x, int32_t y) { return degree(x) > degree(y); });
        }
        for (int32_t i = 0; i < d.n_rows; ++i) {
            const int32_t u = order[i];
            perm[r0 + u] = (int32_t)(r0 + i);
            iperm[r0 + i] = (int32_t)(r0 + u);
            deg_int[r0 + i] = degree(u);
            fixed_int[r0 + i] = fixed[r0 + u];
        }
        for (int32_t i = 0; i < d.n_rows; i += 32) {
            int32_t w = 0;
            for (int32_t l = i; l < std::min(d.n_rows, i + 32); ++l) w = std::max(w, deg_int[r0 + l]);
            slice_ptr.push_back(slots);
            width.push_back(w);
            slots += w;
        }
        // A system of one block of rows whose blocks fit in shared memory runs resident.
        int32_t maxdeg = 0;
        for (int32_t r = 0; r < d.n_rows; ++r) maxdeg = std::max(maxdeg, degree(r));
        const bool fits = d.n_rows <= kThreads && maxdeg <= kResMaxDeg &&
                          resident_smem_bytes(kThreads, d.nnzb, kResMaxDeg) <= smem_cap;
        if (o.executor == OC_EXEC_RESIDENT && !fits) {
            bsr_fail(s, OC_ERR_UNSUPPORTED, who_of(k) + "too large for the resident executor");
            return bail(OC_ERR_UNSUPPORTED);
        }
        if (fits && o.executor != OC_EXEC_STREAMED && o.executor != OC_EXEC_PLAIN) {
            sp.blk0 = 0;
            sp.nblk = 0;
            res_ids.push_back(k);
            s->res_nnzb_max = std::max<int64_t>(s->res_nnzb_max, d.nnzb);
            s->res_stride = std::max(s->res_stride, std::max(maxdeg, 1));
            s->res_threads = std::max(s->res_threads, (d.n_rows + 31) / 32 * 32);
            s->res_rows += d.n_rows;
            s->res_nnzb += d.nnzb;
            continue;
        }
        s->any_iter = s->any_iter || d.cg_max_iter > 0;
        s->st_rows += d.n_rows;
        s->st_nnzb += d.nnzb;
        sp.blk0 = (int32_t)blocks.size();
        sp.nblk = (d.n_rows + kRowsPerBlock - 1) / kRowsPerBlock;
        for (int32_t b = 0; b < sp.nblk; ++b) {
            BlockInfo bi;
            bi.inst = k;
            bi.gblk = (int32_t)blocks.size();
            bi.v_begin = r0 + (int64_t)b * kRowsPerBlock;
            bi.v_end = std::min<int64_t>(r0 + d.n_rows, bi.v_begin + kRowsPerBlock);
            blocks.push_back(bi);
        }
    }
    s->n_slots = slots;
    std::vector<int32_t> scol((size_t)slots * 32, -1);
    for (int32_t k = 0; k < n_systems; ++k) {
        const oc_bsr_desc& d = descs[k];
        const int64_t r0 = s->row_off[k];
        for (int32_t r = 0; r < d.n_rows; ++r) {
            const int64_t i = perm[r0 + r] - r0;
            const int64_t sl = sys[k].slice0 + i / 32;
            for (int32_t e = d.row_ptr[r]; e < d.row_ptr[r + 1]; ++e)
                scol[(size_t)((slice_ptr[sl] + (e - d.row_ptr[r])) * 32 + (i & 31))] = perm[r0 + d.col[e]];
        }
    }
    s->n_blocks = (int32_t)blocks.size();

    BsrArgs& a = s->args;
    BlockInfo* d_blocks = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_blocks, blocks));
    a.blocks = d_blocks;
    BsrParams* d_sys = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_sys, sys));
    a.sys = d_sys;
    BSR_CREATE_TRY(bsr_alloc(s, &a.state, (size_t)n_systems));
    BSR_CREATE_TRY(cudaMemset(a.state, 0, sizeof(BsrState) * n_systems));
    int64_t* d_slice_ptr = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_slice_ptr, slice_ptr));
    a.slice_ptr = d_slice_ptr;
    int32_t* d_width = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_width, width));
    a.width = d_width;
    int32_t* d_scol = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_scol, scol));
    a.sb2_col = d_scol;
    const size_t plane = std::max<size_t>((size_t)slots * 32, 1);
    BSR_CREATE_TRY(bsr_alloc(s, &a.sb0, plane));
    BSR_CREATE_TRY(bsr_alloc(s, &a.sb1, plane));
    BSR_CREATE_TRY(bsr_alloc(s, &a.sb2, plane));
    BSR_CREATE_TRY(cudaMemset(a.sb0, 0, plane * sizeof(float4)));
    BSR_CREATE_TRY(cudaMemset(a.sb1, 0, plane * sizeof(float4)));
    BSR_CREATE_TRY(cudaMemset(a.sb2, 0, plane * sizeof(float2)));
    BSR_CREATE_TRY(bsr_upload(s, &s->d_row_ptr, row_ptr));
    a.row_ptr = s->d_row_ptr;
    BSR_CREATE_TRY(bsr_upload(s, &s->d_fixed, fixed_int));
    a.fixed = s->d_fixed;
    int32_t* d_iperm = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_iperm, iperm));
    a.iperm = d_iperm;
    int32_t* d_deg = nullptr;
    BSR_CREATE_TRY(bsr_upload(s, &d_deg, deg_int));
    a.deg = d_deg;
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_cblk, 9 * std::max<size_t>((size_t)nnzb, 1)));
    BSR_CREATE_TRY(cudaMemset(s->d_cblk, 0, 9 * std::max<size_t>((size_t)nnzb, 1) * sizeof(float)));
    a.cblk = s->d_cblk;
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_b, 3 * (size_t)rows));
    BSR_CREATE_TRY(cudaMemset(s->d_b, 0, 3 * (size_t)rows * sizeof(float)));
    a.b = s->d_b;
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_stage_blk, 9 * std::max<size_t>((size_t)nnzb, 1)));
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_stage_b, 3 * (size_t)rows));
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_stage_x, 3 * (size_t)rows));
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_out, 6 * (size_t)rows));
    BSR_CREATE_TRY(bsr_upload(s, &s->d_fixed_caller, fixed));
    BSR_CREATE_TRY(bsr_upload(s, &s->d_perm, perm));
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_flag, 1));
    BSR_CREATE_TRY(cudaMallocHost(&s->h_flag, sizeof(int)));
    const size_t stride = (size_t)((rows + 63) / 64) * 64;
    float* vec = nullptr;
    BSR_CREATE_TRY(bsr_alloc(s, &vec, 6 * stride));
    BSR_CREATE_TRY(cudaMemset(vec, 0, 6 * stride * sizeof(float)));
    for (int k = 0; k < 3; ++k) {
        a.x[k] = vec + k * stride;
        a.q[k] = vec + (3 + k) * stride;
    }
    BSR_CREATE_TRY(bsr_alloc(s, &a.r4, (size_t)rows));
    BSR_CREATE_TRY(bsr_alloc(s, &a.p4, (size_t)rows));
    BSR_CREATE_TRY(cudaMemset(a.r4, 0, (size_t)rows * sizeof(float4)));
    BSR_CREATE_TRY(cudaMemset(a.p4, 0, (size_t)rows * sizeof(float4)));
    BSR_CREATE_TRY(bsr_alloc(s, &a.partials, 2 * (size_t)s->n_blocks));
    BSR_CREATE_TRY(bsr_alloc(s, &a.unfinished, 1));
    BSR_CREATE_TRY(bsr_alloc(s, &a.grid_ticket, 1));
    BSR_CREATE_TRY(bsr_alloc(s, &a.loop_count, 1));
    BSR_CREATE_TRY(cudaMemset(a.unfinished, 0, sizeof(int32_t)));
    BSR_CREATE_TRY(cudaMemset(a.grid_ticket, 0, sizeof(uint32_t)));
    BSR_CREATE_TRY(cudaMemset(a.loop_count, 0, sizeof(unsigned long long)));
    BSR_CREATE_TRY(cudaMallocHost(&s->h_loop, sizeof(unsigned long long)));
    s->n_res = (int32_t)res_ids.size();
    if (s->n_res > 0) {
        BSR_CREATE_TRY(bsr_upload(s, &s->d_res_ids, res_ids));
        s->res_smem = resident_smem_bytes(s->res_threads, s->res_nnzb_max, s->res_stride);
        // Where each caller block goes: internal local row, slot, internal local column.
        std::vector<uint32_t> map((size_t)std::max<int64_t>(nnzb, 1), 0u);
        for (int32_t k : res_ids) {
            const oc_bsr_desc& d = descs[k];
            const int64_t r0 = s->row_off[k], e0 = s->nnz_off[k];
            for (int32_t r = 0; r < d.n_rows; ++r)
                for (int32_t e = d.row_ptr[r]; e < d.row_ptr[r + 1]; ++e)
                    map[(size_t)(e0 + e)] = (uint32_t)(perm[r0 + r] - r0) | (uint32_t)(e - d.row_ptr[r]) << 8 |
                                            (uint32_t)(perm[r0 + d.col[e]] - r0) << 16;
        }
        BSR_CREATE_TRY(bsr_upload(s, &s->d_res_map, map));
        BSR_CREATE_TRY(cudaFuncSetAttribute(k_bsr_resident, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)s->res_smem));
    }
    BSR_CREATE_TRY(cudaDeviceSynchronize());
#undef BSR_CREATE_TRY
    *out = s;
    return OC_OK;
}

void oc_bsr_destroy(oc_bsr_solver* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    bsr_release(s);
    delete s;
}

const char* oc_bsr_last_error(const oc_bsr_solver* s) { return s ? s->err.c_str() : "null handle"; }

oc_status oc_bsr_get_counts(const oc_bsr_solver* s, int64_t* rows, int64_t* nnzb, int32_t* n_systems) {
    if (!bsr_valid(s)) return OC_ERR_INVALID_ARGUMENT;
    if (rows) *rows = s->n_rows;
    if (nnzb) *nnzb = s->nnzb;
    if (n_systems) *n_systems = s->n_sys;
    return OC_OK;
}

oc_status oc_bsr_set_system(oc_bsr_solver* s, const float* blocks, const float* b, const float* x) {
    if (!bsr_valid(s)) return OC_ERR_INVALID_ARGUMENT;
    if (!blocks && !b && !x) return OC_OK;
    BSR_TRY(cudaSetDevice(s->device));
    // The host arrays go to staging buffers in the caller's order, and a kernel checks
    // them: non-finite values are allowed only where the reference has them, in the rows
    // of fixed vertices (their lumped mass is FLT_MAX, FEM:392-393), which the CG skips.
    // Nothing is committed when the check fails.
    const int64_t rows = s->n_rows;
    if (blocks)
        BSR_TRY(cudaMemcpyAsync(s->d_stage_blk, blocks, sizeof(float) * 9 * s->nnzb, cudaMemcpyHostToDevice,
                                s->stream));
    if (b) BSR_TRY(cudaMemcpyAsync(s->d_stage_b, b, sizeof(float) * 3 * rows, cudaMemcpyHostToDevice, s->stream));
    if (x) BSR_TRY(cudaMemcpyAsync(s->d_stage_x, x, sizeof(float) * 3 * rows, cudaMemcpyHostToDevice, s->stream));
    BSR_TRY(cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream));
    const int grid = row_grid(rows);
    k_bsr_check<<<grid, kThreads, 0, s->stream>>>(blocks ? s->d_stage_blk : nullptr, b ? s->d_stage_b : nullptr,
                                                  x ? s->d_stage_x : nullptr, s->d_row_ptr, s->d_fixed_caller, rows,
                                                  s->d_flag);
    BSR_TRY(cudaGetLastError());
    BSR_TRY(cudaMemcpyAsync(s->h_flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    BSR_TRY(cudaStreamSynchronize(s->stream));
    const int bad = *s->h_flag;
    if (bad & 1) return bsr_fail(s, OC_ERR_NON_FINITE, "oc_bsr_set_system: non-finite block in a free row");
    if (bad & 2) return bsr_fail(s, OC_ERR_NON_FINITE, "oc_bsr_set_system: non-finite b in a free row");
    if (bad & 4) return bsr_fail(s, OC_ERR_NON_FINITE, "oc_bsr_set_system: non-finite x");
    // Commit, stream-ordered before the next solve: the blocks as given, b and x into the
    // internal row order (x as planes).
    if (blocks)
        BSR_TRY(cudaMemcpyAsync(s->d_cblk, s->d_stage_blk, sizeof(float) * 9 * s->nnzb, cudaMemcpyDeviceToDevice,
                                s->stream));
    if (b || x) {
        k_bsr_commit<<<grid, kThreads, 0, s->stream>>>(s->args, s->d_b, b ? s->d_stage_b : nullptr,
                                                       x ? s->d_stage_x : nullptr, s->d_perm, rows);
        BSR_TRY(cudaGetLastError());
    }
    return OC_OK;
}

oc_status oc_bsr_solve(oc_bsr_solver* s) {
    if (!bsr_valid(s)) return OC_ERR_INVALID_ARGUMENT;
    BSR_TRY(cudaSetDevice(s->device));
    if (s->use_graph) {
        if (!s->exec) {
            oc_status st = bsr_build_graph(s);
            if (st != OC_OK) return st;
        }
        BSR_TRY(cudaGraphLaunch(s->exec, s->stream));
        s->launches += (s->n_blocks > 0 ? 2 : 0) + (s->n_res > 0 ? 1 : 0);
        return OC_OK;
    }
    BsrArgs a = s->args;
    a.use_cond = 0;
    if (s->n_res > 0) {
        launch_resident(s, a);
        BSR_TRY(cudaGetLastError());
        s->launches += 1;
    }
    if (s->n_blocks == 0) return OC_OK;
    BSR_TRY(cudaMemsetAsync(a.unfinished, 0, sizeof(int32_t), s->stream));
    launch(k_bsr_pack, a, s->n_blocks, s->stream);
    launch(k_bsr_init, a, s->n_blocks, s->stream);
    BSR_TRY(cudaGetLastError());
    s->launches += 2;
    int32_t* h = nullptr;
    BSR_TRY(cudaMallocHost(&h, sizeof(int32_t)));
    for (;;) {
        cudaError_t e = cudaMemcpyAsync(h, a.unfinished, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            cudaFreeHost(h);
            return bsr_fail_cuda(s, e, "oc_bsr_solve");
        }
        if (*h <= 0) break;
        launch(s->spmv, a, s->n_blocks, s->stream);
        launch(k_bsr_update, a, s->n_blocks, s->stream);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            cudaFreeHost(h);
            return bsr_fail_cuda(s, e, "oc_bsr_solve");
        }
    }
    cudaFreeHost(h);
    return OC_OK;
}

oc_status oc_bsr_profile(oc_bsr_solver* s, int32_t n_solves, int32_t max_kernels, char* names, double* ms_total,
                         int64_t* launches, double* algorithmic_bytes, int32_t* n_kernels) {
    if (!bsr_valid(s) || n_solves < 0 || max_kernels < 0) return OC_ERR_INVALID_ARGUMENT;
    BSR_TRY(cudaSetDevice(s->device));
    // Algorithmic bytes of one launch, each array element once in the device layout (r and
    // p are 16-byte records), over the systems the kernel runs: pack 72 B per block (read
    // and write 36) + 8 B per row; init 40 B per block (block + column) + 61 B per row (b,
    // V, r and p out, fixed, row_ptr); spmv 40 B per block + 53 B per row (fixed, row_ptr,
    // r, p in, q out); update 109 B per row (fixed, r, p, x, q in; x, r, p out); resident
    // 40 B per block (block + column, read once) + 85 B per row (row tables, fixed, b, V in
    // and out, r and p out): its iterations stay on chip.
    const double nb = (double)s->st_nnzb, nr = (double)s->st_rows;
    const double rb = (double)s->res_nnzb, rr = (double)s->res_rows;
    constexpr int K = 5;
    const char* kname[K] = {"k_bsr_pack", "k_bsr_init", "k_bsr_spmv", "k_bsr_update", "k_bsr_resident"};
    const double kbytes[K] = {72.0 * nb + 8.0 * nr, 40.0 * nb + 61.0 * nr, 40.0 * nb + 53.0 * nr, 109.0 * nr,
                              40.0 * rb + 85.0 * rr};
    double ms[K] = {0, 0, 0, 0, 0};
    int64_t cnt[K] = {0, 0, 0, 0, 0};
    cudaEvent_t e0, e1;
    BSR_TRY(cudaEventCreate(&e0));
    BSR_TRY(cudaEventCreate(&e1));
    BsrArgs a = s->args;
    a.use_cond = 0;
    void (*kfn[4])(BsrArgs) = {k_bsr_pack, k_bsr_init, s->spmv, k_bsr_update};
    int32_t* h = nullptr;
    cudaError_t e = cudaMallocHost(&h, sizeof(int32_t));
    auto timed = [&](int k) -> cudaError_t {
        cudaError_t x = cudaEventRecord(e0, s->stream);
        if (k < 4)
            launch(kfn[k], a, s->n_blocks, s->stream);
        else
            launch_resident(s, a);
        if (x == cudaSuccess) x = cudaGetLastError();
        if (x == cudaSuccess) x = cudaEventRecord(e1, s->stream);
        if (x == cudaSuccess) x = cudaEventSynchronize(e1);
        float t = 0.0f;
        if (x == cudaSuccess) x = cudaEventElapsedTime(&t, e0, e1);
        ms[k] += t;
        cnt[k] += 1;
        return x;
    };
    for (int32_t i = 0; i < n_solves && e == cudaSuccess; ++i) {
        if (s->n_res > 0) e = timed(4);
        if (s->n_blocks == 0) continue;
        if (e == cudaSuccess) e = cudaMemsetAsync(a.unfinished, 0, sizeof(int32_t), s->stream);
        if (e == cudaSuccess) e = timed(0);
        if (e == cudaSuccess) e = timed(1);
        for (;;) {
            if (e == cudaSuccess) e = cudaMemcpyAsync(h, a.unfinished, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess || *h <= 0) break;
            e = timed(2);
            if (e == cudaSuccess) e = timed(3);
        }
    }
    if (h) cudaFreeHost(h);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return bsr_fail_cuda(s, e, "oc_bsr_profile");
    int32_t n = 0;
    for (int k = 0; k < K && n < max_kernels; ++k, ++n) {
        if (names) {
            std::memset(names + 32 * n, 0, 32);
            std::strncpy(names + 32 * n, kname[k], 31);
        }
        if (ms_total) ms_total[n] = ms[k];
        if (launches) launches[n] = cnt[k];
        if (algorithmic_bytes) algorithmic_bytes[n] = kbytes[k] * (double)cnt[k];
    }
    if (n_kernels) *n_kernels = n;
    return OC_OK;
}

oc_status oc_bsr_get_solution(oc_bsr_solver* s, float* x, float* residual) {
    if (!bsr_valid(s)) return OC_ERR_INVALID_ARGUMENT;
    if (!x && !residual) return OC_OK;
    BSR_TRY(cudaSetDevice(s->device));
    const int64_t rows = s->n_rows;
    float* dx = s->d_out;
    float* dr = s->d_out + 3 * rows;
    k_bsr_gather_out<<<row_grid(rows), kThreads, 0, s->stream>>>(s->args, s->d_perm, rows, x ? dx : nullptr,
                                                                 residual ? dr : nullptr);
    BSR_TRY(cudaGetLastError());
    if (x) BSR_TRY(cudaMemcpyAsync(x, dx, sizeof(float) * 3 * rows, cudaMemcpyDeviceToHost, s->stream));
    if (residual)
        BSR_TRY(cudaMemcpyAsync(residual, dr, sizeof(float) * 3 * rows, cudaMemcpyDeviceToHost, s->stream));
    BSR_TRY(cudaStreamSynchronize(s->stream));
    return OC_OK;
}

oc_status oc_bsr_get_launch_count(oc_bsr_solver* s, int64_t* kernels_launched) {
    if (!bsr_valid(s) || !kernels_launched) return OC_ERR_INVALID_ARGUMENT;
    BSR_TRY(cudaSetDevice(s->device));
    BSR_TRY(cudaMemcpyAsync(s->h_loop, s->args.loop_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            s->stream));
    BSR_TRY(cudaStreamSynchronize(s->stream));
    *kernels_launched = s->launches + 2 * (int64_t)*s->h_loop;
    return OC_OK;
}

oc_status oc_bsr_synchronize(oc_bsr_solver* s) {
    if (!bsr_valid(s)) return OC_ERR_INVALID_ARGUMENT;
    BSR_TRY(cudaStreamSynchronize(s->stream));
    return OC_OK;
}

}  // extern "C"
