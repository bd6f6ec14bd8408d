// Batched block-sparse conjugate gradient with the FEM demo's semantics:
// ConjugateGradientSolver of OpenCloth_CoRotated_Linear_FEM/.../main.cpp (FEM:837-922),
// on the same engine shape as the cloth step (fixed-order per-system reductions, a
// CUDA-graph WHILE loop, batches of independent systems).
//
// The reference keeps each block row as a std::map<int, mat3> and walks it in ascending
// column order.  Here the rows of a system are cut into slices of 32 consecutive rows
// (one warp) stored slot-major (sliced ELL): slot j of lane l of slice s holds the j-th
// block of that row, each of the 9 components in its own plane, so every load of a
// warp is one coalesced 128-byte line; the columns are a static table built at create
// time, and each solve first packs the caller's CSR blocks into the planes.  Each lane
// sums its own row's products in slot order (the reference's order).
//
//   k_bsr_pack    CSR blocks -> sliced planes
//   k_bsr_init    r = b - A V, p = r               (FEM:841-859)
//   k_bsr_spmv    p = r + d4 p (not in the first pass, FEM:913-917, rebuilt for the
//                 neighbours from their r and p); q = A p; d = r.r, d2 = p.q  (FEM:865-883)
//   k_bsr_update  d3 = d / d2; V += d3 p; r -= d3 q; d1 = r.r  (FEM:885-901), d4 = d1 / d
//
// FP32 vector arithmetic in the reference's order (--fmad=false); the dot products sum
// FP32 per-row terms in error-free float pairs within a warp and FP64 above, and
// d3 = d / d2, d4 = d1 / d are FP64 quotients rounded to FP32, after the reference's
// `tiny` clamps (FEM:885-886, 908-909).  Exactly i_max iterations run: the reference's
// exit test (FEM:905) cannot fire inside its loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerBlock = 2048;  // 8 rows per thread

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
    int32_t blk0, nblk;  // the system's blocks in the block table
    int64_t row0;         // first (global) row
    int64_t slice0;       // first slice
};

struct BsrArgs {
    const BlockInfo* blocks;
    const BsrParams* sys;
    BsrState* state;
    const int64_t* slice_ptr;  // slot offset of each slice (units of 32 entries)
    const int32_t* width;      // slots of each slice
    const int32_t* scol;       // sliced column (global row), -1 for padding
    float* sblk[9];            // sliced block components
    const int32_t* row_ptr;    // caller's CSR (global, over all systems)
    const float* cblk;         // caller's CSR blocks (9 per block)
    const uint8_t* fixed;
    const float* b;            // 3 per row
    float* x[3];               // V (unknown) planes
    float* r[3];
    float* p[3];
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

__global__ void __launch_bounds__(kThreads) k_bsr_pack(const BsrArgs a) {
    const BlockInfo bi = a.blocks[blockIdx.x];
    const BsrParams& sp = a.sys[bi.inst];
    for (int64_t g = bi.v_begin + threadIdx.x; g < bi.v_end; g += blockDim.x) {
        const int32_t e0 = a.row_ptr[g], e1 = a.row_ptr[g + 1];
        for (int32_t e = e0; e < e1; ++e) {
            const int64_t pos = slot_pos(a, sp, g, e - e0);
#pragma unroll
            for (int c = 0; c < 9; ++c) a.sblk[c][pos] = a.cblk[9 * (size_t)e + c];
        }
    }
}

// Two-value last-block epilogue (per system), and the grid-wide WHILE condition.
template <int KIND>
__device__ void bsr_finish(const BsrArgs& a, int blk, int inst, bool participates, Acc p0, Acc p1) {
    __shared__ int s_last;
    if (participates) {
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
            const double tot1 = block_sum(t1);
            if (threadIdx.x == 0) {
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
            const int n = a.row_ptr[g + 1] - a.row_ptr[g];
            for (int j = 0; j < n; ++j) {
                const int64_t pos = slot_pos(a, sp, g, j);
                const int32_t c = a.scol[pos];
                float m[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) m[k] = a.sblk[k][pos];
                float o0, o1, o2;
                block_mv(m, a.x[0][c], a.x[1][c], a.x[2][c], o0, o1, o2);
                r0 = r0 - o0;
                r1 = r1 - o1;
                r2 = r2 - o2;
            }
        }
        a.r[0][g] = r0;
        a.r[1][g] = r1;
        a.r[2][g] = r2;
        a.p[0][g] = r0;
        a.p[1][g] = r1;
        a.p[2][g] = r2;
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

__global__ void __launch_bounds__(kThreads) k_bsr_spmv(const BsrArgs a) {
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
            const float r0 = a.r[0][g], r1 = a.r[1][g], r2 = a.r[2][g];
            float n0 = a.p[0][g], n1 = a.p[1][g], n2 = a.p[2][g];
            if (!first) {
                n0 = r0 + n0 * d4;
                n1 = r1 + n1 * d4;
                n2 = r2 + n2 * d4;
            }
            float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f;
            const int n = a.row_ptr[g + 1] - a.row_ptr[g];
            for (int j = 0; j < n; ++j) {
                const int64_t pos = slot_pos(a, sp, g, j);
                const int32_t c = a.scol[pos];
                float m[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) m[k] = a.sblk[k][pos];
                float v0 = a.p[0][c], v1 = a.p[1][c], v2 = a.p[2][c];
                if (!first) {
                    v0 = a.r[0][c] + v0 * d4;
                    v1 = a.r[1][c] + v1 * d4;
                    v2 = a.r[2][c] + v2 * d4;
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
            float r[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float rk = a.r[k][g];
                float pk = a.p[k][g];
                if (!first) pk = rk + pk * d4;
                a.x[k][g] = a.x[k][g] + pk * d3;  // V += p d3, FEM:895
                r[k] = rk - a.q[k][g] * d3;       // r -= q d3, FEM:896
                a.r[k][g] = r[k];
                a.p[k][g] = pk;
            }
            acc_add(pd1, r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        }
    }
    bsr_finish<1>(a, bi.gblk, bi.inst, active, pd1, acc_zero());
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
    std::vector<uint8_t> fixed_host;
    bool any_iter = false;  // some system has cg_max_iter > 0
    std::vector<int32_t> row_ptr_host;  // global CSR row pointer
    BsrArgs args{};
    std::vector<void*> allocs;
    uint8_t* d_fixed = nullptr;
    int32_t* d_row_ptr = nullptr;
    float* d_cblk = nullptr;  // staging of the caller's CSR blocks
    float* d_b = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
    unsigned long long* h_loop = nullptr;
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
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
}

bool bsr_valid(const oc_bsr_solver* s) { return s != nullptr && s->n_sys > 0; }

void launch(void (*k)(BsrArgs), const BsrArgs& a, int n, cudaStream_t stream) {
    if (n > 0) k<<<n, kThreads, 0, stream>>>(a);
}

oc_status bsr_build_graph(oc_bsr_solver* s) {
    cudaGraph_t g = nullptr;
    BSR_TRY(cudaGraphCreate(&g, 0));
    s->graph = g;
    // The loop condition starts every launch at "some system iterates" (nothing before
    // the loop sets it); the last block of each update pass sets it from then on.
    cudaGraphConditionalHandle handle = 0;
    BSR_TRY(cudaGraphConditionalHandleCreate(&handle, g, s->any_iter ? 1u : 0u, cudaGraphCondAssignDefault));
    BsrArgs a = s->args;
    a.use_cond = 1;
    a.cond = (unsigned long long)handle;
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
    cudaGraphNode_t n_reset, n_pack, n_init, n_loop, n_spmv, n_upd;
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
    p = kp(k_bsr_spmv);
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

    // Global CSR, fixed flags, systems, blocks of rows, slices.
    std::vector<int32_t> row_ptr(1, 0);
    std::vector<uint8_t> fixed;
    std::vector<BsrParams> sys(n_systems);
    std::vector<BlockInfo> blocks;
    std::vector<int64_t> slice_ptr;
    std::vector<int32_t> width, scol_dummy;
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
        s->any_iter = s->any_iter || d.cg_max_iter > 0;
        sp.tiny = d.tiny;
        sp.row0 = r0;
        sp.slice0 = (int64_t)slice_ptr.size();
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
        for (int32_t r = 0; r < d.n_rows; ++r) {
            row_ptr.push_back((int32_t)(e0 + d.row_ptr[r + 1]));
            fixed.push_back(d.fixed ? (d.fixed[r] ? 1 : 0) : 0);
        }
        for (int32_t r = 0; r < d.n_rows; r += 32) {
            int32_t w = 0;
            for (int32_t l = r; l < std::min(d.n_rows, r + 32); ++l) w = std::max(w, d.row_ptr[l + 1] - d.row_ptr[l]);
            slice_ptr.push_back(slots);
            width.push_back(w);
            slots += w;
        }
    }
    s->n_slots = slots;
    std::vector<int32_t> scol((size_t)slots * 32, -1);
    for (int32_t k = 0; k < n_systems; ++k) {
        const oc_bsr_desc& d = descs[k];
        for (int32_t r = 0; r < d.n_rows; ++r) {
            const int64_t sl = sys[k].slice0 + r / 32;
            for (int32_t e = d.row_ptr[r]; e < d.row_ptr[r + 1]; ++e)
                scol[(size_t)((slice_ptr[sl] + (e - d.row_ptr[r])) * 32 + (r & 31))] = (int32_t)(s->row_off[k] + d.col[e]);
        }
    }
    s->fixed_host = fixed;
    s->row_ptr_host = row_ptr;
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
    a.scol = d_scol;
    float* sblk = nullptr;
    const size_t plane = std::max<size_t>((size_t)slots * 32, 1);
    BSR_CREATE_TRY(bsr_alloc(s, &sblk, 9 * plane));
    BSR_CREATE_TRY(cudaMemset(sblk, 0, 9 * plane * sizeof(float)));
    for (int c = 0; c < 9; ++c) a.sblk[c] = sblk + c * plane;
    BSR_CREATE_TRY(bsr_upload(s, &s->d_row_ptr, row_ptr));
    a.row_ptr = s->d_row_ptr;
    BSR_CREATE_TRY(bsr_upload(s, &s->d_fixed, fixed));
    a.fixed = s->d_fixed;
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_cblk, 9 * std::max<size_t>((size_t)nnzb, 1)));
    BSR_CREATE_TRY(cudaMemset(s->d_cblk, 0, 9 * std::max<size_t>((size_t)nnzb, 1) * sizeof(float)));
    a.cblk = s->d_cblk;
    BSR_CREATE_TRY(bsr_alloc(s, &s->d_b, 3 * (size_t)rows));
    BSR_CREATE_TRY(cudaMemset(s->d_b, 0, 3 * (size_t)rows * sizeof(float)));
    a.b = s->d_b;
    const size_t stride = (size_t)((rows + 63) / 64) * 64;
    float* vec = nullptr;
    BSR_CREATE_TRY(bsr_alloc(s, &vec, 12 * stride));
    BSR_CREATE_TRY(cudaMemset(vec, 0, 12 * stride * sizeof(float)));
    for (int k = 0; k < 3; ++k) {
        a.x[k] = vec + k * stride;
        a.r[k] = vec + (3 + k) * stride;
        a.p[k] = vec + (6 + k) * stride;
        a.q[k] = vec + (9 + k) * stride;
    }
    BSR_CREATE_TRY(bsr_alloc(s, &a.partials, 2 * (size_t)s->n_blocks));
    BSR_CREATE_TRY(bsr_alloc(s, &a.unfinished, 1));
    BSR_CREATE_TRY(bsr_alloc(s, &a.grid_ticket, 1));
    BSR_CREATE_TRY(bsr_alloc(s, &a.loop_count, 1));
    BSR_CREATE_TRY(cudaMemset(a.unfinished, 0, sizeof(int32_t)));
    BSR_CREATE_TRY(cudaMemset(a.grid_ticket, 0, sizeof(uint32_t)));
    BSR_CREATE_TRY(cudaMemset(a.loop_count, 0, sizeof(unsigned long long)));
    BSR_CREATE_TRY(cudaMallocHost(&s->h_loop, sizeof(unsigned long long)));
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
    // Non-finite values are allowed only where the reference has them: in the rows of
    // fixed vertices (their lumped mass is FLT_MAX, FEM:392-393), which the CG skips.
    for (int64_t r = 0; r < s->n_rows; ++r) {
        if (s->fixed_host[r]) continue;
        if (blocks)
            for (int64_t e = s->row_ptr_host[r]; e < s->row_ptr_host[r + 1]; ++e)
                for (int c = 0; c < 9; ++c)
                    if (!std::isfinite(blocks[9 * e + c]))
                        return bsr_fail(s, OC_ERR_NON_FINITE, "oc_bsr_set_system: non-finite block in a free row");
        if (b)
            for (int c = 0; c < 3; ++c)
                if (!std::isfinite(b[3 * r + c]))
                    return bsr_fail(s, OC_ERR_NON_FINITE, "oc_bsr_set_system: non-finite b in a free row");
    }
    if (x)
        for (int64_t e = 0; e < 3 * s->n_rows; ++e)
            if (!std::isfinite(x[e])) return bsr_fail(s, OC_ERR_NON_FINITE, "oc_bsr_set_system: non-finite x");
    BSR_TRY(cudaSetDevice(s->device));
    if (blocks)
        BSR_TRY(cudaMemcpyAsync(s->d_cblk, blocks, sizeof(float) * 9 * s->nnzb, cudaMemcpyHostToDevice, s->stream));
    if (b) BSR_TRY(cudaMemcpyAsync(s->d_b, b, sizeof(float) * 3 * s->n_rows, cudaMemcpyHostToDevice, s->stream));
    if (x) {
        // interleaved triples -> planes, through the r planes as staging
        std::vector<float> planes(3 * (size_t)s->n_rows);
        for (int64_t r = 0; r < s->n_rows; ++r)
            for (int c = 0; c < 3; ++c) planes[(size_t)c * s->n_rows + r] = x[3 * r + c];
        for (int c = 0; c < 3; ++c)
            BSR_TRY(cudaMemcpyAsync(s->args.x[c], planes.data() + (size_t)c * s->n_rows, sizeof(float) * s->n_rows,
                                    cudaMemcpyHostToDevice, s->stream));
        BSR_TRY(cudaStreamSynchronize(s->stream));  // `planes` goes out of scope
    }
    BSR_TRY(cudaStreamSynchronize(s->stream));
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
        s->launches += 2;
        return OC_OK;
    }
    BsrArgs a = s->args;
    a.use_cond = 0;
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
        launch(k_bsr_spmv, a, s->n_blocks, s->stream);
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

oc_status oc_bsr_get_solution(oc_bsr_solver* s, float* x, float* residual) {
    if (!bsr_valid(s)) return OC_ERR_INVALID_ARGUMENT;
    BSR_TRY(cudaSetDevice(s->device));
    std::vector<float> planes(3 * (size_t)s->n_rows);
    for (int which = 0; which < 2; ++which) {
        float* out = which == 0 ? x : residual;
        if (!out) continue;
        float* const* src = which == 0 ? s->args.x : s->args.r;
        for (int c = 0; c < 3; ++c)
            BSR_TRY(cudaMemcpyAsync(planes.data() + (size_t)c * s->n_rows, src[c], sizeof(float) * s->n_rows,
                                    cudaMemcpyDeviceToHost, s->stream));
        BSR_TRY(cudaStreamSynchronize(s->stream));
        for (int64_t r = 0; r < s->n_rows; ++r)
            for (int c = 0; c < 3; ++c) out[3 * r + c] = planes[(size_t)c * s->n_rows + r];
    }
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
