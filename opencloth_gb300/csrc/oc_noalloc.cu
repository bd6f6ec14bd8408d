// oc_pcg_solve_noalloc: the step's preconditioned CG on a caller-assembled system,
// with no device allocation.
//
// Some callers cannot call cudaMalloc/cudaFree around a solve.  Examples: an engine
// that hands this library a fixed device-memory budget it manages itself, or a
// real-time frame loop where an allocation (which may synchronise the device or
// fragment a shared pool) is not acceptable.  This entry point takes device
// inputs/outputs from the caller.  Its scratch is a file-scope static __device__
// array of fixed size, so no call allocates.
//
// Scratch: one array per GPU that loads the library, held until process exit, sized
// for OC_NOALLOC_MAX_VERTICES vertices (about 3.8 MB).  All calls on a device share it
// and it keeps the last call's contents; each call clears the parts that must start at
// zero (tickets, counters, CG scalars).  Calls whose GPU work overlaps (two host
// threads, or two streams) race on it and must be serialised by the caller.
//
// The first call on a device looks the array up (cudaGetSymbolAddress with that
// device current) and caches the address; make that first call before any stream
// capture.  Two host threads making their first calls on one device at the same time
// both look it up and store the same address; the cache entries are atomics.
//
// The call is synchronous: it waits on the stream between CG iterations (the host reads
// whether the system is still iterating) and before it returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>

#include "oc_device.cuh"
#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaVertsPerBlock = kNaThreads * 8;  // the step's streamed block shape
constexpr int kNaMaxBlocks = (OC_NOALLOC_MAX_VERTICES + kNaVertsPerBlock - 1) / kNaVertsPerBlock;

struct NoAllocScratch {
    float planes[15][OC_NOALLOC_MAX_VERTICES];  // A (6), x (3), r (3), d (3)
    double partials[kNaMaxBlocks];
    InstParams inst;
    InstState state;
    BlockInfo blocks[kNaMaxBlocks];
    int32_t unconverged;
    uint32_t grid_ticket;
    unsigned long long loop_count;
};

// The scratch.  Host code must not take this name as an address (it is a host-side
// stand-in); it uses the address cudaGetSymbolAddress returns per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kMaxDevices = 64;
std::atomic<NoAllocScratch*> g_scratch_ptr[kMaxDevices] = {};

// CG set-up of IMP:310-318 on a given system: A (glm column-major, 9 floats per
// vertex, symmetric part used), b and the warm start x (float triples), pinned rows
// filtered out.  Per vertex this is the arithmetic of the set-up inside the step's
// assembly, and delta0's terms are summed as the step sums them (error-free float pairs
// per thread and warp, FP64 above).  The blocks here hold 2048 vertices each, which need
// not be the step's partition of the same vertices, so delta0 can differ from the step's
// by the FP64 rounding of a different grouping (about 2^-48 relative).  A pinned row
// gets a zero direction without a reciprocal of its diagonal, so its A may be anything
// finite, zero included.
__global__ void __launch_bounds__(kNaThreads) k_noalloc_setup(const StepArgs a, const float* A9, const float* b,
                                                               const float* x3, const uint8_t* pinned, int32_t n) {
    const int blk = blockIdx.x;
    const int64_t v0 = (int64_t)blk * kNaVertsPerBlock;
    const int64_t v1 = min((int64_t)n, v0 + kNaVertsPerBlock);
    Acc part = acc_zero();
    for (int64_t g = v0 + threadIdx.x; g < v1; g += blockDim.x) {
        const float* m = A9 + 9 * g;
        const float A[6] = {m[0], m[1], m[2], m[4], m[5], m[8]};
        const bool pin = pinned != nullptr && pinned[g] != 0;
        float x0 = x3[3 * g], x1 = x3[3 * g + 1], x2 = x3[3 * g + 2];
        if (pin) x0 = x1 = x2 = 0.0f;
        const float ax = A[0] * x0 + A[1] * x1 + A[2] * x2;
        const float ay = A[1] * x0 + A[3] * x1 + A[4] * x2;
        const float az = A[2] * x0 + A[4] * x1 + A[5] * x2;
        float r0 = b[3 * g] - ax, r1 = b[3 * g + 1] - ay, r2 = b[3 * g + 2] - az;
        if (pin) r0 = r1 = r2 = 0.0f;
        const float pr0 = A[0] * r0, pr1 = A[3] * r1, pr2 = A[5] * r2;
        float d0 = 0.0f, d1 = 0.0f, d2 = 0.0f;
        if (!pin) {
            const float pi0 = 1.0f / A[0], pi1 = 1.0f / A[3], pi2 = 1.0f / A[5];
            d0 = pi0 * r0;
            d1 = pi1 * r1;
            d2 = pi2 * r2;
        }
        acc_add(part, pin ? 0.0f : r0 * pr0 + r1 * pr1 + r2 * pr2);
#pragma unroll
        for (int k = 0; k < 6; ++k) a.A[k][g] = A[k];
        a.x[0][g] = x0;
        a.x[1][g] = x1;
        a.x[2][g] = x2;
        a.r[0][g] = r0;
        a.r[1][g] = r1;
        a.r[2][g] = r2;
        a.d[0][g] = d0;
        a.d[1][g] = d1;
        a.d[2][g] = d2;
    }
    // One instance: the last block sums the partials in order and primes the loop.
    __shared__ int s_last;
    const double bsum = block_sum_acc(part);
    if (threadIdx.x == 0) {
        a.partials[blk] = bsum;
        __threadfence();
        s_last = atomicAdd(&a.state->ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        double acc = 0.0;
        for (int j = threadIdx.x; j < (int)gridDim.x; j += blockDim.x) acc += __ldcg(a.partials + j);
        const double total = block_sum(acc);
        if (threadIdx.x == 0) {
            InstState& st = *a.state;
            st.ticket = 0;
            st.delta0 = total;
            st.delta_new = total;
            st.dq = 0.0;
            st.alpha = 0.0f;
            st.beta = 0.0f;
            st.iter = 0;
            st.flags = 0u;
            bool run = (0 < a.inst->imax) && (total > (double)a.inst->eps2 * total);
            if (!isfinite(total)) {
                st.flags |= OC_FLAG_NON_FINITE;
                run = false;
            }
            st.active = run ? 1 : 0;
            *a.unconverged = run ? 1 : 0;
            __threadfence();
        }
    }
}

__global__ void k_noalloc_out(const StepArgs a, float* x3, int32_t n) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
        x3[3 * g] = a.x[0][g];
        x3[3 * g + 1] = a.x[1][g];
        x3[3 * g + 2] = a.x[2][g];
    }
}

}  // namespace
}  // namespace oc

using namespace oc;

extern "C" oc_status oc_pcg_solve_noalloc(const float* A9, const float* b, float* x, const uint8_t* pinned,
                                          int32_t n_vertices, int32_t cg_max_iter, float cg_tol, int32_t* cg_iters,
                                          uint32_t* flags, void* stream) {
    if (!A9 || !b || !x || n_vertices < 1 || cg_max_iter < 0 || cg_max_iter > OC_MAX_CG_ITER ||
        !std::isfinite(cg_tol) || cg_tol < 0.0f)
        return OC_ERR_INVALID_ARGUMENT;
    if (n_vertices > OC_NOALLOC_MAX_VERTICES) return OC_ERR_UNSUPPORTED;  // beyond the static scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return OC_ERR_CUDA;
    NoAllocScratch* sc = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!sc) {
        // Set-up, once per device, with that device current.
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return OC_ERR_CUDA;
        sc = static_cast<NoAllocScratch*>(p);
        g_scratch_ptr[dev].store(sc, std::memory_order_release);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nblk = (n_vertices + kNaVertsPerBlock - 1) / kNaVertsPerBlock;

    StepArgs a{};
    for (int k = 0; k < 6; ++k) a.A[k] = sc->planes[k];
    for (int k = 0; k < 3; ++k) {
        a.x[k] = sc->planes[6 + k];
        a.r[k] = sc->planes[9 + k];
        a.d[k] = sc->planes[12 + k];
    }
    a.partials = sc->partials;
    a.inst = &sc->inst;
    a.state = &sc->state;
    a.blocks = sc->blocks;
    a.unconverged = &sc->unconverged;
    a.grid_ticket = &sc->grid_ticket;
    a.loop_count = &sc->loop_count;

    // Per-call constants from the host stack (copied before the call returns).
    InstParams ip{};
    const float eps = cg_tol;
    ip.eps2 = eps * eps;
    ip.imax = cg_max_iter;
    ip.blk0 = 0;
    ip.nblk = nblk;
    ip.v_off = 0;
    ip.nv = n_vertices;
    BlockInfo blocks[kNaMaxBlocks];
    for (int k = 0; k < nblk; ++k) {
        blocks[k].inst = 0;
        blocks[k].gblk = k;
        blocks[k].v_begin = (int64_t)k * kNaVertsPerBlock;
        blocks[k].v_end = std::min<int64_t>(n_vertices, (int64_t)(k + 1) * kNaVertsPerBlock);
    }
    // What must start at zero: CG scalars and ticket, loop counter, grid ticket.
    if (cudaMemsetAsync(&sc->state, 0, sizeof(InstState), st) != cudaSuccess ||
        cudaMemsetAsync(&sc->unconverged, 0, sizeof(sc->unconverged), st) != cudaSuccess ||
        cudaMemsetAsync(&sc->grid_ticket, 0, sizeof(sc->grid_ticket), st) != cudaSuccess ||
        cudaMemsetAsync(&sc->loop_count, 0, sizeof(sc->loop_count), st) != cudaSuccess ||
        cudaMemcpyAsync(&sc->inst, &ip, sizeof(ip), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(sc->blocks, blocks, sizeof(BlockInfo) * nblk, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return OC_ERR_CUDA;
    k_noalloc_setup<<<nblk, kNaThreads, 0, st>>>(a, A9, b, x, pinned, n_vertices);
    if (cudaGetLastError() != cudaSuccess) return OC_ERR_CUDA;
    for (int32_t it = 0; it <= cg_max_iter; ++it) {
        int32_t running = 0;
        if (cudaMemcpyAsync(&running, &sc->unconverged, sizeof(running), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return OC_ERR_CUDA;
        if (running <= 0) break;
        if (launch_kernel(K_CG_DIR, a, nblk, st) != cudaSuccess || launch_kernel(K_CG_UPDATE, a, nblk, st) != cudaSuccess)
            return OC_ERR_CUDA;
    }
    k_noalloc_out<<<std::min(nblk * 8, 1024), kNaThreads, 0, st>>>(a, x, n_vertices);
    InstState out{};
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&out, &sc->state, sizeof(out), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return OC_ERR_CUDA;
    if (cg_iters) *cg_iters = out.iter;
    if (flags) *flags = out.flags;
    return OC_OK;
}
