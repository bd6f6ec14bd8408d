// C ABI (include/opencloth_gb.h): handle lifetime, state transfer, and the three ways
// of running a step — a CUDA graph (the assemblies; the CG of up to 16 streamed cloths
// as one cooperative launch, of more as a device-driven WHILE node; the resident
// buckets beside them), the same kernels launched directly with the loop driven from
// the host, and the plain one-cloth-per-launch sequence.  Also the adjoint tape, the
// stencil refit after new spring parameters, and the interaction entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "oc_internal.h"

using namespace oc;

struct oc_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int32_t executor = OC_EXEC_STREAMED;
    bool use_graph = true;
    int32_t n_inst = 0;
    int64_t nv = 0, ns = 0;
    int64_t n_inc = 0;  // incidence records (2 per spring)
    int32_t n_blocks = 0;
    int32_t vertices_per_block = 0;
    std::vector<int64_t> v_off;
    std::vector<InstParams> inst_host;
    std::vector<int64_t> ns_inst;  // springs per instance
    // Resident executor: cloths grouped by launch shape; the streamed kernels of a step
    // run over the blocks of the remaining (streamed) cloths only.
    struct Bucket {
        int threads, cluster, vcta, n;
        int32_t* d_ids;
    };
    std::vector<Bucket> buckets;
    std::vector<uint8_t> resident;  // per instance
    // OC_RESIDENT_FUSED=1: resident cloths assemble inside the resident kernel (no
    // k_assemble pass over them).  Off by default: on 4096 cloths of 64 to 16,384 vertices
    // the fused step measured 4.97 ms against 4.37 ms for the separate passes (the
    // resident CTAs, 3 per SM by shared memory, assemble and then wait in the CG in
    // step with each other, so the assembly runs at lower occupancy and overlaps nothing).
    bool resident_fused = false;
    BlockInfo* d_streamed_blocks = nullptr;
    int32_t n_streamed_blocks = 0;
    // Block tables of a step: k_assemble over the REFERENCE cloths (resident and
    // streamed), the coupled kernels over the COUPLED cloths, k_integrate over the
    // streamed REFERENCE and the COUPLED cloths.  Without COUPLED cloths the first is the
    // full table and the last is the streamed one.
    BlockInfo* d_asm_blocks = nullptr;  // REFERENCE cloths on the CSR gather
    int32_t n_asm_blocks = 0;
    BlockInfo* d_grid_blocks = nullptr;  // REFERENCE grid cloths on the stencil gather
    int32_t n_grid_blocks = 0;
    // Grid cloths on the strip sweep (k_assemble_strip, then k_assemble_finish per cloth):
    // the work items (in args.strip_work), each cloth's range of them and its index in
    // args.strip_ids.
    std::vector<std::pair<int32_t, int32_t>> strip_range;
    std::vector<int32_t> strip_pos;
    // The launch configuration (oc_launch_config) and what re-planning needs: the full
    // block table on the host and the device's cooperative-launch capacity.
    oc_launch_config cfg{};
    std::vector<BlockInfo> h_blocks;
    int sm_count = 0;
    bool coop = false;
    int persist_per_sm = 0;
    // Grid cloths' stencil data on the host, to refit the parameter slots when
    // oc_set_spring_params changes Ks or Kd, and each cloth's grid shape as detected
    // ({0, 0}: not a grid).
    std::vector<int32_t> h_st_data;
    std::vector<float4> h_st_param;
    std::vector<int2> grid_shape;
    BlockInfo* d_cpl_blocks = nullptr;
    int32_t n_cpl_blocks = 0;
    BlockInfo* d_upd_blocks = nullptr;
    int32_t n_upd_blocks = 0;
    bool any_coupled = false;
    // The CG loop of the streamed REFERENCE cloths as one cooperative launch (k_cg_persist)
    // when there is no COUPLED cloth; otherwise the WHILE loop.
    bool persist = false;
    int persist_grid = 0;
    // k_assemble_finish runs when a strip-swept cloth is resident or the streamed CG is
    // not the persistent one; otherwise k_cg_persist forms their delta0 itself.
    bool strip_finish = true;
    unsigned* d_words = nullptr;  // k_cg_persist: one arrival count per cloth
    int* d_perr = nullptr;        // bit 0: a wait of k_cg_persist gave up
    // The adjoint solve (every cloth iterates) as one cooperative launch of k_cg_persist
    // without the update, when the handle has no COUPLED cloth.
    bool adj_persist = false;
    int adj_persist_grid = 0;
    bool any_provot = false;  // some cloth has OC_PASS_PROVOT: k_provot follows the update
    bool any_passes = false;  // some cloth has a pass after the update
    // Resident buckets run concurrently: forked from the handle's stream onto these.
    // Differentiation: spring ids, own-spring incidence, gradient planes and the tape.
    AdjArgs adj{};
    float* d_ks = nullptr;  // per spring, for oc_set_spring_params
    float* d_kd = nullptr;
    size_t stride = 0;      // plane stride (vertices)
    struct Tape {
        int32_t n_steps = 0, every = 0;
        float dt = 0.0f;
        // REPLAY (OC_TAPE_REPLAY): dV of every step (three planes of `stride` floats per
        // step) and per cloth its state every tc[i].every steps plus a segment buffer, in
        // one arena; the reverse pass rebuilds the states by replaying the update.
        bool replay = false;
        float* dvt = nullptr;
        size_t dvt_cap = 0;  // floats
        float4* arena = nullptr;
        size_t arena_cap = 0;  // float4s
        TapeCloth* d_tc = nullptr;
        std::vector<TapeCloth> tc;
        // RECOMPUTE (OC_TAPE_RECOMPUTE, when the dV of every step does not fit the
        // budget): every cloth's state every `every` steps (n_ck checkpoints); segment
        // buffers of every step's X, V and dV, n_buf of them: the last n_keep segments
        // are kept from the taped forward, the others are recomputed with the step into
        // buffer 0 (absent when n_keep = n_ck).
        int32_t n_ck = 0, n_buf = 0, n_keep = 0, cap_ck = 0, cap_slots = 0;
        float4 *ckX = nullptr, *ckV = nullptr, *segX = nullptr, *segV = nullptr, *finX = nullptr, *finV = nullptr;
        float *ckx = nullptr, *segx = nullptr, *finx = nullptr;
        float* planes = nullptr;  // gX 3, gV 3, gF 3, gOwn 6, gExt 3, dV 3
        float* gK = nullptr;      // gKs, gKd
        cudaGraph_t graph = nullptr;  // the adjoint solve as a WHILE loop (many cloths)
        cudaGraphExec_t exec = nullptr;
        cudaGraphNode_t n_seed = nullptr;  // k_adj_seed_own: its arguments change every step
        cudaGraphConditionalHandle handle = 0;
        float graph_dt = 0.0f;
        bool valid = false;
        // Displacement mode (oc_set_tape_mode): the start positions, the springs' start
        // constants and the final displacement of the last taped forward.
        int32_t mode = OC_TAPE_POSITIONS;
        bool gm_valid = false;
        float4* Xbase = nullptr;
        float2* gm_inc = nullptr;
        float2* gm_own = nullptr;
        float4* finU = nullptr;
    } tape;
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> aux_done;
    cudaEvent_t fork_ev = nullptr;
    std::vector<void*> allocs;
    StepArgs args{};
    float* stage = nullptr;         // device staging: 3 x 3 * nv floats
    int32_t* d_err = nullptr;       // device validation flag
    InstState* h_state = nullptr;   // pinned host mirror of the instance states
    int32_t* h_scalar = nullptr;    // pinned host scalar for loop control
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    float graph_dt = 0.0f;
    int64_t host_launches = 0;  // k_assemble, k_integrate, k_resident, k_provot launches enqueued
    unsigned long long* h_loop = nullptr;
    std::string err;
};

namespace {

// Floats between the staging planes of X, V and dV (three floats per vertex, rounded up
// to 64 so that every plane is 256-byte aligned for the float4 check of k_state_check4).
size_t stage_stride(int64_t nv) { return (3 * (size_t)nv + 63) / 64 * 64; }

oc_status fail(oc_solver* s, oc_status code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}

oc_status fail_cuda(oc_solver* s, cudaError_t e, const char* what) {
    const oc_status code = (e == cudaErrorMemoryAllocation) ? OC_ERR_OUT_OF_MEMORY : OC_ERR_CUDA;
    return fail(s, code, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define OC_TRY(call)                                          \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return fail_cuda(s, e_, #call); \
    } while (0)

// Polls of a cloth's arrival count before a wait of k_cg_persist gives up (about half
// a second with its 32 ns back-off).
constexpr uint32_t kDefaultBarrierPolls = 1u << 22;

// A wait of k_cg_persist that gave up (the stream is synchronised).  The error word is
// cleared once reported and the cloths' CG state (which the abandoned launch left part
// updated) is zeroed: every step's assembly sets it up again, and the next launch starts
// from zeroed arrival counts, so the handle steps on.
oc_status check_device_error(oc_solver* s) {
    if (!s->d_perr) return OC_OK;
    int h = 0;
    OC_TRY(cudaMemcpy(&h, s->d_perr, sizeof(int), cudaMemcpyDeviceToHost));
    if (h != 0) {
        OC_TRY(cudaMemset(s->d_perr, 0, sizeof(int)));
        OC_TRY(cudaMemset(s->args.state, 0, sizeof(InstState) * (size_t)s->n_inst));
        return fail(s, OC_ERR_DEVICE_TIMEOUT,
                    "k_cg_persist: a wait gave up (cloths whose solve had not ended were not updated)");
    }
    return OC_OK;
}

// k_cg_persist over block table a.blocks[0, n): its cloths' arrival counts zeroed, then
// the cooperative launch.
cudaError_t persist_cg(oc_solver* s, const StepArgs& a, int32_t n, int grid) {
    cudaError_t e = cudaMemsetAsync(s->d_words, 0, sizeof(unsigned) * (size_t)s->n_inst, s->stream);
    return e == cudaSuccess ? launch_cg_persist(a, n, grid, s->d_words, s->d_perr, s->stream) : e;
}


// Whether a grid cloth that may take the strip sweep should: its warps own 28 columns
// each, so narrow cloths leave lanes idle.  With cfg.strip = 0 every grid cloth stays on
// k_assemble_grid (both give the same bits).
bool strip_wanted(const oc_launch_config& cfg, const InstParams& ip) {
    if (!cfg.strip || !ip.strip_ok || ip.grid_cols <= 0 || ip.coupled) return false;
    const int32_t cols = ip.grid_cols;
    const int32_t strips = (cols + kStripOwned - 1) / kStripOwned;
    return cols >= 20 && 2 * cols >= 32 * strips;  // at least half the lanes own a vertex
}

int strip_blocks(int32_t n_work) { return (n_work + kStripThreads / 32 - 1) / (kStripThreads / 32); }

template <class T>
cudaError_t dalloc(oc_solver* s, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) s->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return e;
}

// The persistent CG's words (once per handle).
oc_status alloc_persist_words(oc_solver* s) {
    if (s->d_words) return OC_OK;
    OC_TRY(dalloc(s, &s->d_words, (size_t)s->n_inst));
    OC_TRY(cudaMemset(s->d_words, 0, sizeof(unsigned) * (size_t)s->n_inst));
    OC_TRY(dalloc(s, &s->d_perr, 1));
    OC_TRY(cudaMemset(s->d_perr, 0, sizeof(int)));
    return OC_OK;
}

template <class T>
cudaError_t upload(oc_solver* s, T** p, const std::vector<T>& v) {
    cudaError_t e = dalloc(s, p, v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// Frees a table of the handle (re-planning replaces its tables).
template <class T>
void dfree(oc_solver* s, T** p) {
    if (*p) {
        auto it = std::find(s->allocs.begin(), s->allocs.end(), (void*)*p);
        if (it != s->allocs.end()) {
            cudaFree((void*)*p);
            s->allocs.erase(it);
        }
        *p = nullptr;
    }
}

// upload() into a pointer that may hold an earlier table of the handle, which is freed.
template <class T>
cudaError_t reupload(oc_solver* s, T** p, const std::vector<T>& v) {
    dfree(s, p);
    return upload(s, p, v);
}

void release(oc_solver* s) {
    if (!s) return;
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    for (void* p : s->allocs) cudaFree(p);
    s->allocs.clear();
    if (s->h_state) cudaFreeHost(s->h_state);
    if (s->h_scalar) cudaFreeHost(s->h_scalar);
    if (s->h_loop) cudaFreeHost(s->h_loop);
    if (s->tape.exec) cudaGraphExecDestroy(s->tape.exec);
    if (s->tape.graph) cudaGraphDestroy(s->tape.graph);
    for (cudaStream_t x : s->aux) cudaStreamDestroy(x);
    for (cudaEvent_t e : s->aux_done) cudaEventDestroy(e);
    if (s->fork_ev) cudaEventDestroy(s->fork_ev);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
}

// One step with the CG loop driven from the host.  per_cloth: launch each instance's
// blocks separately (the plain one-cloth-per-launch baseline).  timer: optional
// per-kernel timing callback around every launch.
struct KernelTimer {
    cudaEvent_t ev[2] = {nullptr, nullptr};
    double ms[K_COUNT] = {0};
    int64_t launches[K_COUNT] = {0};
    double bytes[K_COUNT] = {0};  // algorithmic bytes moved (active instances only)
};

// Algorithmic bytes of one step, from each instance's CG iteration count: every array
// element a kernel must read or write counted once, in the device layout (X/V float4,
// 16-byte incidence records, FP32 planes).  Per vertex: k_assemble 120 B plus 32 B per
// spring, k_assemble_grid 116 B (plus the row pointer 4 B and 4 B per incidence when rest
// lengths are read per incidence), first k_cg_dir pass 36 B, later passes 60 B, k_cg_update 84 B, k_integrate 76 B
// (the ellipsoid pass adds no traffic), k_provot 53 B plus 32 B per spring.
void account_step_bytes(const oc_solver* s, KernelTimer* t) {
    for (int32_t k = 0; k < s->n_inst; ++k) {
        const double nv = (double)s->inst_host[k].nv, ns = (double)s->ns_inst[k];
        const InstState& st = s->h_state[k];
        // Assembled by k_resident (fused) or by the COUPLED kernels: no assembly bytes here.
        const bool fused = (s->resident[k] && s->resident_fused) || s->inst_host[k].coupled;
        if (!fused && s->inst_host[k].strip) {
            // The strip sweep: k_assemble_grid's bytes, rest lengths (when they vary) as six
            // planes by anchor.
            t->bytes[K_ASSEMBLE_STRIP] += 116.0 * nv + (s->inst_host[k].st_rest ? 24.0 * nv : 0.0);
        } else if (!fused && s->inst_host[k].grid_cols > 0)  // no incidence records, no row pointer
            t->bytes[K_ASSEMBLE_GRID] +=              // unless rest lengths are per incidence
                116.0 * nv + (s->inst_host[k].st_rest ? 4.0 * nv + 8.0 * ns : 0.0);
        else if (!fused)
            t->bytes[K_ASSEMBLE] += 120.0 * nv + 32.0 * ns;
        // k_provot: X 16, V 32 in and out, pin flag 1, row pointer 4; 16-byte records (a
        // grid cloth reads its stencil instead, and rest lengths per incidence if they vary).
        if (s->inst_host[k].passes & OC_PASS_PROVOT) {
            const InstParams& ip = s->inst_host[k];
            t->bytes[K_PROVOT] += ip.grid_cols > 0 ? 49.0 * nv + (ip.st_rest ? 4.0 * nv + 8.0 * ns : 0.0)
                                                   : 53.0 * nv + 32.0 * ns;
        }
        if (s->inst_host[k].coupled) {
            // k_cpl_assemble 112 B + 72 B per spring (record in, block out at both ends);
            // k_cpl_dir 37 B (first pass) or 53 B plus 48 B per spring (other vertex and
            // block at both ends; z and d are 16-byte records); k_cpl_update 132 B (first)
            // or 148 B; k_integrate 76 B.
            const InstParams& cp = s->inst_host[k];  // a grid cloth reads its stencil, not records
            t->bytes[K_CPL_ASSEMBLE] += cp.grid_cols > 0 ? 112.0 * nv + 40.0 * ns + (cp.st_rest ? 4.0 * nv + 8.0 * ns : 0.0)
                                                         : 112.0 * nv + 72.0 * ns;
            const double it = (double)st.iter;
            double dirs = it > 0 ? 37.0 * nv + 53.0 * nv * (it - 1.0) + 48.0 * ns * it : 0.0;
            if (st.flags & OC_FLAG_BREAKDOWN) dirs += (it > 0 ? 53.0 : 37.0) * nv + 48.0 * ns;
            t->bytes[K_CPL_DIR] += dirs;
            t->bytes[K_CPL_UPDATE] += it > 0 ? 132.0 * nv + 148.0 * nv * (it - 1.0) : 0.0;
            t->bytes[K_INTEGRATE] += 76.0 * nv;
            continue;
        }
        if (s->resident[k]) {
            if (s->resident_fused) {
                // X, V 32 in and out, spring i 24, warm start 12 in and out, plus the
                // gather's row pointer and records (or stencil rest lengths); the CG
                // iterations run in shared memory.
                const InstParams& ip = s->inst_host[k];
                double gather = 4.0 * nv + 32.0 * ns;
                if (ip.grid_cols > 0) gather = ip.st_rest ? 4.0 * nv + 8.0 * ns : 0.0;
                t->bytes[K_RESIDENT] += 112.0 * nv + gather;
            } else {
                // CG state in (A 24 + x, r, d 36), X, V 32 in and out, dV 12 out; the CG
                // iterations run in shared memory.
                t->bytes[K_RESIDENT] += 136.0 * nv;
            }
            continue;
        }
        const double it = (double)st.iter;
        double dirs = it > 0 ? 36.0 * nv + 60.0 * nv * (it - 1.0) : 0.0;
        if (st.flags & OC_FLAG_BREAKDOWN) dirs += (it > 0 ? 60.0 : 36.0) * nv;
        if (s->persist) {  // k_cg_persist: the same passes and the update in one launch
            t->bytes[K_CG_PERSIST] += dirs + 84.0 * nv * it + 76.0 * nv;
            continue;
        }
        t->bytes[K_INTEGRATE] += 76.0 * nv;
        t->bytes[K_CG_UPDATE] += 84.0 * nv * it;
        t->bytes[K_CG_DIR] += dirs;
    }
}

oc_status launch_timed(oc_solver* s, KernelKind k, const StepArgs& a, int nblocks, KernelTimer* t) {
    if (t) OC_TRY(cudaEventRecord(t->ev[0], s->stream));
    OC_TRY(launch_kernel(k, a, nblocks, s->stream));
    if (t) {
        OC_TRY(cudaEventRecord(t->ev[1], s->stream));
        OC_TRY(cudaEventSynchronize(t->ev[1]));
        float ms = 0.0f;
        OC_TRY(cudaEventElapsedTime(&ms, t->ev[0], t->ev[1]));
        t->ms[k] += ms;
        t->launches[k] += 1;
    }
    return OC_OK;
}

// The resident cloths' launches (one per bucket).  With a.cg_only they run unfused: the
// adjoint solve of each resident cloth on chip.
oc_status launch_resident_all(oc_solver* s, const StepArgs& a, KernelTimer* t) {
    if (!t && !s->aux.empty()) {
        // Fork: every bucket on its own stream, joined back into the handle's stream.
        OC_TRY(cudaEventRecord(s->fork_ev, s->stream));
        for (size_t i = 0; i < s->aux.size(); ++i) OC_TRY(cudaStreamWaitEvent(s->aux[i], s->fork_ev, 0));
        for (size_t i = 0; i < s->buckets.size(); ++i) {
            const auto& b = s->buckets[i];
            ResidentLaunch L{b.d_ids, b.cluster, b.vcta, (s->resident_fused && !a.cg_only) ? 1 : 0};
            OC_TRY(launch_resident(a, L, b.threads, b.n, s->aux[i % s->aux.size()]));
            s->host_launches += 1;
        }
        for (size_t i = 0; i < s->aux.size(); ++i) {
            OC_TRY(cudaEventRecord(s->aux_done[i], s->aux[i]));
            OC_TRY(cudaStreamWaitEvent(s->stream, s->aux_done[i], 0));
        }
        return OC_OK;
    }
    for (const auto& b : s->buckets) {
        if (t) OC_TRY(cudaEventRecord(t->ev[0], s->stream));
        ResidentLaunch L{b.d_ids, b.cluster, b.vcta, (s->resident_fused && !a.cg_only) ? 1 : 0};
        OC_TRY(launch_resident(a, L, b.threads, b.n, s->stream));
        s->host_launches += 1;
        if (t) {
            OC_TRY(cudaEventRecord(t->ev[1], s->stream));
            OC_TRY(cudaEventSynchronize(t->ev[1]));
            float ms = 0.0f;
            OC_TRY(cudaEventElapsedTime(&ms, t->ev[0], t->ev[1]));
            t->ms[K_RESIDENT] += ms;
            t->launches[K_RESIDENT] += 1;
        }
    }
    return OC_OK;
}

oc_status step_host_driven(oc_solver* s, float dt, bool per_cloth, KernelTimer* t) {
    StepArgs a = s->args;
    a.dt = dt;
    a.use_cond = 0;
    a.cond = 0;
    OC_TRY(cudaMemsetAsync(a.unconverged, 0, sizeof(int32_t), s->stream));
    oc_status st = OC_OK;
    if (per_cloth) {
        // The plain baseline: every cloth on its own, streamed kernels, host-driven loop.
        for (int grp = 0; grp < s->n_inst; ++grp) {
            a.blk_base = s->inst_host[grp].blk0;
            const int nb = s->inst_host[grp].nblk;
            const bool cpl = s->inst_host[grp].coupled != 0;
            if (s->inst_host[grp].strip && !cpl) {
                StepArgs w = a;
                w.strip_work = s->args.strip_work + s->strip_range[(size_t)grp].first;
                w.n_strip_work = s->strip_range[(size_t)grp].second;
                w.strip_item0 = s->strip_range[(size_t)grp].first;
                if ((st = launch_timed(s, K_ASSEMBLE_STRIP, w, strip_blocks(w.n_strip_work), t)) != OC_OK) return st;
                StepArgs fa = a;
                fa.strip_ids = s->args.strip_ids + s->strip_pos[(size_t)grp];
                if ((st = launch_timed(s, K_ASSEMBLE_FINISH, fa, 1, t)) != OC_OK) return st;
                s->host_launches += 1;
            } else {
                const KernelKind ka =
                    cpl ? K_CPL_ASSEMBLE : (s->inst_host[grp].grid_cols > 0 ? K_ASSEMBLE_GRID : K_ASSEMBLE);
                if ((st = launch_timed(s, ka, a, nb, t)) != OC_OK) return st;
            }
            s->host_launches += s->any_provot ? 3 : 2;
            for (;;) {
                OC_TRY(cudaMemcpyAsync(s->h_scalar, &s->args.state[grp].active, sizeof(int32_t),
                                       cudaMemcpyDeviceToHost, s->stream));
                OC_TRY(cudaStreamSynchronize(s->stream));
                if (*s->h_scalar <= 0) break;
                if ((st = launch_timed(s, cpl ? K_CPL_DIR : K_CG_DIR, a, nb, t)) != OC_OK) return st;
                if ((st = launch_timed(s, cpl ? K_CPL_UPDATE : K_CG_UPDATE, a, nb, t)) != OC_OK) return st;
            }
            if ((st = launch_timed(s, K_INTEGRATE, a, nb, t)) != OC_OK) return st;
            if (s->any_provot && (st = launch_timed(s, K_PROVOT, a, nb, t)) != OC_OK) return st;
        }
    } else {
        // Assembly over every cloth, then the resident CG launches and the streamed loop.
        a.blk_base = 0;
        StepArgs aa = a, ga = a, ca = a, sa = a, ua = a;
        aa.blocks = s->d_asm_blocks;
        ga.blocks = s->d_grid_blocks;
        ca.blocks = s->d_cpl_blocks;
        sa.blocks = s->d_streamed_blocks;
        ua.blocks = s->d_upd_blocks;
        if (s->n_asm_blocks > 0) {
            if ((st = launch_timed(s, K_ASSEMBLE, aa, s->n_asm_blocks, t)) != OC_OK) return st;
            s->host_launches += 1;
        }
        if (s->n_grid_blocks > 0) {
            if ((st = launch_timed(s, K_ASSEMBLE_GRID, ga, s->n_grid_blocks, t)) != OC_OK) return st;
            s->host_launches += 1;
        }
        if (s->args.n_strip_work > 0) {
            if ((st = launch_timed(s, K_ASSEMBLE_STRIP, a, strip_blocks(a.n_strip_work), t)) != OC_OK) return st;
            s->host_launches += 1;
            if (s->strip_finish) {
                if ((st = launch_timed(s, K_ASSEMBLE_FINISH, a, a.n_strip_ids, t)) != OC_OK) return st;
                s->host_launches += 1;
            }
        }
        if (s->n_cpl_blocks > 0) {
            if ((st = launch_timed(s, K_CPL_ASSEMBLE, ca, s->n_cpl_blocks, t)) != OC_OK) return st;
            s->host_launches += 1;
        }
        if ((st = launch_resident_all(s, a, t)) != OC_OK) return st;
        const int nb = s->n_streamed_blocks, nc = s->n_cpl_blocks;
        if (s->persist) {
            if (t) OC_TRY(cudaEventRecord(t->ev[0], s->stream));
            sa.persist_d0 = 1;
            OC_TRY(persist_cg(s, sa, nb, s->persist_grid));
            s->host_launches += 1;
            if (t) {
                OC_TRY(cudaEventRecord(t->ev[1], s->stream));
                OC_TRY(cudaEventSynchronize(t->ev[1]));
                float ms = 0.0f;
                OC_TRY(cudaEventElapsedTime(&ms, t->ev[0], t->ev[1]));
                t->ms[K_CG_PERSIST] += ms;
                t->launches[K_CG_PERSIST] += 1;
            }
        } else if (nb > 0 || nc > 0) {
            for (;;) {
                OC_TRY(cudaMemcpyAsync(s->h_scalar, a.unconverged, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                       s->stream));
                OC_TRY(cudaStreamSynchronize(s->stream));
                if (*s->h_scalar <= 0) break;
                if (nb > 0) {
                    if ((st = launch_timed(s, K_CG_DIR, sa, nb, t)) != OC_OK) return st;
                    if ((st = launch_timed(s, K_CG_UPDATE, sa, nb, t)) != OC_OK) return st;
                }
                if (nc > 0) {
                    if ((st = launch_timed(s, K_CPL_DIR, ca, nc, t)) != OC_OK) return st;
                    if ((st = launch_timed(s, K_CPL_UPDATE, ca, nc, t)) != OC_OK) return st;
                }
            }
            if ((st = launch_timed(s, K_INTEGRATE, ua, s->n_upd_blocks, t)) != OC_OK) return st;
            s->host_launches += 1;
        }
        if (s->any_provot) {  // after every cloth's update, resident and streamed
            if ((st = launch_timed(s, K_PROVOT, a, s->n_blocks, t)) != OC_OK) return st;
            s->host_launches += 1;
        }
    }
    if (t) {
        OC_TRY(cudaMemcpyAsync(s->h_state, s->args.state, sizeof(InstState) * s->n_inst, cudaMemcpyDeviceToHost,
                               s->stream));
        OC_TRY(cudaStreamSynchronize(s->stream));
        account_step_bytes(s, t);
    }
    return OC_OK;
}

oc_status build_graph(oc_solver* s, float dt) {
    if (s->exec) {
        cudaGraphExecDestroy(s->exec);
        s->exec = nullptr;
    }
    if (s->graph) {
        cudaGraphDestroy(s->graph);
        s->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    OC_TRY(cudaGraphCreate(&g, 0));
    s->graph = g;
    const bool persist = s->persist;
    const bool streamed = s->n_streamed_blocks > 0 && !persist, coupled = s->n_cpl_blocks > 0;
    const bool loop = streamed || coupled;
    // The WHILE loop's handle exists only when there are streamed cloths (a handle that
    // no conditional node uses makes the graph fail to instantiate).
    cudaGraphConditionalHandle handle = 0;
    if (loop) OC_TRY(cudaGraphConditionalHandleCreate(&handle, g, 0, 0));

    StepArgs a = s->args;  // full block table (the passes)
    a.dt = dt;
    a.blk_base = 0;
    a.use_cond = loop ? 1 : 0;
    a.cond = (unsigned long long)handle;
    StepArgs aa = a, ga = a, sa = a, ca = a, ua = a;
    aa.blocks = s->d_asm_blocks;       // REFERENCE cloths: k_assemble
    ga.blocks = s->d_grid_blocks;      // REFERENCE grid cloths: k_assemble_grid
    sa.blocks = s->d_streamed_blocks;  // streamed REFERENCE cloths: CG loop
    ca.blocks = s->d_cpl_blocks;       // COUPLED cloths
    ua.blocks = s->d_upd_blocks;       // k_integrate
    void* params_all[] = {&a};
    void* params_asm[] = {&aa};
    void* params_grid[] = {&ga};
    void* params_str[] = {&sa};
    void* params_cpl[] = {&ca};
    void* params_upd[] = {&ua};
    enum Table { T_ALL, T_ASM, T_STR, T_CPL, T_UPD, T_GRID, T_STRIP, T_SFIN };
    auto kparams = [&](KernelKind k, Table tab) {
        cudaKernelNodeParams kp{};
        kp.func = const_cast<void*>(kernel_fn(k, a));
        const int n[] = {s->n_blocks, s->n_asm_blocks, s->n_streamed_blocks, s->n_cpl_blocks, s->n_upd_blocks,
                         s->n_grid_blocks, strip_blocks(s->args.n_strip_work), s->args.n_strip_ids};
        void** pp[] = {params_all, params_asm, params_str, params_cpl, params_upd, params_grid, params_all, params_all};
        kp.gridDim = dim3((unsigned)n[tab]);
        kp.blockDim = dim3((unsigned)kernel_block_threads());
        kp.sharedMemBytes = (unsigned)kernel_smem_bytes(k, a);
        kp.kernelParams = pp[tab];
        kp.extra = nullptr;
        return kp;
    };

    cudaGraphNode_t n_reset, n_asm;
    cudaMemsetParams mp{};
    mp.dst = a.unconverged;
    mp.value = 0;
    mp.elementSize = sizeof(int32_t);
    mp.width = 1;
    mp.height = 1;
    mp.pitch = sizeof(int32_t);
    OC_TRY(cudaGraphAddMemsetNode(&n_reset, g, nullptr, 0, &mp));
    cudaKernelNodeParams kp{};
    n_asm = n_reset;
    if (s->n_asm_blocks > 0) {
        kp = kparams(K_ASSEMBLE, T_ASM);
        OC_TRY(cudaGraphAddKernelNode(&n_asm, g, &n_reset, 1, &kp));
    }
    if (s->n_grid_blocks > 0) {  // serialised after k_assemble: both end in the same counters
        cudaGraphNode_t prev = n_asm;
        kp = kparams(K_ASSEMBLE_GRID, T_GRID);
        OC_TRY(cudaGraphAddKernelNode(&n_asm, g, &prev, 1, &kp));
    }
    if (s->args.n_strip_work > 0) {  // the strip sweep, then its cloths' delta0 totals
        cudaGraphNode_t prev = n_asm;
        kp = kparams(K_ASSEMBLE_STRIP, T_STRIP);
        OC_TRY(cudaGraphAddKernelNode(&n_asm, g, &prev, 1, &kp));
        if (s->strip_finish) {
            prev = n_asm;
            kp = kparams(K_ASSEMBLE_FINISH, T_SFIN);
            OC_TRY(cudaGraphAddKernelNode(&n_asm, g, &prev, 1, &kp));
        }
    }
    cudaGraphNode_t n_last = n_asm;  // the loop waits for every assembly
    if (coupled) {
        kp = kparams(K_CPL_ASSEMBLE, T_CPL);
        OC_TRY(cudaGraphAddKernelNode(&n_last, g, &n_asm, 1, &kp));
    }
    std::vector<cudaGraphNode_t> updates;  // the nodes that write X and V

    if (loop) {
        cudaGraphNode_t n_loop, n_int;
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        OC_TRY(cudaGraphAddNode(&n_loop, g, &n_last, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        // Body: the REFERENCE pair, then the COUPLED pair; the last update kernel's last
        // block sets the condition from the counter both loops decrement.
        cudaGraphNode_t prev = nullptr;
        auto add_body = [&](KernelKind k, Table tab) -> cudaError_t {
            cudaKernelNodeParams bp = kparams(k, tab);
            cudaGraphNode_t n;
            cudaError_t e = cudaGraphAddKernelNode(&n, body, prev ? &prev : nullptr, prev ? 1 : 0, &bp);
            prev = n;
            return e;
        };
        if (streamed) {
            OC_TRY(add_body(K_CG_DIR, T_STR));
            OC_TRY(add_body(K_CG_UPDATE, T_STR));
        }
        if (coupled) {
            OC_TRY(add_body(K_CPL_DIR, T_CPL));
            OC_TRY(add_body(K_CPL_UPDATE, T_CPL));
        }
        kp = kparams(K_INTEGRATE, T_UPD);
        OC_TRY(cudaGraphAddKernelNode(&n_int, g, &n_loop, 1, &kp));
        updates.push_back(n_int);
    }
    if (persist) {
        // The streamed cloths' whole CG loop and update: the memset of their completion
        // words and the cooperative launch, captured into a child graph.
        cudaGraphNode_t n_pc;
        cudaGraph_t pg = nullptr;
        OC_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        StepArgs pa = sa;
        pa.blocks = s->d_streamed_blocks;
        pa.use_cond = 0;
        pa.persist_d0 = 1;
        cudaError_t le = persist_cg(s, pa, s->n_streamed_blocks, s->persist_grid);
        cudaError_t ce = cudaStreamEndCapture(s->stream, &pg);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (pg) cudaGraphDestroy(pg);
            return fail_cuda(s, le != cudaSuccess ? le : ce, "capture of k_cg_persist");
        }
        cudaError_t e = cudaGraphAddChildGraphNode(&n_pc, g, &n_last, 1, pg);
        cudaGraphDestroy(pg);
        if (e != cudaSuccess) return fail_cuda(s, e, "cudaGraphAddChildGraphNode");
        updates.push_back(n_pc);
    }
    if (!s->buckets.empty()) {
        // The resident launches (concurrent, fork/join) captured into a child graph that
        // runs beside the streamed cloths' kernels (they touch disjoint cloths): after the
        // assembly when that pass builds the resident cloths' systems, else from the start.
        cudaGraph_t rg = nullptr;
        OC_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        StepArgs ra = a;
        ra.use_cond = 0;
        const int64_t launches_before = s->host_launches;
        oc_status rs = launch_resident_all(s, ra, nullptr);
        s->host_launches = launches_before;
        cudaError_t ce = cudaStreamEndCapture(s->stream, &rg);
        if (rs != OC_OK) {
            if (rg) cudaGraphDestroy(rg);
            return rs;
        }
        if (ce != cudaSuccess) return fail_cuda(s, ce, "cudaStreamEndCapture");
        cudaGraphNode_t n_res;
        cudaError_t e = cudaGraphAddChildGraphNode(&n_res, g, s->resident_fused ? &n_reset : &n_asm, 1, rg);
        cudaGraphDestroy(rg);
        if (e != cudaSuccess) return fail_cuda(s, e, "cudaGraphAddChildGraphNode");
        updates.push_back(n_res);
    }
    if (s->any_provot) {
        cudaGraphNode_t n_prov;
        kp = kparams(K_PROVOT, T_ALL);
        OC_TRY(cudaGraphAddKernelNode(&n_prov, g, updates.data(), updates.size(), &kp));
    }
    OC_TRY(cudaGraphInstantiate(&s->exec, g, 0));
    s->graph_dt = dt;
    return OC_OK;
}

// Launch shape of a resident cloth: up to 1024 vertices one CTA (vertex capacity the
// next power of two, at least 128); beyond, clusters of CTAs of 1024 vertices each, up
// to max_vertices and kResidentMaxCluster CTAs.
constexpr int kResidentDefaultVcta = 1024;

// The per-CTA vertex capacity and thread count come from the launch configuration
// (resident_vcta, resident_threads).
bool resident_shape(int nv, int max_vertices, int base, int thr, int* threads, int* cluster, int* vcta) {
    if (nv < 1 || nv > max_vertices) return false;
    if (nv <= base) {
        int v = 128;
        while (v < nv) v <<= 1;
        *cluster = 1;
        *vcta = v;
        *threads = v < thr ? v : thr;
        return true;
    }
    const int c = (nv + base - 1) / base;
    if (c > kResidentMaxCluster) {
        const int c2 = (nv + kResidentMaxVcta - 1) / kResidentMaxVcta;
        if (c2 > kResidentMaxCluster) return false;
        *cluster = c2;
        *vcta = kResidentMaxVcta;
        *threads = 512;
        return true;
    }
    *cluster = c;
    *vcta = base;
    *threads = thr;
    return true;
}

bool valid_solver(const oc_solver* s) { return s != nullptr && s->nv > 0; }

// Copies of the state triple (X, V float4; the warm-start planes) between the solver
// and a tape slot.
oc_status copy_state(oc_solver* s, float4* dX, float4* dV, float* dx, const float4* sX, const float4* sV,
                     const float* sx) {
    const size_t n4 = sizeof(float4) * (size_t)s->nv;
    OC_TRY(cudaMemcpyAsync(dX, sX, n4, cudaMemcpyDeviceToDevice, s->stream));
    OC_TRY(cudaMemcpyAsync(dV, sV, n4, cudaMemcpyDeviceToDevice, s->stream));
    if (dx && sx) OC_TRY(cudaMemcpyAsync(dx, sx, 3 * s->stride * sizeof(float), cudaMemcpyDeviceToDevice, s->stream));
    return OC_OK;
}

float* xplanes(oc_solver* s) { return s->args.x[0]; }  // the three x planes are contiguous

// The segment buffer of segment c: a kept segment's own buffer, or -1 for a segment the
// reverse pass recomputes (into buffer 0).
int32_t tape_buffer(const oc_solver::Tape& T, int32_t c) {
    const int32_t first_kept = T.n_ck - T.n_keep;
    if (c < first_kept) return -1;
    return (c - first_kept) + (T.n_keep < T.n_ck ? 1 : 0);
}

// The handle's arguments in the tape's displacement mode (X then holds u).
StepArgs gm_args(const oc_solver* s, float dt) {
    StepArgs a = s->args;
    a.dt = dt;
    a.blk_base = 0;
    a.use_cond = 0;
    a.all_streamed = 1;
    a.gm = 1;
    a.Xbase = s->tape.Xbase;
    a.gm_inc = s->tape.gm_inc;
    a.gm_own = s->tape.gm_own;
    return a;
}

// The CG alone (no update) of every cloth, from the CG state set up in the planes and
// the cloths' states: the resident cloths on chip (k_resident unfused, one launch per
// bucket, beside) and the streamed ones in one cooperative launch of k_cg_persist over
// the streamed block table.  A handle whose plan has no resident bucket runs every cloth
// in k_cg_persist.
oc_status solve_only(oc_solver* s, const StepArgs& a) {
    StepArgs pa = a;
    pa.cg_only = 1;
    if (s->buckets.empty()) {
        OC_TRY(persist_cg(s, pa, s->n_blocks, s->adj_persist_grid));
        s->host_launches += 1;
        return OC_OK;
    }
    if (oc_status r = launch_resident_all(s, pa, nullptr)) return r;
    if (s->n_streamed_blocks > 0) {
        pa.blocks = s->d_streamed_blocks;
        const int grid = std::min(s->persist_per_sm * s->sm_count, std::max(1, s->n_streamed_blocks));
        OC_TRY(persist_cg(s, pa, s->n_streamed_blocks, grid));
        s->host_launches += 1;
    }
    return OC_OK;
}

// One step in displacement mode: the assembly over every cloth, the CG of every cloth
// without the update, then the displacement update.
oc_status gm_step(oc_solver* s, float dt) {
    const StepArgs a = gm_args(s, dt);
    OC_TRY(cudaMemsetAsync(a.unconverged, 0, sizeof(int32_t), s->stream));
    OC_TRY(launch_gm(1, a, s->n_blocks, s->stream));
    if (oc_status r = solve_only(s, a)) return r;
    OC_TRY(launch_gm(2, a, s->n_blocks, s->stream));
    s->host_launches += 2;
    return OC_OK;
}

// The adjoint solve of one step as a graph (positions mode, a handle without the
// cooperative CG): reset the loop counter, rebuild the system's diagonal blocks and set
// up the CG on the adjoint right-hand side (k_adj_seed_own), iterate (WHILE node) over
// every cloth.
oc_status build_adjoint_graph(oc_solver* s, float dt) {
    auto& T = s->tape;
    if (T.exec) {
        cudaGraphExecDestroy(T.exec);
        T.exec = nullptr;
    }
    if (T.graph) {
        cudaGraphDestroy(T.graph);
        T.graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    OC_TRY(cudaGraphCreate(&g, 0));
    T.graph = g;
    cudaGraphConditionalHandle handle;
    OC_TRY(cudaGraphConditionalHandleCreate(&handle, g, 0, 0));
    StepArgs a = s->args;
    a.dt = dt;
    a.blk_base = 0;
    a.use_cond = 1;
    a.cond = (unsigned long long)handle;
    a.all_streamed = 1;
    AdjArgs j = s->adj;
    void* params_seed[] = {&a, &j};
    void* params_cg[] = {&a};
    cudaGraphNode_t n_reset, n_seed, n_loop, n_dir, n_upd;
    cudaMemsetParams mp{};
    mp.dst = a.unconverged;
    mp.value = 0;
    mp.elementSize = sizeof(int32_t);
    mp.width = 1;
    mp.height = 1;
    mp.pitch = sizeof(int32_t);
    OC_TRY(cudaGraphAddMemsetNode(&n_reset, g, nullptr, 0, &mp));
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(adjoint_seed_own_fn());
    kp.gridDim = dim3((unsigned)s->n_blocks);
    kp.blockDim = dim3(256);
    kp.kernelParams = params_seed;
    OC_TRY(cudaGraphAddKernelNode(&n_seed, g, &n_reset, 1, &kp));
    T.n_seed = n_seed;
    T.handle = handle;
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    OC_TRY(cudaGraphAddNode(&n_loop, g, &n_seed, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    kp.func = const_cast<void*>(kernel_fn(K_CG_DIR, s->args));
    kp.gridDim = dim3((unsigned)s->n_blocks);
    kp.blockDim = dim3((unsigned)kernel_block_threads());
    kp.kernelParams = params_cg;
    OC_TRY(cudaGraphAddKernelNode(&n_dir, body, nullptr, 0, &kp));
    kp.func = const_cast<void*>(kernel_fn(K_CG_UPDATE, s->args));
    OC_TRY(cudaGraphAddKernelNode(&n_upd, body, &n_dir, 1, &kp));
    OC_TRY(cudaGraphInstantiate(&T.exec, g, 0));
    T.graph_dt = dt;
    return OC_OK;
}

// The strip sweep's work items: per cloth on the sweep, bands of rows times strips of 28
// columns, one warp each, a band's strips adjacent so a CTA's warps share rows.  Each warp
// walks its band row by row, so short bands give more warps to hide the memory latency of
// each row, and long bands recompute fewer springs (a band recomputes the springs of the
// two rows above it): R rows per band, R chosen for about four waves of 16 warps per SM,
// between 4 and 16, unless the launch configuration sets it (strip_rows).
oc_status build_strip_work(oc_solver* s) {
    std::vector<StripWork> work;
    s->strip_range.assign((size_t)s->n_inst, std::make_pair(0, 0));
    // Band height: a warp walks R + 2 rows for R owned ones, and the warps run in waves of
    // (SMs x CTAs per SM x 8): take the R of 4 ... 64 that minimises waves x (R + 2).
    const int64_t per_wave = (int64_t)std::max(1, s->sm_count) * s->cfg.strip_variant * (kStripThreads / 32);
    int32_t R = 16;
    double best = 0.0;
    for (int32_t r = 4; r <= 64; ++r) {
        int64_t items = 0;
        for (int32_t k = 0; k < s->n_inst; ++k) {
            const InstParams& ip = s->inst_host[(size_t)k];
            if (ip.strip)
                items += (int64_t)((ip.grid_cols + kStripOwned - 1) / kStripOwned) * ((ip.grid_rows + r - 1) / r);
        }
        const double cost = (double)((items + per_wave - 1) / per_wave) * (double)(r + 2);
        if (items > 0 && (best == 0.0 || cost < best)) {
            best = cost;
            R = r;
        }
    }
    if (s->cfg.strip_rows > 0) R = s->cfg.strip_rows;
    for (int32_t k = 0; k < s->n_inst; ++k) {
        InstParams& ip = s->inst_host[(size_t)k];
        ip.strip_w0 = ip.strip_nw = 0;
        if (!ip.strip) continue;
        const int32_t first = (int32_t)work.size();
        const int32_t rows = ip.grid_rows, band = std::min(R, rows);
        for (int32_t r0 = 0; r0 < rows; r0 += band)
            for (int32_t c0 = 0; c0 < ip.grid_cols; c0 += kStripOwned)
                work.push_back(StripWork{k, c0, r0, std::min(rows, r0 + band)});
        s->strip_range[(size_t)k] = std::make_pair(first, (int32_t)work.size() - first);
        ip.strip_w0 = first;
        ip.strip_nw = (int32_t)work.size() - first;
    }
    StripWork* d = const_cast<StripWork*>(s->args.strip_work);
    OC_TRY(reupload(s, &d, work));
    s->args.strip_work = d;
    s->args.n_strip_work = (int32_t)work.size();
    s->args.strip_item0 = 0;
    dfree(s, &s->args.strip_part);
    OC_TRY(dalloc(s, &s->args.strip_part, std::max<size_t>(work.size(), 1)));
    std::vector<int32_t> ids;
    s->strip_pos.assign((size_t)s->n_inst, -1);
    for (int32_t k = 0; k < s->n_inst; ++k)
        if (s->inst_host[(size_t)k].strip) {
            s->strip_pos[(size_t)k] = (int32_t)ids.size();
            ids.push_back(k);
        }
    int32_t* di = const_cast<int32_t*>(s->args.strip_ids);
    OC_TRY(reupload(s, &di, ids));
    s->args.strip_ids = di;
    s->args.n_strip_ids = (int32_t)ids.size();
    return OC_OK;
}

bool launch_config_valid(const oc_launch_config& c) {
    const int v = c.resident_vcta, t = c.resident_threads;
    const bool pow2 = v == 256 || v == 512 || v == 1024 || v == 2048;
    return c.resident_max_vertices >= 0 && pow2 && v <= kResidentMaxVcta && (t == 128 || t == 256 || t == 512) &&
           v <= kResidentVpt * t && (c.resident_fused == 0 || c.resident_fused == 1) &&
           (c.persist == 0 || c.persist == 1) && c.gather_variant >= 0 && c.gather_variant <= 6 &&
           (c.strip == 0 || c.strip == 1) && c.strip_rows >= 0 && c.strip_rows <= 64 &&
           (c.strip_variant == 2 || c.strip_variant == 3);
}

void drop_graphs(oc_solver* s) {
    if (s->exec) {
        cudaGraphExecDestroy(s->exec);
        s->exec = nullptr;
    }
    if (s->graph) {
        cudaGraphDestroy(s->graph);
        s->graph = nullptr;
    }
}

// The launch plan from the handle's cloths and its launch configuration: which cloths run
// resident (one cluster per cloth, the whole step on chip) and which streamed, resident
// cloths grouped by launch shape into buckets, the assembly tables (record gather,
// stencil, strip sweep), the update table, and the persistent CG of the streamed cloths.
// Run at create and again by oc_set_launch_config (an earlier plan's tables are freed).
oc_status plan_execution(oc_solver* s) {
    const oc_launch_config& cfg = s->cfg;
    StepArgs& a = s->args;
    a.gather_variant = cfg.gather_variant;
    a.strip_variant = cfg.strip_variant;
    s->resident_fused = cfg.resident_fused != 0;
    const int max_res = cfg.resident_max_vertices;
    s->resident.assign((size_t)s->n_inst, 0);
    for (oc_solver::Bucket& b : s->buckets) dfree(s, &b.d_ids);
    s->buckets.clear();
    std::vector<BlockInfo> streamed, asm_ref, cpl, upd, grid;
    std::map<std::tuple<int, int, int>, std::vector<int32_t>> groups;
    for (int32_t k = 0; k < s->n_inst; ++k) {
        InstParams& ip = s->inst_host[(size_t)k];
        const bool cpl_k = ip.coupled != 0;
        if (s->executor == OC_EXEC_RESIDENT && cpl_k)
            return fail(s, OC_ERR_UNSUPPORTED,
                        "instance " + std::to_string(k) + " is COUPLED: the resident executor runs REFERENCE cloths");
        int threads = 0, cluster = 0, vcta = 0;
        const bool want = !cpl_k && (s->executor == OC_EXEC_RESIDENT || s->executor == OC_EXEC_AUTO) &&
                          resident_shape(ip.nv, max_res, cfg.resident_vcta, cfg.resident_threads, &threads, &cluster,
                                         &vcta);
        if (s->executor == OC_EXEC_RESIDENT && !want)
            return fail(s, OC_ERR_UNSUPPORTED, "instance " + std::to_string(k) + " (" + std::to_string(ip.nv) +
                                                   " vertices) is too large for the resident executor");
        const BlockInfo* kb = s->h_blocks.data() + ip.blk0;
        ip.strip = 0;
        ip.resident = want ? 1 : 0;
        if (cpl_k) {
            cpl.insert(cpl.end(), kb, kb + ip.nblk);
            upd.insert(upd.end(), kb, kb + ip.nblk);
            continue;
        }
        if (!(want && s->resident_fused)) {
            ip.strip = strip_wanted(cfg, ip) ? 1 : 0;
            if (!ip.strip) {  // a cloth on the strip sweep is in no block table of the assembly
                auto& tab = ip.grid_cols > 0 ? grid : asm_ref;
                tab.insert(tab.end(), kb, kb + ip.nblk);
            }
        }
        if (want) {
            s->resident[(size_t)k] = 1;
            groups[std::make_tuple(threads, cluster, vcta)].push_back(k);
        } else {
            streamed.insert(streamed.end(), kb, kb + ip.nblk);
            upd.insert(upd.end(), kb, kb + ip.nblk);
        }
    }
    s->n_asm_blocks = (int32_t)asm_ref.size();
    OC_TRY(reupload(s, &s->d_asm_blocks, asm_ref));
    s->n_grid_blocks = (int32_t)grid.size();
    OC_TRY(reupload(s, &s->d_grid_blocks, grid));
    s->n_cpl_blocks = (int32_t)cpl.size();
    OC_TRY(reupload(s, &s->d_cpl_blocks, cpl));
    s->n_upd_blocks = (int32_t)upd.size();
    OC_TRY(reupload(s, &s->d_upd_blocks, upd));
    s->n_streamed_blocks = (int32_t)streamed.size();
    OC_TRY(reupload(s, &s->d_streamed_blocks, streamed));
    if (oc_status r = build_strip_work(s)) return r;
    std::vector<std::pair<std::tuple<int, int, int>, std::vector<int32_t>>> ordered(groups.begin(), groups.end());
    // Largest buckets first, so their clusters start before the small ones fill in.
    std::stable_sort(ordered.begin(), ordered.end(), [](const auto& x, const auto& y) {
        const double wx = (double)x.second.size() * std::get<1>(x.first) * std::get<2>(x.first);
        const double wy = (double)y.second.size() * std::get<1>(y.first) * std::get<2>(y.first);
        return wx > wy;
    });
    for (auto& kv : ordered) {
        oc_solver::Bucket b{};
        b.threads = std::get<0>(kv.first);
        b.cluster = std::get<1>(kv.first);
        b.vcta = std::get<2>(kv.first);
        b.n = (int)kv.second.size();
        OC_TRY(upload(s, &b.d_ids, kv.second));
        s->buckets.push_back(b);
    }
    OC_TRY(cudaMemcpy(const_cast<InstParams*>(a.inst), s->inst_host.data(), sizeof(InstParams) * s->inst_host.size(),
                      cudaMemcpyHostToDevice));
    if (!s->buckets.empty()) {
        OC_TRY(prepare_resident());
        const size_t naux = std::min<size_t>(s->buckets.size(), 8);
        if (!s->fork_ev) OC_TRY(cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming));
        while (s->aux.size() < naux) {
            cudaStream_t x = nullptr;
            cudaEvent_t e = nullptr;
            OC_TRY(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
            s->aux.push_back(x);
            OC_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            s->aux_done.push_back(e);
        }
    }
    // Persistent CG for the streamed REFERENCE cloths, any number of them: no COUPLED
    // cloth, a cooperative launch fits, and the configuration allows it.
    bool any_streamed = false, any_coupled = false;
    for (int32_t k = 0; k < s->n_inst; ++k) {
        any_coupled |= s->inst_host[(size_t)k].coupled != 0;
        any_streamed |= !s->resident[(size_t)k] && !s->inst_host[(size_t)k].coupled;
    }
    s->persist = false;
    const int pgrid = std::min(s->persist_per_sm * s->sm_count, std::max(1, s->n_streamed_blocks));
    if (cfg.persist && s->coop && s->persist_per_sm > 0 && any_streamed && !any_coupled &&
        (int64_t)s->n_streamed_blocks <= (int64_t)persist_max_entries_per_block() * pgrid) {
        s->persist = true;
        s->persist_grid = pgrid;
        if (oc_status r = alloc_persist_words(s)) return r;
    }
    s->strip_finish = false;
    for (int32_t k = 0; k < s->n_inst; ++k)
        if (s->inst_host[(size_t)k].strip && (s->resident[(size_t)k] || !s->persist)) s->strip_finish = true;
    drop_graphs(s);
    return OC_OK;
}

// After a cloth moved between the gathers (its grid_cols changed): the plan again, which
// rebuilds the assembly tables and the strip work from the current grid_cols.
oc_status rebuild_assembly_tables(oc_solver* s) { return plan_execution(s); }

// After new per-spring Ks / Kd: a grid cloth reads them from its stencil's parameter
// slots, so either every spring of each slot still shares one (Ks, Kd) and the slots take
// the new values, or the cloth moves to the CSR gather (which reads the records).  A cloth
// whose values fit again moves back.  Either move rebuilds the tables and the graph.
oc_status refit_stencils(oc_solver* s) {
    bool any = false;
    for (const int2& g : s->grid_shape) any |= g.x > 0;
    if (!any) return OC_OK;
    std::vector<int32_t> rowptr((size_t)s->nv + 1), sid((size_t)s->n_inc);
    std::vector<float> ks((size_t)s->ns), kd((size_t)s->ns);
    OC_TRY(cudaMemcpy(rowptr.data(), s->args.rowptr, sizeof(int32_t) * rowptr.size(), cudaMemcpyDeviceToHost));
    OC_TRY(cudaMemcpy(sid.data(), s->adj.inc_sid, sizeof(int32_t) * sid.size(), cudaMemcpyDeviceToHost));
    OC_TRY(cudaMemcpy(ks.data(), s->d_ks, sizeof(float) * ks.size(), cudaMemcpyDeviceToHost));
    OC_TRY(cudaMemcpy(kd.data(), s->d_kd, sizeof(float) * kd.size(), cudaMemcpyDeviceToHost));
    bool moved = false, slots_changed = false;
    for (int32_t k = 0; k < s->n_inst; ++k) {
        const int2 shape = s->grid_shape[(size_t)k];
        if (shape.x <= 0) continue;
        InstParams& ip = s->inst_host[(size_t)k];
        const int32_t* st = s->h_st_data.data() + ip.st_off;
        int32_t slot_ks[kStencilSlots], slot_kd[kStencilSlots];
        bool seen[kStencilSlots] = {false};
        bool fits = true;
        const int64_t vo = s->v_off[(size_t)k];
        for (int32_t l = 0; l < ip.nv && fits; ++l) {
            const int cl = stencil_class_1d(l / shape.x, shape.y) * 6 + stencil_class_1d(l % shape.x, shape.x);
            const int32_t e0 = st[cl], e1 = st[cl + 1], k0 = rowptr[(size_t)(vo + l)];
            for (int32_t e = e0; e < e1 && fits; ++e) {
                const int q = st[e] >> 7;
                const int32_t sp = sid[(size_t)(k0 + (e - e0))];
                int32_t bk, bd;
                std::memcpy(&bk, &ks[(size_t)sp], 4);
                std::memcpy(&bd, &kd[(size_t)sp], 4);
                if (!seen[q]) {
                    seen[q] = true;
                    slot_ks[q] = bk;
                    slot_kd[q] = bd;
                } else if (slot_ks[q] != bk || slot_kd[q] != bd) {
                    fits = false;
                }
            }
        }
        if (fits)
            for (int q = 0; q < kStencilSlots; ++q) {
                if (!seen[q]) continue;
                float4& f = s->h_st_param[(size_t)(ip.st_par + q)];
                int32_t ok_, od_;
                std::memcpy(&ok_, &f.y, 4);
                std::memcpy(&od_, &f.z, 4);
                if (ok_ != slot_ks[q] || od_ != slot_kd[q]) {
                    std::memcpy(&f.y, &slot_ks[q], 4);
                    std::memcpy(&f.z, &slot_kd[q], 4);
                    slots_changed = true;
                }
            }
        const int32_t cols = fits ? shape.x : 0;
        if (cols != ip.grid_cols) {
            ip.grid_cols = cols;
            ip.grid_rows = fits ? shape.y : 0;
            moved = true;
        }
    }
    if (slots_changed)
        OC_TRY(cudaMemcpy(const_cast<float4*>(s->args.st_param), s->h_st_param.data(),
                          sizeof(float4) * s->h_st_param.size(), cudaMemcpyHostToDevice));
    if (moved) {
        OC_TRY(cudaMemcpy(const_cast<InstParams*>(s->args.inst), s->inst_host.data(),
                          sizeof(InstParams) * s->inst_host.size(), cudaMemcpyHostToDevice));
        if (oc_status r = rebuild_assembly_tables(s)) return r;
        if (s->exec) {
            cudaGraphExecDestroy(s->exec);
            s->exec = nullptr;
        }
        if (s->graph) {
            cudaGraphDestroy(s->graph);
            s->graph = nullptr;
        }
    }
    return OC_OK;
}

}  // namespace

extern "C" {

void oc_default_options(oc_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->executor = OC_EXEC_AUTO;
    o->device = 0;
    o->stream = nullptr;
    o->use_graph = 1;
}

const char* oc_status_string(oc_status st) {
    switch (st) {
        case OC_OK: return "OC_OK";
        case OC_ERR_INVALID_ARGUMENT: return "OC_ERR_INVALID_ARGUMENT";
        case OC_ERR_BAD_INDEX: return "OC_ERR_BAD_INDEX";
        case OC_ERR_NON_FINITE: return "OC_ERR_NON_FINITE";
        case OC_ERR_DEGENERATE: return "OC_ERR_DEGENERATE";
        case OC_ERR_CUDA: return "OC_ERR_CUDA";
        case OC_ERR_OUT_OF_MEMORY: return "OC_ERR_OUT_OF_MEMORY";
        case OC_ERR_UNSUPPORTED: return "OC_ERR_UNSUPPORTED";
        case OC_ERR_DEVICE_TIMEOUT: return "OC_ERR_DEVICE_TIMEOUT";
        default: return "OC_ERR_UNKNOWN";
    }
}

const char* oc_last_error(const oc_solver* s) { return s ? s->err.c_str() : "NULL solver"; }

oc_status oc_create(const oc_cloth_desc* descs, int32_t n_instances, const oc_options* opts, oc_solver** out) {
    if (!out) return OC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    oc_options o;
    oc_default_options(&o);
    if (opts) o = *opts;
    if (o.executor < OC_EXEC_AUTO || o.executor > OC_EXEC_PLAIN) return OC_ERR_INVALID_ARGUMENT;
    if (o.vertices_per_thread < 0 || o.vertices_per_thread > 64 || o.block_threads < 0) return OC_ERR_INVALID_ARGUMENT;
    if (o.block_threads != 0 && o.block_threads != kernel_block_threads()) return OC_ERR_UNSUPPORTED;

    oc_solver* s = new (std::nothrow) oc_solver();
    if (!s) return OC_ERR_OUT_OF_MEMORY;
    // Block size: up to eight vertices per thread (2048-vertex blocks): fewer, longer-lived
    // blocks amortise the per-block reduction epilogue.  When the whole batch would fill
    // less than a few waves, the size is chosen so the block count is a multiple of the
    // resident capacity (4 blocks per SM), so every SM gets the same work: a 1M-vertex
    // cloth gets 608 blocks of 1728 vertices instead of 514 of 2048.
    int vpb = kernel_block_threads() * (o.vertices_per_thread > 0 ? o.vertices_per_thread : 8);
    if (o.vertices_per_thread <= 0) {
        int n_sm = 0;
        if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, o.device) != cudaSuccess || n_sm <= 0)
            n_sm = 152;
        int64_t total = 0;
        for (int32_t k = 0; k < n_instances; ++k) total += std::max(0, descs[k].n_vertices);
        const int64_t slots = 4LL * n_sm;
        if (total > 0 && total <= 3 * slots * (int64_t)vpb) {
            const int64_t waves = (total + slots * vpb - 1) / (slots * vpb);  // 1..3
            int64_t want = (total + waves * slots - 1) / (waves * slots);
            want = (want + 31) / 32 * 32;
            vpb = (int)std::min<int64_t>(std::max<int64_t>(want, 256), vpb);
        }
    }
    const int vpt = (vpb + kernel_block_threads() - 1) / kernel_block_threads();
    PackedHost P;
    oc_status st = pack_instances(descs, n_instances, vpb, &P, &s->err);
    if (st != OC_OK) {
        // The message is only reachable through a handle; print it for the caller.
        std::fprintf(stderr, "oc_create: %s\n", s->err.c_str());
        delete s;
        return st;
    }
    // OC_STENCIL=0 keeps grid cloths on the CSR gather (a diagnostic switch: both paths
    // give the same bits).
    if (const char* e = std::getenv("OC_STENCIL"))
        if (std::atoi(e) == 0)
            for (InstParams& ip : P.inst) ip.grid_cols = ip.grid_rows = 0;
    build_strip_tables(&P);
    auto bail = [&](oc_status code) {
        std::fprintf(stderr, "oc_create: %s\n", s->err.c_str());
        release(s);
        delete s;
        return code;
    };
#define OC_CREATE_TRY(call)                                           \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return bail(fail_cuda(s, e_, #call));  \
    } while (0)

    s->device = o.device;
    s->executor = o.executor;
    if (const char* rf = std::getenv("OC_RESIDENT_FUSED")) s->resident_fused = std::atoi(rf) != 0;
    s->use_graph = o.use_graph != 0;
    s->n_inst = P.n_inst;
    s->nv = P.nv;
    s->ns = P.ns;
    s->n_inc = (int64_t)P.inc.size();
    s->v_off = P.v_off;
    s->inst_host = P.inst;
    s->ns_inst.resize(P.n_inst);
    for (int32_t k = 0; k < P.n_inst; ++k) s->ns_inst[k] = P.s_off[k + 1] - P.s_off[k];
    s->n_blocks = (int32_t)P.blocks.size();
    s->vertices_per_block = P.vertices_per_block;
    OC_CREATE_TRY(cudaSetDevice(o.device));
    OC_CREATE_TRY(prepare_kernels());
    if (o.stream) {
        s->stream = static_cast<cudaStream_t>(o.stream);
    } else {
        OC_CREATE_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }

    StepArgs& a = s->args;
    OC_CREATE_TRY(upload(s, &a.X, P.X0));
    OC_CREATE_TRY(upload(s, &a.V, P.V0));
    float4* fext = nullptr;
    if (!P.fext.empty()) OC_CREATE_TRY(upload(s, &fext, P.fext));
    a.fext = fext;
    int32_t* rowptr = nullptr;
    int4* inc = nullptr;
    int2* own_ends = nullptr;
    float4* own_par = nullptr;
    OC_CREATE_TRY(upload(s, &rowptr, P.rowptr));
    OC_CREATE_TRY(upload(s, &inc, P.inc));
    OC_CREATE_TRY(upload(s, &own_ends, P.own_ends));
    OC_CREATE_TRY(upload(s, &own_par, P.own_par));
    a.rowptr = rowptr;
    a.inc = inc;
    {
        s->h_st_data = P.st_data;
        s->h_st_param = P.st_param;
        s->grid_shape.resize((size_t)P.n_inst);
        for (int32_t k = 0; k < P.n_inst; ++k) s->grid_shape[(size_t)k] = make_int2(P.inst[k].grid_cols, P.inst[k].grid_rows);
        int32_t* d_st = nullptr;
        OC_CREATE_TRY(upload(s, &d_st, P.st_data));
        a.st_data = d_st;
        float4* d_sp = nullptr;
        OC_CREATE_TRY(upload(s, &d_sp, P.st_param));
        a.st_param = d_sp;
        if (P.any_st_rest) {
            std::vector<float> rest(P.inc.size());
            for (size_t k = 0; k < P.inc.size(); ++k) std::memcpy(&rest[k], &P.inc[k].y, 4);
            float* d_rest = nullptr;
            OC_CREATE_TRY(upload(s, &d_rest, rest));
            a.rest_inc = d_rest;
        }
        if (!P.strip_slot.empty()) {
            uint32_t* d_ss = nullptr;
            OC_CREATE_TRY(upload(s, &d_ss, P.strip_slot));
            a.strip_slot = d_ss;
            if (!P.strip_rest.empty()) {
                float* d_sr = nullptr;
                OC_CREATE_TRY(upload(s, &d_sr, P.strip_rest));
                a.strip_rest = d_sr;
            }
        }
    }
    a.own_ends = own_ends;
    a.own_par = own_par;
    const size_t stride = (size_t)((P.nv + 63) / 64) * 64;
    s->stride = stride;
    {
        int32_t *inc_sid = nullptr, *own_sid = nullptr, *own_rowptr = nullptr, *own_ent = nullptr;
        OC_CREATE_TRY(upload(s, &inc_sid, P.inc_sid));
        OC_CREATE_TRY(upload(s, &own_sid, P.own_sid));
        OC_CREATE_TRY(upload(s, &own_rowptr, P.own_rowptr));
        OC_CREATE_TRY(upload(s, &own_ent, P.own_ent));
        s->adj.inc_sid = inc_sid;
        s->adj.own_sid = own_sid;
        s->adj.own_rowptr = own_rowptr;
        s->adj.own_ent = own_ent;
        if (const char* e = std::getenv("OC_ADJ_SPRINGS_VARIANT")) s->adj.springs_variant = std::atoi(e);
        if (const char* e = std::getenv("OC_ADJ_VERTEX_VARIANT")) s->adj.vertex_variant = std::atoi(e);
    }
    float* planes = nullptr;
    OC_CREATE_TRY(dalloc(s, &planes, 15 * stride));
    OC_CREATE_TRY(cudaMemset(planes, 0, 15 * stride * sizeof(float)));
    for (int k = 0; k < 6; ++k) a.A[k] = planes + k * stride;
    for (int k = 0; k < 3; ++k) {
        a.x[k] = planes + (6 + k) * stride;
        a.r[k] = planes + (9 + k) * stride;
        a.d[k] = planes + (12 + k) * stride;
    }
    OC_CREATE_TRY(dalloc(s, &a.partials, 2 * P.blocks.size()));
    a.partials_b = a.partials + P.blocks.size();
    InstParams* inst = nullptr;
    OC_CREATE_TRY(upload(s, &inst, P.inst));
    a.inst = inst;
    OC_CREATE_TRY(dalloc(s, &a.state, (size_t)P.n_inst));
    OC_CREATE_TRY(cudaMemset(a.state, 0, sizeof(InstState) * P.n_inst));
    BlockInfo* blocks = nullptr;
    OC_CREATE_TRY(upload(s, &blocks, P.blocks));
    a.blocks = blocks;
    for (const InstParams& ip : P.inst) s->any_passes = s->any_passes || ip.passes != 0;
    s->any_provot = P.any_provot;
    s->any_coupled = P.any_coupled;
    if (P.any_coupled) {
        // Slot-major per-incidence layout: slices of 32 vertices, each as wide as its
        // largest degree (padding slots hold the vertex itself and are never read).
        const int64_t n_slices = (P.nv + 31) / 32;
        std::vector<int64_t> slice((size_t)n_slices + 1, 0);
        for (int64_t sl = 0; sl < n_slices; ++sl) {
            int32_t width = 0;
            for (int64_t g = 32 * sl; g < std::min<int64_t>(P.nv, 32 * sl + 32); ++g)
                width = std::max(width, P.rowptr[g + 1] - P.rowptr[g]);
            slice[(size_t)sl + 1] = slice[(size_t)sl] + 32 * (int64_t)width;
        }
        const size_t slots = std::max<size_t>((size_t)slice[(size_t)n_slices], 1);
        std::vector<int32_t> other(slots, 0);
        for (int64_t g = 0; g < P.nv; ++g) {
            const int64_t base = slice[(size_t)(g >> 5)] + (g & 31);
            const int32_t deg = P.rowptr[g + 1] - P.rowptr[g];
            for (int32_t e = 0; e < deg; ++e) other[(size_t)(base + 32 * e)] = P.inc[P.rowptr[g] + e].x & 0x7fffffff;
        }
        int64_t* d_slice = nullptr;
        OC_CREATE_TRY(upload(s, &d_slice, slice));
        a.cpl_slice = d_slice;
        int32_t* d_other = nullptr;
        OC_CREATE_TRY(upload(s, &d_other, other));
        a.cpl_o = d_other;
        float* cplanes = nullptr;
        OC_CREATE_TRY(dalloc(s, &cplanes, 5 * slots));
        for (int k = 0; k < 5; ++k) a.cpl_c[k] = cplanes + (size_t)k * slots;
        float* vplanes = nullptr;
        OC_CREATE_TRY(dalloc(s, &vplanes, 4 * stride));
        OC_CREATE_TRY(cudaMemset(vplanes, 0, 4 * stride * sizeof(float)));
        a.cpl_m = vplanes;
        for (int k = 0; k < 3; ++k) a.q[k] = vplanes + (1 + k) * stride;
        OC_CREATE_TRY(dalloc(s, &a.cpl_z, (size_t)P.nv));
        OC_CREATE_TRY(dalloc(s, &a.cpl_d, (size_t)P.nv));
        OC_CREATE_TRY(cudaMemset(a.cpl_z, 0, sizeof(float4) * (size_t)P.nv));
        OC_CREATE_TRY(cudaMemset(a.cpl_d, 0, sizeof(float4) * (size_t)P.nv));
    }
    {
        std::vector<uint8_t> pins((size_t)P.nv);
        for (int64_t g = 0; g < P.nv; ++g) pins[g] = P.V0[g].w != 0.0f ? 1 : 0;
        uint8_t* d_pins = nullptr;
        OC_CREATE_TRY(upload(s, &d_pins, pins));
        a.pinflag = d_pins;
    }

    // The launch configuration: the options and the environment's diagnostic switches
    // over the measured defaults, then the plan (resident buckets, block tables, strip
    // work, persistent CG).
    {
        oc_launch_config& c = s->cfg;
        c.resident_max_vertices = o.resident_max_vertices > 0 ? o.resident_max_vertices
                                                              : kResidentMaxCluster * kResidentDefaultVcta;
        c.resident_vcta = kResidentDefaultVcta;
        c.resident_threads = 256;
        if (const char* e = std::getenv("OC_RESIDENT_SHAPE")) {
            int v = 0, t = 0;
            if (std::sscanf(e, "%d:%d", &v, &t) == 2) {
                c.resident_vcta = v;
                c.resident_threads = t;
            }
        }
        c.resident_fused = s->resident_fused ? 1 : 0;
        const char* pe = std::getenv("OC_PERSIST");
        c.persist = (pe && std::atoi(pe) == 0) ? 0 : 1;
        const char* gv = std::getenv("OC_GATHER_VARIANT");
        c.gather_variant = gv ? std::atoi(gv) : 6;
        // The strip sweep is off by default: on GB300 it measured level with the stencil
        // gather on the 1M-vertex cloth (its delta0 reduction costs what its single spring
        // evaluations save) and slower on the 4096-cloth batch; the autotuner tries it.
        const char* se = std::getenv("OC_STRIP");
        c.strip = (se && std::atoi(se) != 0) ? 1 : 0;
        const char* sr = std::getenv("OC_STRIP_ROWS");
        c.strip_rows = sr ? std::max(0, std::atoi(sr)) : 0;
        const char* sv = std::getenv("OC_STRIP_VARIANT");
        c.strip_variant = (sv && std::atoi(sv) == 3) ? 3 : 2;
        if (!launch_config_valid(c)) {
            s->err = "oc_create: invalid launch configuration from the environment";
            return bail(OC_ERR_INVALID_ARGUMENT);
        }
        OC_CREATE_TRY(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device));
        int coop = 0;
        OC_CREATE_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->device));
        s->coop = coop != 0;
        s->persist_per_sm = s->executor != OC_EXEC_PLAIN ? persist_blocks_per_sm() : 0;
        s->h_blocks = P.blocks;
        if (oc_status r = plan_execution(s)) return bail(r);
    }
    {
        const char* pe = std::getenv("OC_PERSIST");
        const bool allowed = !(pe && std::atoi(pe) == 0) && s->executor != OC_EXEC_PLAIN;
        const int per_sm = allowed ? s->persist_per_sm : 0;
        const int n_sm = s->sm_count;
        const int coop = s->coop ? 1 : 0;
        // The adjoint solve runs every cloth's CG over the full block table: one
        // cooperative launch without the update, any number of cloths.
        const int adj_grid = std::min(per_sm * n_sm, std::max(1, s->n_blocks));
        if (allowed && coop && per_sm > 0 && !P.any_coupled &&
            (int64_t)s->n_blocks <= (int64_t)persist_max_entries_per_block() * adj_grid) {
            s->adj_persist = true;
            s->adj_persist_grid = adj_grid;
            if (oc_status r = alloc_persist_words(s)) return bail(r);
        }
    }
    OC_CREATE_TRY(dalloc(s, &a.unconverged, 1));
    OC_CREATE_TRY(dalloc(s, &a.grid_ticket, 1));
    OC_CREATE_TRY(dalloc(s, &a.loop_count, 1));
    OC_CREATE_TRY(cudaMemset(a.loop_count, 0, sizeof(unsigned long long)));
    OC_CREATE_TRY(cudaMallocHost(&s->h_loop, sizeof(unsigned long long)));
    OC_CREATE_TRY(cudaMemset(a.unconverged, 0, sizeof(int32_t)));
    OC_CREATE_TRY(cudaMemset(a.grid_ticket, 0, sizeof(uint32_t)));
    OC_CREATE_TRY(dalloc(s, &s->stage, 3 * stage_stride(P.nv)));
    OC_CREATE_TRY(dalloc(s, &s->d_err, 1));
    OC_CREATE_TRY(cudaMallocHost(&s->h_state, sizeof(InstState) * P.n_inst));
    OC_CREATE_TRY(cudaMallocHost(&s->h_scalar, sizeof(int32_t)));
    a.vpt = vpt;
    a.barrier_polls = kDefaultBarrierPolls;
    a.withhold_block = -1;
    OC_CREATE_TRY(cudaDeviceSynchronize());
#undef OC_CREATE_TRY
    *out = s;
    return OC_OK;
}

void oc_destroy(oc_solver* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    release(s);
    delete s;
}

oc_status oc_get_counts(const oc_solver* s, int64_t* total_vertices, int64_t* total_springs, int32_t* n_instances) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    if (total_vertices) *total_vertices = s->nv;
    if (total_springs) *total_springs = s->ns;
    if (n_instances) *n_instances = s->n_inst;
    return OC_OK;
}

oc_status oc_get_vertex_offsets(const oc_solver* s, int64_t* offsets) {
    if (!valid_solver(s) || !offsets) return OC_ERR_INVALID_ARGUMENT;
    std::memcpy(offsets, s->v_off.data(), sizeof(int64_t) * s->v_off.size());
    return OC_OK;
}

oc_status oc_set_state_device(oc_solver* s, const float* X, const float* V, const float* dV) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaMemsetAsync(s->d_err, 0, sizeof(int32_t), s->stream));
    OC_TRY(launch_state_in(s->args, X, V, dV, s->nv, s->d_err, s->stream));
    return OC_OK;
}

oc_status oc_get_state_device(oc_solver* s, float* X, float* V, float* dV) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(launch_state_out(s->args, X, V, dV, s->nv, s->stream));
    return OC_OK;
}

namespace {

// Copies the caller's host triples into the staging buffer and checks them on the device,
// writing nothing into the state; returns OC_ERR_NON_FINITE when one holds a NaN or Inf.
// The staged arrays are left in *sx, *sv, *sd (NULL where the caller passed NULL) for a
// commit with launch_state_in.
oc_status stage_checked(oc_solver* s, const float* X, const float* V, const float* dV, float** sx, float** sv,
                        float** sd, const char* who) {
    const size_t n3 = 3 * (size_t)s->nv;
    const size_t ps = stage_stride(s->nv);
    *sx = X ? s->stage : nullptr;
    *sv = V ? s->stage + ps : nullptr;
    *sd = dV ? s->stage + 2 * ps : nullptr;
    if (X) OC_TRY(cudaMemcpyAsync(*sx, X, n3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    if (V) OC_TRY(cudaMemcpyAsync(*sv, V, n3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    if (dV) OC_TRY(cudaMemcpyAsync(*sd, dV, n3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    OC_TRY(cudaMemsetAsync(s->d_err, 0, sizeof(int32_t), s->stream));
    OC_TRY(launch_state_check(*sx, *sv, *sd, s->nv, s->d_err, s->stream));
    OC_TRY(cudaMemcpyAsync(s->h_scalar, s->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    if (*s->h_scalar != 0)
        return fail(s, OC_ERR_NON_FINITE, std::string(who) + ": non-finite value in the input state (nothing changed)");
    return OC_OK;
}

}  // namespace

oc_status oc_set_state(oc_solver* s, const float* X, const float* V, const float* dV) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    float *sx, *sv, *sd;
    if (oc_status st = stage_checked(s, X, V, dV, &sx, &sv, &sd, "oc_set_state")) return st;
    OC_TRY(launch_state_in(s->args, sx, sv, sd, s->nv, s->d_err, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    return OC_OK;
}

oc_status oc_get_state(oc_solver* s, float* X, float* V, float* dV) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    const size_t n3 = 3 * (size_t)s->nv;
    const size_t ps = stage_stride(s->nv);
    float* sx = X ? s->stage : nullptr;
    float* sv = V ? s->stage + ps : nullptr;
    float* sd = dV ? s->stage + 2 * ps : nullptr;
    OC_TRY(launch_state_out(s->args, sx, sv, sd, s->nv, s->stream));
    if (X) OC_TRY(cudaMemcpyAsync(X, sx, n3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    if (V) OC_TRY(cudaMemcpyAsync(V, sv, n3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    if (dV) OC_TRY(cudaMemcpyAsync(dV, sd, n3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
}

oc_status oc_step_host(oc_solver* s, float dt, int32_t n_steps, float* X, float* V) {
    if (!valid_solver(s) || n_steps < 0 || !std::isfinite(dt)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    const size_t n3 = 3 * (size_t)s->nv;
    // The input is staged and checked before anything is committed: a NaN or Inf leaves
    // the device state and the caller's arrays as they were.
    float *sx, *sv, *sd;
    if (oc_status st = stage_checked(s, X, V, nullptr, &sx, &sv, &sd, "oc_step_host")) return st;
    OC_TRY(launch_state_in(s->args, sx, sv, nullptr, s->nv, s->d_err, s->stream));
    if (oc_status st = oc_step(s, dt, n_steps)) return st;
    OC_TRY(launch_state_out(s->args, sx, sv, nullptr, s->nv, s->stream));
    if (X) OC_TRY(cudaMemcpyAsync(X, sx, n3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    if (V) OC_TRY(cudaMemcpyAsync(V, sv, n3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
}

oc_status oc_step(oc_solver* s, float dt, int32_t n_steps) {
    if (!valid_solver(s) || n_steps < 0 || !std::isfinite(dt)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    if (s->executor == OC_EXEC_PLAIN) {
        for (int32_t i = 0; i < n_steps; ++i) {
            oc_status st = step_host_driven(s, dt, true, nullptr);
            if (st != OC_OK) return st;
        }
        return OC_OK;
    }
    if (!s->use_graph) {
        for (int32_t i = 0; i < n_steps; ++i) {
            oc_status st = step_host_driven(s, dt, false, nullptr);
            if (st != OC_OK) return st;
        }
        return OC_OK;
    }
    if (!s->exec || s->graph_dt != dt) {
        oc_status st = build_graph(s, dt);
        if (st != OC_OK) return st;
    }
    for (int32_t i = 0; i < n_steps; ++i) OC_TRY(cudaGraphLaunch(s->exec, s->stream));
    // assemblies, the persistent CG (which includes the update) or the update kernel,
    // the resident launches and the Provot pass; the WHILE loop's launches are counted on
    // the device (loop_count).
    const int64_t per_step = (s->n_asm_blocks > 0 ? 1 : 0) + (s->n_grid_blocks > 0 ? 1 : 0) +
                             (s->args.n_strip_work > 0 ? (s->strip_finish ? 2 : 1) : 0) + (s->n_cpl_blocks > 0 ? 1 : 0) +
                             (s->persist ? 1 : (s->n_upd_blocks > 0 ? 1 : 0)) + (int64_t)s->buckets.size() +
                             (s->any_provot ? 1 : 0);
    s->host_launches += per_step * (int64_t)n_steps;
    return OC_OK;
}

oc_status oc_set_passes(oc_solver* s, int32_t instance, int32_t passes) {
    if (!valid_solver(s) || instance < -1 || instance >= s->n_inst ||
        (passes & ~(OC_PASS_ELLIPSOID | OC_PASS_PROVOT)))
        return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    const int32_t k0 = instance < 0 ? 0 : instance, k1 = instance < 0 ? s->n_inst : instance + 1;
    for (int32_t k = k0; k < k1; ++k) {
        const InstParams& ip = s->inst_host[k];
        if (passes & OC_PASS_ELLIPSOID)
            for (int i = 0; i < 16; ++i)
                if (!std::isfinite(ip.ellipsoid[i]) || !std::isfinite(ip.ellipsoid_inv[i]))
                    return fail(s, OC_ERR_NON_FINITE, "oc_set_passes: ellipsoid matrix not finite");
    }
    for (int32_t k = k0; k < k1; ++k) s->inst_host[k].passes = passes;
    OC_TRY(cudaStreamSynchronize(s->stream));  // no step in flight reads the parameters
    OC_TRY(cudaMemcpy(const_cast<InstParams*>(s->args.inst), s->inst_host.data(), sizeof(InstParams) * s->n_inst,
                      cudaMemcpyHostToDevice));
    s->any_passes = s->any_provot = false;
    for (const InstParams& ip : s->inst_host) {
        s->any_passes = s->any_passes || ip.passes != 0;
        s->any_provot = s->any_provot || (ip.passes & OC_PASS_PROVOT);
    }
    if (s->exec) {  // the graph's node set depends on the passes
        cudaGraphExecDestroy(s->exec);
        s->exec = nullptr;
    }
    return OC_OK;
}

oc_status oc_apply_passes(oc_solver* s, int32_t passes) {
    if (!valid_solver(s) || (passes & ~(OC_PASS_ELLIPSOID | OC_PASS_PROVOT))) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    StepArgs a = s->args;
    a.blk_base = 0;
    if (passes & OC_PASS_ELLIPSOID) {
        a.only_passes = OC_PASS_ELLIPSOID;
        OC_TRY(launch_kernel(K_ELLIPSOID, a, s->n_blocks, s->stream));
        s->host_launches += 1;
    }
    if (passes & OC_PASS_PROVOT) {
        a.only_passes = OC_PASS_PROVOT;
        OC_TRY(launch_kernel(K_PROVOT, a, s->n_blocks, s->stream));
        s->host_launches += 1;
    }
    return OC_OK;
}

oc_status oc_pick_vertex(oc_solver* s, int32_t instance, const float point[3], double radius, int32_t* index) {
    if (!valid_solver(s) || !point || !index || instance < 0 || instance >= s->n_inst || !std::isfinite(radius))
        return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaMemsetAsync(s->d_err, 0x7f, sizeof(int32_t), s->stream));  // 0x7f7f7f7f: "none"
    OC_TRY(launch_pick(s->args.X, s->v_off[instance], s->v_off[instance + 1] - s->v_off[instance], point, radius,
                       s->d_err, s->stream));
    OC_TRY(cudaMemcpyAsync(s->h_scalar, s->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    *index = *s->h_scalar == 0x7f7f7f7f ? -1 : *s->h_scalar;
    return OC_OK;
}

oc_status oc_drag_vertex(oc_solver* s, int32_t instance, int32_t index, const float delta[3]) {
    if (!valid_solver(s) || !delta || instance < 0 || instance >= s->n_inst) return OC_ERR_INVALID_ARGUMENT;
    if (index < 0 || index >= s->v_off[instance + 1] - s->v_off[instance])
        return fail(s, OC_ERR_BAD_INDEX, "oc_drag_vertex: index outside the cloth");
    if (!std::isfinite(delta[0]) || !std::isfinite(delta[1]) || !std::isfinite(delta[2]))
        return fail(s, OC_ERR_NON_FINITE, "oc_drag_vertex: delta not finite");
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(launch_drag(s->args.X, s->args.V, s->v_off[instance] + index, delta, s->stream));
    return OC_OK;
}

oc_status oc_set_vertices(oc_solver* s, int32_t n, const int64_t* indices, const float* X, const float* V) {
    if (!valid_solver(s) || n < 0 || (n > 0 && !indices)) return OC_ERR_INVALID_ARGUMENT;
    if ((int64_t)n > s->nv) return fail(s, OC_ERR_INVALID_ARGUMENT, "oc_set_vertices: more entries than vertices");
    for (int32_t k = 0; k < n; ++k)
        if (indices[k] < 0 || indices[k] >= s->nv) return fail(s, OC_ERR_BAD_INDEX, "oc_set_vertices: bad index");
    {
        std::vector<int64_t> sorted(indices, indices + n);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
            return fail(s, OC_ERR_INVALID_ARGUMENT, "oc_set_vertices: an index appears twice");
    }
    for (const float* p : {X, V})
        if (p)
            for (size_t k = 0; k < 3 * (size_t)n; ++k)
                if (!std::isfinite(p[k])) return fail(s, OC_ERR_NON_FINITE, "oc_set_vertices: value not finite");
    if (n == 0 || (!X && !V)) return OC_OK;
    OC_TRY(cudaSetDevice(s->device));
    // Staging: indices (2 floats each), then X, then V, within the 9 x n_vertices buffer.
    int64_t* d_idx = reinterpret_cast<int64_t*>(s->stage);
    float* d_X = s->stage + 2 * (size_t)n;
    float* d_V = d_X + 3 * (size_t)n;
    OC_TRY(cudaMemcpyAsync(d_idx, indices, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s->stream));
    if (X) OC_TRY(cudaMemcpyAsync(d_X, X, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s->stream));
    if (V) OC_TRY(cudaMemcpyAsync(d_V, V, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s->stream));
    OC_TRY(launch_set_vertices(s->args.X, s->args.V, d_idx, X ? d_X : nullptr, V ? d_V : nullptr, n, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));  // the host arrays may be reused on return
    return OC_OK;
}

oc_status oc_set_pins(oc_solver* s, int32_t instance, const int32_t* pins, int32_t n_pins) {
    if (!valid_solver(s) || instance < 0 || instance >= s->n_inst || n_pins < 0 || (n_pins > 0 && !pins))
        return OC_ERR_INVALID_ARGUMENT;
    const int64_t nv = s->v_off[instance + 1] - s->v_off[instance];
    if (n_pins > nv) return fail(s, OC_ERR_INVALID_ARGUMENT, "oc_set_pins: more pins than vertices");
    for (int32_t k = 0; k < n_pins; ++k)
        if (pins[k] < 0 || pins[k] >= nv) return fail(s, OC_ERR_BAD_INDEX, "oc_set_pins: pin outside the cloth");
    OC_TRY(cudaSetDevice(s->device));
    int32_t* d_pins = reinterpret_cast<int32_t*>(s->stage);
    if (n_pins > 0)
        OC_TRY(cudaMemcpyAsync(d_pins, pins, sizeof(int32_t) * n_pins, cudaMemcpyHostToDevice, s->stream));
    OC_TRY(launch_set_pins(s->args.V, const_cast<uint8_t*>(s->args.pinflag), s->v_off[instance], nv, d_pins, n_pins,
                           s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    s->tape.valid = false;
    return OC_OK;
}

oc_status oc_synchronize(oc_solver* s) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
}

oc_status oc_get_stats(oc_solver* s, int32_t* cg_iters, double* rel_residual, uint32_t* flags) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaMemcpyAsync(s->h_state, s->args.state, sizeof(InstState) * s->n_inst, cudaMemcpyDeviceToHost,
                           s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    if (oc_status e = check_device_error(s)) return e;
    for (int32_t k = 0; k < s->n_inst; ++k) {
        const InstState& st = s->h_state[k];
        if (cg_iters) cg_iters[k] = st.iter;
        if (rel_residual) rel_residual[k] = st.delta0 > 0.0 ? std::sqrt(st.delta_new / st.delta0) : 0.0;
        if (flags) flags[k] = st.flags;
    }
    return OC_OK;
}

oc_status oc_get_launch_count(oc_solver* s, int64_t* kernels_launched) {
    if (!valid_solver(s) || !kernels_launched) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaMemcpyAsync(s->h_loop, s->args.loop_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    *kernels_launched = s->host_launches + 2 * (int64_t)*s->h_loop;
    return OC_OK;
}

oc_status oc_compute_forces(oc_solver* s, float* F) {
    if (!valid_solver(s) || !F) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    StepArgs a = s->args;
    a.dbg_F = s->stage;
    a.blk_base = 0;
    OC_TRY(launch_kernel(K_FORCES, a, s->n_blocks, s->stream));
    OC_TRY(cudaMemcpyAsync(F, s->stage, 3 * (size_t)s->nv * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    return OC_OK;
}

oc_status oc_assemble(oc_solver* s, float dt, float* A9, float* b) {
    if (!valid_solver(s) || !A9 || !b || !std::isfinite(dt)) return OC_ERR_INVALID_ARGUMENT;
    if (s->any_coupled)
        return fail(s, OC_ERR_UNSUPPORTED, "oc_assemble: a COUPLED cloth's system is not block-diagonal");
    OC_TRY(cudaSetDevice(s->device));
    float* dA9 = nullptr;
    OC_TRY(cudaMallocAsync(&dA9, 9 * (size_t)s->nv * sizeof(float), s->stream));
    StepArgs a = s->args;
    a.dt = dt;
    a.blk_base = 0;
    a.use_cond = 0;
    a.dbg_A9 = dA9;
    a.dbg_b = s->stage;
    cudaError_t e = launch_kernel(K_ASSEMBLE, a, s->n_blocks, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(A9, dA9, 9 * (size_t)s->nv * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b, s->stage, 3 * (size_t)s->nv * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
    // The assembly pass also primed the CG loop; leave no instance marked running.
    if (e == cudaSuccess) e = cudaMemsetAsync(s->args.unconverged, 0, sizeof(int32_t), s->stream);
    cudaFreeAsync(dA9, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail_cuda(s, e, "oc_assemble");
    return OC_OK;
}

oc_status oc_profile_steps(oc_solver* s, float dt, int32_t n_steps, int32_t max_kernels, char* names,
                           double* ms_total, int64_t* launches, double* algorithmic_bytes, int32_t* n_kernels) {
    if (!valid_solver(s) || n_steps < 0 || max_kernels < 0 || !std::isfinite(dt)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    KernelTimer t;
    OC_TRY(cudaEventCreate(&t.ev[0]));
    OC_TRY(cudaEventCreate(&t.ev[1]));
    oc_status st = OC_OK;
    for (int32_t i = 0; i < n_steps && st == OC_OK; ++i)
        st = step_host_driven(s, dt, s->executor == OC_EXEC_PLAIN, &t);
    cudaEventDestroy(t.ev[0]);
    cudaEventDestroy(t.ev[1]);
    if (st != OC_OK) return st;
    const KernelKind kinds[] = {K_ASSEMBLE, K_ASSEMBLE_GRID, K_ASSEMBLE_STRIP, K_ASSEMBLE_FINISH, K_CG_DIR,
                                K_CG_UPDATE, K_INTEGRATE, K_CG_PERSIST, K_RESIDENT, K_PROVOT,
                                K_CPL_ASSEMBLE, K_CPL_DIR, K_CPL_UPDATE};
    int32_t n = 0;
    for (KernelKind k : kinds) {
        if (n >= max_kernels) break;
        if (k == K_PROVOT && !s->any_provot) continue;
        if ((k == K_CPL_ASSEMBLE || k == K_CPL_DIR || k == K_CPL_UPDATE) && !s->any_coupled) continue;
        if (k == K_ASSEMBLE_GRID && s->n_grid_blocks == 0) continue;
        if (k == K_CG_PERSIST && !s->persist) continue;
        if ((k == K_CG_DIR || k == K_CG_UPDATE || k == K_INTEGRATE) && s->persist) continue;
        if ((k == K_ASSEMBLE_STRIP || k == K_ASSEMBLE_FINISH) && s->args.n_strip_work == 0) continue;
        if (k == K_ASSEMBLE_FINISH && !s->strip_finish) continue;
        if (k == K_ASSEMBLE && s->n_asm_blocks == 0 && (s->n_grid_blocks > 0 || s->args.n_strip_work > 0)) continue;
        if (names) {
            std::memset(names + 32 * n, 0, 32);
            std::strncpy(names + 32 * n, kernel_name(k), 31);
        }
        if (ms_total) ms_total[n] = t.ms[k];
        if (launches) launches[n] = t.launches[k];
        if (algorithmic_bytes) algorithmic_bytes[n] = t.bytes[k];
        ++n;
    }
    if (n_kernels) *n_kernels = n;
    return OC_OK;
}

oc_status oc_set_spring_params(oc_solver* s, const float* ks, const float* kd) {
    if (!valid_solver(s) || (!ks && !kd)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    const size_t ns = (size_t)s->ns;
    for (size_t k = 0; k < ns; ++k)
        if ((ks && !std::isfinite(ks[k])) || (kd && !std::isfinite(kd[k])))
            return fail(s, OC_ERR_NON_FINITE, "oc_set_spring_params: non-finite parameter");
    if (!s->d_ks) {
        OC_TRY(dalloc(s, &s->d_ks, ns));
        OC_TRY(dalloc(s, &s->d_kd, ns));
        // Current values, read back from the records through the spring ids.
        std::vector<int4> rec(s->n_inc);
        std::vector<int32_t> sid(s->n_inc);
        OC_TRY(cudaMemcpy(rec.data(), s->args.inc, sizeof(int4) * s->n_inc, cudaMemcpyDeviceToHost));
        OC_TRY(cudaMemcpy(sid.data(), s->adj.inc_sid, sizeof(int32_t) * s->n_inc, cudaMemcpyDeviceToHost));
        std::vector<float> hk(ns), hd(ns);
        for (int64_t k = 0; k < s->n_inc; ++k) {
            std::memcpy(&hk[sid[k]], &rec[k].z, 4);
            std::memcpy(&hd[sid[k]], &rec[k].w, 4);
        }
        OC_TRY(cudaMemcpy(s->d_ks, hk.data(), sizeof(float) * ns, cudaMemcpyHostToDevice));
        OC_TRY(cudaMemcpy(s->d_kd, hd.data(), sizeof(float) * ns, cudaMemcpyHostToDevice));
    }
    if (ks) OC_TRY(cudaMemcpyAsync(s->d_ks, ks, sizeof(float) * ns, cudaMemcpyHostToDevice, s->stream));
    if (kd) OC_TRY(cudaMemcpyAsync(s->d_kd, kd, sizeof(float) * ns, cudaMemcpyHostToDevice, s->stream));
    OC_TRY(launch_set_spring_params(s->args, s->adj, s->d_ks, s->d_kd, s->n_inc, s->nv, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    s->tape.valid = false;
    return refit_stencils(s);
}

oc_status oc_set_ext_force(oc_solver* s, const float* ext) {
    if (!valid_solver(s) || !ext) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    const size_t n3 = 3 * (size_t)s->nv;
    for (size_t k = 0; k < n3; ++k)
        if (!std::isfinite(ext[k])) return fail(s, OC_ERR_NON_FINITE, "oc_set_ext_force: non-finite value");
    std::vector<float4> f(s->nv);
    for (int64_t g = 0; g < s->nv; ++g) f[g] = make_float4(ext[3 * g], ext[3 * g + 1], ext[3 * g + 2], 0.f);
    if (!s->args.fext) {
        float4* p = nullptr;
        OC_TRY(dalloc(s, &p, (size_t)s->nv));
        s->args.fext = p;
    }
    OC_TRY(cudaMemcpy(const_cast<float4*>(s->args.fext), f.data(), sizeof(float4) * s->nv, cudaMemcpyHostToDevice));
    bool changed = false;
    for (auto& ip : s->inst_host) {
        changed |= ip.has_ext == 0;
        ip.has_ext = 1;
    }
    if (changed) {
        OC_TRY(cudaMemcpy(const_cast<InstParams*>(s->args.inst), s->inst_host.data(),
                          sizeof(InstParams) * s->n_inst, cudaMemcpyHostToDevice));
    }
    // The step graph holds the old StepArgs; rebuild it on the next step.
    if (s->exec) {
        cudaGraphExecDestroy(s->exec);
        s->exec = nullptr;
    }
    s->tape.valid = false;
    return OC_OK;
}

}  // extern "C"

namespace {

int32_t ceil_div(int32_t a, int32_t b) { return (a + b - 1) / b; }

// Bytes of one state of every cloth as the recompute tape keeps it (X, V and three planes:
// the warm start in a checkpoint, the step's dV in a segment slot); also the final state
// both tapes keep.
double tape_state_bytes(const oc_solver* s) {
    return 2.0 * sizeof(float4) * (double)s->nv + 3.0 * (double)s->stride * sizeof(float);
}

// float4s of one cloth's replay arena for interval e over n steps: its checkpoints and, for
// e > 1, a segment buffer.
size_t replay_cloth_f4(int64_t nv, int32_t n, int32_t e) {
    return 2 * (size_t)nv * ((size_t)ceil_div(n, e) + (e > 1 ? (size_t)e : 0));
}

double replay_bytes(const oc_solver* s, int32_t n, const std::vector<int32_t>& every) {
    double b = tape_state_bytes(s) + (double)n * 3.0 * (double)s->stride * sizeof(float);
    for (int32_t i = 0; i < s->n_inst; ++i)
        b += (double)sizeof(float4) * (double)replay_cloth_f4(s->inst_host[(size_t)i].nv, n, every[(size_t)i]);
    return b;
}

// Buffers both tapes use: the final state, the gradient planes and the spring gradients.
oc_status alloc_tape_common(oc_solver* s) {
    auto& T = s->tape;
    if (T.finX) return OC_OK;
    OC_TRY(dalloc(s, &T.finX, (size_t)s->nv));
    OC_TRY(dalloc(s, &T.finV, (size_t)s->nv));
    OC_TRY(dalloc(s, &T.finx, 3 * s->stride));
    OC_TRY(dalloc(s, &T.planes, 21 * s->stride));
    OC_TRY(dalloc(s, &T.gK, 2 * (size_t)s->ns + 2));
    return OC_OK;
}

void free_recompute(oc_solver* s) {
    auto& T = s->tape;
    dfree(s, &T.ckX);
    dfree(s, &T.ckV);
    dfree(s, &T.ckx);
    dfree(s, &T.segX);
    dfree(s, &T.segV);
    dfree(s, &T.segx);
    T.cap_ck = T.cap_slots = 0;
}

void free_replay(oc_solver* s) {
    auto& T = s->tape;
    dfree(s, &T.arena);
    dfree(s, &T.dvt);
    T.arena_cap = T.dvt_cap = 0;
}

// The replay tape's layout for per-cloth intervals every[i] (1 ... n): offsets, arena, dV.
cudaError_t alloc_replay(oc_solver* s, int32_t n, const std::vector<int32_t>& every) {
    auto& T = s->tape;
    T.tc.assign((size_t)s->n_inst, TapeCloth{});
    size_t off = 0;
    for (int32_t i = 0; i < s->n_inst; ++i) {
        const int64_t nv = s->inst_host[(size_t)i].nv;
        TapeCloth& c = T.tc[(size_t)i];
        c.every = every[(size_t)i];
        c.ck = (int64_t)off;
        off += 2 * (size_t)nv * (size_t)ceil_div(n, c.every);
        c.buf = (int64_t)off;
        if (c.every > 1) off += 2 * (size_t)nv * (size_t)c.every;
    }
    const size_t nd = (size_t)n * 3 * s->stride;
    cudaError_t e = cudaSuccess;
    if (T.arena_cap < off) {
        dfree(s, &T.arena);
        T.arena_cap = 0;
        if ((e = dalloc(s, &T.arena, off)) != cudaSuccess) return e;
        T.arena_cap = off;
    }
    if (T.dvt_cap < nd) {
        dfree(s, &T.dvt);
        T.dvt_cap = 0;
        if ((e = dalloc(s, &T.dvt, nd)) != cudaSuccess) return e;
        T.dvt_cap = nd;
    }
    return reupload(s, &T.d_tc, T.tc);
}

cudaError_t alloc_recompute(oc_solver* s, int32_t n_ck, int32_t every, int32_t n_buf) {
    auto& T = s->tape;
    cudaError_t e = cudaSuccess;
    if (T.cap_ck < n_ck) {
        dfree(s, &T.ckX);
        dfree(s, &T.ckV);
        dfree(s, &T.ckx);
        T.cap_ck = 0;
        if ((e = dalloc(s, &T.ckX, (size_t)s->nv * n_ck)) != cudaSuccess) return e;
        if ((e = dalloc(s, &T.ckV, (size_t)s->nv * n_ck)) != cudaSuccess) return e;
        if ((e = dalloc(s, &T.ckx, 3 * s->stride * n_ck)) != cudaSuccess) return e;
        T.cap_ck = n_ck;
    }
    const int32_t slots = every * n_buf;
    if (T.cap_slots < slots) {
        dfree(s, &T.segX);
        dfree(s, &T.segV);
        dfree(s, &T.segx);
        T.cap_slots = 0;
        if ((e = dalloc(s, &T.segX, (size_t)s->nv * slots)) != cudaSuccess) return e;
        if ((e = dalloc(s, &T.segV, (size_t)s->nv * slots)) != cudaSuccess) return e;
        if ((e = dalloc(s, &T.segx, 3 * s->stride * slots)) != cudaSuccess) return e;
        T.cap_slots = slots;
    }
    return cudaSuccess;
}

// The taped forward of n steps from the handle's state (either tape).
oc_status taped_forward(oc_solver* s, float dt) {
    auto& T = s->tape;
    const bool gm = T.mode == OC_TAPE_DISPLACEMENT;
    T.gm_valid = false;
    if (gm) {  // the start positions and spring constants; the state becomes u = 0
        const StepArgs ga = gm_args(s, dt);
        OC_TRY(launch_gm(0, ga, (int)s->nv, s->stream));
        OC_TRY(launch_gm(4, ga, (int)s->nv, s->stream));
    }
    const size_t st = s->stride;
    for (int32_t t = 0; t < T.n_steps; ++t) {
        int32_t b = -1, q = 0, len = 0;
        float4 *sX = nullptr, *sV = nullptr;
        float* sx = nullptr;
        if (T.replay) {
            OC_TRY(launch_tape_save(s->args, T.d_tc, T.arena, t, s->n_blocks, s->stream));
        } else {
            const int32_t c = t / T.every;
            q = t - c * T.every;
            len = std::min(T.n_steps, (c + 1) * T.every) - c * T.every;
            if (q == 0) {
                oc_status st0 = copy_state(s, T.ckX + (size_t)c * s->nv, T.ckV + (size_t)c * s->nv,
                                           T.ckx + 3 * st * c, s->args.X, s->args.V, xplanes(s));
                if (st0 != OC_OK) return st0;
            }
            b = tape_buffer(T, c);  // a kept segment: its slots as the recompute would fill them
            if (b >= 0) {
                sX = T.segX + (size_t)b * T.every * s->nv;
                sV = T.segV + (size_t)b * T.every * s->nv;
                sx = T.segx + (size_t)b * T.every * 3 * st;
                if (q == 0) OC_TRY(launch_snapshot(s->args.X, s->args.V, sX, sV, nullptr, nullptr, s->nv, 0, s->stream));
            }
        }
        oc_status r = gm ? gm_step(s, dt) : oc_step(s, dt, 1);
        if (r != OC_OK) return r;
        if (T.replay) {
            OC_TRY(cudaMemcpyAsync(T.dvt + (size_t)t * 3 * st, xplanes(s), 3 * st * sizeof(float),
                                   cudaMemcpyDeviceToDevice, s->stream));
        } else if (b >= 0) {
            const bool more = q + 1 < len;
            OC_TRY(launch_snapshot(s->args.X, s->args.V, more ? sX + (size_t)(q + 1) * s->nv : nullptr,
                                   more ? sV + (size_t)(q + 1) * s->nv : nullptr, xplanes(s), sx + 3 * st * q,
                                   s->nv, (int64_t)(3 * st), s->stream));
        }
    }
    if (gm) {  // keep the final displacement, then the state goes back to positions
        OC_TRY(cudaMemcpyAsync(T.finU, s->args.X, sizeof(float4) * (size_t)s->nv, cudaMemcpyDeviceToDevice, s->stream));
        OC_TRY(launch_gm(3, gm_args(s, dt), (int)s->nv, s->stream));
    }
    oc_status r = copy_state(s, T.finX, T.finV, T.finx, s->args.X, s->args.V, xplanes(s));
    if (r != OC_OK) return r;
    OC_TRY(cudaStreamSynchronize(s->stream));
    if ((r = check_device_error(s)) != OC_OK) return r;
    T.valid = true;
    T.gm_valid = gm;
    return OC_OK;
}

// Chooses the tape and its intervals, allocates it and runs the taped forward.
//   every_in != null: the replay tape with those per-cloth intervals.
//   otherwise: every cloth at the interval `checkpoint_every` (0: ceil(sqrt(n)), which
//   minimises each cloth's checkpoints plus segment buffer; the replay's cost does not
//   depend on the interval, and interval 1 would move a copy of the state into every
//   forward step).  The replay tape when it fits the budget (budget <= 0: when its
//   buffers can be had); else the recompute tape, keeping as many segments as fit.
oc_status tape_begin(oc_solver* s, float dt, int32_t n, int32_t checkpoint_every, int64_t budget,
                     const int32_t* every_in) {
    if (!valid_solver(s) || n < 1 || checkpoint_every < 0 || !std::isfinite(dt)) return OC_ERR_INVALID_ARGUMENT;
    if (s->any_passes)
        return fail(s, OC_ERR_UNSUPPORTED, "oc_tape_forward: the adjoint covers the implicit step only, not the "
                                           "passes after it");
    if (s->any_coupled)
        return fail(s, OC_ERR_UNSUPPORTED, "oc_tape_forward: the adjoint covers the REFERENCE Jacobian mode");
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaStreamSynchronize(s->stream));
    auto& T = s->tape;
    T.valid = false;
    int32_t every = checkpoint_every;
    if (every == 0) every = std::max(1, (int32_t)std::ceil(std::sqrt((double)n)));
    every = std::min(every, n);
    std::vector<int32_t> ev((size_t)s->n_inst, every);
    bool replay = true;
    if (every_in) {
        for (int32_t i = 0; i < s->n_inst; ++i) {
            if (every_in[i] < 1) return OC_ERR_INVALID_ARGUMENT;
            ev[(size_t)i] = std::min(every_in[i], n);
        }
    } else if (budget > 0 && replay_bytes(s, n, ev) > (double)budget) {
        replay = false;
    }
    if (replay) {
        free_recompute(s);
        cudaError_t e = alloc_replay(s, n, ev);
        if (e == cudaErrorMemoryAllocation && !every_in && budget <= 0) {
            cudaGetLastError();
            free_replay(s);
            replay = false;
        } else if (e != cudaSuccess) {
            free_replay(s);
            return fail_cuda(s, e, "oc_tape_forward: the replay tape's buffers");
        }
    }
    if (!replay) {
        free_replay(s);
        const int32_t n_ck = ceil_div(n, every);
        const double state = tape_state_bytes(s), buf = state * (double)every;
        const double need = state * (double)(n_ck + 1) + buf;
        if (budget > 0 && need > (double)budget)
            return fail(s, OC_ERR_OUT_OF_MEMORY, "oc_tape_forward: checkpoints need " + std::to_string(need) +
                                                     " bytes, above the budget");
        // The room left after the checkpoints keeps whole segments from this forward, the
        // last ones first, so that the reverse pass need not recompute them.
        int32_t n_buf = 1;
        if (budget > 0) n_buf = (int32_t)std::min<double>(n_ck, 1.0 + std::floor(((double)budget - need) / buf));
        T.n_ck = n_ck;
        T.n_buf = n_buf;
        T.n_keep = n_buf >= n_ck ? n_ck : n_buf - 1;
        cudaError_t e = alloc_recompute(s, n_ck, every, n_buf);
        if (e != cudaSuccess) {
            free_recompute(s);
            return fail_cuda(s, e, "oc_tape_forward: the recompute tape's buffers");
        }
    }
    if (oc_status r = alloc_tape_common(s)) return r;
    T.replay = replay;
    T.n_steps = n;
    T.every = every;
    T.dt = dt;
    return taped_forward(s, dt);
}

}  // namespace

extern "C" {

oc_status oc_tape_forward(oc_solver* s, float dt, int32_t n_steps, int32_t checkpoint_every, int64_t budget_bytes) {
    return tape_begin(s, dt, n_steps, checkpoint_every, budget_bytes, nullptr);
}

oc_status oc_tape_forward_intervals(oc_solver* s, float dt, int32_t n_steps, const int32_t* every) {
    if (!every) return OC_ERR_INVALID_ARGUMENT;
    return tape_begin(s, dt, n_steps, 0, 0, every);
}

oc_status oc_tape_layout(const oc_solver* s, int32_t* kind, int32_t* every) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    const auto& T = s->tape;
    if (!T.valid) return OC_ERR_INVALID_ARGUMENT;
    if (kind) *kind = T.replay ? OC_TAPE_REPLAY : OC_TAPE_RECOMPUTE;
    if (every)
        for (int32_t i = 0; i < s->n_inst; ++i) every[i] = T.replay ? T.tc[(size_t)i].every : T.every;
    return OC_OK;
}

oc_status oc_set_tape_mode(oc_solver* s, int32_t mode) {
    if (!valid_solver(s) || (mode != OC_TAPE_POSITIONS && mode != OC_TAPE_DISPLACEMENT)) return OC_ERR_INVALID_ARGUMENT;
    auto& T = s->tape;
    if (mode == OC_TAPE_DISPLACEMENT) {
        if (!s->adj_persist)
            return fail(s, OC_ERR_UNSUPPORTED, "oc_set_tape_mode: the displacement mode runs every cloth's CG through "
                                               "the cooperative CG (no COUPLED cloth, cooperative launch available)");
        OC_TRY(cudaSetDevice(s->device));
        if (!T.Xbase) {
            OC_TRY(dalloc(s, &T.Xbase, (size_t)s->nv));
            OC_TRY(dalloc(s, &T.gm_inc, (size_t)s->n_inc));
            OC_TRY(dalloc(s, &T.gm_own, (size_t)s->nv));
            OC_TRY(dalloc(s, &T.finU, (size_t)s->nv));
        }
    }
    T.mode = mode;
    T.valid = false;
    T.gm_valid = false;
    return OC_OK;
}

oc_status oc_tape_displacement(oc_solver* s, float* u) {
    if (!valid_solver(s) || !u) return OC_ERR_INVALID_ARGUMENT;
    auto& T = s->tape;
    if (!T.valid || !T.gm_valid)
        return fail(s, OC_ERR_INVALID_ARGUMENT, "oc_tape_displacement: no displacement-mode tape");
    OC_TRY(cudaSetDevice(s->device));
    StepArgs dn = s->args;
    dn.X = T.finU;
    OC_TRY(launch_state_out(dn, s->stage, nullptr, nullptr, s->nv, s->stream));
    OC_TRY(cudaMemcpyAsync(u, s->stage, 3 * (size_t)s->nv * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    return OC_OK;
}

oc_status oc_tape_backward(oc_solver* s, const float* dL_dX, const float* dL_dV, float* dL_dX0, float* dL_dV0,
                           float* dL_dKs, float* dL_dKd, float* dL_dext) {
    if (!valid_solver(s) || !dL_dX) return OC_ERR_INVALID_ARGUMENT;
    auto& T = s->tape;
    if (!T.valid) return fail(s, OC_ERR_INVALID_ARGUMENT, "oc_tape_backward: no tape (run oc_tape_forward first)");
    OC_TRY(cudaSetDevice(s->device));
    const size_t st = s->stride, n3 = 3 * (size_t)s->nv;
    AdjArgs& j = s->adj;
    for (int k = 0; k < 3; ++k) {
        j.gX[k] = T.planes + (0 + k) * st;
        j.gV[k] = T.planes + (3 + k) * st;
        j.gF[k] = T.planes + (6 + k) * st;
        j.gExt[k] = T.planes + (15 + k) * st;
        j.dV[k] = T.planes + (18 + k) * st;
    }
    for (int k = 0; k < 6; ++k) j.gOwn[k] = T.planes + (9 + k) * st;
    j.gKs = T.gK;
    j.gKd = T.gK + s->ns;
    OC_TRY(cudaMemsetAsync(T.planes, 0, 21 * st * sizeof(float), s->stream));
    OC_TRY(cudaMemsetAsync(T.gK, 0, (2 * (size_t)s->ns + 2) * sizeof(float), s->stream));
    // dL/dX_T, dL/dV_T -> gX, gV planes (through the state upload kernel).
    StepArgs up = s->args;
    for (int k = 0; k < 3; ++k) up.x[k] = j.gX[k];
    OC_TRY(cudaMemcpyAsync(s->stage, dL_dX, n3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    OC_TRY(launch_state_in(up, nullptr, nullptr, s->stage, s->nv, s->d_err, s->stream));
    if (dL_dV) {
        for (int k = 0; k < 3; ++k) up.x[k] = j.gV[k];
        float* sv = s->stage + stage_stride(s->nv);
        OC_TRY(cudaMemcpyAsync(sv, dL_dV, n3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        OC_TRY(launch_state_in(up, nullptr, nullptr, sv, s->nv, s->d_err, s->stream));
    }
    if (!s->adj_persist && (!T.exec || T.graph_dt != T.dt)) {
        oc_status r = build_adjoint_graph(s, T.dt);
        if (r != OC_OK) return r;
    }
    const bool gm = T.gm_valid;
    StepArgs a = gm ? gm_args(s, T.dt) : s->args;
    a.dt = T.dt;
    a.blk_base = 0;
    a.use_cond = 0;
    a.all_streamed = 1;
    // One reverse step on the state b.X, b.V with the step's dV at dv (three planes): the
    // system's diagonal blocks rebuilt from spring i as the step formed them, the adjoint
    // seed, lambda = A^-1 g_dV, then the vertex and spring terms.
    auto reverse_step = [&](const StepArgs& b, const float* dv) -> oc_status {
        AdjArgs jj = j;
        for (int k = 0; k < 3; ++k) jj.dV[k] = dv + k * st;
        if (gm) {
            OC_TRY(launch_adjoint(0, b, jj, s->n_blocks, s->stream));
        } else if (s->adj_persist) {
            OC_TRY(launch_adj_seed_own(b, jj, s->n_blocks, s->stream));
        }
        if (s->adj_persist) {
            if (oc_status r = solve_only(s, b)) return r;
        } else {  // the WHILE-loop graph, its seed node pointed at this step
            StepArgs bs = b;
            bs.use_cond = 1;
            bs.cond = (unsigned long long)T.handle;
            void* params_seed[] = {&bs, &jj};
            cudaKernelNodeParams kp{};
            kp.func = const_cast<void*>(adjoint_seed_own_fn());
            kp.gridDim = dim3((unsigned)s->n_blocks);
            kp.blockDim = dim3(256);
            kp.kernelParams = params_seed;
            OC_TRY(cudaGraphExecKernelNodeSetParams(T.exec, T.n_seed, &kp));
            OC_TRY(cudaGraphLaunch(T.exec, s->stream));
        }
        OC_TRY(launch_adjoint(1, b, jj, s->n_blocks, s->stream));
        OC_TRY(launch_adjoint(2, b, jj, s->n_blocks, s->stream));
        return OC_OK;
    };
    if (T.replay) {
        // Each step's state is rebuilt into the handle's X, V (the replay tape's view).
        for (int32_t t = T.n_steps - 1; t >= 0; --t) {
            OC_TRY(launch_tape_view(a, T.d_tc, T.arena, T.dvt, (int64_t)(3 * st), t, T.n_steps, s->n_blocks,
                                    s->stream));
            if (oc_status r = reverse_step(a, T.dvt + (size_t)t * 3 * st)) return r;
        }
    } else {
        for (int32_t c = T.n_ck - 1; c >= 0; --c) {
            const int32_t t0 = c * T.every, t1 = std::min(T.n_steps, t0 + T.every), len = t1 - t0;
            const int32_t kept = tape_buffer(T, c);
            const int32_t buf = kept >= 0 ? kept : 0;
            float4* const segX = T.segX + (size_t)buf * T.every * s->nv;
            float4* const segV = T.segV + (size_t)buf * T.every * s->nv;
            float* const segx = T.segx + (size_t)buf * T.every * 3 * st;
            if (kept < 0) {
                // Recompute the segment from its checkpoint, keeping every step's input state
                // and solution.
                oc_status r = copy_state(s, s->args.X, s->args.V, xplanes(s), T.ckX + (size_t)c * s->nv,
                                         T.ckV + (size_t)c * s->nv, T.ckx + 3 * st * c);
                if (r != OC_OK) return r;
                OC_TRY(launch_snapshot(s->args.X, s->args.V, segX, segV, nullptr, nullptr, s->nv, 0, s->stream));
                for (int32_t q = 0; q < len; ++q) {
                    if ((r = gm ? gm_step(s, T.dt) : oc_step(s, T.dt, 1)) != OC_OK) return r;
                    const bool more = q + 1 < len;
                    OC_TRY(launch_snapshot(s->args.X, s->args.V, more ? segX + (size_t)(q + 1) * s->nv : nullptr,
                                           more ? segV + (size_t)(q + 1) * s->nv : nullptr, xplanes(s),
                                           segx + 3 * st * q, s->nv, (int64_t)(3 * st), s->stream));
                }
            }
            // And walk it backwards: the kernels read the step's state in place in the tape.
            for (int32_t q = len - 1; q >= 0; --q) {
                StepArgs b = a;
                b.X = segX + (size_t)q * s->nv;
                b.V = segV + (size_t)q * s->nv;
                if (oc_status r = reverse_step(b, segx + 3 * st * q)) return r;
            }
        }
    }
    oc_status r = copy_state(s, s->args.X, s->args.V, xplanes(s), T.finX, T.finV, T.finx);
    if (r != OC_OK) return r;
    if ((r = check_device_error(s)) != OC_OK) return r;
    // Gradients out (planes -> packed triples through the state download kernel).
    StepArgs dn = s->args;
    auto planes_out = [&](float* const* pl, float* host) -> oc_status {
        if (!host) return OC_OK;
        for (int k = 0; k < 3; ++k) dn.x[k] = pl[k];
        OC_TRY(launch_state_out(dn, nullptr, nullptr, s->stage, s->nv, s->stream));
        OC_TRY(cudaMemcpyAsync(host, s->stage, n3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        OC_TRY(cudaStreamSynchronize(s->stream));
        return OC_OK;
    };
    if ((r = planes_out(j.gX, dL_dX0)) != OC_OK) return r;
    if ((r = planes_out(j.gV, dL_dV0)) != OC_OK) return r;
    if ((r = planes_out(j.gExt, dL_dext)) != OC_OK) return r;
    if (dL_dKs) OC_TRY(cudaMemcpyAsync(dL_dKs, j.gKs, sizeof(float) * s->ns, cudaMemcpyDeviceToHost, s->stream));
    if (dL_dKd) OC_TRY(cudaMemcpyAsync(dL_dKd, j.gKd, sizeof(float) * s->ns, cudaMemcpyDeviceToHost, s->stream));
    OC_TRY(cudaStreamSynchronize(s->stream));
    return OC_OK;
}

oc_status oc_get_launch_config(const oc_solver* s, oc_launch_config* cfg) {
    if (!valid_solver(s) || !cfg) return OC_ERR_INVALID_ARGUMENT;
    *cfg = s->cfg;
    return OC_OK;
}

oc_status oc_set_launch_config(oc_solver* s, const oc_launch_config* cfg) {
    if (!valid_solver(s) || !cfg || !launch_config_valid(*cfg)) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaStreamSynchronize(s->stream));
    const oc_launch_config old = s->cfg;
    s->cfg = *cfg;
    oc_status r = plan_execution(s);
    if (r != OC_OK) {
        const std::string why = s->err;
        s->cfg = old;
        if (plan_execution(s) != OC_OK) return r;
        return fail(s, r, why);
    }
    s->tape.valid = false;
    if (s->tape.exec) {
        cudaGraphExecDestroy(s->tape.exec);
        s->tape.exec = nullptr;
    }
    if (s->tape.graph) {
        cudaGraphDestroy(s->tape.graph);
        s->tape.graph = nullptr;
    }
    return OC_OK;
}

}  // extern "C"

namespace {

// 64-bit FNV-1a.
uint64_t fnv1a(const void* data, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

// The tuning key: GPU name (spaces as '_'), SM count and the hash of the sorted per-cloth
// signatures (vertices, grid shape, Jacobian mode, passes, strip eligibility).
oc_status make_tune_key(const std::vector<InstParams>& inst, const char* gpu_name, int32_t sm_count, char* key,
                        int32_t key_size) {
    if (!gpu_name || !key || key_size < 96 || sm_count < 0) return OC_ERR_INVALID_ARGUMENT;
    std::vector<std::array<int32_t, 6>> sig;
    sig.reserve(inst.size());
    for (const InstParams& ip : inst)
        sig.push_back({ip.nv, ip.grid_cols, ip.grid_rows, ip.coupled, ip.passes, ip.strip_ok});
    std::sort(sig.begin(), sig.end());
    const uint64_t h = fnv1a(sig.data(), sig.size() * sizeof(sig[0]));
    std::string name(gpu_name);
    for (char& ch : name)
        if (ch == ' ' || ch == '\t' || ch == '\n') ch = '_';
    char buf[64];
    std::snprintf(buf, sizeof buf, ";sm=%d;n=%zu;h=%016llx", sm_count, inst.size(), (unsigned long long)h);
    const std::string k = "gpu=" + name.substr(0, (size_t)std::max(0, key_size - 64)) + buf;
    if ((int32_t)k.size() >= key_size) return OC_ERR_INVALID_ARGUMENT;
    std::memcpy(key, k.c_str(), k.size() + 1);
    return OC_OK;
}

// Device copies of a handle's state (X, V, the warm-start planes), to time candidates
// without advancing the simulation.
struct StateBackup {
    float4* X = nullptr;
    float4* V = nullptr;
    float* x = nullptr;
};

}  // namespace

extern "C" {

oc_status oc_tune_key(const oc_cloth_desc* descs, int32_t n_instances, const char* gpu_name, int32_t sm_count,
                      char* key, int32_t key_size) {
    if (!descs || n_instances < 1) return OC_ERR_INVALID_ARGUMENT;
    PackedHost P;
    std::string err;
    if (oc_status st = pack_instances(descs, n_instances, 2048, &P, &err)) return st;
    build_strip_tables(&P);
    return make_tune_key(P.inst, gpu_name, sm_count, key, key_size);
}

oc_status oc_tune_key_of(const oc_solver* s, char* key, int32_t key_size) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, s->device) != cudaSuccess) return OC_ERR_CUDA;
    return make_tune_key(s->inst_host, prop.name, prop.multiProcessorCount, key, key_size);
}

oc_status oc_tune_cache_lookup(const char* path, const char* key, oc_launch_config* cfg, int32_t* found) {
    if (!path || !key || !cfg || !found) return OC_ERR_INVALID_ARGUMENT;
    *found = 0;
    std::ifstream in(path);
    if (!in) return OC_OK;  // no cache yet
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string k;
        oc_launch_config c{};
        double ms = 0.0;
        if (!(ls >> k >> c.resident_max_vertices >> c.resident_vcta >> c.resident_threads >> c.resident_fused >>
              c.persist >> c.gather_variant >> c.strip >> c.strip_rows >> c.strip_variant >> ms))
            continue;  // not a cache line
        if (k == key && launch_config_valid(c)) {
            *cfg = c;
            *found = 1;
        }
    }
    return OC_OK;
}

oc_status oc_tune_cache_store(const char* path, const char* key, const oc_launch_config* cfg, double ms_per_step) {
    if (!path || !key || !cfg || !launch_config_valid(*cfg) || std::strchr(key, ' ') || std::strchr(key, '\n'))
        return OC_ERR_INVALID_ARGUMENT;
    std::ofstream out(path, std::ios::app);
    if (!out) return OC_ERR_INVALID_ARGUMENT;
    const oc_launch_config& c = *cfg;
    out << key << ' ' << c.resident_max_vertices << ' ' << c.resident_vcta << ' ' << c.resident_threads << ' '
        << c.resident_fused << ' ' << c.persist << ' ' << c.gather_variant << ' ' << c.strip << ' ' << c.strip_rows
        << ' ' << c.strip_variant << ' ' << ms_per_step << '\n';
    return out ? OC_OK : OC_ERR_INVALID_ARGUMENT;
}

oc_status oc_autotune(oc_solver* s, float dt, const char* cache_path, int32_t flags, oc_launch_config* chosen,
                      double* ms_per_step) {
    if (!valid_solver(s) || !std::isfinite(dt) || dt <= 0.0f) return OC_ERR_INVALID_ARGUMENT;
    OC_TRY(cudaSetDevice(s->device));
    char key[256];
    if (oc_status st = oc_tune_key_of(s, key, (int32_t)sizeof key)) return st;
    if (cache_path && (flags & OC_TUNE_USE_CACHE)) {
        oc_launch_config c{};
        int32_t found = 0;
        if (oc_status st = oc_tune_cache_lookup(cache_path, key, &c, &found)) return st;
        if (found && oc_set_launch_config(s, &c) == OC_OK) {
            if (chosen) *chosen = s->cfg;
            if (ms_per_step) *ms_per_step = 0.0;
            return OC_OK;
        }
    }
    OC_TRY(cudaStreamSynchronize(s->stream));
    // Save the state; every candidate starts from it, and it is put back at the end.
    StateBackup B;
    const size_t n4 = sizeof(float4) * (size_t)s->nv, nx = 3 * s->stride * sizeof(float);
    OC_TRY(cudaMalloc(&B.X, n4));
    OC_TRY(cudaMalloc(&B.V, n4));
    OC_TRY(cudaMalloc(&B.x, nx));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&](oc_status st) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(B.X);
        cudaFree(B.V);
        cudaFree(B.x);
        return st;
    };
    if (copy_state(s, B.X, B.V, B.x, s->args.X, s->args.V, xplanes(s)) != OC_OK ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return cleanup(fail(s, OC_ERR_CUDA, "oc_autotune: set-up failed"));
    auto restore = [&]() { return copy_state(s, s->args.X, s->args.V, xplanes(s), B.X, B.V, B.x); };
    int32_t timed_steps = 0;  // fixed after the first candidate (about 20 ms of steps)
    // Time one configuration: re-plan, two warm-up steps from the saved state, then the
    // timed steps from the saved state again.  A configuration the handle cannot run is
    // skipped (returns a negative time).
    auto measure = [&](const oc_launch_config& c) -> double {
        if (oc_set_launch_config(s, &c) != OC_OK) return -1.0;
        if (restore() != OC_OK || oc_step(s, dt, 2) != OC_OK) return -1.0;
        if (cudaEventRecord(e0, s->stream) != cudaSuccess || oc_step(s, dt, 1) != OC_OK ||
            cudaEventRecord(e1, s->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            return -1.0;
        float one = 0.0f;
        cudaEventElapsedTime(&one, e0, e1);
        if (timed_steps == 0) timed_steps = (int32_t)std::min(200.0, std::max(3.0, 20.0 / std::max(one, 1e-3f)));
        if (restore() != OC_OK || cudaEventRecord(e0, s->stream) != cudaSuccess ||
            oc_step(s, dt, timed_steps) != OC_OK || cudaEventRecord(e1, s->stream) != cudaSuccess ||
            cudaEventSynchronize(e1) != cudaSuccess || check_device_error(s) != OC_OK)
            return -1.0;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        return (double)ms / timed_steps;
    };
    // Which knobs matter for these cloths.
    bool any_strip = false, any_small = false, any_records = false;
    for (int32_t k = 0; k < s->n_inst; ++k) {
        const InstParams& ip = s->inst_host[(size_t)k];
        if (ip.coupled) continue;
        any_strip |= ip.strip_ok != 0 && ip.grid_cols > 0;
        any_small |= ip.nv <= kResidentMaxCluster * kResidentDefaultVcta;
        any_records |= ip.grid_cols <= 0;
    }
    oc_launch_config best = s->cfg;
    double t_best = measure(best);
    if (t_best < 0.0) {
        oc_set_launch_config(s, &best);
        restore();
        return cleanup(fail(s, OC_ERR_CUDA, "oc_autotune: the current configuration failed to run"));
    }
    auto consider = [&](oc_launch_config c) {
        if (std::memcmp(&c, &best, sizeof c) == 0 || !launch_config_valid(c)) return;
        const double t = measure(c);
        if (t > 0.0 && t < 0.99 * t_best) {
            best = c;
            t_best = t;
        }
    };
    if (any_strip) {
        for (int32_t v : {1, 0}) {
            oc_launch_config c = best;
            c.strip = v;
            consider(c);
        }
        if (best.strip) {
            for (int32_t rows : {0, 4, 8, 16, 32}) {
                oc_launch_config c = best;
                c.strip_rows = rows;
                consider(c);
            }
            for (int32_t v : {2, 3}) {
                oc_launch_config c = best;
                c.strip_variant = v;
                consider(c);
            }
        }
    }
    if (any_small && s->executor == OC_EXEC_AUTO) {
        for (int32_t m : {kResidentMaxCluster * kResidentDefaultVcta, 4096, 1024, 0}) {
            oc_launch_config c = best;
            c.resident_max_vertices = m;
            consider(c);
        }
    }
    if (any_small && s->executor != OC_EXEC_STREAMED && s->executor != OC_EXEC_PLAIN && !s->buckets.empty()) {
        const int32_t shapes[3][2] = {{1024, 256}, {512, 128}, {2048, 512}};
        for (const auto& sh : shapes) {
            oc_launch_config c = best;
            c.resident_vcta = sh[0];
            c.resident_threads = sh[1];
            consider(c);
        }
        for (int32_t v : {0, 1}) {
            oc_launch_config c = best;
            c.resident_fused = v;
            consider(c);
        }
    }
    for (int32_t v : {1, 0}) {
        oc_launch_config c = best;
        c.persist = v;
        consider(c);
    }
    if (any_records)
        for (int32_t v : {6, 4, 1}) {
            oc_launch_config c = best;
            c.gather_variant = v;
            consider(c);
        }
    oc_status st = oc_set_launch_config(s, &best);
    if (st == OC_OK) st = restore();
    if (st == OC_OK) st = cudaStreamSynchronize(s->stream) == cudaSuccess ? OC_OK : OC_ERR_CUDA;
    if (st == OC_OK && cache_path && (flags & OC_TUNE_STORE)) st = oc_tune_cache_store(cache_path, key, &best, t_best);
    if (chosen) *chosen = best;
    if (ms_per_step) *ms_per_step = t_best;
    return cleanup(st);
}

oc_status oc_test_barrier_timeout(oc_solver* s, int32_t withhold_block, uint32_t max_polls) {
    if (!valid_solver(s) || withhold_block < -1) return OC_ERR_INVALID_ARGUMENT;
    if (!s->persist && !s->adj_persist) return fail(s, OC_ERR_UNSUPPORTED, "the handle runs no persistent CG");
    OC_TRY(cudaSetDevice(s->device));
    OC_TRY(cudaStreamSynchronize(s->stream));
    s->args.withhold_block = withhold_block;
    s->args.barrier_polls = max_polls > 0 ? max_polls : kDefaultBarrierPolls;
    // The step graph holds the launch arguments: rebuild it at the next step.
    if (s->exec) {
        cudaGraphExecDestroy(s->exec);
        s->exec = nullptr;
    }
    if (s->graph) {
        cudaGraphDestroy(s->graph);
        s->graph = nullptr;
    }
    return OC_OK;
}

oc_status oc_test_cr_arith(int32_t device, uint64_t n_pairs, uint64_t seed, uint64_t* mismatches) {
    if (!mismatches || device < 0) return OC_ERR_INVALID_ARGUMENT;
    oc_solver* s = nullptr;  // fail_cuda records the message without a handle
    OC_TRY(cudaSetDevice(device));
    unsigned long long* counts = nullptr;
    OC_TRY(cudaMalloc(&counts, 3 * sizeof(unsigned long long)));
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t e = cudaMemset(counts, 0, sizeof h);
    if (e == cudaSuccess) e = launch_test_cr_arith(counts, n_pairs, seed, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(h, counts, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(counts);
    if (e != cudaSuccess) return fail_cuda(s, e, "oc_test_cr_arith");
    for (int k = 0; k < 3; ++k) mismatches[k] = h[k];
    return OC_OK;
}

oc_status oc_tape_info(const oc_solver* s, int32_t* checkpoint_every, int64_t* tape_bytes) {
    if (!valid_solver(s)) return OC_ERR_INVALID_ARGUMENT;
    const auto& T = s->tape;
    if (checkpoint_every) *checkpoint_every = T.every;
    if (tape_bytes) {
        if (T.replay) {
            std::vector<int32_t> ev((size_t)s->n_inst);
            for (int32_t i = 0; i < s->n_inst; ++i) ev[(size_t)i] = T.tc.empty() ? 1 : T.tc[(size_t)i].every;
            *tape_bytes = (int64_t)replay_bytes(s, T.n_steps, ev);
        } else {
            const double state = tape_state_bytes(s);
            *tape_bytes = (int64_t)(state * (double)(T.n_ck + 1) + state * (double)T.every * (double)T.n_buf);
        }
    }
    return OC_OK;
}

}  // extern "C"
