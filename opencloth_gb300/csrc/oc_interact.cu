// Interaction and constraint entry points on the device state (no host round trip):
//
//   k_pick        the reference's picking loop, IMP:399-405: the first vertex (lowest
//                 index) of a cloth whose distance to a point is below a radius
//   k_drag        the reference's drag, IMP:433-440: V = 0, X moved by a world-space delta
//                 with the y component applied only while it stays above 0
//   k_set_verts   per-step overrides of chosen vertices' positions and velocities
//   k_pins_clear / k_pins_set   a new pin set for one cloth
//
// FP32 arithmetic in the reference's order; compiled with --fmad=false like the step.
#include <cuda_runtime.h>

#include <algorithm>

#include "oc_internal.h"

namespace oc {
namespace {

constexpr int kThreads = 256;

// glm::distance(X[i], pt) < radius: length(pt - X[i]) (GLM/core/func_geometric.inl),
// squares summed left to right, compared in double (the reference compares with the
// double literal 0.1).
__global__ void k_pick(const float4* __restrict__ X, int64_t v0, int64_t nv, float px, float py, float pz,
                       double radius, int32_t* __restrict__ out) {
    int32_t best = 0x7fffffff;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 x = X[v0 + i];
        const float dx = px - x.x, dy = py - x.y, dz = pz - x.z;
        const float d = sqrtf(dx * dx + dy * dy + dz * dz);
        if ((double)d < radius) {
            best = (int32_t)i;
            break;  // later indices of this thread are larger
        }
    }
    if (best != 0x7fffffff) atomicMin(out, best);
}

__global__ void k_drag(float4* X, float4* V, int64_t g, float dx, float dy, float dz) {
    float4 x = X[g], v = V[g];
    v.x = 0.0f;  // V[selected_index] = glm::vec3(0), IMP:433
    v.y = 0.0f;
    v.z = 0.0f;
    x.x = x.x + dx;                 // IMP:434
    const float ny = x.y + dy;      // IMP:435
    if (ny > 0.0f) x.y = ny;        // IMP:436-437
    x.z = x.z + dz;                 // IMP:438
    X[g] = x;
    V[g] = v;
}

__global__ void k_set_verts(float4* X, float4* V, const int64_t* __restrict__ idx, const float* __restrict__ X3,
                            const float* __restrict__ V3, int32_t n) {
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t g = idx[k];
    if (X3) {
        float4 x = X[g];  // keeps the mass in w
        x.x = X3[3 * (size_t)k];
        x.y = X3[3 * (size_t)k + 1];
        x.z = X3[3 * (size_t)k + 2];
        X[g] = x;
    }
    if (V3) {
        float4 v = V[g];  // keeps the pin flag in w
        v.x = V3[3 * (size_t)k];
        v.y = V3[3 * (size_t)k + 1];
        v.z = V3[3 * (size_t)k + 2];
        V[g] = v;
    }
}

__global__ void k_pins_clear(float4* V, uint8_t* pinflag, int64_t v0, int64_t nv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        V[v0 + i].w = 0.0f;
        pinflag[v0 + i] = 0;
    }
}

__global__ void k_pins_set(float4* V, uint8_t* pinflag, int64_t v0, const int32_t* __restrict__ pins, int32_t n) {
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    V[v0 + pins[k]].w = 1.0f;
    pinflag[v0 + pins[k]] = 1;
}

int grid_for(int64_t n) {
    const int64_t b = (n + kThreads - 1) / kThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 8));
}

}  // namespace

cudaError_t launch_pick(const float4* X, int64_t v0, int64_t nv, const float pt[3], double radius, int32_t* out,
                        cudaStream_t stream) {
    k_pick<<<grid_for(nv), kThreads, 0, stream>>>(X, v0, nv, pt[0], pt[1], pt[2], radius, out);
    return cudaGetLastError();
}

cudaError_t launch_drag(float4* X, float4* V, int64_t g, const float delta[3], cudaStream_t stream) {
    k_drag<<<1, 1, 0, stream>>>(X, V, g, delta[0], delta[1], delta[2]);
    return cudaGetLastError();
}

cudaError_t launch_set_vertices(float4* X, float4* V, const int64_t* idx, const float* X3, const float* V3,
                                int32_t n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_set_verts<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(X, V, idx, X3, V3, n);
    return cudaGetLastError();
}

cudaError_t launch_set_pins(float4* V, uint8_t* pinflag, int64_t v0, int64_t nv, const int32_t* pins, int32_t n,
                            cudaStream_t stream) {
    if (nv <= 0) return cudaSuccess;
    k_pins_clear<<<grid_for(nv), kThreads, 0, stream>>>(V, pinflag, v0, nv);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || n <= 0) return e;
    k_pins_set<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(V, pinflag, v0, pins, n);
    return cudaGetLastError();
}

}  // namespace oc
