// Spanning-path test of the convergence check's zero-flux branch on the device (sm_103a), and
// the anchored-cluster phase map of the FP64 refinement.
//
// The reference calls extract_through_feature(mask, 1, 'x') (taufactor/metrics/connectivity.py:
// 138-213, from taufactor/taufactor.py:318-327) on the host: face-connected (6-neighbour)
// labelling without periodic wrap, then whether any cluster touches both x = 0 and x = nx - 1.
// Here: union-find over the voxels of every volume (each voxel links to its conductive +x, +y, +z
// neighbours with atomicMin on the larger root), flattening, and a pass over plane nx - 1. The
// root of a cluster is its smallest flat index [b][x][y][z], so a cluster touches x = 0 exactly
// when its root lies in plane 0. Every retry loop is bounded; running out sets TF_ERR_TIMEOUT.
#include "tf_common.cuh"
#include "tf_internal.h"

namespace tf {

constexpr int CC_LIMIT = 1 << 20;  // bound of every find / union retry loop

__device__ __forceinline__ int cc_find(const int* __restrict__ L, int v, int32_t* err) {
    for (int it = 0; it < CC_LIMIT; ++it) {
        const int p = L[v];
        if (p == v) return v;
        v = p;
    }
    atomicExch(err, TF_ERR_TIMEOUT);
    return v;
}

__device__ __forceinline__ void cc_union(int* L, int a, int b, int32_t* err) {
    for (int it = 0; it < CC_LIMIT; ++it) {
        a = cc_find(L, a, err);
        b = cc_find(L, b, err);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        // link root b under the smaller root a, unless b has been linked meanwhile
        const int old = atomicMin(&L[b], a);
        if (old == b) return;
        b = old;
    }
    atomicExch(err, TF_ERR_TIMEOUT);
}

struct PhaseTable {
    uint8_t conductive[256];
};

__global__ void k_cc_init(const uint8_t* __restrict__ phase, const PhaseTable t, int* __restrict__ L, long long n) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n) return;
    L[v] = t.conductive[phase[v]] ? (int)v : -1;
}

// py / pz: also link the last y (z) row of a plane to its first (periodic faces).
__global__ void k_cc_union(int* __restrict__ L, int nx, int ny, int nz, long long n, int py, int pz, int32_t* err) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n || L[v] < 0) return;
    const int z = (int)(v % nz);
    const int y = (int)((v / nz) % ny);
    const int x = (int)((v / ((long long)nz * ny)) % nx);
    if (z + 1 < nz && L[v + 1] >= 0) cc_union(L, (int)v, (int)(v + 1), err);
    if (y + 1 < ny && L[v + nz] >= 0) cc_union(L, (int)v, (int)(v + nz), err);
    if (x + 1 < nx && L[v + (long long)ny * nz] >= 0) cc_union(L, (int)v, (int)(v + (long long)ny * nz), err);
    if (pz && z == nz - 1 && nz > 1 && L[v - (nz - 1)] >= 0) cc_union(L, (int)v, (int)(v - (nz - 1)), err);
    if (py && y == ny - 1 && ny > 1) {
        const long long w = v - (long long)(ny - 1) * nz;
        if (L[w] >= 0) cc_union(L, (int)v, (int)w, err);
    }
}

__global__ void k_cc_flatten(int* __restrict__ L, long long n, int32_t* err) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n || L[v] < 0) return;
    L[v] = cc_find(L, (int)v, err);
}

// One thread per voxel of plane nx - 1 of volume blockIdx.y: marks the root of its cluster.
__global__ void k_cc_mark_last(const int* __restrict__ L, int nx, int ny, int nz, uint8_t* __restrict__ flags) {
    const long long plane = (long long)ny * nz;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= plane) return;
    const int r = L[(long long)blockIdx.y * nx * plane + (long long)(nx - 1) * plane + i];
    if (r >= 0) flags[r] = 1;
}

// out[v] = phase[v] for voxels of clusters that touch x = 0 (root in plane 0) or x = nx - 1
// (root marked), 0 for every other voxel.
__global__ void k_cc_anchored(const uint8_t* __restrict__ phase, const int* __restrict__ L,
                              const uint8_t* __restrict__ flags, long long vol, long long plane, long long n,
                              uint8_t* __restrict__ out) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int r = L[v];
    const bool keep = r >= 0 && ((long long)r - (v / vol) * vol < plane || flags[r]);
    out[v] = keep ? phase[v] : 0;
}

// One thread per voxel of plane nx - 1 of volume blockIdx.y: spans if its root is in plane 0.
__global__ void k_cc_spans(const int* __restrict__ L, int nx, int ny, int nz, int32_t* __restrict__ spans) {
    const long long plane = (long long)ny * nz;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= plane) return;
    const long long base = (long long)blockIdx.y * nx * plane;
    const int r = L[base + (long long)(nx - 1) * plane + i];
    if (r >= 0 && (long long)r - base < plane) atomicOr(&spans[blockIdx.y], 1);
}

}  // namespace tf

using namespace tf;

extern "C" int tf_spans_x(int batch, int nx, int ny, int nz, const uint8_t* phase_dev, const uint8_t* conductive,
                          int32_t* labels_dev, int32_t* spans_dev, int32_t* err_dev, void* stream) {
    if (batch < 1 || nx < 1 || ny < 1 || nz < 1 || !phase_dev || !conductive || !labels_dev || !spans_dev || !err_dev)
        return TF_ERR_ARG;
    const long long n = (long long)batch * nx * ny * nz;
    if (n > 0x7fffffffLL) return TF_ERR_UNSUPPORTED;  // int32 labels
    cudaStream_t st = (cudaStream_t)stream;
    PhaseTable t;
    for (int i = 0; i < 256; ++i) t.conductive[i] = conductive[i] ? 1 : 0;
    if (cudaMemsetAsync(spans_dev, 0, sizeof(int32_t) * batch, st) != cudaSuccess) return TF_ERR_CUDA;
    const unsigned grid = (unsigned)((n + 255) / 256);
    k_cc_init<<<grid, 256, 0, st>>>(phase_dev, t, labels_dev, n);
    k_cc_union<<<grid, 256, 0, st>>>(labels_dev, nx, ny, nz, n, 0, 0, err_dev);
    k_cc_flatten<<<grid, 256, 0, st>>>(labels_dev, n, err_dev);
    const long long plane = (long long)ny * nz;
    k_cc_spans<<<dim3((unsigned)((plane + 255) / 256), batch), 256, 0, st>>>(labels_dev, nx, ny, nz, spans_dev);
    for (int i = 0; i < 4; ++i) note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

extern "C" int tf_anchored_phase(int batch, int nx, int ny, int nz, int periodic, const uint8_t* phase_dev,
                                 const uint8_t* conductive, int32_t* labels_dev, uint8_t* flags_dev,
                                 uint8_t* out_phase_dev, int32_t* err_dev, void* stream) {
    if (batch < 1 || nx < 1 || ny < 1 || nz < 1 || !phase_dev || !conductive || !labels_dev || !flags_dev ||
        !out_phase_dev || !err_dev)
        return TF_ERR_ARG;
    const long long n = (long long)batch * nx * ny * nz;
    if (n > 0x7fffffffLL) return TF_ERR_UNSUPPORTED;  // int32 labels
    cudaStream_t st = (cudaStream_t)stream;
    PhaseTable t;
    for (int i = 0; i < 256; ++i) t.conductive[i] = conductive[i] ? 1 : 0;
    if (cudaMemsetAsync(flags_dev, 0, (size_t)n, st) != cudaSuccess) return TF_ERR_CUDA;
    const unsigned grid = (unsigned)((n + 255) / 256);
    k_cc_init<<<grid, 256, 0, st>>>(phase_dev, t, labels_dev, n);
    k_cc_union<<<grid, 256, 0, st>>>(labels_dev, nx, ny, nz, n, (periodic & TF_PERIODIC_Y) ? 1 : 0,
                                     (periodic & TF_PERIODIC_Z) ? 1 : 0, err_dev);
    k_cc_flatten<<<grid, 256, 0, st>>>(labels_dev, n, err_dev);
    const long long plane = (long long)ny * nz;
    k_cc_mark_last<<<dim3((unsigned)((plane + 255) / 256), batch), 256, 0, st>>>(labels_dev, nx, ny, nz, flags_dev);
    k_cc_anchored<<<grid, 256, 0, st>>>(phase_dev, labels_dev, flags_dev, (long long)nx * plane, plane, n,
                                        out_phase_dev);
    for (int i = 0; i < 5; ++i) note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}
