// Set-up statistics on the device (sm_103a), one pass over the input as the caller uploaded it:
// for uint8 labels the per-plane counts of label 1 and the largest label (Solver set-up: the 0/1
// label check, taufactor/taufactor.py:387-397, and vol_x = mean(mask, (2, 3)), :42); for a
// per-voxel conductivity the per-plane count of kappa > 0, the per-plane float64 sum and a
// validity flag (KappaSolver set-up).
#include "tf_common.cuh"
#include "tf_internal.h"

namespace tf {

// grid (chunks of a plane, batch * nx planes): each CTA counts the 1s in its chunk of plane
// blockIdx.y with 16-byte loads (byte tail scalar), adds them to counts[plane] and raises
// max_label.
__global__ void __launch_bounds__(256) k_label_stats(const uint8_t* __restrict__ labels, long long plane_bytes,
                                                      unsigned long long* __restrict__ counts,
                                                      int32_t* __restrict__ max_label) {
    const long long plane = blockIdx.y;
    const uint8_t* base = labels + plane * plane_bytes;
    // 16-byte groups of this plane (the plane may start unaligned: peel to the first boundary)
    const long long mis = (long long)((16 - ((uintptr_t)base & 15)) & 15);
    const long long head = mis < plane_bytes ? mis : plane_bytes;
    const long long n16 = (plane_bytes - head) / 16;
    const uint4* v = reinterpret_cast<const uint4*>(base + head);
    unsigned int ones = 0;
    uint32_t mxv = 0;  // per-byte running maximum
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n16; i += (long long)gridDim.x * blockDim.x) {
        const uint4 q = v[i];
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            ones += __popc(__vcmpeq4(w[k], 0x01010101u)) >> 3;  // 0xff per byte equal to 1
            mxv = __vmaxu4(mxv, w[k]);
        }
    }
    unsigned int mx = max(max(mxv & 0xffu, (mxv >> 8) & 0xffu), max((mxv >> 16) & 0xffu, mxv >> 24));
    // scalar head and tail bytes, by the first CTA of the plane
    if (blockIdx.x == 0) {
        const long long tail0 = head + n16 * 16;
        for (long long i = threadIdx.x; i < head + (plane_bytes - tail0); i += blockDim.x) {
            const long long j = i < head ? i : tail0 + (i - head);
            const unsigned int b = base[j];
            ones += b == 1u;
            mx = max(mx, b);
        }
    }
    for (int o = 16; o; o >>= 1) {
        ones += __shfl_down_sync(0xffffffffu, ones, o);
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    __shared__ unsigned int s_ones[8], s_mx[8];
    if ((threadIdx.x & 31) == 0) {
        s_ones[threadIdx.x >> 5] = ones;
        s_mx[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = 0, m = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            t += s_ones[i];
            m = max(m, s_mx[i]);
        }
        if (t) atomicAdd(&counts[plane], (unsigned long long)t);
        atomicMax(max_label, (int)m);
    }
}

}  // namespace tf

using namespace tf;

extern "C" int tf_label_stats(int batch, int nx, int ny, int nz, const uint8_t* labels_dev, uint64_t* plane_counts_dev,
                              int32_t* max_label_dev, void* stream) {
    if (batch < 1 || nx < 1 || ny < 1 || nz < 1 || !labels_dev || !plane_counts_dev || !max_label_dev)
        return TF_ERR_ARG;
    const long long planes = (long long)batch * nx;
    if (planes > 65535) return TF_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    const long long plane_bytes = (long long)ny * nz;
    if (cudaMemsetAsync(plane_counts_dev, 0, sizeof(uint64_t) * planes, st) != cudaSuccess) return TF_ERR_CUDA;
    if (cudaMemsetAsync(max_label_dev, 0, sizeof(int32_t), st) != cudaSuccess) return TF_ERR_CUDA;
    // enough CTAs per plane to cover the machine a few times over, at most one per 4 KB
    long long per_plane = (4LL * sm_count() * 8 + planes - 1) / planes;
    const long long cap = (plane_bytes + 4095) / 4096;
    if (per_plane > cap) per_plane = cap;
    if (per_plane < 1) per_plane = 1;
    k_label_stats<<<dim3((unsigned)per_plane, (unsigned)planes), 256, 0, st>>>(
        labels_dev, plane_bytes, (unsigned long long*)plane_counts_dev, max_label_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

// Per-voxel conductivity statistics (KappaSolver set-up): per plane the count of kappa > 0 and the
// float64 sum of kappa, and a flag for any value that is negative, infinite or NaN. One CTA per
// plane with a fixed-order reduction, so the sums do not depend on scheduling.
namespace tf {

__global__ void __launch_bounds__(256) k_kappa_stats(const float* __restrict__ kappa, long long plane_elems,
                                                      unsigned long long* __restrict__ positive,
                                                      double* __restrict__ sums, int32_t* __restrict__ bad) {
    const long long plane = blockIdx.x;
    const float* base = kappa + plane * plane_elems;
    unsigned int npos = 0;
    double s = 0.0;
    int badf = 0;
    for (long long i = threadIdx.x; i < plane_elems; i += blockDim.x) {
        const float k = base[i];
        badf |= !(k >= 0.0f) || isinf(k);
        npos += k > 0.0f;
        s += (double)k;
    }
    for (int o = 16; o; o >>= 1) {
        npos += __shfl_down_sync(0xffffffffu, npos, o);
        s += __shfl_down_sync(0xffffffffu, s, o);
        badf |= __shfl_down_sync(0xffffffffu, badf, o);
    }
    __shared__ unsigned int s_pos[8];
    __shared__ double s_sum[8];
    __shared__ int s_bad[8];
    if ((threadIdx.x & 31) == 0) {
        s_pos[threadIdx.x >> 5] = npos;
        s_sum[threadIdx.x >> 5] = s;
        s_bad[threadIdx.x >> 5] = badf;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long p = 0;
        double t = 0.0;
        int b = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            p += s_pos[i];
            t += s_sum[i];
            b |= s_bad[i];
        }
        positive[plane] = p;
        sums[plane] = t;
        if (b) atomicOr(bad, 1);
    }
}

}  // namespace tf

extern "C" int tf_kappa_stats(int batch, int nx, int ny, int nz, const float* kappa_dev, uint64_t* plane_positive_dev,
                              double* plane_sums_dev, int32_t* bad_dev, void* stream) {
    if (batch < 1 || nx < 1 || ny < 1 || nz < 1 || !kappa_dev || !plane_positive_dev || !plane_sums_dev || !bad_dev)
        return TF_ERR_ARG;
    const long long planes = (long long)batch * nx;
    if (planes > 0x7fffffffLL) return TF_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(bad_dev, 0, sizeof(int32_t), st) != cudaSuccess) return TF_ERR_CUDA;
    k_kappa_stats<<<(unsigned)planes, 256, 0, st>>>(kappa_dev, (long long)ny * nz,
                                                   (unsigned long long*)plane_positive_dev, plane_sums_dev, bad_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

// Per-voxel lookup of a 256-entry float32 table by uint8 label (MultiPhaseSolver.phase_gradients:
// the conductivity field kappa = D[label]), and per-plane float64 sums of a field over the voxels
// of each label (the per-label sums of dD_eff/dkappa). One thread per voxel in a grid-stride loop
// for the lookup; one CTA per plane for the sums, four label slots per pass accumulated in
// registers and reduced by shuffles and a fixed warp order, so the sums do not depend on
// scheduling.
namespace tf {

__global__ void __launch_bounds__(256) k_label_map(const uint8_t* __restrict__ labels, long long n,
                                                   const float* __restrict__ table, float* __restrict__ out) {
    __shared__ float s_t[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_t[i] = table[i];
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = s_t[labels[i]];
}

__global__ void __launch_bounds__(256) k_label_sums(const uint8_t* __restrict__ labels,
                                                    const double* __restrict__ values, long long plane_elems,
                                                    const int32_t* __restrict__ slot_of, int n_slots,
                                                    double* __restrict__ sums) {
    __shared__ int s_slot[256];
    __shared__ double s_red[8][4];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_slot[i] = slot_of[i];
    __syncthreads();
    const long long plane = blockIdx.x;
    const uint8_t* lab = labels + plane * plane_elems;
    const double* val = values + plane * plane_elems;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int s0 = 0; s0 < n_slots; s0 += 4) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (long long i = threadIdx.x; i < plane_elems; i += blockDim.x) {
            const int k = s_slot[lab[i]] - s0;
            const double v = val[i];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (k == j) acc[j] += v;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_down_sync(0xffffffffu, acc[j], o);
            if (lane == 0) s_red[warp][j] = acc[j];
        }
        __syncthreads();
        if (threadIdx.x < 4 && s0 + (int)threadIdx.x < n_slots) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w][threadIdx.x];
            sums[plane * n_slots + s0 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

}  // namespace tf

extern "C" int tf_label_map(const uint8_t* labels_dev, long long n, const float* table_dev, float* out_dev,
                            void* stream) {
    if (n < 1 || !labels_dev || !table_dev || !out_dev) return TF_ERR_ARG;
    const long long blocks = (n + 255) / 256 < 16LL * sm_count() ? (n + 255) / 256 : 16LL * sm_count();
    k_label_map<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(labels_dev, n, table_dev, out_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

extern "C" int tf_label_sums(int batch, int nx, int ny, int nz, const uint8_t* labels_dev, const double* values_dev,
                             const int32_t* slot_of_dev, int n_slots, double* plane_sums_dev, void* stream) {
    if (batch < 1 || nx < 1 || ny < 1 || nz < 1 || n_slots < 1 || n_slots > 256 || !labels_dev || !values_dev ||
        !slot_of_dev || !plane_sums_dev)
        return TF_ERR_ARG;
    const long long planes = (long long)batch * nx;
    if (planes > 0x7fffffffLL) return TF_ERR_UNSUPPORTED;
    k_label_sums<<<(unsigned)planes, 256, 0, (cudaStream_t)stream>>>(labels_dev, values_dev, (long long)ny * nz,
                                                                      slot_of_dev, n_slots, plane_sums_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}
