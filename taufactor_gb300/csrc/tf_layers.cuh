// Per-plane reductions shared by the single-volume and batched layer-sum kernels.
#pragma once

#include "tf_common.cuh"
#include "tf_update.cuh"

namespace tf {

// Float64 sums over plane x of one volume (f0 / c0 point at plane x) of the x-flux through face
// x|x+1 and of the field, accumulated by this thread over its share of float4 groups. Flux per
// cell as the reference takes it: binary c[x+1]-c[x] where both voxels are updated (divisor <= 8,
// taufactor.py:412-419); anisotropic the same test on the divisor table (which also drops finite
// divisors above 8, :417-418); multiphase face * (c[x+1]-c[x]) (:615-620). The (up to) four cells
// of a group are summed in float32 first (differences and products are float32 in the reference
// too) and then added in float64; the order is fixed, so results do not depend on scheduling.
template <int KIND>
__device__ __forceinline__ void plane_partials(const float* __restrict__ f0, const uint8_t* __restrict__ c0,
                                               const Geo& g, bool has_flux, const float* lut, double& fs,
                                               double& cs) {
    const int gm = (half_len(g.NZ, 0) + 3) >> 2;
    for (int it = threadIdx.x; it < g.NY * 2 * gm; it += blockDim.x) {
        const int gi = it % gm;
        const int r = it / gm;
        const int y = r >> 1, q = r & 1;
        const int nj = half_len(g.NZ, q);
        const int j = 4 * gi;
        if (j >= nj) continue;
        const long long off = (long long)(y + HY) * g.row_f + q * g.ZH + HJ + j;
        const long long offc = (long long)(y + HY) * g.row_c + q * g.ZHC + HJ + j;
        const float4 a = ld4(f0 + off);
        const int n = nj - j < 4 ? nj - j : 4;
        float pc = 0.0f, pf = 0.0f;
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (i < n) pc = __fadd_rn(pc, comp(a, i));
        if (has_flux) {
            const float4 bb = ld4(f0 + g.plane_f + off);
            const uint32_t ca = ld_u32(c0 + offc), cb = ld_u32(c0 + g.plane_c + offc);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (i >= n) continue;
                const float d = __fsub_rn(comp(bb, i), comp(a, i));
                const uint32_t ka = byte_of(ca, i), kb = byte_of(cb, i);
                if (KIND == TF_KIND_MULTIPHASE) pf = __fadd_rn(pf, __fmul_rn(lut[ka * 32 + kb], d));
                else if (KIND == TF_KIND_ANISOTROPIC) pf = (lut[ka] <= 8.0f && lut[kb] <= 8.0f) ? __fadd_rn(pf, d) : pf;
                else pf = (ka != 0 && kb != 0) ? __fadd_rn(pf, d) : pf;
            }
        }
        cs += (double)pc;
        fs += (double)pf;
    }
}

// Block-wide sums of two float64 values (blockDim.x a multiple of 32, at most 1024); the result
// is valid in thread 0.
__device__ __forceinline__ void block_sum_pair(double& a, double& b) {
    __shared__ double red[2][32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = a;
        red[1][w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            a += red[0][i];
            b += red[1][i];
        }
    }
}

}  // namespace tf
