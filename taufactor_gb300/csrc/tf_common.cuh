// Shared definitions of the taufactor_gb300 kernels (sm_103a).
//
// Layout ("z-parity split"): voxel (x, y, z) of volume b is stored at
//   field[((b*nx + x)*yp + (y + HY))*2*zh + (z & 1)*zh + (z >> 1) + HJ]
// i.e. each (b, x, y) row holds the even-z half-row followed by the odd-z half-row, each padded
// by HJ ghost cells on both sides; each x-plane has HY ghost rows on both y sides. In a
// red-black sweep every cell of one half-row has the same colour, and a cell's x and y
// neighbours sit at the same position of the same half-row of the adjacent plane/row, so a
// float4 of one half-row is four updates whose x/y neighbours are four-wide loads too.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/taufactor_gb300.h"

namespace tf {

constexpr int HY = TF_MAX_HALF_SWEEPS;  // ghost rows per y side
constexpr int HJ = 4;                   // ghost cells per side of each half-row (one float4)

struct Geo {
    int B, NX, NY, NZ, YP, ZH, ZHC;
    long long row_f, plane_f, vol_f;  // float strides
    long long row_c, plane_c, vol_c;  // byte strides of the code buffer
};

inline Geo make_geo(const tf_geom& g) {
    Geo o;
    o.B = g.batch; o.NX = g.nx; o.NY = g.ny; o.NZ = g.nz; o.YP = g.yp; o.ZH = g.zh; o.ZHC = g.zhc;
    o.row_f = 2LL * g.zh; o.plane_f = o.row_f * g.yp; o.vol_f = o.plane_f * g.nx;
    o.row_c = 2LL * g.zhc; o.plane_c = o.row_c * g.yp; o.vol_c = o.plane_c * g.nx;
    return o;
}

// Number of valid (interior) cells in the half-row of parity q.
__host__ __device__ __forceinline__ int half_len(int nz, int q) { return q ? (nz >> 1) : ((nz + 1) >> 1); }

__host__ __device__ __forceinline__ int wrap(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

// ---------------------------------------------------------------- PTX helpers (TMA, mbarrier)
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory accesses before later async-proxy (TMA)
// accesses of the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase: gives up after ~2^31 SM cycles (about a second).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > (1LL << 31)) return false;
    }
    return true;
}

// 3-D tiled TMA load (global -> this CTA's shared memory), completion counted on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}

// ---------------------------------------------------------------- arithmetic of one update
// The reference evaluates (taufactor.py:176-181), per voxel and in float32 with one rounding
// per operation: inc = sum / div; inc -= c; inc *= omega; c += inc. The _rn intrinsics keep
// the compiler from contracting the multiply-add into an FMA.
__device__ __forceinline__ float sor_finish(float c, float quot, float omega) {
    float inc = __fsub_rn(quot, c);
    inc = __fmul_rn(inc, omega);
    return __fadd_rn(c, inc);
}

// sum / div for an arbitrary positive divisor, inf allowed. A finite sum over an infinite
// divisor is a signed zero, and 0 / div is a signed zero; both are returned without dividing,
// which keeps the division on its fast path.
__device__ __forceinline__ float quotient(float sum, float div) {
    if (div == __int_as_float(0x7f800000) || sum == 0.0f) return __fmul_rn(sum, 0.0f);
    return __fdiv_rn(sum, div);
}

// Correctly rounded sum / n for n in 1..8 given r = RN(1/n): one multiply and two fused
// multiply-adds (Brisebarre, Muller, Raina, "Accelerating correctly rounded floating-point
// division when the divisor is known in advance", IEEE Trans. Computers 53(8), 2004):
// q = RN(s*r); e = s - q*n (exact by FMA); result = RN(q + e*r), or q itself when e is 0
// (q is then exact, and returning it keeps the sign of a zero quotient). For these divisors the
// result equals IEEE division for finite float32 s with |s| >= 2^-90 (below that the product
// e*r may underflow); div_small_exact() adds IEEE division for the tiny range.
// tf_check_small_division() verifies div_small_exact exhaustively against the hardware division
// on the GPU. (Infinite s never occurs: the dividend is a sum of finite field values.)
__device__ __forceinline__ float div_small(float s, float n, float r) {
    const float q = __fmul_rn(s, r);
    const float e = __fmaf_rn(-q, n, s);
    return e == 0.0f ? q : __fmaf_rn(e, r, q);
}

// div_small without the zero test, as the binary sweeps use it: RN(q + e*r) also when e == 0.
// It differs from IEEE division only for s = -0 (it returns +0 instead of -0), and the SOR step
// c + omega * (quot - c) gives the same float32 bits for either zero quotient (quot - c is -c
// for c != 0, and a zero c ends as +0 both ways), so the field stays bit-exact.
__device__ __forceinline__ float div_small_fast(float s, float n, float r) {
    const float q = __fmul_rn(s, r);
    return __fmaf_rn(__fmaf_rn(-q, n, s), r, q);
}

// div_small with the tiny-dividend fallback: exact for every finite s.
__device__ __forceinline__ float div_small_exact(float s, float n, float r) {
    return (s != 0.0f && fabsf(s) < 0x1p-90f) ? __fdiv_rn(s, n) : div_small(s, n, r);
}

}  // namespace tf
