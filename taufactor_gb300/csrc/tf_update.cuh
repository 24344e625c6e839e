// Per-voxel update arithmetic shared by the sweep kernels (sm_103a).
#pragma once

#include "tf_common.cuh"

namespace tf {

struct SweepArgs {
    Geo g;
    float* out;
    float omega, glo, ghi, ky, kz;
    int first_colour, n_half, periodic;
    int x_chunks;      // x-chunks per tile column of the fused sweep (grid z = batch * x_chunks)
    int32_t* err;
    const float* rhs;  // right-hand side of a correction solve (split layout), or null
};

SweepArgs make_args(const Geo& g, const tf_operator& op, float* out, int first_colour, int n_half, int32_t* err);

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float comp(const float4& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set_comp(float4& v, int i, float f) {
    if (i == 0) v.x = f; else if (i == 1) v.y = f; else if (i == 2) v.z = f; else v.w = f;
}
__device__ __forceinline__ uint32_t byte_of(uint32_t w, int i) { return (w >> (8 * i)) & 0xffu; }
__device__ __forceinline__ uint32_t ld_u32(const unsigned char* p) { return *reinterpret_cast<const uint32_t*>(p); }

// Binary division table: entry n = (n, RN(1/n)) for n = 1..8, entry 0 = (1, 0).
__device__ __forceinline__ void fill_division_table(float2* tab, int tid) {
    if (tid < 16) tab[tid] = tid == 0 ? make_float2(1.0f, 0.0f)
                           : make_float2(static_cast<float>(tid), __frcp_rn(static_cast<float>(tid)));
}

// Quotients sum / n by IEEE division, for the (rare) group in which some |sum| < 2^-90; kept
// out of line so the sweeps' hot code stays small.
static __device__ __noinline__ float4 tiny_quotients(float4 sum, float4 n, float4 r) {
    float4 q;
    q.x = r.x == 0.0f ? __fmul_rn(sum.x, 0.0f) : __fdiv_rn(sum.x, n.x);
    q.y = r.y == 0.0f ? __fmul_rn(sum.y, 0.0f) : __fdiv_rn(sum.y, n.y);
    q.z = r.z == 0.0f ? __fmul_rn(sum.z, 0.0f) : __fdiv_rn(sum.z, n.z);
    q.w = r.w == 0.0f ? __fmul_rn(sum.w, 0.0f) : __fdiv_rn(sum.w, n.w);
    return q;
}

#define TF_LANES(OP) OP(x) OP(y) OP(z) OP(w)

// Binary / periodic update of a float4 group, written lane-interleaved so the four dependency
// chains overlap: sum in the order of taufactor.py:97-102 (x+1, x-1, y+1, y-1, z+1, z-1),
// exact division by the neighbour count (table entry (n, RN(1/n)); code 0 -> (1, 0) gives the
// reference's sum/inf = signed zero), then inc = q - c; inc *= omega; c += inc (:177-181).
template <bool RHS>
__device__ __forceinline__ float4 update4_binary(float4 c, const float4& xp, const float4& xm, const float4& yp,
                                                 const float4& ym, const float4& zp, const float4& zm, uint32_t cc,
                                                 float omega, const float2* tab, const float4& rv) {
    float4 s, n, r, q;
#define TF_S1(L) s.L = __fadd_rn(xp.L, xm.L);
#define TF_S2(L) s.L = __fadd_rn(s.L, yp.L);
#define TF_S3(L) s.L = __fadd_rn(s.L, ym.L);
#define TF_S4(L) s.L = __fadd_rn(s.L, zp.L);
#define TF_S5(L) s.L = __fadd_rn(s.L, zm.L);
    TF_LANES(TF_S1) TF_LANES(TF_S2) TF_LANES(TF_S3) TF_LANES(TF_S4) TF_LANES(TF_S5)
    if (RHS) {
#define TF_S6(L) s.L = __fadd_rn(s.L, rv.L);
        TF_LANES(TF_S6)
#undef TF_S6
    }
    const float2 t0 = tab[cc & 0xffu], t1 = tab[(cc >> 8) & 0xffu], t2 = tab[(cc >> 16) & 0xffu], t3 = tab[cc >> 24];
    n = make_float4(t0.x, t1.x, t2.x, t3.x);
    r = make_float4(t0.y, t1.y, t2.y, t3.y);
#define TF_Q(L) q.L = div_small_fast(s.L, n.L, r.L);
    TF_LANES(TF_Q)
    // 0 < |sum| < 2^-90: the correction term can underflow, take IEEE division (never in practice;
    // a zero sum is exact on the fast path)
    const float tiny = 0x1p-90f;
    const float m = fminf(fminf(fabsf(s.x) == 0.0f ? 1.0f : fabsf(s.x), fabsf(s.y) == 0.0f ? 1.0f : fabsf(s.y)),
                          fminf(fabsf(s.z) == 0.0f ? 1.0f : fabsf(s.z), fabsf(s.w) == 0.0f ? 1.0f : fabsf(s.w)));
    if (m < tiny) q = tiny_quotients(s, n, r);
#define TF_F1(L) q.L = __fsub_rn(q.L, c.L);
#define TF_F2(L) q.L = __fmul_rn(q.L, omega);
#define TF_F3(L) c.L = __fadd_rn(c.L, q.L);
    TF_LANES(TF_F1) TF_LANES(TF_F2) TF_LANES(TF_F3)
#undef TF_S1
#undef TF_S2
#undef TF_S3
#undef TF_S4
#undef TF_S5
#undef TF_Q
#undef TF_F1
#undef TF_F2
#undef TF_F3
    return c;
}

// One float4 group of a colour-c half-row: 4 updates.
//   c        the 4 cells; xp/xm/yp/ym their x+1, x-1, y+1, y-1 neighbours;
//   zp/zm    their z+1, z-1 neighbours; codes: 4 code bytes of the cells and of each neighbour
//            set (multiphase needs them for the faces); at_lo/at_hi: plane is x = 0 / x = nx-1.
//   lut      anisotropic: divisor per code; multiphase: face table [32][32];
//   tab      binary: (n, RN(1/n)) per code n = 1..8; entry 0 = (1, 0) makes the quotient of a
//            frozen voxel (the reference's inf divisor) a signed zero without a branch.
template <int KIND, bool RHS = false>
__device__ __forceinline__ float4 update4(float4 c, const float4& xp, const float4& xm, const float4& yp,
                                          const float4& ym, const float4& zp, const float4& zm, uint32_t cc,
                                          uint32_t cxp, uint32_t cxm, uint32_t cyp, uint32_t cym, uint32_t czp,
                                          uint32_t czm, bool at_lo, bool at_hi, float omega, float ky, float kz,
                                          const float* lut, const float2* tab,
                                          const float4& rv = make_float4(0.f, 0.f, 0.f, 0.f)) {
    if (KIND == TF_KIND_BINARY) return update4_binary<RHS>(c, xp, xm, yp, ym, zp, zm, cc, omega, tab, rv);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float ci = comp(c, i);
        float sum, quot;
        if (KIND == TF_KIND_BINARY) {
            // sum order of taufactor.py:97-102: x+1, x-1, y+1, y-1, z+1, z-1
            sum = __fadd_rn(comp(xp, i), comp(xm, i));
            sum = __fadd_rn(sum, comp(yp, i));
            sum = __fadd_rn(sum, comp(ym, i));
            sum = __fadd_rn(sum, comp(zp, i));
            sum = __fadd_rn(sum, comp(zm, i));
            const float2 nr = tab[byte_of(cc, i)];
            quot = div_small(sum, nr.x, nr.y);
            // below 2^-90 the correction term can underflow; take IEEE division there
            if (fabsf(sum) < 0x1p-90f) quot = nr.y == 0.0f ? __fmul_rn(sum, 0.0f) : __fdiv_rn(sum, nr.x);
        } else if (KIND == TF_KIND_ANISOTROPIC) {
            // taufactor.py:475-477: (x+1 + x-1) + Ky*(y+1 + y-1) + Kz*(z+1 + z-1)
            sum = __fadd_rn(comp(xp, i), comp(xm, i));
            sum = __fadd_rn(sum, __fmul_rn(ky, __fadd_rn(comp(yp, i), comp(ym, i))));
            sum = __fadd_rn(sum, __fmul_rn(kz, __fadd_rn(comp(zp, i), comp(zm, i))));
            if (RHS) sum = __fadd_rn(sum, comp(rv, i));
            quot = quotient(sum, lut[byte_of(cc, i)]);
        } else {
            // taufactor.py:607-612 (products first, then left-to-right sum) and the factor of
            // :598-603 (lower x face, upper x face, y lower/upper, z lower/upper, +boundary faces).
            const uint32_t a = byte_of(cc, i);
            const float* row = lut + a * 32;
            const float fxp = at_hi ? row[a] : row[byte_of(cxp, i)];
            const float fxm = at_lo ? row[a] : row[byte_of(cxm, i)];
            const float fyp = row[byte_of(cyp, i)];
            const float fym = row[byte_of(cym, i)];
            const float fzp = row[byte_of(czp, i)];
            const float fzm = row[byte_of(czm, i)];
            sum = __fadd_rn(__fmul_rn(comp(xp, i), fxp), __fmul_rn(comp(xm, i), fxm));
            sum = __fadd_rn(sum, __fmul_rn(comp(yp, i), fyp));
            sum = __fadd_rn(sum, __fmul_rn(comp(ym, i), fym));
            sum = __fadd_rn(sum, __fmul_rn(comp(zp, i), fzp));
            sum = __fadd_rn(sum, __fmul_rn(comp(zm, i), fzm));
            if (RHS) sum = __fadd_rn(sum, comp(rv, i));
            float div = __fadd_rn(fxm, fxp);
            div = __fadd_rn(div, fym);
            div = __fadd_rn(div, fyp);
            div = __fadd_rn(div, fzm);
            div = __fadd_rn(div, fzp);
            if (at_lo) div = __fadd_rn(div, fxm);
            if (at_hi) div = __fadd_rn(div, fxp);
            if (div == 0.0f) div = __int_as_float(0x7f800000);
            quot = quotient(sum, div);
        }
        set_comp(c, i, sor_finish(ci, quot, omega));
    }
    return c;
}

// z-neighbours of the 4 cells of a half-row group from the other-parity half-row.
// Even half-row (q = 0), cell j: z-1 = odd[j-1], z+1 = odd[j]. Odd (q = 1): z-1 = even[j],
// z+1 = even[j+1]. `o` = other[j..j+3]; `e` = other[j-1] (q = 0) or other[j+4] (q = 1).
__device__ __forceinline__ void z_neighbours(int q, const float4& o, float e, float4& zp, float4& zm) {
    if (q == 0) {
        zm = make_float4(e, o.x, o.y, o.z);
        zp = o;
    } else {
        zm = o;
        zp = make_float4(o.y, o.z, o.w, e);
    }
}
__device__ __forceinline__ void z_codes(int q, uint32_t o, uint32_t e, uint32_t& czp, uint32_t& czm) {
    if (q == 0) {
        czm = (o << 8) | (e & 0xffu);
        czp = o;
    } else {
        czm = o;
        czp = (o >> 8) | ((e & 0xffu) << 24);
    }
}

}  // namespace tf
