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
    // KIND_FACES: the packed per-voxel faces and factor (k_kappa_face_pack's layout), else null
    const float *fx, *fy, *fz, *dv;
};

// Internal operator kind of the fused sweep: per-voxel faces and factor read from the packed
// arrays of SweepArgs instead of derived from codes (the per-voxel conductivity operator, and
// MultiPhaseSolver's with kappa = D[label]).
constexpr int KIND_FACES = 16;

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

// Two float32 values in one 64-bit register pair, for the packed f32x2 instructions of
// sm_100+ (each lane rounds exactly like the scalar instruction). Never feed mul2 into add2 or
// sub2 where the product's own rounding matters: the assembler may fuse that pair.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(f32x2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Binary division table for two cells at once: pair e = lo * 9 + hi of neighbour counts lo, hi
// in 0..8 holds (-n_lo, -n_hi, RN(1/n_lo), RN(1/n_hi)) with n = count, except count 0 -> n = 1,
// 1/n = 0 (a frozen voxel: the reference's division by inf). Each pair is stored 8 times
// (float4 at e * 8 + lane % 8), so the 8 threads of one phase of a 128-bit shared load always
// hit different banks. 81 * 8 float4 = 10368 bytes. Counts are masked to 4 bits before the
// lookup, which keeps any index inside the CTA's shared memory.
constexpr int DIV_PAIRS = 81;
constexpr int DIV_COPIES = 8;
constexpr int DIV_TABLE_BYTES = DIV_PAIRS * DIV_COPIES * 16;
__device__ __forceinline__ void fill_division_table(float4* tab, int tid, int nthreads) {
    for (int i = tid; i < DIV_PAIRS * DIV_COPIES; i += nthreads) {
        const int e = i / DIV_COPIES, lo = e / 9, hi = e - 9 * (e / 9);
        const float nl = lo ? static_cast<float>(lo) : 1.0f, nh = hi ? static_cast<float>(hi) : 1.0f;
        tab[i] = make_float4(-nl, -nh, lo ? __frcp_rn(nl) : 0.0f, hi ? __frcp_rn(nh) : 0.0f);
    }
}
// Electrode operator: the divisor of every code of one volume into lut[0..255]. code = 1 + nn +
// 8 nr (0: not conductive); factor nn + nr * k_0 in float32 as the reference forms it
// (electrode.py:46-62, taufactor.py:47-55), inf where it is 0 or the voxel is not conductive.
__device__ __forceinline__ void fill_electrode_divisors(float* lut, float k0, int tid, int nthreads) {
    for (int i = tid; i < 256; i += nthreads) {
        float d = __int_as_float(0x7f800000);
        if (i != 0) {
            const uint32_t m = (uint32_t)i - 1u;
            const float f = __fadd_rn(static_cast<float>(m & 7u), __fmul_rn(static_cast<float>(m >> 3), k0));
            if (f != 0.0f) d = f;
        }
        lut[i] = d;
    }
}
// This thread's copy of the table (copy lane % 8).
__device__ __forceinline__ const float4* division_copy(const float4* tab) { return tab + (threadIdx.x & 7); }

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

// Binary / periodic update of a float4 group as two packed lane pairs (x, y) and (z, w): sum
// in the order of taufactor.py:97-102 (x+1, x-1, y+1, y-1, z+1, z-1), exact division by the
// neighbour count (div_small_fast with the pair table; count 0 gives the reference's
// sum/inf = signed zero), then inc = q - c; inc *= omega; c += inc (:177-181). Every packed
// instruction rounds each lane like its scalar counterpart, so the result is the scalar one.
// `tab` is this thread's copy of the division table (division_copy).
template <bool RHS>
__device__ __forceinline__ float4 update4_binary(float4 c, const float4& xp, const float4& xm, const float4& yp,
                                                 const float4& ym, const float4& zp, const float4& zm, uint32_t cc,
                                                 float omega, const float4* tab, const float4& rv) {
    f32x2 s0 = add2(pk2(xp.x, xp.y), pk2(xm.x, xm.y));
    f32x2 s1 = add2(pk2(xp.z, xp.w), pk2(xm.z, xm.w));
    s0 = add2(s0, pk2(yp.x, yp.y));
    s1 = add2(s1, pk2(yp.z, yp.w));
    s0 = add2(s0, pk2(ym.x, ym.y));
    s1 = add2(s1, pk2(ym.z, ym.w));
    s0 = add2(s0, pk2(zp.x, zp.y));
    s1 = add2(s1, pk2(zp.z, zp.w));
    s0 = add2(s0, pk2(zm.x, zm.y));
    s1 = add2(s1, pk2(zm.z, zm.w));
    if (RHS) {
        s0 = add2(s0, pk2(rv.x, rv.y));
        s1 = add2(s1, pk2(rv.z, rv.w));
    }
    // pair index 9 lo + hi of the 4-bit-masked counts, one byte dot product per pair
    const int cm = static_cast<int>(cc & 0x0f0f0f0fu);
    const float4 t0 = tab[__dp4a(cm, 0x00000109, 0) * DIV_COPIES];
    const float4 t1 = tab[__dp4a(cm, 0x01090000, 0) * DIV_COPIES];
    const f32x2 r0 = pk2(t0.z, t0.w), r1 = pk2(t1.z, t1.w);
    f32x2 q0 = mul2(s0, r0), q1 = mul2(s1, r1);
    q0 = fma2(fma2(q0, pk2(t0.x, t0.y), s0), r0, q0);
    q1 = fma2(fma2(q1, pk2(t1.x, t1.y), s1), r1, q1);
    // 0 < |sum| <= 2^-90: the correction term can underflow, take IEEE division (never in
    // practice; a zero sum is exact on the fast path). Each lane's bit pattern minus one is
    // |sum| less one ulp in magnitude, or a NaN for +-0, which fminf skips.
    float4 s;
    upk2(s0, s.x, s.y);
    upk2(s1, s.z, s.w);
    const float m = fminf(fminf(fabsf(__int_as_float(__float_as_int(s.x) - 1)), fabsf(__int_as_float(__float_as_int(s.y) - 1))),
                          fminf(fabsf(__int_as_float(__float_as_int(s.z) - 1)), fabsf(__int_as_float(__float_as_int(s.w) - 1))));
    if (m < 0x1p-90f) {
        const float4 q = tiny_quotients(s, make_float4(-t0.x, -t0.y, -t1.x, -t1.y), make_float4(t0.z, t0.w, t1.z, t1.w));
        q0 = pk2(q.x, q.y);
        q1 = pk2(q.z, q.w);
    }
    // inc * omega with scalar mul.rn: a packed multiply feeding the packed add below can be
    // merged into one fused operation by the assembler (its .rn does not prevent that), which
    // would skip the rounding of the product; scalar mul.rn is never contracted
    const f32x2 c0 = pk2(c.x, c.y), c1 = pk2(c.z, c.w);
    float i0, i1, i2, i3;
    upk2(sub2(q0, c0), i0, i1);
    upk2(sub2(q1, c1), i2, i3);
    q0 = add2(c0, pk2(__fmul_rn(i0, omega), __fmul_rn(i1, omega)));
    q1 = add2(c1, pk2(__fmul_rn(i2, omega), __fmul_rn(i3, omega)));
    upk2(q0, c.x, c.y);
    upk2(q1, c.z, c.w);
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
                                          const float* lut, const float4* tab,
                                          const float4& rv = make_float4(0.f, 0.f, 0.f, 0.f)) {
    if (KIND == TF_KIND_BINARY) return update4_binary<RHS>(c, xp, xm, yp, ym, zp, zm, cc, omega, tab, rv);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float ci = comp(c, i);
        float sum, quot;
        if (KIND == TF_KIND_ELECTRODE) {
            // the default neighbour sum (taufactor.py:95-103) over the divisor
            // factor = nn + nr * k_0 in float32, inf where 0 (:47-55, electrode.py:46-62),
            // looked up by code in lut (fill_electrode_divisors)
            sum = __fadd_rn(comp(xp, i), comp(xm, i));
            sum = __fadd_rn(sum, comp(yp, i));
            sum = __fadd_rn(sum, comp(ym, i));
            sum = __fadd_rn(sum, comp(zp, i));
            sum = __fadd_rn(sum, comp(zm, i));
            if (RHS) sum = __fadd_rn(sum, comp(rv, i));
            // lut[code]: the divisor nn + nr * k_0 of the code, inf where 0 or not conductive
            quot = quotient(sum, lut[byte_of(cc, i)]);
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

// One float4 group from packed faces: k_kappa_sweep4's arithmetic (taufactor.py:607-612, products
// then the left-to-right sum, over the packed factor; inf where frozen), so the same bits.
template <bool RHS>
__device__ __forceinline__ float4 update4_faces(float4 c, const float4& xp, const float4& xm, const float4& yp,
                                                const float4& ym, const float4& zp, const float4& zm,
                                                const float4& fxp, const float4& fxm, const float4& fyp,
                                                const float4& fym, const float4& fzp, const float4& fzm,
                                                const float4& d, float omega, const float4& rv) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float s = __fadd_rn(__fmul_rn(comp(xp, i), comp(fxp, i)), __fmul_rn(comp(xm, i), comp(fxm, i)));
        s = __fadd_rn(s, __fmul_rn(comp(yp, i), comp(fyp, i)));
        s = __fadd_rn(s, __fmul_rn(comp(ym, i), comp(fym, i)));
        s = __fadd_rn(s, __fmul_rn(comp(zp, i), comp(fzp, i)));
        s = __fadd_rn(s, __fmul_rn(comp(zm, i), comp(fzm, i)));
        if (RHS) s = __fadd_rn(s, comp(rv, i));
        set_comp(c, i, sor_finish(comp(c, i), quotient(s, comp(d, i)), omega));
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
