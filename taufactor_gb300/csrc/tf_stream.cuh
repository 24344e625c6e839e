// Register-streaming red-black SOR wavefront: K half-sweeps per launch (sm_103a).
//
// Each CTA owns a TY x TZ tile of the (y, z) plane (plus K ghost rows and one ghost float4
// group on each side of every half-row) and marches along x. Planes are staged into a
// shared-memory ring by TMA (cp.async.bulk.tensor + mbarrier, D planes ahead).
//
// One thread per (tile row, float4 group). A thread keeps its own 2 x 4 cells (even-z and odd-z
// half-row groups) of the K+2 planes in flight in registers, indexed by *relative colour*
// (colour XOR the launch's first colour), so half-sweep s of the launch always updates the
// relative-colour (s-1)&1 registers: every register index is a compile-time constant after
// unrolling. Half-sweep s is applied to plane t-s at step t (wavefront in x). x- and z-
// neighbours come from the thread's registers; y-neighbours and the z-edge cell of the
// adjacent group come from the plane's shared-memory slot, where every update is published.
// Within a step no half-sweep reads shared memory written in the same step, so one CTA barrier
// per plane suffices. The region updated by half-sweep s shrinks by one row per half-sweep, so
// the tile interior is exact; it is written from registers to the other ping-pong buffer (plus
// periodic ghost copies). The result is K reference iterations of taufactor.py:174-182,
// bit for bit.
//
// A CTA may own only the planes [x0, x1) of its tile column (x-chunks, to even out the last
// wave of CTAs): it streams planes [x0-K, x1+K) clipped to the volume. Below x0 the missing
// x-1 neighbour corrupts one more plane per half-sweep, i.e. exactly the K margin planes; above
// x1 the margin planes are only read, never needed at a later time. Planes [x0, x1) are exact.
#pragma once

#include <mutex>

#include "tf_common.cuh"
#include "tf_internal.h"
#include "tf_update.cuh"

namespace tf {

template <int TY, int TZ, int K>
struct StreamShape {
    static constexpr int TJ = TZ / 2;                // interior cells per half-row
    static constexpr int G = TJ / 4 + 2;             // float4 groups per staged half-row
    static constexpr int WJ = 4 * G;                 // floats per staged half-row
    static constexpr int WJC = (WJ + 15) / 16 * 16;  // bytes per staged code half-row
    static constexpr int ROWS = TY + 2 * K;          // staged rows: K ghost rows per side
    static constexpr int NT = ROWS * G;              // one thread per (row, group)
    static constexpr int R = K + 2;                  // planes held in registers
    static constexpr int D = 3;                      // planes loaded ahead
    static constexpr int NS = K + 1 + D;             // shared-memory slots
    static constexpr int FBYTES = 2 * ROWS * WJ * 4;
    static constexpr int CBYTES = 2 * ROWS * WJC;
    static constexpr int GUARD = 128;                // readable guard around each field slot
    static constexpr int FSPAN = (GUARD + FBYTES + GUARD + 127) / 128 * 128;
    static constexpr int SLOT = FSPAN + (CBYTES + 127) / 128 * 128;
    // operator table: multiphase faces (4 KB), anisotropic divisors or the binary division table
    static constexpr int LUT_BYTES = (DIV_TABLE_BYTES > 32 * 32 * 4 ? DIV_TABLE_BYTES : 32 * 32 * 4) / 128 * 128 + 128;
    static constexpr int HEAD = 128 + LUT_BYTES + 128;  // mbarriers, LUT (binary: division table)
    static constexpr int SMEM = HEAD + NS * SLOT;
    static_assert(TJ % 16 == 0, "tile z-extent must keep TMA box starts 16-byte aligned for codes");
    static_assert(K >= 1 && K <= HY, "half-sweeps per launch exceed the ghost rows");
};

// Periodic ghost copies of one written float4 group for faces whose half-row length is not a
// multiple of 4 (the common case is handled inline with float4 stores). Out of line.
static __device__ __noinline__ void ghost_copies_scalar(float* outp, long long row_f, int zh, int ny, int nz, int y,
                                                        int q, int j, int nj, float4 v, bool py) {
    const int hz = nz >> 1;
    const int ys = py && y < HY ? y + ny : (py && y >= ny - HY ? y - ny : y);
    for (int pass = 0; pass < (ys != y ? 2 : 1); ++pass) {
        const int yy = pass ? ys : y;
        float* rowp = outp + (long long)(yy + HY) * row_f + q * zh + HJ;
        for (int c = 0; c < 4 && j + c < nj; ++c) {
            const int jc = j + c;
            const float val = comp(v, c);
            if (pass) rowp[jc] = val;
            if (jc < HJ) rowp[jc + hz] = val;
            else if (jc >= hz - HJ) rowp[jc - hz] = val;
        }
    }
}

// Offsets (elements) of one thread's cells within a plane's shared-memory slot for the half-row
// q updated in a step: its own group (`me`; the y-neighbours are me -+ 2 WJ) and the z-edge cell
// of the adjacent group in the other half-row (`e`). The same for every half-sweep of the step.
struct SlotOffsets {
    int me, e;
};
__device__ __forceinline__ SlotOffsets slot_offsets(int ty, int jj, int q, int W) {
    SlotOffsets o;
    o.me = (2 * ty + q) * W + jj;
    o.e = (2 * ty + (q ^ 1)) * W + (q ? jj + 4 : jj - 1);
    return o;
}

// One half-sweep on the thread's float4 group at plane p (relative colour held in `self`).
//   xp/xm: x-neighbour groups (registers; Dirichlet ghost planes are part of the ring);
//   zo: the other half-row group of this plane (registers); y-neighbours and the z-edge cell of
//   the adjacent group are read from the plane's shared-memory slot (field offsets fo, code
//   offsets co), and the result is published there.
__device__ __forceinline__ void prefetch_l2(const float* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// KIND_FACES: the packed faces and factor of a thread's group at global offset `go` (the group's
// first padded cell of half-row 0, or -1 outside the padded plane: no faces, factor inf);
// `ym_ok`: the row above exists in the padded plane; `zm_ok`: the cell before the group does.
struct GroupFaces {
    float4 xp, xm, yp, ym, zp, zm, d;
};
__device__ __forceinline__ GroupFaces load_faces(const SweepArgs& a, long long go, int b, int q, bool ym_ok,
                                                 bool zm_ok) {
    GroupFaces f;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (go < 0) {
        f.xp = f.xm = f.yp = f.ym = f.zp = f.zm = zero4;
        const float inf = __int_as_float(0x7f800000);
        f.d = make_float4(inf, inf, inf, inf);
        return f;
    }
    const Geo& g = a.g;
    const long long o = go + q * g.ZH, oo = go + (q ^ 1) * g.ZH;  // this half-row, the other one
    const long long ox = o + (long long)b * g.plane_f;           // fx plane p: the face to p - 1
    f.xm = __ldg(reinterpret_cast<const float4*>(a.fx + ox));
    f.xp = __ldg(reinterpret_cast<const float4*>(a.fx + ox + g.plane_f));
    f.yp = __ldg(reinterpret_cast<const float4*>(a.fy + o));
    f.ym = ym_ok ? __ldg(reinterpret_cast<const float4*>(a.fy + o - g.row_f)) : zero4;
    f.zp = __ldg(reinterpret_cast<const float4*>(a.fz + o));
    const float4 fo = __ldg(reinterpret_cast<const float4*>(a.fz + oo));
    // the face between z - 1 and z, stored at cell z - 1 (other half-row, j - 1 for q = 0)
    f.zm = q ? fo : make_float4(zm_ok ? __ldg(a.fz + oo - 1) : 0.0f, fo.x, fo.y, fo.z);
    f.d = __ldg(reinterpret_cast<const float4*>(a.dv + o));
    return f;
}

template <int KIND, bool RHS>
__device__ __forceinline__ void stage_update(float4& self, const float4& xp, const float4& xm, const float4& zo,
                                             uint32_t cc, uint32_t cxp, uint32_t cxm, uint32_t czo, float* Fp,
                                             const unsigned char* Cp, SlotOffsets fo, SlotOffsets co, int q, int WJ,
                                             int WJC, bool at_lo, bool at_hi, const SweepArgs& a, const float* lut,
                                             const float4* tab, const float* rhs_row, long long go = -1, int b = 0,
                                             bool ym_ok = false, bool zm_ok = false) {
    // right-hand side of a correction solve (A e = r): the thread's 4 cells, read-only path
    float4 rv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (RHS && rhs_row) rv = __ldg(reinterpret_cast<const float4*>(rhs_row + q * a.g.ZH));
    const float4 yp = ld4(Fp + fo.me + 2 * WJ);
    const float4 ym = ld4(Fp + fo.me - 2 * WJ);
    const float e = Fp[fo.e];
    float4 zp, zm;
    z_neighbours(q, zo, e, zp, zm);
    if (KIND == KIND_FACES) {
        const GroupFaces f = load_faces(a, go, b, q, ym_ok, zm_ok);
        self = update4_faces<RHS>(self, xp, xm, yp, ym, zp, zm, f.xp, f.xm, f.yp, f.ym, f.zp, f.zm, f.d, a.omega, rv);
        st4(Fp + fo.me, self);
        return;
    }
    uint32_t cyp = 0, cym = 0, czp = 0, czm = 0;
    if (KIND == TF_KIND_MULTIPHASE) {
        cyp = ld_u32(Cp + co.me + 2 * WJC);
        cym = ld_u32(Cp + co.me - 2 * WJC);
        // z-edge code: inside the slot for every thread (a halo group may read the edge code of
        // the neighbouring staged row, which only affects halo cells)
        const uint32_t ce = Cp[co.e];
        z_codes(q, czo, ce, czp, czm);
    }
    self = update4<KIND, RHS>(self, xp, xm, yp, ym, zp, zm, cc, cxp, cxm, cyp, cym, czp, czm, at_lo, at_hi, a.omega,
                              a.ky, a.kz, lut, tab, rv);
    st4(Fp + fo.me, self);
}

// The CTA's work: one tile (j0 = first staged padded j, y0 = first interior row, volume b of
// the batch described by `a`, written planes [x0, x1)) for K half-sweeps. `op` may be null for
// the binary operator.
// `tmf` / `tmc` are tensor maps of the input field and the codes (kernel parameter or global
// memory). Shared memory: StreamShape::SMEM bytes at `smem` (128-byte aligned).
template <int KIND, int TY, int TZ, int K, bool RHS>
__device__ __forceinline__ void stream_tile(const CUtensorMap* tmf, const CUtensorMap* tmc, const SweepArgs& a,
                                            const tf_operator* op, int j0, int y0, int b, int x0, int x1,
                                            unsigned char* smem) {
    using S = StreamShape<TY, TZ, K>;
    constexpr int G = S::G, WJ = S::WJ, WJC = S::WJC, NS = S::NS, D = S::D, R = S::R, NT = S::NT;
    constexpr int ROWS = S::ROWS;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    int* s_fail = reinterpret_cast<int*>(smem + 8 * NS);
    float* lut = reinterpret_cast<float*>(smem + 128);
    // binary: the pair division table in the LUT area (the LUT serves the other operators)
    float4* tab_all = reinterpret_cast<float4*>(smem + 128);
    const float4* tab = division_copy(tab_all);
    float* const F0 = reinterpret_cast<float*>(smem + S::HEAD + S::GUARD);
    unsigned char* const C0 = smem + S::HEAD + S::FSPAN;

    const Geo& g = a.g;
    const int tid = threadIdx.x;
    const int ty = tid / G;
    const int gi = tid - ty * G;
    const int jj = 4 * gi;
    const int NX = g.NX;
    const int y = y0 - K + ty;  // interior y of this thread's row (may lie in a ghost band)
    const int row0 = 2 * (y0 + HY - K);  // first staged row of the TMA box (padded coordinates)
    const int c0 = a.first_colour;
    const float4 glo4 = make_float4(a.glo, a.glo, a.glo, a.glo);
    const float4 ghi4 = make_float4(a.ghi, a.ghi, a.ghi, a.ghi);

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
        *s_fail = 0;
    }
    if (KIND == TF_KIND_ANISOTROPIC)
        for (int i = tid; i < 256; i += NT) lut[i] = op->divisor[i];
    if (KIND == TF_KIND_ELECTRODE) fill_electrode_divisors(lut, op->divisor[b & 255], tid, NT);  // k_0 of volume b
    if (KIND == TF_KIND_MULTIPHASE)
        for (int i = tid; i < 32 * 32; i += NT) lut[i] = op->face[i];
    if (KIND == TF_KIND_BINARY) fill_division_table(tab_all, tid, NT);
    for (int s = 0; s < NS; ++s) {
        float* f = F0 + s * (S::SLOT / 4);
        for (int i = tid; i < S::GUARD / 4; i += NT) {
            f[-1 - i] = 0.0f;
            f[S::FBYTES / 4 + i] = 0.0f;
        }
    }
    __syncthreads();

    // streamed planes [xs, xe); plane x uses slot (x - xs) % NS, its ((x - xs) / NS)-th use
    const int xs = x0 > K ? x0 - K : 0;
    const int xe = x1 + K < NX ? x1 + K : NX;
    auto issue = [&](int x) {
        const int s = (int)((unsigned)(x - xs) % NS);
        mbar_arrive_expect_tx(&bar[s], S::FBYTES + (KIND == KIND_FACES ? 0 : S::CBYTES));
        tma_load_3d(F0 + s * (S::SLOT / 4), tmf, &bar[s], j0, row0, b * NX + x);
        if (KIND != KIND_FACES) tma_load_3d(C0 + s * S::SLOT, tmc, &bar[s], j0, row0, b * NX + x);
    };
    if (tid == 0)
        for (int x = xs; x < xs + D && x < xe; ++x) issue(x);

    // own cells by relative colour (V0, V1) and their codes (K0, K1); ring index = (plane - xs) % R.
    // Plane -1 (ring slot R-1 until plane R-1 arrives) and plane NX are the Dirichlet ghost
    // planes 2*bc, so x-neighbours need no boundary selects (a chunk starting above 0 reads the
    // same constant as its plane xs-1: a margin plane).
    float4 V0[R], V1[R];
    uint32_t K0[R], K1[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        V0[r] = V1[r] = glo4;
        K0[r] = K1[r] = 0u;
    }

    const bool interior_group = gi >= 1 && gi < G - 1;
    // bit s: this row lies in the region [s, ROWS - s) of half-sweep s
    uint32_t stage_rows = 0;
#pragma unroll
    for (int s = 1; s <= K; ++s) stage_rows |= (ty >= s && ty < ROWS - s) ? (1u << s) : 0u;
    const bool py = a.periodic & TF_PERIODIC_Y, pz = a.periodic & TF_PERIODIC_Z;

    // write-back invariants: this thread's interior group (if any), its row in plane 0 of the
    // output, and whether both half-row groups are whole and need no periodic ghost copy (the
    // common case: one pointer select and one 128-bit store per half-row and step)
    const int jw = j0 + 4 * (gi - 1);
    const bool writes = interior_group && ty >= K && ty < K + TY && y < g.NY;
    const bool wb_plain = writes && jw + 4 <= half_len(g.NZ, 1) && !(py && (y < HY || y >= g.NY - HY)) &&
                          !(pz && (jw < HJ || jw + 4 > (g.NZ >> 1) - HJ));
    float* const wb_row = a.out + (long long)b * g.vol_f + (long long)(y + HY) * g.row_f + HJ + jw;

    // steps: the last chunk runs K past the volume (Dirichlet plane NX), the others stop at xe
    const int total = xe == NX ? NX + K : xe;
    for (int t0 = xs; t0 < total; t0 += R) {
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int t = t0 + i;
            if (t < total) {
                if (tid == 0 && t + D < xe) issue(t + D);
                if (KIND == KIND_FACES && t < NX && y >= -HY && y < g.NY + HY && j0 + jj + 4 <= g.ZH) {
                    // the faces of plane t, first used one step later: into L2 now, so that the
                    // stages' loads do not wait on DRAM in the middle of their dependent chain
                    const long long go = (long long)b * g.vol_f + (long long)t * g.plane_f +
                                         (long long)(y + HY) * g.row_f + j0 + jj;
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const long long o = go + q * g.ZH;
                        prefetch_l2(a.fx + o + (long long)b * g.plane_f);
                        prefetch_l2(a.fy + o);
                        prefetch_l2(a.fz + o);
                        prefetch_l2(a.dv + o);
                    }
                }
                if (t < xe) {
                    const int slot = (int)((unsigned)(t - xs) % NS);
                    if (!mbar_wait_bounded(&bar[slot], ((unsigned)(t - xs) / NS) & 1)) *s_fail = 1;
                    const float* Fs = F0 + slot * (S::SLOT / 4);
                    const unsigned char* Cs = C0 + slot * S::SLOT;
                    const float4 e4 = ld4(Fs + (2 * ty) * WJ + jj);
                    const float4 o4 = ld4(Fs + (2 * ty + 1) * WJ + jj);
                    // (KIND_FACES stages no codes)
                    const uint32_t ce = KIND == KIND_FACES ? 0u : ld_u32(Cs + (2 * ty) * WJC + jj);
                    const uint32_t co = KIND == KIND_FACES ? 0u : ld_u32(Cs + (2 * ty + 1) * WJC + jj);
                    const bool even0 = ((t + y + c0) & 1) == 0;  // even-z cells have relative colour 0
                    V0[i] = even0 ? e4 : o4;
                    V1[i] = even0 ? o4 : e4;
                    K0[i] = even0 ? ce : co;
                    K1[i] = even0 ? co : ce;
                } else if (t == NX) {
                    V0[i] = V1[i] = ghi4;
                }
                // every half-sweep of step t updates half-row (t + y + c0 + 1) & 1 of its plane: the
                // relative colour (s-1)&1 sits in half-row (p + y + c0) & 1 ^ (s-1)&1, p = t - s
                const int qs = (t + y + c0 + 1) & 1;
                const SlotOffsets fo = slot_offsets(ty, jj, qs, WJ);
                const SlotOffsets co = slot_offsets(ty, jj, qs, WJC);
#pragma unroll
                for (int s = 1; s <= K; ++s) {
                    const int p = t - s;
                    const int ip = (i - s + 2 * R) % R;
                    const int ipn = (i - s + 1 + 2 * R) % R;
                    const int ipp = (i - s - 1 + 2 * R) % R;
                    // rows [s, ROWS - s) form the region of half-sweep s: it shrinks by one row per
                    // half-sweep so the tile interior is exact after K of them
                    if (p >= xs && p < NX && (stage_rows & (1u << s))) {
                        const int ps = (int)((unsigned)(p - xs) % NS);  // p >= xs here
                        float* Fp = F0 + ps * (S::SLOT / 4);
                        const unsigned char* Cp = C0 + ps * S::SLOT;
                        const bool at_lo = p == 0, at_hi = p == NX - 1;
                        // global address of this thread's group in the right-hand side (padded
                        // coordinates; rows beyond the ghost bands and groups past the row read 0)
                        const bool in_plane = y >= -HY && y < g.NY + HY && j0 + jj + 4 <= g.ZH;
                        const float* rhs_row = nullptr;
                        if (RHS && in_plane)
                            rhs_row = a.rhs + (long long)b * g.vol_f + (long long)p * g.plane_f +
                                      (long long)(y + HY) * g.row_f + j0 + jj;
                        // KIND_FACES: global offset of the group's faces (half-row 0), -1 if none
                        const long long go = KIND == KIND_FACES && in_plane
                                                 ? (long long)b * g.vol_f + (long long)p * g.plane_f +
                                                       (long long)(y + HY) * g.row_f + j0 + jj
                                                 : -1LL;
                        const bool ym_ok = y + HY > 0, zm_ok = j0 + jj > 0;
                        if (((s - 1) & 1) == 0) {
                            const uint32_t cxp = at_hi ? K0[ip] : K1[ipn], cxm = at_lo ? K0[ip] : K1[ipp];
                            stage_update<KIND, RHS>(V0[ip], V1[ipn], V1[ipp], V1[ip], K0[ip], cxp, cxm, K1[ip], Fp,
                                                    Cp, fo, co, qs, WJ, WJC, at_lo, at_hi, a, lut, tab, rhs_row, go,
                                                    b, ym_ok, zm_ok);
                        } else {
                            const uint32_t cxp = at_hi ? K1[ip] : K0[ipn], cxm = at_lo ? K1[ip] : K0[ipp];
                            stage_update<KIND, RHS>(V1[ip], V0[ipn], V0[ipp], V0[ip], K1[ip], cxp, cxm, K0[ip], Fp,
                                                    Cp, fo, co, qs, WJ, WJC, at_lo, at_hi, a, lut, tab, rhs_row, go,
                                                    b, ym_ok, zm_ok);
                        }
                    }
                }
                // write back plane t-K from registers
                const int pw = t - K;
                const int iw = (i - K + 2 * R) % R;
                if (pw >= x0 && pw < x1 && wb_plain) {
                    // V0 holds relative colour 0: the even-z half-row when pw + y + c0 is even
                    float* const wp = wb_row + (long long)pw * g.plane_f;
                    const bool even0 = ((pw + y + c0) & 1) == 0;
                    st4(even0 ? wp : wp + g.ZH, V0[iw]);
                    st4(even0 ? wp + g.ZH : wp, V1[iw]);
                } else if (pw >= x0 && pw < x1 && writes) {
                    const bool even0 = ((pw + y + c0) & 1) == 0;
                    const float4 ev = even0 ? V0[iw] : V1[iw];
                    const float4 od = even0 ? V1[iw] : V0[iw];
                    const int j = jw;
                    float* outp = a.out + (long long)b * g.vol_f + (long long)pw * g.plane_f;
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const float4 v = q ? od : ev;
                        const int nj = half_len(g.NZ, q);
                        if (j >= nj) continue;
                        float* rowp = outp + (long long)(y + HY) * g.row_f + q * g.ZH + HJ;
                        if (j + 4 <= nj) {
                            st4(rowp + j, v);
                        } else {
                            for (int c = 0; c < nj - j; ++c) rowp[j + c] = comp(v, c);
                        }
                        if (py || pz) {
                            const int hz = g.NZ >> 1;
                            if ((hz & 3) == 0) {
                                // periodic ghost copies as whole aligned groups
                                const bool yb = py && (y < HY || y >= g.NY - HY);
                                const int ys = y < HY ? y + g.NY : y - g.NY;
                                const bool zb = pz && (j == 0 || j == hz - 4);
                                const int jz = j == 0 ? hz : -4;
                                float* rows_ = outp + (long long)(ys + HY) * g.row_f + q * g.ZH + HJ;
                                if (yb) st4(rows_ + j, v);
                                if (zb) st4(rowp + jz, v);
                                if (yb && zb) st4(rows_ + jz, v);
                            } else if ((py && (y < HY || y >= g.NY - HY)) || (pz && (j < HJ || j + 4 > hz - HJ))) {
                                ghost_copies_scalar(outp, g.row_f, g.ZH, g.NY, g.NZ, y, q, j, nj, v, py);
                            }
                        }
                    }
                }
                fence_proxy_async_smem();
                __syncthreads();
                if (*s_fail) {
                    if (tid == 0) {
                        for (int x = t + 1; x < t + 1 + D && x < xe; ++x)
                            mbar_wait_bounded(&bar[(x - xs) % NS], ((x - xs) / NS) & 1);
                        if (a.err) atomicExch(a.err, TF_ERR_TIMEOUT);
                    }
                    return;
                }
            }
        }
    }
}

template <int KIND, int TY, int TZ, int K, bool RHS>
__global__ void __launch_bounds__(StreamShape<TY, TZ, K>::NT, StreamShape<TY, TZ, K>::NT <= 256 ? 2 : 1)
    k_stream(const __grid_constant__ CUtensorMap tmf, const __grid_constant__ CUtensorMap tmc, const SweepArgs a,
             const __grid_constant__ tf_operator op) {
    // dynamic shared memory: the runtime aligns it to at least 128 bytes (no static shared
    // variables precede it in this kernel); every pointer below stays in the shared window
    extern __shared__ __align__(128) unsigned char smem[];
    const int b = blockIdx.z / a.x_chunks, c = blockIdx.z - b * a.x_chunks;
    const int x0 = (int)((long long)c * a.g.NX / a.x_chunks), x1 = (int)((long long)(c + 1) * a.g.NX / a.x_chunks);
    stream_tile<KIND, TY, TZ, K, RHS>(&tmf, &tmc, a, &op, blockIdx.x * (TZ / 2), blockIdx.y * TY, b, x0, x1, smem);
}

// ------------------------------------------------------------------------------ host side
// Number of x-chunks per tile column: minimises (waves of CTAs) x (steps per CTA), where a
// chunk of nx/c planes costs nx/c + 2K steps and `slots` CTAs run at once. 1 when the
// columns already fill the last wave well.
inline int x_chunks_for(long long columns, int nx, int k, int slots) {
    if (slots <= 0) return 1;
    int best = 1;
    double best_cost = 1e300;
    for (int c = 1; c <= 8 && nx / c >= 8 * k; ++c) {
        const long long waves = (columns * c + slots - 1) / slots;
        const double cost = (double)waves * ((double)nx / c + (c > 1 ? 2 * k : k));
        if (cost < best_cost * 0.995) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

// One-time set-up of a kernel on the current device: the dynamic shared-memory limit (an
// attribute that applies to the device current when it is set) and the number of CTAs of the
// kernel resident per SM. Kept per device and per kernel, guarded by a mutex; returns the
// resident count, or 0 if the set-up failed (it is then tried again at the next call).
template <auto KERN>
static int prepare_kernel(int threads, int smem) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static int resident[MAX_DEVICES];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return 0;
    std::lock_guard<std::mutex> lock(mu);
    if (resident[dev] == 0) {
        if (cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 0;
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, KERN, threads, smem) != cudaSuccess || n <= 0)
            return 0;  // the kernel cannot run with this block on this device
        resident[dev] = n;
    }
    return resident[dev];
}

template <int KIND, int TY, int TZ, int K, bool RHS>
static int launch_stream(const tf_geom& gg, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                         const float* rhs, int first_colour, int32_t* err, cudaStream_t st,
                         const float* const* faces = nullptr) {
    using S = StreamShape<TY, TZ, K>;
    CUtensorMap tmf, tmc;
    int rc = encode_map_3d(&tmf, in, 4, gg.zh, 2 * gg.yp, (long long)gg.batch * gg.nx, (long long)gg.zh * 4,
                           (long long)gg.zh * 4 * 2 * gg.yp, S::WJ, 2 * S::ROWS);
    if (rc) return rc;
    if (KIND == KIND_FACES) {
        if (!faces) return TF_ERR_ARG;
        tmc = tmf;  // no codes: the map is passed but never read
    } else {
        rc = encode_map_3d(&tmc, code, 1, gg.zhc, 2 * gg.yp, (long long)gg.batch * gg.nx, gg.zhc,
                           (long long)gg.zhc * 2 * gg.yp, S::WJC, 2 * S::ROWS);
        if (rc) return rc;
    }
    constexpr auto kern = k_stream<KIND, TY, TZ, K, RHS>;
    const int resident = prepare_kernel<kern>(S::NT, S::SMEM);  // CTAs of this kernel per SM
    if (resident <= 0) return TF_ERR_CUDA;
    SweepArgs a = make_args(make_geo(gg), op, out, first_colour, K, err);
    a.rhs = rhs;
    if (faces) {
        a.fx = faces[0];
        a.fy = faces[1];
        a.fz = faces[2];
        a.dv = faces[3];
    }
    const long long columns = (long long)((gg.nz + TZ - 1) / TZ) * ((gg.ny + TY - 1) / TY) * gg.batch;
    a.x_chunks = x_chunks_for(columns, gg.nx, K, resident * sm_count());
    if ((long long)gg.batch * a.x_chunks > 65535) a.x_chunks = 1;  // grid z limit
    dim3 grid((gg.nz + TZ - 1) / TZ, (gg.ny + TY - 1) / TY, gg.batch * a.x_chunks);
    kern<<<grid, S::NT, S::SMEM, st>>>(tmf, tmc, a, op);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

template <int KIND, int TY, int TZ, bool RHS>
static int dispatch_k(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                      const float* rhs, int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    switch (n_half) {
        case 1: return launch_stream<KIND, TY, TZ, 1, RHS>(g, op, in, out, code, rhs, first_colour, err, st);
        case 2: return launch_stream<KIND, TY, TZ, 2, RHS>(g, op, in, out, code, rhs, first_colour, err, st);
        case 3: return launch_stream<KIND, TY, TZ, 3, RHS>(g, op, in, out, code, rhs, first_colour, err, st);
        case 4: return launch_stream<KIND, TY, TZ, 4, RHS>(g, op, in, out, code, rhs, first_colour, err, st);
    }
    return TF_ERR_ARG;
}

// Tile shapes (op.tile) of the binary operator: 0 = 16x64, 1 = 16x128, 2 = 32x64 (rows x
// z-cells); shapes 1 and 2 fuse 2..4 half-sweeps (a single half-sweep runs on shape 0). The
// multiphase and anisotropic operators, and every correction solve with a right-hand side, use
// shape 0. Each shape's instantiations live in their own translation unit.
template <int KIND>
static int dispatch_kind(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                         const float* rhs, int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    if (rhs) return dispatch_k<KIND, 16, 64, true>(g, op, in, out, code, rhs, first_colour, n_half, err, st);
    return dispatch_k<KIND, 16, 64, false>(g, op, in, out, code, nullptr, first_colour, n_half, err, st);
}

// K = 2..4 on one tile shape (shapes 1 and 2 of the binary operator).
template <int TY, int TZ>
static int dispatch_k234(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                         int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    switch (n_half) {
        case 2: return launch_stream<TF_KIND_BINARY, TY, TZ, 2, false>(g, op, in, out, code, nullptr, first_colour, err, st);
        case 3: return launch_stream<TF_KIND_BINARY, TY, TZ, 3, false>(g, op, in, out, code, nullptr, first_colour, err, st);
        case 4: return launch_stream<TF_KIND_BINARY, TY, TZ, 4, false>(g, op, in, out, code, nullptr, first_colour, err, st);
    }
    return TF_ERR_ARG;
}

}  // namespace tf
