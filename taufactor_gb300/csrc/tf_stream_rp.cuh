// Row-pair register-streaming wavefront for the binary operator: K (even) half-sweeps per launch
// (sm_103a). Same TMA plane ring, x-wavefront and one-barrier-per-plane protocol as k_stream
// (tf_stream.cuh); what changes is how threads map onto the tile.
//
// A thread owns two adjacent rows (a row pair) at one float2 group (2 cells) of both half-rows.
// In a red-black half-sweep the half-row whose cells are updated in a row is (x + y + colour)&1,
// so the two rows of a pair always update opposite half-rows. Call P the row of the pair for
// which (x0 + y + first colour) is even (the same choice for every pair of the CTA) and Q the
// other: at unrolled step i of the march P updates half-row (i+1)&1 and Q half-row i&1. Both are
// compile-time constants, so the z-neighbour pattern of each update (the even half-row's cell j
// sits between odd cells j-1 and j, the odd one's between even cells j and j+1) needs no selects,
// and neither does the split of a loaded plane into relative colours.
//
// Warps: warp w < NP holds pair w (its 32 lanes are the pair's 32 interior groups of a 128-cell
// tile), so the shrinking row region of the half-sweeps is a warp-uniform test. One more warp
// holds the z-halo groups (HG float2 groups per side, enough for the K/2-cell dependency cone in
// each half-row) of all pairs; its spare lanes repeat the first halo groups and store nothing.
// Rows outside a half-sweep's region may be computed (a pair straddling the region edge): their
// values are never read by a row inside a later region, so the interior stays exact. Rows -1
// and ROWS of a slot are zero guards in shared memory.
//
// The update is the binary one of update4_binary (sum in the reference's order, exact division
// by the neighbour count, SOR finish) on one f32x2 lane pair per row, bit for bit the reference
// (taufactor.py:95-103, :174-182).
#pragma once

#include <type_traits>

#include "tf_stream.cuh"

namespace tf {

template <int TY, int TZ, int K>
struct RowPairShape {
    static constexpr int TJ = TZ / 2;                  // interior cells per half-row
    static constexpr int WJ = TJ + 2 * HJ;             // staged floats per half-row (one float4 ghost group per side)
    static constexpr int WJC = (WJ + 15) / 16 * 16;    // bytes per staged code half-row
    static constexpr int ROWS = TY + 2 * K;            // staged rows: K ghost rows per side
    static constexpr int NP = ROWS / 2;                // row pairs
    static constexpr int HG = (K + 3) / 4;             // halo float2 groups per side (2 HG >= K/2 cells)
    static constexpr int GM = TJ / 2;                  // interior float2 groups per half-row
    static constexpr int WM = GM / 32;                 // warps per pair for the interior groups
    static constexpr int NHALO = 2 * HG * NP;          // halo threads
    static constexpr int NW = NP * WM + (NHALO + 31) / 32;
    static constexpr int NT = 32 * NW;
    static constexpr int R = K + 2;                    // planes held in registers = ring slots in shared memory
    static constexpr int D = R / 2;                    // TMA staging buffers (D - 1 planes in flight ahead)
    static constexpr int FBYTES = 2 * ROWS * WJ * 4;   // one staged plane of the field
    static constexpr int CBYTES = 2 * ROWS * WJC;      // one staged plane of the codes
    static constexpr int GUARD = (2 * WJ * 4 + 127) / 128 * 128;  // one zero row (both half-rows)
    static constexpr int RSTRIDE = (FBYTES + 127) / 128 * 128 + GUARD;  // ring slot + following guard
    static constexpr int SSTRIDE = (FBYTES + 127) / 128 * 128 + (CBYTES + 127) / 128 * 128;
    static constexpr int TAB = (DIV_TABLE_BYTES + 127) / 128 * 128;
    static constexpr int HEAD = 128 + TAB;             // mbarriers + failure flag, division table
    static constexpr int RING0 = HEAD + GUARD;         // ring slot r: RING0 + r * RSTRIDE, a guard on each side
    static constexpr int STAGE0 = RING0 + R * RSTRIDE; // staging buffer d: STAGE0 + d * SSTRIDE (field, codes)
    static constexpr int SMEM = STAGE0 + D * SSTRIDE;
    static_assert(TJ % 64 == 0, "a pair's interior groups must fill whole warps");
    static_assert(K % 2 == 0 && K >= 2 && K <= HY, "row pairs fuse an even number of half-sweeps");
    static_assert(R % D == 0 && (R / D) % 2 == 0, "staging parity must repeat with the unrolled march");
    static_assert(4 * HG >= K && 2 * HG <= HJ, "z halo must cover the dependency cone inside the staged ghosts");
    static_assert(8 * D <= 120, "mbarriers and the failure flag must fit the head");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
    static_assert(151 * 16 * DIV_COPIES < 65536, "table offsets must fit 16 bits");
    static_assert(HEAD % 16 == 0 && STAGE0 % 16 == 0, "ring zeroed as float4");
};

__device__ __forceinline__ f32x2 ld_pair(const float* p) { return *reinterpret_cast<const f32x2*>(p); }
__device__ __forceinline__ void st_pair(float* p, f32x2 v) { *reinterpret_cast<f32x2*>(p) = v; }
__device__ __forceinline__ uint32_t ld_u16(const unsigned char* p) {
    return *reinterpret_cast<const unsigned short*>(p);
}
__device__ __forceinline__ float lo_of(f32x2 v) { float l, h; upk2(v, l, h); return l; }
__device__ __forceinline__ float hi_of(f32x2 v) { float l, h; upk2(v, l, h); return h; }

// Neighbour sum of one row's float2 group updating half-row q, in the reference's order
// (x+1, x-1, y+1, y-1, z+1, z-1). `zo` is the group of the other half-row (registers), `e` the
// z-edge cell of the adjacent group (odd j-1 for q = 0, even j+2 for q = 1). q is a constant
// after unrolling.
__device__ __forceinline__ f32x2 rp_sum(int q, f32x2 xp, f32x2 xm, f32x2 yp, f32x2 ym, f32x2 zo, float e) {
    f32x2 s = add2(xp, xm);
    s = add2(s, yp);
    s = add2(s, ym);
    if (q == 0) {
        // even cells j, j+1: z+1 = odd j, j+1 (zo); z-1 = odd j-1 (edge), odd j
        s = add2(s, zo);
        s = add2(s, pk2(e, lo_of(zo)));
    } else {
        // odd cells j, j+1: z+1 = even j+1, j+2 (edge); z-1 = even j, j+1 (zo)
        s = add2(s, pk2(hi_of(zo), e));
        s = add2(s, zo);
    }
    return s;
}

// Quotients sum / neighbour count of one row's lane pair, correctly rounded (Brisebarre, Muller,
// Raina with the pair table, as update4_binary); `t` = the table entry (-n_lo, -n_hi, RN(1/n_lo),
// RN(1/n_hi)) of the two cells.
__device__ __forceinline__ f32x2 rp_quotient(f32x2 s, float4 t) {
    const f32x2 r = pk2(t.z, t.w);
    f32x2 q = mul2(s, r);
    q = fma2(fma2(q, pk2(t.x, t.y), s), r, q);
    return q;
}

// SOR finish c + omega * (q - c) of a lane pair (taufactor.py:177-181).
__device__ __forceinline__ f32x2 rp_sor(f32x2 c, f32x2 q, float omega) {
    float i0, i1;
    upk2(sub2(q, c), i0, i1);
    // scalar mul.rn: never contracted into the following add (see update4_binary)
    return add2(c, pk2(__fmul_rn(i0, omega), __fmul_rn(i1, omega)));
}

// IEEE quotients of one lane pair (the tiny-sum path of update4_binary).
__device__ __forceinline__ f32x2 rp_tiny(f32x2 s, float4 t) {
    float a, b;
    upk2(s, a, b);
    const float4 q = tiny_quotients(make_float4(a, b, 0.f, 0.f), make_float4(-t.x, -t.y, 1.f, 1.f),
                                    make_float4(t.z, t.w, 1.f, 1.f));
    return pk2(q.x, q.y);
}

// |bits - 1| of a lane: +-0 becomes a NaN (skipped by fminf), anything else loses one ulp.
__device__ __forceinline__ float tiny_key(float v) { return fabsf(__int_as_float(__float_as_int(v) - 1)); }

// Writes one row's two half-row groups of plane `pw` (with periodic ghost copies).
__device__ __forceinline__ void rp_write_row(const SweepArgs& a, int b, int pw, int y, int j, f32x2 ev, f32x2 od,
                                             bool py, bool pz) {
    const Geo& g = a.g;
    float* outp = a.out + (long long)b * g.vol_f + (long long)pw * g.plane_f;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const f32x2 v = q ? od : ev;
        const int nj = half_len(g.NZ, q);
        if (j >= nj) continue;
        float* rowp = outp + (long long)(y + HY) * g.row_f + q * g.ZH + HJ;
        if (j + 2 <= nj) st_pair(rowp + j, v);
        else rowp[j] = lo_of(v);
        if (py || pz) {
            const int hz = g.NZ >> 1;
            if ((hz & 1) == 0) {
                const bool yb = py && (y < HY || y >= g.NY - HY);
                const int ys = y < HY ? y + g.NY : y - g.NY;
                const bool zb = pz && (j < HJ || j >= hz - HJ);
                const int jz = j < HJ ? j + hz : j - hz;
                float* rows_ = outp + (long long)(ys + HY) * g.row_f + q * g.ZH + HJ;
                if (yb) st_pair(rows_ + j, v);
                if (zb) st_pair(rowp + jz, v);
                if (yb && zb) st_pair(rows_ + jz, v);
            } else if ((py && (y < HY || y >= g.NY - HY)) || (pz && (j < HJ || j + 2 > hz - HJ))) {
                // odd half-row length: cell by cell
                float l, h;
                upk2(v, l, h);
                ghost_copies_scalar(outp, g.row_f, g.ZH, g.NY, g.NZ, y, q, j, j + 2 < nj ? j + 2 : nj,
                                    make_float4(l, h, 0.f, 0.f), py);
            }
        }
    }
}

// One CTA's tile (j0 = first staged padded j, y0 = first interior row, volume b, written planes
// [x0, x1)) for K half-sweeps. RPAR = (x0-chunk start + y0 - K + first colour) & 1: which row
// of every pair is P (0: the lower one). Shared memory: RowPairShape::SMEM bytes at `smem`.
//
// Planes arrive by TMA in D staging buffers, D - 1 ahead; at step t every thread copies its own
// cells of plane t into ring slot (t - xs) mod R (and its codes into registers), where the K
// half-sweeps of the following steps read y-neighbours and z-edges and publish their updates.
// R and D divide the unrolled march, so every slot, buffer and mbarrier phase is a
// compile-time constant.
template <int TY, int TZ, int K, int RPAR>
__device__ __forceinline__ void stream_tile_rp(const CUtensorMap* tmf, const CUtensorMap* tmc, const SweepArgs& a,
                                               int j0, int y0, int b, int x0, int x1, unsigned char* smem) {
    using S = RowPairShape<TY, TZ, K>;
    constexpr int WJ = S::WJ, WJC = S::WJC, D = S::D, R = S::R, NT = S::NT, NP = S::NP;
    constexpr int RS = S::RSTRIDE / 4, SS = S::SSTRIDE / 4;  // floats between ring slots / staging buffers
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    int* s_fail = reinterpret_cast<int*>(smem + 120);
    float4* tab_all = reinterpret_cast<float4*>(smem + 128);

    const Geo& g = a.g;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int NX = g.NX;

    // thread -> (pair k, float2 group gi); halo lanes beyond the halo threads repeat them (dup)
    int k, gi;
    bool halo = false, dup = false;
    if (warp < NP * S::WM) {
        k = warp / S::WM;
        gi = S::HG + (warp % S::WM) * 32 + lane;
    } else {
        int h = (warp - NP * S::WM) * 32 + lane;
        if (h >= S::NHALO) {
            h -= S::NHALO;
            dup = true;
        }
        halo = true;
        k = h / (2 * S::HG);
        const int e = h - k * (2 * S::HG);
        gi = e < S::HG ? e : S::GM + e;
    }
    const int jj = HJ - 2 * S::HG + 2 * gi;  // staged float index of the group's first cell
    // float offset of the pair's lower row (half-row 0) at the group; the upper row is + 2 WJ
    const int base = 4 * k * WJ + jj;
    float* const ring = reinterpret_cast<float*>(smem + S::RING0) + base;
    const float* const stage_f = reinterpret_cast<const float*>(smem + S::STAGE0) + base;
    const unsigned char* const stage_c = smem + S::STAGE0 + S::FBYTES + 4 * k * WJC + jj;
    // byte offset of this thread's copy of the division table, added to 16 * DIV_COPIES * index
    const uint32_t copy_off = 16u * (uint32_t)(tid & (DIV_COPIES - 1));

    if (tid == 0) {
        for (int d = 0; d < D; ++d) mbar_init(&bar[d], 1);
        fence_mbar_init();
        *s_fail = 0;
    }
    fill_division_table(tab_all, tid, NT);
    // zero the guard before ring slot 0 and the whole ring with its guards: rows -1 and ROWS
    // read zeros, and so do the staged ghost cells no thread owns (positions < HJ - 2 HG and
    // >= WJ - HJ + 2 HG of every half-row, read as z-edges by the halo groups), which would
    // otherwise hold whatever the shared memory held before
    {
        float4* z = reinterpret_cast<float4*>(smem + S::HEAD);
        for (int i = tid; i < (S::STAGE0 - S::HEAD) / 16; i += NT) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();

    const int xs = x0 > K ? x0 - K : 0;
    const int xe = x1 + K < NX ? x1 + K : NX;
    const int row0 = 2 * (y0 + HY - K);
    auto issue = [&](int x, int d) {
        mbar_arrive_expect_tx(&bar[d], S::FBYTES + S::CBYTES);
        float* dst = reinterpret_cast<float*>(smem + S::STAGE0 + d * S::SSTRIDE);
        tma_load_3d(dst, tmf, &bar[d], j0, row0, b * NX + x);
        tma_load_3d(reinterpret_cast<unsigned char*>(dst) + S::FBYTES, tmc, &bar[d], j0, row0, b * NX + x);
    };
    if (tid == 0)
        for (int x = xs; x < xs + D - 1 && x < xe; ++x) issue(x, x - xs);

    // rows of the pair: P is the lower row when RPAR == 0
    constexpr int LP = RPAR ? 2 * WJ : 0, LQ = RPAR ? 0 : 2 * WJ;    // float offsets of rows P, Q
    constexpr int CP = RPAR ? 2 * WJC : 0, CQ = RPAR ? 0 : 2 * WJC;  // their code byte offsets
    const int yL = y0 - K + 2 * k;  // interior y of the lower row
    const int yP = yL + (RPAR ? 1 : 0), yQ = yL + (RPAR ? 0 : 1);
    // bit s: the pair takes part in half-sweep s (a row of it lies in [s, ROWS - s)); the halo
    // warp takes part in every half-sweep
    uint32_t stage_mask = 0;
#pragma unroll
    for (int s = 1; s <= K; ++s)
        stage_mask |= (halo || (2 * k + 1 >= s && 2 * k < S::ROWS - s)) ? (1u << s) : 0u;
    const bool wP = !halo && (2 * k + (RPAR ? 1 : 0)) >= K && (2 * k + (RPAR ? 1 : 0)) < K + TY && yP < g.NY;
    const bool wQ = !halo && (2 * k + (RPAR ? 0 : 1)) >= K && (2 * k + (RPAR ? 0 : 1)) < K + TY && yQ < g.NY;
    const int jglob = j0 + jj - HJ;  // interior index of the group's first cell
    const bool py = a.periodic & TF_PERIODIC_Y, pz = a.periodic & TF_PERIODIC_Z;
    const float omega = a.omega;

    // ring by relative colour: P0/P1 (row P), Q0/Q1 (row Q); TP/TQ: byte offsets of the division
    // table entries of the row's even (low 16 bits) and odd (high 16 bits) half-row groups
    f32x2 P0[R], P1[R], Q0[R], Q1[R];
    uint32_t TP[R], TQ[R];
    const f32x2 glo = pk2(a.glo, a.glo), ghi = pk2(a.ghi, a.ghi);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        P0[r] = P1[r] = Q0[r] = Q1[r] = glo;
        TP[r] = TQ[r] = 0u;
    }
    const unsigned char* const tab_base = smem + 128;

    const int total = xe == NX ? NX + K : xe;
    // One block of R steps starting at t0 (t0 - xs a multiple of R). CHECKED: any block; else a
    // block in the steady state (t0 >= x0 + K and t0 + R <= xe), where every step loads its
    // plane, runs all K half-sweeps and writes back, so the range checks drop out.
    auto block = [&](auto checked, int t0) -> bool {
        constexpr bool CK = decltype(checked)::value;
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int t = t0 + i;
            if (CK && t >= total) continue;
            if (tid == 0 && t + D - 1 < xe) issue(t + D - 1, (i + D - 1) % D);
            if (!CK || t < xe) {
                const int d = i % D;
                if (!mbar_wait_bounded(&bar[d], (i / D) & 1)) *s_fail = 1;
                const float* fs = stage_f + d * SS;
                const unsigned char* cs = stage_c + d * S::SSTRIDE;
                float* fr = ring + i * RS;
                const f32x2 eP = ld_pair(fs + LP), oP = ld_pair(fs + LP + WJ);
                const f32x2 eQ = ld_pair(fs + LQ), oQ = ld_pair(fs + LQ + WJ);
                st_pair(fr + LP, eP);
                st_pair(fr + LP + WJ, oP);
                st_pair(fr + LQ, eQ);
                st_pair(fr + LQ + WJ, oQ);
                // counts masked to 4 bits: table offsets stay inside shared memory whatever
                // the code bytes hold
                const uint32_t cP = (ld_u16(cs + CP) | (ld_u16(cs + CP + WJC) << 16)) & 0x0f0f0f0fu;
                const uint32_t cQ = (ld_u16(cs + CQ) | (ld_u16(cs + CQ + WJC) << 16)) & 0x0f0f0f0fu;
                constexpr uint32_t ENT = 16u * DIV_COPIES;  // bytes per table entry (all copies)
                TP[i] = ((uint32_t)__dp4a((int)cP, 0x0109, 0) * ENT + copy_off) |
                        (((uint32_t)__dp4a((int)cP, 0x01090000, 0) * ENT + copy_off) << 16);
                TQ[i] = ((uint32_t)__dp4a((int)cQ, 0x0109, 0) * ENT + copy_off) |
                        (((uint32_t)__dp4a((int)cQ, 0x01090000, 0) * ENT + copy_off) << 16);
                // relative colour 0 of row P is its even half-row at even i; row Q the opposite
                if ((i & 1) == 0) {
                    P0[i] = eP; P1[i] = oP; Q0[i] = oQ; Q1[i] = eQ;
                } else {
                    P0[i] = oP; P1[i] = eP; Q0[i] = eQ; Q1[i] = oQ;
                }
            } else if (t == NX) {
                P0[i] = P1[i] = Q0[i] = Q1[i] = ghi;
            }
            const int qp = (i + 1) & 1;  // half-row updated by row P in this step
            const int qq = 1 - qp;
#pragma unroll
            for (int s = 1; s <= K; ++s) {
                const int p = t - s;
                const int ip = (i - s + 2 * R) % R;
                const int ipn = (i - s + 1 + 2 * R) % R;
                const int ipp = (i - s - 1 + 2 * R) % R;
                if ((!CK || (p >= xs && p < NX)) && __any_sync(0xffffffffu, (stage_mask >> s) & 1u)) {
                    float* fr = ring + ip * RS;
                    const int rc = (s - 1) & 1;
                    f32x2& cP = rc ? P1[ip] : P0[ip];
                    f32x2& cQ = rc ? Q1[ip] : Q0[ip];
                    const f32x2 oP = rc ? P0[ip] : P1[ip], oQ = rc ? Q0[ip] : Q1[ip];
                    const f32x2 xpP = rc ? P0[ipn] : P1[ipn], xmP = rc ? P0[ipp] : P1[ipp];
                    const f32x2 xpQ = rc ? Q0[ipn] : Q1[ipn], xmQ = rc ? Q0[ipp] : Q1[ipp];
                    // y-neighbours: the pair's other row from registers (its cells in the
                    // updated half-row have the other colour), the far side from the slot
                    f32x2 ypP, ymP, ypQ, ymQ;
                    if (RPAR == 0) {  // P lower, Q upper
                        ypP = oQ;
                        ymP = ld_pair(fr + LP - 2 * WJ + qp * WJ);
                        ypQ = ld_pair(fr + LQ + 2 * WJ + qq * WJ);
                        ymQ = oP;
                    } else {  // P upper, Q lower
                        ypP = ld_pair(fr + LP + 2 * WJ + qp * WJ);
                        ymP = oQ;
                        ypQ = oP;
                        ymQ = ld_pair(fr + LQ - 2 * WJ + qq * WJ);
                    }
                    // z-edges: odd j-1 for an even half-row, even j+2 for an odd one
                    const float eP = qp == 0 ? fr[LP + WJ - 1] : fr[LP + 2];
                    const float eQ = qq == 0 ? fr[LQ + WJ - 1] : fr[LQ + 2];
                    const f32x2 sP = rp_sum(qp, xpP, xmP, ypP, ymP, oP, eP);
                    const f32x2 sQ = rp_sum(qq, xpQ, xmQ, ypQ, ymQ, oQ, eQ);
                    const uint32_t offP = qp ? (TP[ip] >> 16) : (TP[ip] & 0xffffu);
                    const uint32_t offQ = qq ? (TQ[ip] >> 16) : (TQ[ip] & 0xffffu);
                    const float4 tP = *reinterpret_cast<const float4*>(tab_base + offP);
                    const float4 tQ = *reinterpret_cast<const float4*>(tab_base + offQ);
                    f32x2 quP = rp_quotient(sP, tP);
                    f32x2 quQ = rp_quotient(sQ, tQ);
                    // 0 < |sum| <= 2^-90: the correction term may underflow; IEEE division
                    // for the whole warp instead (never in practice)
                    const float m = fminf(fminf(tiny_key(lo_of(sP)), tiny_key(hi_of(sP))),
                                          fminf(tiny_key(lo_of(sQ)), tiny_key(hi_of(sQ))));
                    if (__any_sync(0xffffffffu, m < 0x1p-90f)) {
                        quP = rp_tiny(sP, tP);
                        quQ = rp_tiny(sQ, tQ);
                    }
                    cP = rp_sor(cP, quP, omega);
                    cQ = rp_sor(cQ, quQ, omega);
                    if (!dup) {
                        st_pair(fr + LP + qp * WJ, cP);
                        st_pair(fr + LQ + qq * WJ, cQ);
                    }
                }
            }
            // write back plane t-K from registers: even half-row of P is relative colour 0 at even i
            const int pw = t - K;
            const int iw = (i - K + 2 * R) % R;
            if (!CK || (pw >= x0 && pw < x1)) {
                if (wP) {
                    if ((i & 1) == 0) rp_write_row(a, b, pw, yP, jglob, P0[iw], P1[iw], py, pz);
                    else rp_write_row(a, b, pw, yP, jglob, P1[iw], P0[iw], py, pz);
                }
                if (wQ) {
                    if ((i & 1) == 0) rp_write_row(a, b, pw, yQ, jglob, Q1[iw], Q0[iw], py, pz);
                    else rp_write_row(a, b, pw, yQ, jglob, Q0[iw], Q1[iw], py, pz);
                }
            }
            // the staging buffer read above is refilled by TMA after the barrier
            fence_proxy_async_smem();
            __syncthreads();
            if (*s_fail) {
                if (tid == 0) {
                    for (int x = t + 1; x < t + D && x < xe; ++x)
                        mbar_wait_bounded(&bar[(x - xs) % D], ((x - xs) / D) & 1);
                    if (a.err) atomicExch(a.err, TF_ERR_TIMEOUT);
                }
                return false;
            }
        }
        return true;
    };
    for (int t0 = xs; t0 < total; t0 += R) {
        const bool ok = (t0 >= x0 + K && t0 + R <= xe) ? block(std::false_type{}, t0) : block(std::true_type{}, t0);
        if (!ok) return;
    }
}

// 13 warps: one SM sub-partition holds 4 of them, which caps a thread at 128 registers.
template <int TY, int TZ, int K>
__global__ void __launch_bounds__(RowPairShape<TY, TZ, K>::NT, 1)
    k_stream_rp(const __grid_constant__ CUtensorMap tmf, const __grid_constant__ CUtensorMap tmc, const SweepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int b = blockIdx.z / a.x_chunks, c = blockIdx.z - b * a.x_chunks;
    const int x0 = (int)((long long)c * a.g.NX / a.x_chunks), x1 = (int)((long long)(c + 1) * a.g.NX / a.x_chunks);
    const int xs = x0 > K ? x0 - K : 0;
    const int y0 = blockIdx.y * TY;
    // CTA-uniform: which row of each pair has (xs + y + first colour) even
    if (((xs + y0 - K + a.first_colour) & 1) == 0)
        stream_tile_rp<TY, TZ, K, 0>(&tmf, &tmc, a, blockIdx.x * (TZ / 2), y0, b, x0, x1, smem);
    else
        stream_tile_rp<TY, TZ, K, 1>(&tmf, &tmc, a, blockIdx.x * (TZ / 2), y0, b, x0, x1, smem);
}

template <int TY, int TZ, int K>
static int launch_stream_rp(const tf_geom& gg, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                            int first_colour, int32_t* err, cudaStream_t st) {
    using S = RowPairShape<TY, TZ, K>;
    CUtensorMap tmf, tmc;
    int rc = encode_map_3d(&tmf, in, 4, gg.zh, 2 * gg.yp, (long long)gg.batch * gg.nx, (long long)gg.zh * 4,
                           (long long)gg.zh * 4 * 2 * gg.yp, S::WJ, 2 * S::ROWS);
    if (rc) return rc;
    rc = encode_map_3d(&tmc, code, 1, gg.zhc, 2 * gg.yp, (long long)gg.batch * gg.nx, gg.zhc,
                       (long long)gg.zhc * 2 * gg.yp, S::WJC, 2 * S::ROWS);
    if (rc) return rc;
    constexpr auto kern = k_stream_rp<TY, TZ, K>;
    const int resident = prepare_kernel<kern>(S::NT, S::SMEM);
    if (resident <= 0) return TF_ERR_CUDA;
    SweepArgs a = make_args(make_geo(gg), op, out, first_colour, K, err);
    const long long columns = (long long)((gg.nz + TZ - 1) / TZ) * ((gg.ny + TY - 1) / TY) * gg.batch;
    a.x_chunks = x_chunks_for(columns, gg.nx, K, resident * sm_count());
    if ((long long)gg.batch * a.x_chunks > 65535) a.x_chunks = 1;  // grid z limit
    dim3 grid((gg.nz + TZ - 1) / TZ, (gg.ny + TY - 1) / TY, gg.batch * a.x_chunks);
    kern<<<grid, S::NT, S::SMEM, st>>>(tmf, tmc, a);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

}  // namespace tf
