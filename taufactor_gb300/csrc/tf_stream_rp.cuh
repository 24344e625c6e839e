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
    static constexpr int R = K + 2;                    // planes held in registers
    static constexpr int D = 3;                        // planes loaded ahead
    static constexpr int NS = K + 1 + D;               // shared-memory slots
    static constexpr int FBYTES = 2 * ROWS * WJ * 4;
    static constexpr int GUARD = (2 * WJ * 4 + 127) / 128 * 128;  // one zero row (both half-rows)
    static constexpr int FSTRIDE = (FBYTES + 127) / 128 * 128 + GUARD;
    static constexpr int CBYTES = 2 * ROWS * WJC;
    static constexpr int CSTRIDE = (CBYTES + 127) / 128 * 128;
    static constexpr int LUT_BYTES = (DIV_TABLE_BYTES + 127) / 128 * 128;
    static constexpr int HEAD = 128 + LUT_BYTES;       // mbarriers + failure flag, division table
    static constexpr int FIELD0 = HEAD + GUARD;        // slot s: FIELD0 + s * FSTRIDE, a guard on each side
    static constexpr int CODE0 = FIELD0 + NS * FSTRIDE;
    static constexpr int SMEM = CODE0 + NS * CSTRIDE;
    static_assert(TJ % 64 == 0, "a pair's interior groups must fill whole warps");
    static_assert(K % 2 == 0 && K >= 2 && K <= HY, "row pairs fuse an even number of half-sweeps");
    static_assert(4 * HG >= K && 2 * HG <= HJ, "z halo must cover the dependency cone inside the staged ghosts");
    static_assert(8 * NS <= 120, "mbarriers and the failure flag must fit the head");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};

__device__ __forceinline__ f32x2 ld_pair(const float* p) { return *reinterpret_cast<const f32x2*>(p); }
__device__ __forceinline__ void st_pair(float* p, f32x2 v) { *reinterpret_cast<f32x2*>(p) = v; }
__device__ __forceinline__ uint32_t ld_u16(const unsigned char* p) {
    return *reinterpret_cast<const unsigned short*>(p);
}
__device__ __forceinline__ float lo_of(f32x2 v) { float l, h; upk2(v, l, h); return l; }
__device__ __forceinline__ float hi_of(f32x2 v) { float l, h; upk2(v, l, h); return h; }

// Neighbour sum of one row's float2 group updating half-row q, in the reference's order
// (x+1, x-1, y+1, y-1, z+1, z-1). `f` points at the group in half-row q of the row's slot;
// `zo` is the group of the other half-row (registers). q is a constant after unrolling.
template <int WJ>
__device__ __forceinline__ f32x2 rp_sum(int q, f32x2 xp, f32x2 xm, f32x2 zo, const float* f) {
    const f32x2 yp = ld_pair(f + 2 * WJ);
    const f32x2 ym = ld_pair(f - 2 * WJ);
    f32x2 s = add2(xp, xm);
    s = add2(s, yp);
    s = add2(s, ym);
    if (q == 0) {
        // even cells j, j+1: z+1 = odd j, j+1 (zo); z-1 = odd j-1 (edge), odd j
        const float e = f[WJ - 1];
        s = add2(s, zo);
        s = add2(s, pk2(e, lo_of(zo)));
    } else {
        // odd cells j, j+1: z+1 = even j+1, j+2 (edge); z-1 = even j, j+1 (zo)
        const float e = f[-WJ + 2];
        s = add2(s, pk2(hi_of(zo), e));
        s = add2(s, zo);
    }
    return s;
}

// Quotients sum / neighbour count of one row's lane pair, correctly rounded (Brisebarre, Muller,
// Raina with the pair table, as update4_binary); `idx` = 9 n_lo + n_hi of the two cells.
__device__ __forceinline__ f32x2 rp_quotient(f32x2 s, uint32_t idx, const float4* tab) {
    const float4 t = tab[idx * DIV_COPIES];
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
__device__ __forceinline__ f32x2 rp_tiny(f32x2 s, uint32_t idx, const float4* tab) {
    const float4 t = tab[idx * DIV_COPIES];
    float a, b;
    upk2(s, a, b);
    const float4 q = tiny_quotients(make_float4(a, b, 0.f, 0.f), make_float4(-t.x, -t.y, 1.f, 1.f),
                                    make_float4(t.z, t.w, 1.f, 1.f));
    return pk2(q.x, q.y);
}

// |bits - 1| of a lane: +-0 becomes a NaN (skipped by fminf), anything else loses one ulp.
__device__ __forceinline__ float tiny_key(float v) { return fabsf(__int_as_float(__float_as_int(v) - 1)); }

// One half-sweep of both rows of the pair: P updates half-row qp, Q half-row 1 - qp (qp is a
// constant after unrolling).
// `ki` holds the plane's four table indices, one byte each: row P even / odd half-row, then
// row Q even / odd half-row.
template <int WJ>
__device__ __forceinline__ void rp_stage(int qp, f32x2& cP, f32x2 xpP, f32x2 xmP, f32x2 zoP, float* fP,
                                         f32x2& cQ, f32x2 xpQ, f32x2 xmQ, f32x2 zoQ, float* fQ, uint32_t ki,
                                         float omega, const float4* tab, bool store) {
    const int qq = 1 - qp;
    const uint32_t iP = (ki >> (8 * qp)) & 0xffu, iQ = (ki >> (16 + 8 * qq)) & 0xffu;
    const f32x2 sP = rp_sum<WJ>(qp, xpP, xmP, zoP, fP);
    const f32x2 sQ = rp_sum<WJ>(qq, xpQ, xmQ, zoQ, fQ);
    f32x2 qP = rp_quotient(sP, iP, tab);
    f32x2 qQ = rp_quotient(sQ, iQ, tab);
    // 0 < |sum| <= 2^-90: the correction term may underflow; IEEE division instead (never in practice)
    const float m = fminf(fminf(tiny_key(lo_of(sP)), tiny_key(hi_of(sP))), fminf(tiny_key(lo_of(sQ)), tiny_key(hi_of(sQ))));
    if (m < 0x1p-90f) {
        qP = rp_tiny(sP, iP, tab);
        qQ = rp_tiny(sQ, iQ, tab);
    }
    cP = rp_sor(cP, qP, omega);
    cQ = rp_sor(cQ, qQ, omega);
    if (store) {
        st_pair(fP, cP);
        st_pair(fQ, cQ);
    }
}

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

template <int TY, int TZ, int K>
__device__ __forceinline__ void stream_tile_rp(const CUtensorMap* tmf, const CUtensorMap* tmc, const SweepArgs& a,
                                               int j0, int y0, int b, int x0, int x1, unsigned char* smem) {
    using S = RowPairShape<TY, TZ, K>;
    constexpr int WJ = S::WJ, WJC = S::WJC, NS = S::NS, D = S::D, R = S::R, NT = S::NT, NP = S::NP;
    constexpr int FS = S::FSTRIDE / 4;  // floats between slots
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    int* s_fail = reinterpret_cast<int*>(smem + 120);
    float4* tab_all = reinterpret_cast<float4*>(smem + 128);
    const float4* tab = division_copy(tab_all);
    float* const F0 = reinterpret_cast<float*>(smem + S::FIELD0);
    unsigned char* const C0 = smem + S::CODE0;

    const Geo& g = a.g;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int NX = g.NX;
    const int c0 = a.first_colour;

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

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
        *s_fail = 0;
    }
    fill_division_table(tab_all, tid, NT);
    // zero guards: [HEAD, FIELD0) before slot 0, and from the end of each slot's field to the
    // next slot (rows -1 and ROWS of every slot read zeros)
    for (int s = -1; s < NS; ++s) {
        const int lo = s < 0 ? S::HEAD : S::FIELD0 + s * S::FSTRIDE + S::FBYTES;
        const int hi = S::FIELD0 + (s + 1) * S::FSTRIDE;
        float* gp = reinterpret_cast<float*>(smem + lo);
        for (int i = tid; i < (hi - lo) / 4; i += NT) gp[i] = 0.0f;
    }
    __syncthreads();

    const int xs = x0 > K ? x0 - K : 0;
    const int xe = x1 + K < NX ? x1 + K : NX;
    const int row0 = 2 * (y0 + HY - K);
    auto issue = [&](int x) {
        const int s = (int)((unsigned)(x - xs) % NS);
        mbar_arrive_expect_tx(&bar[s], S::FBYTES + S::CBYTES);
        tma_load_3d(F0 + s * FS, tmf, &bar[s], j0, row0, b * NX + x);
        tma_load_3d(C0 + s * S::CSTRIDE, tmc, &bar[s], j0, row0, b * NX + x);
    };
    if (tid == 0)
        for (int x = xs; x < xs + D && x < xe; ++x) issue(x);

    // rows of the pair: P has (xs + y + c0) even
    const int rp = (xs + y0 - K + c0) & 1;
    const int rP = 2 * k + rp, rQ = 2 * k + 1 - rp;
    const int yP = y0 - K + rP, yQ = y0 - K + rQ;
    const int offP = 2 * rP * WJ + jj, offQ = 2 * rQ * WJ + jj;     // half-row 0 of each row (floats)
    const int coP = 2 * rP * WJC + jj, coQ = 2 * rQ * WJC + jj;     // code bytes
    // bit s: the pair takes part in half-sweep s (a row of it lies in [s, ROWS - s)); the halo warp
    // takes part in every half-sweep
    uint32_t stage_mask = 0;
#pragma unroll
    for (int s = 1; s <= K; ++s)
        stage_mask |= (halo || (2 * k + 1 >= s && 2 * k < S::ROWS - s)) ? (1u << s) : 0u;
    const bool wP = !halo && rP >= K && rP < K + TY && yP < g.NY;
    const bool wQ = !halo && rQ >= K && rQ < K + TY && yQ < g.NY;
    const int jglob = j0 + jj - HJ;  // interior index of the group's first cell
    const bool py = a.periodic & TF_PERIODIC_Y, pz = a.periodic & TF_PERIODIC_Z;
    const float omega = a.omega;

    // ring by relative colour: P0/P1 (row P), Q0/Q1 (row Q); KI: the division-table indices of
    // the plane's four half-row groups (bytes: P even, P odd, Q even, Q odd)
    f32x2 P0[R], P1[R], Q0[R], Q1[R];
    uint32_t KI[R];
    const f32x2 glo = pk2(a.glo, a.glo), ghi = pk2(a.ghi, a.ghi);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        P0[r] = P1[r] = Q0[r] = Q1[r] = glo;
        KI[r] = 0u;
    }

    const int total = xe == NX ? NX + K : xe;
    for (int t0 = xs; t0 < total; t0 += R) {
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int t = t0 + i;
            if (t < total) {
                if (tid == 0 && t + D < xe) issue(t + D);
                if (t < xe) {
                    const int slot = (int)((unsigned)(t - xs) % NS);
                    if (!mbar_wait_bounded(&bar[slot], ((unsigned)(t - xs) / NS) & 1)) *s_fail = 1;
                    const float* Fs = F0 + slot * FS;
                    const unsigned char* Cs = C0 + slot * S::CSTRIDE;
                    const f32x2 eP = ld_pair(Fs + offP), oP = ld_pair(Fs + offP + WJ);
                    const f32x2 eQ = ld_pair(Fs + offQ), oQ = ld_pair(Fs + offQ + WJ);
                    // 9 n_lo + n_hi per half-row group, counts masked to 4 bits (index <= 150:
                    // inside the CTA's shared memory whatever the code bytes hold)
                    const uint32_t cP = (ld_u16(Cs + coP) | (ld_u16(Cs + coP + WJC) << 16)) & 0x0f0f0f0fu;
                    const uint32_t cQ = (ld_u16(Cs + coQ) | (ld_u16(Cs + coQ + WJC) << 16)) & 0x0f0f0f0fu;
                    KI[i] = (uint32_t)__dp4a((int)cP, 0x0109, 0) | ((uint32_t)__dp4a((int)cP, 0x01090000, 0) << 8) |
                            ((uint32_t)__dp4a((int)cQ, 0x0109, 0) << 16) |
                            ((uint32_t)__dp4a((int)cQ, 0x01090000, 0) << 24);
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
#pragma unroll
                for (int s = 1; s <= K; ++s) {
                    const int p = t - s;
                    const int ip = (i - s + 2 * R) % R;
                    const int ipn = (i - s + 1 + 2 * R) % R;
                    const int ipp = (i - s - 1 + 2 * R) % R;
                    if (p >= xs && p < NX && (stage_mask & (1u << s))) {
                        float* Fp = F0 + (int)((unsigned)(p - xs) % NS) * FS;
                        if (((s - 1) & 1) == 0) {
                            rp_stage<WJ>(qp, P0[ip], P1[ipn], P1[ipp], P1[ip], Fp + offP + qp * WJ,
                                         Q0[ip], Q1[ipn], Q1[ipp], Q1[ip], Fp + offQ + (1 - qp) * WJ, KI[ip],
                                         omega, tab, !dup);
                        } else {
                            rp_stage<WJ>(qp, P1[ip], P0[ipn], P0[ipp], P0[ip], Fp + offP + qp * WJ,
                                         Q1[ip], Q0[ipn], Q0[ipp], Q0[ip], Fp + offQ + (1 - qp) * WJ, KI[ip],
                                         omega, tab, !dup);
                        }
                    }
                }
                // write back plane t-K from registers: even half-row of P is relative colour 0 at even i
                const int pw = t - K;
                const int iw = (i - K + 2 * R) % R;
                if (pw >= x0 && pw < x1) {
                    if (wP) {
                        if ((i & 1) == 0) rp_write_row(a, b, pw, yP, jglob, P0[iw], P1[iw], py, pz);
                        else rp_write_row(a, b, pw, yP, jglob, P1[iw], P0[iw], py, pz);
                    }
                    if (wQ) {
                        if ((i & 1) == 0) rp_write_row(a, b, pw, yQ, jglob, Q1[iw], Q0[iw], py, pz);
                        else rp_write_row(a, b, pw, yQ, jglob, Q0[iw], Q1[iw], py, pz);
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

// 13 warps: one SM sub-partition holds 4 of them, which caps a thread at 128 registers.
template <int TY, int TZ, int K>
__global__ void __launch_bounds__(RowPairShape<TY, TZ, K>::NT, 1)
    k_stream_rp(const __grid_constant__ CUtensorMap tmf, const __grid_constant__ CUtensorMap tmc, const SweepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int b = blockIdx.z / a.x_chunks, c = blockIdx.z - b * a.x_chunks;
    const int x0 = (int)((long long)c * a.g.NX / a.x_chunks), x1 = (int)((long long)(c + 1) * a.g.NX / a.x_chunks);
    stream_tile_rp<TY, TZ, K>(&tmf, &tmc, a, blockIdx.x * (TZ / 2), blockIdx.y * TY, b, x0, x1, smem);
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
