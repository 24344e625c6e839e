// Red-black SOR half-sweeps on the 7-point stencil (sm_103a).
//
// k_tiled   : several half-sweeps per launch. Each CTA owns a TY x TZ tile of the (y, z)
//             plane and marches along x. Planes of the tile plus HY ghost rows / HJ ghost cells
//             are staged into a shared-memory ring by TMA (cp.async.bulk.tensor, mbarrier
//             completion, D planes ahead). Half-sweep s of the launch is applied to plane t-s at
//             step t (a wavefront in x), on a region that shrinks by one cell per half-sweep so
//             the tile interior is exact; the interior of the final plane is written to the
//             other ping-pong buffer (plus periodic ghost copies). Result = n_half reference
//             iterations of taufactor.py:174-182, bit for bit.
// k_plain   : one half-sweep in place straight from global memory; used where the tiled kernel
//             does not apply (periodic faces of odd or tiny size), followed by k_ghosts, which
//             refreshes periodic ghost cells like PeriodicSolver.apply_boundary_conditions
//             (taufactor.py:501-505).
#include "tf_common.cuh"
#include "tf_internal.h"

namespace tf {

struct SweepArgs {
    Geo g;
    float* out;
    float omega, glo, ghi, ky, kz;
    int first_colour, n_half;
    int32_t* err;
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float comp(const float4& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set_comp(float4& v, int i, float f) {
    if (i == 0) v.x = f; else if (i == 1) v.y = f; else if (i == 2) v.z = f; else v.w = f;
}
__device__ __forceinline__ uint32_t byte_of(uint32_t w, int i) { return (w >> (8 * i)) & 0xffu; }

// One float4 group of a colour-c half-row: 4 updates.
//   c        the 4 cells; xp/xm/yp/ym their x+1, x-1, y+1, y-1 neighbours;
//   zp/zm    their z+1, z-1 neighbours; codes: 4 code bytes of the cells and of each neighbour
//            set (multiphase needs them for the faces); at_lo/at_hi: plane is x = 0 / x = nx-1.
template <int KIND>
__device__ __forceinline__ float4 update4(float4 c, const float4& xp, const float4& xm, const float4& yp,
                                          const float4& ym, const float4& zp, const float4& zm, uint32_t cc,
                                          uint32_t cxp, uint32_t cxm, uint32_t cyp, uint32_t cym, uint32_t czp,
                                          uint32_t czm, bool at_lo, bool at_hi, float omega, float ky, float kz,
                                          const float* lut) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float ci = comp(c, i);
        float sum, div;
        if (KIND == TF_KIND_BINARY) {
            // sum order of taufactor.py:97-102: x+1, x-1, y+1, y-1, z+1, z-1
            sum = __fadd_rn(comp(xp, i), comp(xm, i));
            sum = __fadd_rn(sum, comp(yp, i));
            sum = __fadd_rn(sum, comp(ym, i));
            sum = __fadd_rn(sum, comp(zp, i));
            sum = __fadd_rn(sum, comp(zm, i));
            const uint32_t n = byte_of(cc, i);
            div = n ? static_cast<float>(n) : __int_as_float(0x7f800000);
        } else if (KIND == TF_KIND_ANISOTROPIC) {
            // taufactor.py:475-477: (x+1 + x-1) + Ky*(y+1 + y-1) + Kz*(z+1 + z-1)
            sum = __fadd_rn(comp(xp, i), comp(xm, i));
            sum = __fadd_rn(sum, __fmul_rn(ky, __fadd_rn(comp(yp, i), comp(ym, i))));
            sum = __fadd_rn(sum, __fmul_rn(kz, __fadd_rn(comp(zp, i), comp(zm, i))));
            div = lut[byte_of(cc, i)];
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
            div = __fadd_rn(fxm, fxp);
            div = __fadd_rn(div, fym);
            div = __fadd_rn(div, fyp);
            div = __fadd_rn(div, fzm);
            div = __fadd_rn(div, fzp);
            if (at_lo) div = __fadd_rn(div, fxm);
            if (at_hi) div = __fadd_rn(div, fxp);
            if (div == 0.0f) div = __int_as_float(0x7f800000);
        }
        set_comp(c, i, sor_update(ci, sum, div, omega));
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

// ------------------------------------------------------------------------------ tiled kernel
template <int TY, int TZ>
struct TiledShape {
    static constexpr int TJ = TZ / 2;                 // interior cells per half-row
    static constexpr int WJ = TJ + 2 * HJ;            // floats per staged half-row
    static constexpr int WJC = (WJ + 15) / 16 * 16;   // bytes per staged code half-row
    static constexpr int ROWS = 2 * (TY + 2 * HY);    // staged half-rows per plane
    static constexpr int D = 2;                       // planes loaded ahead
    static constexpr int NS = HY + 2 + D;             // ring slots
    static constexpr int FBYTES = ROWS * WJ * 4;
    static constexpr int CBYTES = ROWS * WJC;
    static constexpr int GUARD = 128;                 // readable guard around each field slot
    static constexpr int FSPAN = (GUARD + FBYTES + GUARD + 127) / 128 * 128;
    static constexpr int SLOT = FSPAN + (CBYTES + 127) / 128 * 128;
    static constexpr int LUT_BYTES = 32 * 32 * 4;
    static constexpr int HEAD = 128 + LUT_BYTES;      // mbarriers + LUT
    static constexpr int SMEM = HEAD + NS * SLOT + 128;  // +128: base alignment slack
    static constexpr int NT = 256;
};

template <int KIND, int TY, int TZ, bool PY, bool PZ>
__global__ void __launch_bounds__(256, 2)
    k_tiled(const __grid_constant__ CUtensorMap tmf, const __grid_constant__ CUtensorMap tmc, const SweepArgs a,
            const __grid_constant__ tf_operator op) {
    using S = TiledShape<TY, TZ>;
    constexpr int NT = S::NT, WJ = S::WJ, WJC = S::WJC, NS = S::NS, D = S::D, TJ = S::TJ;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    float* lut = reinterpret_cast<float*>(smem + 128);
    __shared__ int s_fail;
    auto F = [&](int slot) { return reinterpret_cast<float*>(smem + S::HEAD + slot * S::SLOT + S::GUARD); };
    auto C = [&](int slot) { return smem + S::HEAD + slot * S::SLOT + S::FSPAN; };

    const Geo& g = a.g;
    const int tid = threadIdx.x;
    const int j0 = blockIdx.x * TJ;
    const int y0 = blockIdx.y * TY;
    const int b = blockIdx.z;
    const int NX = g.NX;
    const int k = a.n_half;

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
        s_fail = 0;
    }
    if (KIND == TF_KIND_ANISOTROPIC)
        for (int i = tid; i < 256; i += NT) lut[i] = op.divisor[i];
    if (KIND == TF_KIND_MULTIPHASE)
        for (int i = tid; i < 32 * 32; i += NT) lut[i] = op.face[i];
    // zero the guards once: stale guard contents only feed cells that are never written back
    for (int s = 0; s < NS; ++s) {
        float* f = F(s);
        for (int i = tid; i < S::GUARD / 4; i += NT) {
            f[-1 - i] = 0.0f;
            f[S::FBYTES / 4 + i] = 0.0f;
        }
    }
    __syncthreads();

    auto issue = [&](int x) {
        const int s = x % NS;
        mbar_arrive_expect_tx(&bar[s], S::FBYTES + S::CBYTES);
        tma_load_3d(F(s), &tmf, &bar[s], j0, 2 * y0, b * NX + x);
        tma_load_3d(C(s), &tmc, &bar[s], j0, 2 * y0, b * NX + x);
    };
    if (tid == 0)
        for (int x = 0; x < D && x < NX; ++x) issue(x);

    const float omega = a.omega;
    for (int t = 0; t < NX + k; ++t) {
        if (tid == 0 && t + D < NX) issue(t + D);
        if (t < NX) {
            if (!mbar_wait_bounded(&bar[t % NS], (t / NS) & 1)) s_fail = 1;
        }
        __syncthreads();
        if (s_fail) {
            // drain loads still in flight (bounded), report, leave
            if (tid == 0) {
                for (int x = t + 1; x < t + 1 + D && x < NX; ++x) mbar_wait_bounded(&bar[x % NS], (x / NS) & 1);
                if (a.err) atomicExch(a.err, TF_ERR_TIMEOUT);
            }
            return;
        }
        for (int s = 1; s <= k; ++s) {
            const int p = t - s;
            if (p >= 0 && p < NX) {
                const int colour = (a.first_colour + s - 1) & 1;
                const int rlo = HY - (k - s);
                const int nrows = TY + 2 * (k - s);
                constexpr int G = WJ / 4;
                const float* Fm = p > 0 ? F((p - 1) % NS) : nullptr;
                const float* Fx = p + 1 < NX ? F((p + 1) % NS) : nullptr;
                const unsigned char* Cm = p > 0 ? C((p - 1) % NS) : nullptr;
                const unsigned char* Cx = p + 1 < NX ? C((p + 1) % NS) : nullptr;
                float* Fp = F(p % NS);
                const unsigned char* Cp = C(p % NS);
                const float4 glo4 = make_float4(a.glo, a.glo, a.glo, a.glo);
                const float4 ghi4 = make_float4(a.ghi, a.ghi, a.ghi, a.ghi);
                for (int it = tid; it < nrows * G; it += NT) {
                    const int r = it / G;
                    const int gi = it - r * G;
                    const int ty = rlo + r;
                    const int y = y0 - HY + ty;
                    const int q = (p + y + colour) & 1;
                    const int row = 2 * ty + q, orow = 2 * ty + (q ^ 1);
                    const int jj = 4 * gi;
                    const float4 c = ld4(Fp + row * WJ + jj);
                    const float4 xp = Fx ? ld4(Fx + row * WJ + jj) : ghi4;
                    const float4 xm = Fm ? ld4(Fm + row * WJ + jj) : glo4;
                    const float4 yp = ld4(Fp + (row + 2) * WJ + jj);
                    const float4 ym = ld4(Fp + (row - 2) * WJ + jj);
                    const float4 o = ld4(Fp + orow * WJ + jj);
                    const float e = q ? Fp[orow * WJ + jj + 4] : Fp[orow * WJ + jj - 1];
                    float4 zp, zm;
                    z_neighbours(q, o, e, zp, zm);
                    const uint32_t cc = *reinterpret_cast<const uint32_t*>(Cp + row * WJC + jj);
                    uint32_t cxp = 0, cxm = 0, cyp = 0, cym = 0, czp = 0, czm = 0;
                    if (KIND == TF_KIND_MULTIPHASE) {
                        cxp = Cx ? *reinterpret_cast<const uint32_t*>(Cx + row * WJC + jj) : cc;
                        cxm = Cm ? *reinterpret_cast<const uint32_t*>(Cm + row * WJC + jj) : cc;
                        cyp = *reinterpret_cast<const uint32_t*>(Cp + (row + 2) * WJC + jj);
                        cym = *reinterpret_cast<const uint32_t*>(Cp + (row - 2) * WJC + jj);
                        const uint32_t co = *reinterpret_cast<const uint32_t*>(Cp + orow * WJC + jj);
                        // the edge byte: jj-1 / jj+4 stay inside the code slot except at its two
                        // ends, where the value only feeds cells that are never written back
                        const int ei = q ? jj + 4 : jj - 1;
                        const uint32_t ce = (ei >= 0 && ei < WJC) ? Cp[orow * WJC + ei] : 0u;
                        z_codes(q, co, ce, czp, czm);
                    }
                    const float4 nv = update4<KIND>(c, xp, xm, yp, ym, zp, zm, cc, cxp, cxm, cyp, cym, czp, czm,
                                                    p == 0, p == NX - 1, omega, a.ky, a.kz, lut);
                    st4(Fp + row * WJ + jj, nv);
                }
            }
            __syncthreads();
        }
        const int p = t - k;
        if (p >= 0 && p < NX) {
            // write back the tile interior of plane p (+ periodic ghost copies)
            constexpr int GI = TJ / 4;
            const float* Fp = F(p % NS);
            float* outp = a.out + (long long)b * g.vol_f + (long long)p * g.plane_f;
            for (int it = tid; it < TY * 2 * GI; it += NT) {
                const int gi = it % GI;
                const int rq = it / GI;
                const int q = rq & 1;
                const int y = y0 + (rq >> 1);
                const int j = j0 + 4 * gi;
                const int nj = half_len(g.NZ, q);
                if (y >= g.NY || j >= nj) continue;
                const float4 v = ld4(Fp + (2 * (HY + (rq >> 1)) + q) * WJ + HJ + 4 * gi);
                float* dst = outp + (long long)(y + HY) * g.row_f + q * g.ZH + HJ + j;
                if (j + 4 <= nj) {
                    st4(dst, v);
                } else {
                    for (int i = 0; i < nj - j; ++i) dst[i] = comp(v, i);
                }
                if (PY || PZ) {
                    // periodic ghost copies; the tiled kernel runs periodic faces of even size
                    // >= the ghost width only, so a single wrap suffices and parity is kept
                    const int hz = g.NZ >> 1;
                    int ys[2] = {y, y};
                    int nys = 1;
                    if (PY && y < HY) ys[nys++] = y + g.NY;
                    else if (PY && y >= g.NY - HY) ys[nys++] = y - g.NY;
                    for (int yi = 0; yi < nys; ++yi) {
                        float* rowp = outp + (long long)(ys[yi] + HY) * g.row_f + q * g.ZH + HJ;
                        for (int i = 0; i < 4 && j + i < nj; ++i) {
                            const int jj = j + i;
                            if (yi > 0) rowp[jj] = comp(v, i);
                            if (PZ && jj < HJ) rowp[jj + hz] = comp(v, i);
                            else if (PZ && jj >= hz - HJ) rowp[jj - hz] = comp(v, i);
                        }
                    }
                }
            }
        }
        fence_proxy_async_smem();
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------ plain kernel
template <int KIND>
__global__ void __launch_bounds__(256) k_plain(float* __restrict__ f, const uint8_t* __restrict__ code,
                                               const SweepArgs a, const __grid_constant__ tf_operator op, int colour) {
    __shared__ float lut[32 * 32];
    if (KIND == TF_KIND_ANISOTROPIC)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = op.divisor[i];
    if (KIND == TF_KIND_MULTIPHASE)
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) lut[i] = op.face[i];
    __syncthreads();
    const Geo& g = a.g;
    const int gmax = (half_len(g.NZ, 0) + 3) >> 2;
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int bx = blockIdx.z;  // b*NX + x
    const int x = bx % g.NX;
    const int b = bx / g.NX;
    if (gi >= gmax) return;
    const int q = (x + y + colour) & 1;
    const int nj = half_len(g.NZ, q);
    const int j = 4 * gi;
    if (j >= nj) return;
    const long long base = (long long)b * g.vol_f + (long long)x * g.plane_f + (long long)(y + HY) * g.row_f;
    const long long cbase = (long long)b * g.vol_c + (long long)x * g.plane_c + (long long)(y + HY) * g.row_c;
    const float* row = f + base + q * g.ZH + HJ;
    const float* orow = f + base + (q ^ 1) * g.ZH + HJ;
    const uint8_t* crow = code + cbase + q * g.ZHC + HJ;
    const uint8_t* corow = code + cbase + (q ^ 1) * g.ZHC + HJ;
    const float4 c = ld4(row + j);
    const float4 xp = x + 1 < g.NX ? ld4(row + g.plane_f + j) : make_float4(a.ghi, a.ghi, a.ghi, a.ghi);
    const float4 xm = x > 0 ? ld4(row - g.plane_f + j) : make_float4(a.glo, a.glo, a.glo, a.glo);
    const float4 yp = ld4(row + g.row_f + j);
    const float4 ym = ld4(row - g.row_f + j);
    const float4 o = ld4(orow + j);
    const float e = q ? orow[j + 4] : orow[j - 1];
    float4 zp, zm;
    z_neighbours(q, o, e, zp, zm);
    auto ld_code = [](const uint8_t* p) {
        return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    };
    const uint32_t cc = ld_code(crow + j);
    uint32_t cxp = 0, cxm = 0, cyp = 0, cym = 0, czp = 0, czm = 0;
    if (KIND == TF_KIND_MULTIPHASE) {
        cxp = x + 1 < g.NX ? ld_code(crow + g.plane_c + j) : cc;
        cxm = x > 0 ? ld_code(crow - g.plane_c + j) : cc;
        cyp = ld_code(crow + g.row_c + j);
        cym = ld_code(crow - g.row_c + j);
        z_codes(q, ld_code(corow + j), q ? corow[j + 4] : corow[j - 1], czp, czm);
    }
    const float4 nv = update4<KIND>(c, xp, xm, yp, ym, zp, zm, cc, cxp, cxm, cyp, cym, czp, czm, x == 0,
                                    x == g.NX - 1, a.omega, a.ky, a.kz, lut);
    float* dst = f + base + q * g.ZH + HJ + j;
    for (int i = 0; i < 4 && j + i < nj; ++i) dst[i] = comp(nv, i);
}

// Periodic ghost cells <- wrapped interior (any size; also odd). One thread per row position.
__global__ void k_ghosts(float* __restrict__ f, Geo g, int periodic) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q*ZH + jp within the row
    const int Y = blockIdx.y;                               // padded row
    const int bx = blockIdx.z;
    if (pos >= 2 * g.ZH) return;
    const int q = pos >= g.ZH ? 1 : 0;
    const int jp = pos - q * g.ZH;
    const int y = Y - HY;
    const int z = 2 * (jp - HJ) + q;
    const bool yin = y >= 0 && y < g.NY;
    const bool zin = z >= 0 && z < g.NZ && (jp - HJ) >= 0;
    if (yin && zin) return;
    const bool py = periodic & TF_PERIODIC_Y, pz = periodic & TF_PERIODIC_Z;
    if ((!yin && !py) || (!zin && !pz)) return;
    const int ys = yin ? y : wrap(y, g.NY);
    const int zs = zin ? z : wrap(z, g.NZ);
    const long long plane = (long long)bx * g.plane_f;
    f[plane + (long long)Y * g.row_f + pos] =
        f[plane + (long long)(ys + HY) * g.row_f + (zs & 1) * g.ZH + HJ + (zs >> 1)];
}

// ------------------------------------------------------------------------------ host side
template <int KIND, int TY, int TZ, bool PY, bool PZ>
static int launch_tiled_t(const CUtensorMap& tmf, const CUtensorMap& tmc, const SweepArgs& a,
                          const tf_operator& op, cudaStream_t st) {
    using S = TiledShape<TY, TZ>;
    static bool attr_set = false;
    auto kern = k_tiled<KIND, TY, TZ, PY, PZ>;
    if (!attr_set) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM) != cudaSuccess)
            return TF_ERR_CUDA;
        attr_set = true;
    }
    dim3 grid((a.g.NZ + TZ - 1) / TZ, (a.g.NY + TY - 1) / TY, a.g.B);
    kern<<<grid, S::NT, S::SMEM, st>>>(tmf, tmc, a, op);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

template <int KIND>
static int launch_tiled_k(const CUtensorMap& tmf, const CUtensorMap& tmc, const SweepArgs& a,
                          const tf_operator& op, cudaStream_t st) {
    const bool py = op.periodic & TF_PERIODIC_Y, pz = op.periodic & TF_PERIODIC_Z;
    if (py && pz) return launch_tiled_t<KIND, TILE_Y, TILE_Z, true, true>(tmf, tmc, a, op, st);
    if (py) return launch_tiled_t<KIND, TILE_Y, TILE_Z, true, false>(tmf, tmc, a, op, st);
    if (pz) return launch_tiled_t<KIND, TILE_Y, TILE_Z, false, true>(tmf, tmc, a, op, st);
    return launch_tiled_t<KIND, TILE_Y, TILE_Z, false, false>(tmf, tmc, a, op, st);
}

static SweepArgs make_args(const Geo& g, const tf_operator& op, float* out, int first_colour, int n_half,
                           int32_t* err) {
    SweepArgs a;
    a.g = g; a.out = out; a.omega = op.omega; a.glo = op.ghost_lo; a.ghi = op.ghost_hi;
    a.ky = op.ky; a.kz = op.kz; a.first_colour = first_colour & 1; a.n_half = n_half; a.err = err;
    return a;
}

int sweep_tiled(const tf_geom& gg, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    using S = TiledShape<TILE_Y, TILE_Z>;
    const Geo g = make_geo(gg);
    CUtensorMap tmf, tmc;
    // field: dims {zh, 2*yp, batch*nx}; box {WJ, ROWS, 1}
    int rc = encode_map_3d(&tmf, in, /*elem bytes*/ 4, gg.zh, 2 * gg.yp, (long long)gg.batch * gg.nx,
                           (long long)gg.zh * 4, (long long)gg.zh * 4 * 2 * gg.yp, S::WJ, S::ROWS);
    if (rc) return rc;
    rc = encode_map_3d(&tmc, code, 1, gg.zhc, 2 * gg.yp, (long long)gg.batch * gg.nx, gg.zhc,
                       (long long)gg.zhc * 2 * gg.yp, S::WJC, S::ROWS);
    if (rc) return rc;
    const SweepArgs a = make_args(g, op, out, first_colour, n_half, err);
    switch (op.kind) {
        case TF_KIND_BINARY: return launch_tiled_k<TF_KIND_BINARY>(tmf, tmc, a, op, st);
        case TF_KIND_ANISOTROPIC: return launch_tiled_k<TF_KIND_ANISOTROPIC>(tmf, tmc, a, op, st);
        case TF_KIND_MULTIPHASE: return launch_tiled_k<TF_KIND_MULTIPHASE>(tmf, tmc, a, op, st);
    }
    return TF_ERR_ARG;
}

int sweep_plain(const tf_geom& gg, const tf_operator& op, float* f, const uint8_t* code, int colour,
                cudaStream_t st) {
    const Geo g = make_geo(gg);
    const SweepArgs a = make_args(g, op, f, colour, 1, nullptr);
    const int gmax = (half_len(g.NZ, 0) + 3) >> 2;
    dim3 block(gmax >= 128 ? 128 : (gmax >= 32 ? 64 : 32));
    dim3 grid((gmax + block.x - 1) / block.x, g.NY, g.B * g.NX);
    switch (op.kind) {
        case TF_KIND_BINARY: k_plain<TF_KIND_BINARY><<<grid, block, 0, st>>>(f, code, a, op, colour); break;
        case TF_KIND_ANISOTROPIC: k_plain<TF_KIND_ANISOTROPIC><<<grid, block, 0, st>>>(f, code, a, op, colour); break;
        case TF_KIND_MULTIPHASE: k_plain<TF_KIND_MULTIPHASE><<<grid, block, 0, st>>>(f, code, a, op, colour); break;
        default: return TF_ERR_ARG;
    }
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    if (op.periodic) return refresh_ghosts(gg, op.periodic, f, st);
    return TF_OK;
}

int refresh_ghosts(const tf_geom& gg, int periodic, float* f, cudaStream_t st) {
    const Geo g = make_geo(gg);
    dim3 block(128);
    dim3 grid((2 * g.ZH + 127) / 128, g.YP, g.B * g.NX);
    k_ghosts<<<grid, block, 0, st>>>(f, g, periodic);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tiled_smem_bytes() { return TiledShape<TILE_Y, TILE_Z>::SMEM; }

}  // namespace tf
