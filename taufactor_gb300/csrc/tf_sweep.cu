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
#include "tf_update.cuh"

namespace tf {

// ------------------------------------------------------------------------------ plain kernel
template <int KIND, bool RHS>
__global__ void __launch_bounds__(256) k_plain(float* __restrict__ f, const uint8_t* __restrict__ code,
                                               const SweepArgs a, const __grid_constant__ tf_operator op, int colour) {
    __shared__ float lut[32 * 32];
    __shared__ float4 tab[DIV_PAIRS * DIV_COPIES];
    if (KIND == TF_KIND_ANISOTROPIC)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = op.divisor[i];
    if (KIND == TF_KIND_ELECTRODE)
        fill_electrode_divisors(lut, op.divisor[(blockIdx.z / a.g.NX) & 255], threadIdx.x, blockDim.x);
    if (KIND == TF_KIND_MULTIPHASE)
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) lut[i] = op.face[i];
    if (KIND == TF_KIND_BINARY) fill_division_table(tab, threadIdx.x, blockDim.x);
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
    float4 rv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (RHS) rv = *reinterpret_cast<const float4*>(a.rhs + base + q * g.ZH + HJ + j);
    const float4 nv = update4<KIND, RHS>(c, xp, xm, yp, ym, zp, zm, cc, cxp, cxm, cyp, cym, czp, czm, x == 0,
                                         x == g.NX - 1, a.omega, a.ky, a.kz, lut, division_copy(tab), rv);
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

// Exhaustive check of div_small_exact against IEEE division for divisor n over every finite float32
// bit pattern. Counts mismatching results (bitwise, so signed zeros count) into *bad.
__global__ void k_check_division(int n, unsigned long long* bad) {
    const float nf = static_cast<float>(n);
    const float r = __frcp_rn(nf);
    unsigned long long local = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < (1ull << 32); u += stride) {
        const float s = __uint_as_float(static_cast<uint32_t>(u));
        if (!isfinite(s)) continue;
        const float a = div_small_exact(s, nf, r);
        const float b = __fdiv_rn(s, nf);
        if (__float_as_uint(a) != __float_as_uint(b)) ++local;
        // the sweeps' form: equal up to the sign of a zero quotient ...
        const float f = (s != 0.0f && fabsf(s) < 0x1p-90f) ? __fdiv_rn(s, nf) : div_small_fast(s, nf, r);
        if (__float_as_uint(f) != __float_as_uint(b) && !(f == 0.0f && b == 0.0f)) ++local;
        // ... which the SOR step maps to the same bits (s taken as the old value c)
        const float w = 1.0f + 0.125f * static_cast<float>(n);
        if (__float_as_uint(sor_finish(s, 0.0f, w)) != __float_as_uint(sor_finish(s, -0.0f, w))) ++local;
    }
    if (local) atomicAdd(bad, local);
}

int check_small_division(int n, unsigned long long* bad_dev, cudaStream_t st) {
    k_check_division<<<152 * 8, 256, 0, st>>>(n, bad_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

// ------------------------------------------------------------------------------ host side
SweepArgs make_args(const Geo& g, const tf_operator& op, float* out, int first_colour, int n_half,
                           int32_t* err) {
    SweepArgs a;
    a.g = g; a.out = out; a.omega = op.omega; a.glo = op.ghost_lo; a.ghi = op.ghost_hi;
    a.ky = op.ky; a.kz = op.kz; a.first_colour = first_colour & 1; a.n_half = n_half; a.err = err;
    a.periodic = op.periodic;
    a.x_chunks = 1;
    a.rhs = nullptr;
    a.fx = a.fy = a.fz = a.dv = nullptr;
    return a;
}

int sweep_plain(const tf_geom& gg, const tf_operator& op, float* f, const uint8_t* code, const float* rhs,
                int colour, cudaStream_t st) {
    const Geo g = make_geo(gg);
    SweepArgs a = make_args(g, op, f, colour, 1, nullptr);
    a.rhs = rhs;
    const int gmax = (half_len(g.NZ, 0) + 3) >> 2;
    dim3 block(gmax >= 128 ? 128 : (gmax >= 32 ? 64 : 32));
    dim3 grid((gmax + block.x - 1) / block.x, g.NY, g.B * g.NX);
#define TF_PLAIN(K)                                                                        \
    (rhs ? k_plain<K, true><<<grid, block, 0, st>>>(f, code, a, op, colour)                  \
         : k_plain<K, false><<<grid, block, 0, st>>>(f, code, a, op, colour))
    switch (op.kind) {
        case TF_KIND_BINARY: TF_PLAIN(TF_KIND_BINARY); break;
        case TF_KIND_ANISOTROPIC: TF_PLAIN(TF_KIND_ANISOTROPIC); break;
        case TF_KIND_MULTIPHASE: TF_PLAIN(TF_KIND_MULTIPHASE); break;
        case TF_KIND_ELECTRODE: TF_PLAIN(TF_KIND_ELECTRODE); break;
        default: return TF_ERR_ARG;
    }
#undef TF_PLAIN
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


}  // namespace tf
