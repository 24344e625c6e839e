// Setup, layout conversion and per-layer reductions (sm_103a).
//
// k_pack        phase indices (natural layout) -> code buffer + initial field in the split
//               layout, ghost cells included (taufactor.py:282-291 init_field, :402-410 /
//               :493-499 / :459-471 neighbour counts, :585-592 label map).
// k_unpack      split layout -> the reference's padded field [B][nx+2][ny+2][nz+2]
//               (taufactor.py:228-238, :501-505).
// k_repack      padded reference layout -> split layout (resume from a user field).
// k_layer_sums  per-plane float64 sums of the x-flux and of the field (taufactor.py:294-296,
//               :307, :412-419, :615-620); one CTA per (plane, volume), fixed summation order,
//               so the result does not depend on scheduling.
#include "tf_common.cuh"
#include "tf_internal.h"
#include "tf_layers.cuh"

namespace tf {

struct PackArgs {
    Geo g;
    int kind, periodic;
};

__device__ __forceinline__ bool src_cell(const Geo& g, int periodic, int y, int z, int& ys, int& zs) {
    const bool yin = y >= 0 && y < g.NY;
    const bool zin = z >= 0 && z < g.NZ;
    if (!yin && !(periodic & TF_PERIODIC_Y)) return false;
    if (!zin && !(periodic & TF_PERIODIC_Z)) return false;
    ys = yin ? y : wrap(y, g.NY);
    zs = zin ? z : wrap(z, g.NZ);
    return true;
}

// value of the mask "phase == ph" at a neighbour (0 outside closed faces, wrapped on periodic)
__device__ __forceinline__ int mask_at(const uint8_t* P, const Geo& g, int periodic, int x, int y, int z,
                                       int ph = 1) {
    int ys, zs;
    if (!src_cell(g, periodic, y, z, ys, zs)) return 0;
    return P[((long long)x * g.NY + ys) * g.NZ + zs] == ph;
}

__global__ void k_pack(const uint8_t* __restrict__ phase, const float* __restrict__ profile,
                       uint8_t* __restrict__ code, float* __restrict__ field, const PackArgs a,
                       const __grid_constant__ tf_operator op) {
    const Geo& g = a.g;
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q*ZHC + jp
    if (pos >= 2 * g.ZHC) return;
    const int Y = blockIdx.y;
    const int bx = blockIdx.z;
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = pos >= g.ZHC ? 1 : 0;
    const int jp = pos - q * g.ZHC;
    const int y = Y - HY;
    const int z = 2 * (jp - HJ) + q;
    const uint8_t* P = phase + (long long)b * g.NX * g.NY * g.NZ;
    uint8_t cd = 0;
    float fv = 0.0f;
    int ys, zs;
    if (jp < g.ZH && src_cell(g, a.periodic, y, z, ys, zs)) {
        const int ph = P[((long long)x * g.NY + ys) * g.NZ + zs];
        if (a.kind == TF_KIND_MULTIPHASE) {
            cd = (uint8_t)ph;
            fv = op.conductive[ph & 31] ? profile[x] : 0.0f;
        } else if (ph == 1 && a.kind == TF_KIND_ELECTRODE) {
            // taufactor/electrode.py:46-62: conductive neighbours with the mask padded 2 at the
            // inlet and 0 at the (closed) outlet, reactive neighbours (phase 2) padded 0
            const int per = a.periodic;
            const long long ox = ((long long)x * g.NY + ys) * g.NZ + zs, sx = (long long)g.NY * g.NZ;
            const int xm = x > 0 ? (P[ox - sx] == 1) : 2;
            const int xp = x + 1 < g.NX ? (P[ox + sx] == 1) : 0;
            const int nn = xm + xp + mask_at(P, g, per, x, ys - 1, zs) + mask_at(P, g, per, x, ys + 1, zs) +
                           mask_at(P, g, per, x, ys, zs - 1) + mask_at(P, g, per, x, ys, zs + 1);
            const int rxm = x > 0 ? (P[ox - sx] == 2) : 0;
            const int rxp = x + 1 < g.NX ? (P[ox + sx] == 2) : 0;
            const int nr = rxm + rxp + mask_at(P, g, per, x, ys - 1, zs, 2) + mask_at(P, g, per, x, ys + 1, zs, 2) +
                           mask_at(P, g, per, x, ys, zs - 1, 2) + mask_at(P, g, per, x, ys, zs + 1, 2);
            cd = (uint8_t)(1 + nn + 8 * nr);
            fv = profile[x];
        } else if (ph == 1) {
            const int per = a.periodic;
            const int xm = x > 0 ? (P[((long long)(x - 1) * g.NY + ys) * g.NZ + zs] == 1) : 2;
            const int xp = x + 1 < g.NX ? (P[((long long)(x + 1) * g.NY + ys) * g.NZ + zs] == 1) : 2;
            const int ym = mask_at(P, g, per, x, ys - 1, zs), yp = mask_at(P, g, per, x, ys + 1, zs);
            const int zm = mask_at(P, g, per, x, ys, zs - 1), zp = mask_at(P, g, per, x, ys, zs + 1);
            if (a.kind == TF_KIND_BINARY) {
                cd = (uint8_t)(xm + xp + ym + yp + zm + zp);
            } else {
                cd = (uint8_t)(1 + xm + 3 * xp + 9 * ym + 18 * yp + 36 * zm + 72 * zp);
            }
            fv = profile[x];
        }
    }
    const long long rowc = ((long long)bx * g.YP + Y) * 2 * g.ZHC;
    code[rowc + pos] = cd;
    if (jp < g.ZH) field[((long long)bx * g.YP + Y) * 2 * g.ZH + q * g.ZH + jp] = fv;
}

__global__ void k_unpack(const float* __restrict__ field, float* __restrict__ out, const Geo g, int periodic,
                         float glo, float ghi) {
    const int Z = blockIdx.x * blockDim.x + threadIdx.x;
    if (Z >= g.NZ + 2) return;
    const int Y = blockIdx.y;
    const int bX = blockIdx.z;  // b*(NX+2) + X
    const int X = bX % (g.NX + 2), b = bX / (g.NX + 2);
    float v = 0.0f;
    const bool yin = Y >= 1 && Y <= g.NY, zin = Z >= 1 && Z <= g.NZ;
    if (X == 0 || X == g.NX + 1) {
        if ((yin && zin) || periodic) v = X == 0 ? glo : ghi;
    } else {
        int ys, zs;
        if (src_cell(g, periodic, Y - 1, Z - 1, ys, zs)) {
            v = field[(long long)b * g.vol_f + (long long)(X - 1) * g.plane_f + (long long)(ys + HY) * g.row_f +
                      (zs & 1) * g.ZH + HJ + (zs >> 1)];
        }
    }
    out[(((long long)bX * (g.NY + 2)) + Y) * (g.NZ + 2) + Z] = v;
}

__global__ void k_repack(const float* __restrict__ padded, float* __restrict__ field, const Geo g, int periodic) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q*ZH + jp
    if (pos >= 2 * g.ZH) return;
    const int Y = blockIdx.y;
    const int bx = blockIdx.z;
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = pos >= g.ZH ? 1 : 0;
    const int jp = pos - q * g.ZH;
    const int y = Y - HY, z = 2 * (jp - HJ) + q;
    float v = 0.0f;
    int ys, zs;
    if (src_cell(g, periodic, y, z, ys, zs))
        v = padded[(((long long)b * (g.NX + 2) + x + 1) * (g.NY + 2) + ys + 1) * (g.NZ + 2) + zs + 1];
    field[((long long)bx * g.YP + Y) * 2 * g.ZH + pos] = v;
}

template <int KIND>
__global__ void __launch_bounds__(256) k_layer_sums(const float* __restrict__ field, const uint8_t* __restrict__ code,
                                                    double* __restrict__ flux, double* __restrict__ csum,
                                                    const Geo g, const __grid_constant__ tf_operator op) {
    __shared__ float lut[32 * 32];
    if (KIND == TF_KIND_MULTIPHASE)
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) lut[i] = op.face[i];
    if (KIND == TF_KIND_ANISOTROPIC)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = op.divisor[i];
    __syncthreads();
    const int x = blockIdx.x, b = blockIdx.y;
    const bool has_flux = x + 1 < g.NX;
    double fs = 0.0, cs = 0.0;
    plane_partials<KIND>(field + (long long)b * g.vol_f + (long long)x * g.plane_f,
                         code + (long long)b * g.vol_c + (long long)x * g.plane_c, g, has_flux, lut, fs, cs);
    block_sum_pair(fs, cs);
    if (threadIdx.x == 0) {
        if (has_flux) flux[(long long)b * (g.NX - 1) + x] = fs;
        csum[(long long)b * g.NX + x] = cs;
    }
}

// ------------------------------------------------------------------------------ host side
int pack(const tf_geom& gg, const tf_operator& op, const uint8_t* phase, const float* profile, uint8_t* code,
         float* field, cudaStream_t st) {
    PackArgs a;
    a.g = make_geo(gg);
    a.kind = op.kind;
    a.periodic = op.periodic;
    dim3 block(128);
    dim3 grid((2 * gg.zhc + 127) / 128, gg.yp, gg.batch * gg.nx);
    k_pack<<<grid, block, 0, st>>>(phase, profile, code, field, a, op);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int unpack(const tf_geom& gg, const tf_operator& op, const float* field, float* padded, cudaStream_t st) {
    const Geo g = make_geo(gg);
    dim3 block(128);
    dim3 grid((gg.nz + 2 + 127) / 128, gg.ny + 2, gg.batch * (gg.nx + 2));
    k_unpack<<<grid, block, 0, st>>>(field, padded, g, op.periodic, op.ghost_lo, op.ghost_hi);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int repack(const tf_geom& gg, const tf_operator& op, const float* padded, float* field, cudaStream_t st) {
    const Geo g = make_geo(gg);
    dim3 block(128);
    dim3 grid((2 * gg.zh + 127) / 128, gg.yp, gg.batch * gg.nx);
    k_repack<<<grid, block, 0, st>>>(padded, field, g, op.periodic);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

// ElectrodeSolver's per-plane fluxes (taufactor/electrode.py:70-74) and field sums, one CTA per
// (plane, volume): plane 0 (left_bc - c) / 0.5, plane x > 0 c[x-1] - c[x] (the float32 values of
// -field[x] + field[x-1]), 0 where c or c[x-1] is 0; summed in float64 in a fixed order.
__global__ void __launch_bounds__(256) k_layer_sums_electrode(const float* __restrict__ field, double* __restrict__ flux,
                                                              double* __restrict__ csum, const Geo g, float glo) {
    const int x = blockIdx.x, b = blockIdx.y;
    const float left = 0.5f * glo;
    const float* P = field + (long long)b * g.vol_f + (long long)x * g.plane_f;
    double fs = 0.0, cs = 0.0;
    const int rowlen = 2 * g.ZH;
    for (long long it = threadIdx.x; it < (long long)g.NY * rowlen; it += blockDim.x) {
        const int y = (int)(it / rowlen), pos = (int)(it - (long long)y * rowlen);
        const int q = pos >= g.ZH ? 1 : 0, j = pos - q * g.ZH - HJ;
        if (j < 0 || j >= half_len(g.NZ, q)) continue;
        const long long o = (long long)(y + HY) * g.row_f + pos;
        const float c = P[o];
        const float cm = x > 0 ? P[o - g.plane_f] : glo;
        float f = x > 0 ? __fsub_rn(cm, c) : __fdiv_rn(__fsub_rn(left, c), 0.5f);
        if (c == 0.0f || cm == 0.0f) f = 0.0f;
        fs += (double)f;
        cs += (double)c;
    }
    block_sum_pair(fs, cs);
    if (threadIdx.x == 0) {
        flux[(long long)b * g.NX + x] = fs;
        csum[(long long)b * g.NX + x] = cs;
    }
}

int layer_sums(const tf_geom& gg, const tf_operator& op, const float* field, const uint8_t* code, double* flux,
               double* csum, cudaStream_t st) {
    const Geo g = make_geo(gg);
    dim3 grid(gg.nx, gg.batch);
    if (op.kind == TF_KIND_ELECTRODE)
        k_layer_sums_electrode<<<grid, 256, 0, st>>>(field, flux, csum, g, op.ghost_lo);
    else if (op.kind == TF_KIND_MULTIPHASE)
        k_layer_sums<TF_KIND_MULTIPHASE><<<grid, 256, 0, st>>>(field, code, flux, csum, g, op);
    else if (op.kind == TF_KIND_ANISOTROPIC)
        k_layer_sums<TF_KIND_ANISOTROPIC><<<grid, 256, 0, st>>>(field, code, flux, csum, g, op);
    else
        k_layer_sums<TF_KIND_BINARY><<<grid, 256, 0, st>>>(field, code, flux, csum, g, op);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

}  // namespace tf
