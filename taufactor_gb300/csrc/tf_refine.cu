// FP64 defect correction (sm_103a): r = b - A c in float64 around the float32 sweeps.
//
// The reference iterates c <- c + omega (S(c)/d - c) in float32 only (taufactor.py:174-182); its
// fixed point solves A c = b with A c = d c - S_in(c) (S_in: weighted sum of in-volume
// neighbours, d: the divisor nn / factor) and b = the Dirichlet ghost terms. Mixed-precision
// refinement keeps c in float64, forms r = b - A c in float64, solves A e = r approximately by
// the float32 sweeps with a right-hand side, and adds e to c in float64.
//
// k_widen / k_narrow  float32 <-> float64 split-layout fields (narrow rebuilds periodic ghosts)
// k_residual          per-cell float64 residual -> float32 right-hand side (+ ghost copies via
//                     k_ghosts), with per-plane float64 sums of r^2 and b^2 (one CTA per plane,
//                     fixed summation order)
// k_axpy              c64 += e32
// k_layer_sums_f64    the layer sums of tf_pack.cu's k_layer_sums on a float64 field
#include "tf_common.cuh"
#include "tf_internal.h"

namespace tf {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sums of two values, result valid in thread 0 (blockDim.x a multiple of 32, <= 1024)
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double red[2][32];
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
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

__global__ void k_widen(const float* __restrict__ f32, double* __restrict__ f64, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        f64[i] = (double)f32[i];
}

__global__ void k_narrow(const double* __restrict__ f64, float* __restrict__ f32, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        f32[i] = (float)f64[i];
}

__global__ void k_axpy(double* __restrict__ c, const float* __restrict__ e, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c[i] += (double)e[i];
}

// value of the float64 field at interior (x, y, z) with the solver's boundary rules in y/z:
// wrapped on periodic faces, 0 beyond closed faces. `ok` = the neighbour is inside the volume.
struct F64View {
    const double* f;
    const uint8_t* code;
    Geo g;
    int periodic;
    __device__ __forceinline__ bool cell(int y, int z, int& ys, int& zs) const {
        ys = y;
        zs = z;
        if (y < 0 || y >= g.NY) {
            if (!(periodic & TF_PERIODIC_Y)) return false;
            ys = wrap(y, g.NY);
        }
        if (z < 0 || z >= g.NZ) {
            if (!(periodic & TF_PERIODIC_Z)) return false;
            zs = wrap(z, g.NZ);
        }
        return true;
    }
    __device__ __forceinline__ long long off(int x, int y, int z) const {
        return (long long)x * g.plane_f + (long long)(y + HY) * g.row_f + (z & 1) * g.ZH + HJ + (z >> 1);
    }
    __device__ __forceinline__ long long offc(int x, int y, int z) const {
        return (long long)x * g.plane_c + (long long)(y + HY) * g.row_c + (z & 1) * g.ZHC + HJ + (z >> 1);
    }
};

__global__ void __launch_bounds__(256) k_residual(const double* __restrict__ c64, const uint8_t* __restrict__ code,
                                                  float* __restrict__ r32, double* __restrict__ r2,
                                                  double* __restrict__ b2, const Geo g,
                                                  const __grid_constant__ tf_operator op) {
    __shared__ float lut[32 * 32];
    if (op.kind == TF_KIND_MULTIPHASE) {
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) lut[i] = op.face[i];
    } else {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = op.divisor[i];
    }
    __syncthreads();
    const int x = blockIdx.x, b = blockIdx.y;
    F64View v{c64 + (long long)b * g.vol_f, code + (long long)b * g.vol_c, g, op.periodic};
    float* rb = r32 + (long long)b * g.vol_f;
    double rs = 0.0, bs = 0.0;
    const long long ncell = (long long)g.NY * g.NZ;
    for (long long it = threadIdx.x; it < ncell; it += blockDim.x) {
        const int y = (int)(it / g.NZ), z = (int)(it - (long long)y * g.NZ);
        const long long o = v.off(x, y, z);
        const int cd = v.code[v.offc(x, y, z)];
        double res = 0.0, rhs = 0.0;
        const double c = v.f[o];
        if (op.kind == TF_KIND_MULTIPHASE) {
            // faces as the sweep sees them; the diagonal is the reference's float32 factor
            // (taufactor.py:598-603: lower x, upper x, y lower/upper, z lower/upper, then the
            // boundary faces once more), promoted to float64
            const float* row = lut + cd * 32;
            int ys, zs;
            const float fxm = x > 0 ? row[v.code[v.offc(x - 1, y, z)]] : row[cd];
            const float fxp = x + 1 < g.NX ? row[v.code[v.offc(x + 1, y, z)]] : row[cd];
            const float fyp = v.cell(y + 1, z, ys, zs) ? row[v.code[v.offc(x, ys, zs)]] : 0.0f;
            const double cyp = v.cell(y + 1, z, ys, zs) ? v.f[v.off(x, ys, zs)] : 0.0;
            const float fym = v.cell(y - 1, z, ys, zs) ? row[v.code[v.offc(x, ys, zs)]] : 0.0f;
            const double cym = v.cell(y - 1, z, ys, zs) ? v.f[v.off(x, ys, zs)] : 0.0;
            const float fzp = v.cell(y, z + 1, ys, zs) ? row[v.code[v.offc(x, ys, zs)]] : 0.0f;
            const double czp = v.cell(y, z + 1, ys, zs) ? v.f[v.off(x, ys, zs)] : 0.0;
            const float fzm = v.cell(y, z - 1, ys, zs) ? row[v.code[v.offc(x, ys, zs)]] : 0.0f;
            const double czm = v.cell(y, z - 1, ys, zs) ? v.f[v.off(x, ys, zs)] : 0.0;
            float div = __fadd_rn(fxm, fxp);
            div = __fadd_rn(div, fym);
            div = __fadd_rn(div, fyp);
            div = __fadd_rn(div, fzm);
            div = __fadd_rn(div, fzp);
            if (x == 0) div = __fadd_rn(div, fxm);
            if (x == g.NX - 1) div = __fadd_rn(div, fxp);
            if (div > 0.0f) {
                double s = (double)fyp * cyp + (double)fym * cym + (double)fzp * czp + (double)fzm * czm;
                if (x > 0) s += (double)fxm * v.f[v.off(x - 1, y, z)];
                else rhs += (double)fxm * (double)op.ghost_lo;
                if (x + 1 < g.NX) s += (double)fxp * v.f[v.off(x + 1, y, z)];
                else rhs += (double)fxp * (double)op.ghost_hi;
                res = rhs - ((double)div * c - s);
            }
        } else {
            // divisor: the table entry of the code; for the electrode kind the sweep's float32
            // nn + nr * k_0 (code 1 + nn + 8 nr, k_0 of volume b in the table; taufactor.py:47-55)
            double d;
            if (op.kind == TF_KIND_ELECTRODE) {
                d = 1e300;
                if (cd != 0) {
                    const int m = cd - 1;
                    const float df = __fadd_rn(static_cast<float>(m & 7), __fmul_rn(static_cast<float>(m >> 3), lut[b & 255]));
                    if (df != 0.0f) d = (double)df;
                }
            } else {
                d = (double)lut[cd];
            }
            if (d < 1e30) {  // conductive, non-isolated
                const double ky = op.kind == TF_KIND_ANISOTROPIC ? (double)op.ky : 1.0;
                const double kz = op.kind == TF_KIND_ANISOTROPIC ? (double)op.kz : 1.0;
                double s = 0.0;
                int ys, zs;
                if (x > 0) s += v.f[v.off(x - 1, y, z)];
                else rhs += (double)op.ghost_lo;
                if (x + 1 < g.NX) s += v.f[v.off(x + 1, y, z)];
                else rhs += (double)op.ghost_hi;
                double sy = 0.0, sz = 0.0;
                if (v.cell(y + 1, z, ys, zs)) sy += v.f[v.off(x, ys, zs)];
                if (v.cell(y - 1, z, ys, zs)) sy += v.f[v.off(x, ys, zs)];
                if (v.cell(y, z + 1, ys, zs)) sz += v.f[v.off(x, ys, zs)];
                if (v.cell(y, z - 1, ys, zs)) sz += v.f[v.off(x, ys, zs)];
                res = rhs - (d * c - (s + ky * sy + kz * sz));
            }
        }
        rb[o] = (float)res;
        rs += res * res;
        bs += rhs * rhs;
    }
    block_sum2(rs, bs);
    if (threadIdx.x == 0) {
        r2[(long long)b * g.NX + x] = rs;
        b2[(long long)b * g.NX + x] = bs;
    }
}

__global__ void __launch_bounds__(256) k_layer_sums_f64(const double* __restrict__ field,
                                                        const uint8_t* __restrict__ code, double* __restrict__ flux,
                                                        double* __restrict__ csum, const Geo g,
                                                        const __grid_constant__ tf_operator op) {
    __shared__ float lut[32 * 32];
    if (op.kind == TF_KIND_MULTIPHASE) {
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) lut[i] = op.face[i];
    } else {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = op.divisor[i];
    }
    __syncthreads();
    const int x = blockIdx.x, b = blockIdx.y;
    const bool has_flux = x + 1 < g.NX;
    F64View v{field + (long long)b * g.vol_f, code + (long long)b * g.vol_c, g, op.periodic};
    double fs = 0.0, cs = 0.0;
    const long long ncell = (long long)g.NY * g.NZ;
    for (long long it = threadIdx.x; it < ncell; it += blockDim.x) {
        const int y = (int)(it / g.NZ), z = (int)(it - (long long)y * g.NZ);
        const double a = v.f[v.off(x, y, z)];
        cs += a;
        if (op.kind == TF_KIND_ELECTRODE) {
            // ElectrodeSolver's plane fluxes (taufactor/electrode.py:70-74) in float64: plane 0
            // (left_bc - c) / 0.5, plane x > 0 c[x-1] - c[x]; 0 where either value is 0
            const double am = x > 0 ? v.f[v.off(x - 1, y, z)] : (double)op.ghost_lo;
            double f = x > 0 ? am - a : (0.5 * (double)op.ghost_lo - a) / 0.5;
            if (a == 0.0 || am == 0.0) f = 0.0;
            fs += f;
        } else if (has_flux) {
            const double d = v.f[v.off(x + 1, y, z)] - a;
            const int ca = v.code[v.offc(x, y, z)], cb = v.code[v.offc(x + 1, y, z)];
            if (op.kind == TF_KIND_MULTIPHASE) fs += (double)lut[ca * 32 + cb] * d;
            else if (lut[ca] <= 8.0f && lut[cb] <= 8.0f) fs += d;
        }
    }
    block_sum2(fs, cs);
    if (threadIdx.x == 0) {
        if (op.kind == TF_KIND_ELECTRODE) flux[(long long)b * g.NX + x] = fs;  // one flux per plane
        else if (has_flux) flux[(long long)b * (g.NX - 1) + x] = fs;
        csum[(long long)b * g.NX + x] = cs;
    }
}

static dim3 grid_for(long long n) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    return dim3((unsigned)(blocks > 0 ? blocks : 1));
}

int widen(const tf_geom& gg, const float* f32, double* f64, cudaStream_t st) {
    k_widen<<<grid_for(gg.field_elems), 256, 0, st>>>(f32, f64, gg.field_elems);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int narrow(const tf_geom& gg, const tf_operator& op, const double* f64, float* f32, cudaStream_t st) {
    k_narrow<<<grid_for(gg.field_elems), 256, 0, st>>>(f64, f32, gg.field_elems);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    return op.periodic ? refresh_ghosts(gg, op.periodic, f32, st) : TF_OK;
}

int axpy(const tf_geom& gg, double* c64, const float* e32, cudaStream_t st) {
    k_axpy<<<grid_for(gg.field_elems), 256, 0, st>>>(c64, e32, gg.field_elems);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int residual(const tf_geom& gg, const tf_operator& op, const double* c64, const uint8_t* code, float* r32, double* r2,
             double* b2, cudaStream_t st) {
    const Geo g = make_geo(gg);
    k_residual<<<dim3(gg.nx, gg.batch), 256, 0, st>>>(c64, code, r32, r2, b2, g, op);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    return op.periodic ? refresh_ghosts(gg, op.periodic, r32, st) : TF_OK;
}

int layer_sums_f64(const tf_geom& gg, const tf_operator& op, const double* f64, const uint8_t* code, double* flux,
                   double* csum, cudaStream_t st) {
    const Geo g = make_geo(gg);
    k_layer_sums_f64<<<dim3(gg.nx, gg.batch), 256, 0, st>>>(f64, code, flux, csum, g, op);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

}  // namespace tf
