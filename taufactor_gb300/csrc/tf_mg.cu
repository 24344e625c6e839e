// Geometric multigrid and conjugate-gradient building blocks for the per-voxel conductivity
// operator (sm_103a). No reference counterpart: the reference solves only by red-black SOR
// (taufactor.py:156-191); these kernels serve the float32 inner solve A e = r of the FP64 defect
// correction, where any convergent method may replace the SOR sweeps.
//
// Every level keeps the split field layout of its own geometry (tf_geometry) and the packed
// faces of k_kappa_face_pack (fx [b][x'][plane] with x' = 0..nx, fy, fz, factor dv), so the
// smoother of every level is the packed-face half-sweep of tf_kappa_advance_faces.
//
// Coarse operator: cell aggregation by 2 along every axis that the coarse level halves (the last
// aggregate of an odd extent has one cell; an axis whose extent stays is aggregated 1:1); a
// coarse face is the sum of the fine faces across the coarse interface, times `scale` if its
// normal axis is halved (scale 1/2 re-discretises the operator on the doubled spacing); the
// coarse factor is the sum of the six coarse faces in the fine order, the Dirichlet x faces
// counted twice.
// Restriction sums the fine residuals of the aggregate, prolongation adds the coarse value to
// every cell of the aggregate (its transpose), so a V-cycle with a palindromic smoother is a
// symmetric preconditioner.
//
// k_mg_coarsen   coarse faces and factor from the fine ones
// k_mg_restrict  coarse right-hand side = sum over the aggregate of (rhs - A e)
// k_mg_prolong   e += coarse e on every cell of the aggregate
// k_mg_apply     out = A in (interior cells; 0 on cells without a finite factor)
// k_mg_dot_rows / k_mg_dot_sum   per-volume float64 dot products over interior cells, in a fixed order
// k_pcg_xr / k_pcg_p             the conjugate-gradient vector updates with per-volume scalars
#include "tf_common.cuh"
#include "tf_internal.h"
#include "tf_update.cuh"

namespace tf {

namespace {

// offset of interior or ghost cell (x, y, z) of volume b; y >= -HY, z >= -2 HJ
__device__ __forceinline__ long long cell(const Geo& g, int b, int x, int y, int z) {
    return (long long)b * g.vol_f + (long long)x * g.plane_f + (long long)(y + HY) * g.row_f + (z & 1) * g.ZH + HJ +
           (z >> 1);
}
// offset of the x-face plane xp (0..NX) at cell (y, z) of volume b
__device__ __forceinline__ long long xface(const Geo& g, int b, int xp, int y, int z) {
    return ((long long)b * (g.NX + 1) + xp) * g.plane_f + (long long)(y + HY) * g.row_f + (z & 1) * g.ZH + HJ +
           (z >> 1);
}

constexpr float kInf = __builtin_huge_valf();

// 1 where the coarse level halves the axis, 0 where it keeps the fine extent
struct Shift {
    int x, y, z;
};

// rhs - A e at interior cell (x, y, z) with homogeneous Dirichlet x ghosts; 0 where the factor
// is not finite (a cell outside the system).
__device__ __forceinline__ float residual_at(const Geo& g, int b, int x, int y, int z, const float* __restrict__ e,
                                             const float* __restrict__ rhs, const float* __restrict__ fx,
                                             const float* __restrict__ fy, const float* __restrict__ fz,
                                             const float* __restrict__ dv) {
    const long long o = cell(g, b, x, y, z);
    const float d = dv[o];
    if (!(d < kInf)) return 0.0f;
    float s = x + 1 < g.NX ? fx[xface(g, b, x + 1, y, z)] * e[o + g.plane_f] : 0.0f;
    if (x > 0) s += fx[xface(g, b, x, y, z)] * e[o - g.plane_f];
    s += fy[o] * e[o + g.row_f];
    s += fy[o - g.row_f] * e[o - g.row_f];
    s += fz[o] * e[cell(g, b, x, y, z + 1)];
    const long long om = cell(g, b, x, y, z - 1);
    s += fz[om] * e[om];
    if (rhs) s += rhs[o];
    return s - d * e[o];
}

}  // namespace

// One thread per padded position of the coarse level; periodic ghost positions hold the faces
// of the wrapped cell, closed ghost positions 0 (factor inf), as k_kappa_face_pack writes them.
__global__ void k_mg_coarsen(const float* __restrict__ fx, const float* __restrict__ fy, const float* __restrict__ fz,
                             const Geo f, float* __restrict__ cfx, float* __restrict__ cfy, float* __restrict__ cfz,
                             float* __restrict__ cdv, const Geo c, const Shift sh, int periodic, float scale) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q * ZH + jp
    if (pos >= 2 * c.ZH) return;
    const int Y = blockIdx.y;
    const int bx = blockIdx.z;  // b * NX + x of the coarse level
    const int xc = bx % c.NX, b = bx / c.NX;
    const int q = pos >= c.ZH ? 1 : 0;
    const int jp = pos - q * c.ZH;
    int yc = Y - HY, zc = 2 * (jp - HJ) + q;
    const bool interior = yc >= 0 && yc < c.NY && zc >= 0 && zc < c.NZ;
    bool ok = true;
    if (yc < 0 || yc >= c.NY) {
        ok = ok && (periodic & TF_PERIODIC_Y);
        yc = wrap(yc, c.NY);
    }
    if (zc < 0 || zc >= c.NZ) {
        ok = ok && (periodic & TF_PERIODIC_Z);
        zc = wrap(zc, c.NZ);
    }
    const long long o = (long long)bx * c.plane_f + (long long)Y * c.row_f + pos;
    const long long ox = ((long long)b * (c.NX + 1) + xc) * c.plane_f + (long long)Y * c.row_f + pos;
    if (!ok) {
        cfy[o] = 0.0f;
        cfz[o] = 0.0f;
        cdv[o] = kInf;
        cfx[ox + c.plane_f] = 0.0f;
        if (xc == 0) cfx[ox] = 0.0f;
        return;
    }
    // the aggregate: fine cells [x0, xl] x [y0, yl] x [z0, zl]
    const int x0 = xc << sh.x, y0 = yc << sh.y, z0 = zc << sh.z;
    const int xl = sh.x && x0 + 1 < f.NX ? x0 + 1 : x0;
    const int yl = sh.y && y0 + 1 < f.NY ? y0 + 1 : y0;
    const int zl = sh.z && z0 + 1 < f.NZ ? z0 + 1 : z0;
    float sxm = 0.0f, sxp = 0.0f, sym = 0.0f, syp = 0.0f, szm = 0.0f, szp = 0.0f;
    for (int y = y0; y <= yl; ++y)
        for (int z = z0; z <= zl; ++z) {
            sxm += fx[xface(f, b, x0, y, z)];
            sxp += fx[xface(f, b, xl + 1, y, z)];
        }
    for (int x = x0; x <= xl; ++x)
        for (int z = z0; z <= zl; ++z) {
            sym += fy[cell(f, b, x, y0 - 1, z)];
            syp += fy[cell(f, b, x, yl, z)];
        }
    for (int x = x0; x <= xl; ++x)
        for (int y = y0; y <= yl; ++y) {
            szm += fz[cell(f, b, x, y, z0 - 1)];
            szp += fz[cell(f, b, x, y, zl)];
        }
    const float kx = sh.x ? scale : 1.0f, ky = sh.y ? scale : 1.0f, kz = sh.z ? scale : 1.0f;
    const float xm = kx * sxm, xp = kx * sxp, ym = ky * sym, yp = ky * syp, zm = kz * szm, zp = kz * szp;
    cfy[o] = yp;
    cfz[o] = zp;
    cfx[ox + c.plane_f] = xp;
    if (xc == 0) cfx[ox] = xm;
    float d = kInf;
    if (interior) {
        d = xm + xp;
        d += ym;
        d += yp;
        d += zm;
        d += zp;
        if (xc == 0) d += xm;
        if (xc == c.NX - 1) d += xp;
        if (d == 0.0f) d = kInf;
    }
    cdv[o] = d;
}

// One thread per interior cell of the coarse level (blockIdx.y = volume): the sum over the
// aggregate of the fine residual, children in a fixed order.
__global__ void __launch_bounds__(256) k_mg_restrict(const float* __restrict__ e, const float* __restrict__ rhs,
                                                     const float* __restrict__ fx, const float* __restrict__ fy,
                                                     const float* __restrict__ fz, const float* __restrict__ dv,
                                                     const Geo f, float* __restrict__ rc, const Geo c, const Shift sh) {
    const long long n = (long long)c.NX * c.NY * c.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = blockIdx.y;
    const int xc = (int)(i / ((long long)c.NY * c.NZ));
    const int rem = (int)(i - (long long)xc * c.NY * c.NZ);
    const int yc = rem / c.NZ, zc = rem - yc * c.NZ;
    const int x0 = xc << sh.x, y0 = yc << sh.y, z0 = zc << sh.z;
    const int xl = sh.x && x0 + 1 < f.NX ? x0 + 1 : x0;
    const int yl = sh.y && y0 + 1 < f.NY ? y0 + 1 : y0;
    const int zl = sh.z && z0 + 1 < f.NZ ? z0 + 1 : z0;
    float acc = 0.0f;
    for (int x = x0; x <= xl; ++x)
        for (int y = y0; y <= yl; ++y)
            for (int z = z0; z <= zl; ++z) acc += residual_at(f, b, x, y, z, e, rhs, fx, fy, fz, dv);
    rc[cell(c, b, xc, yc, zc)] = acc;
}

// One thread per interior cell of the fine level: e += coarse e of its aggregate.
__global__ void __launch_bounds__(256) k_mg_prolong(const float* __restrict__ ec, const Geo c, float* __restrict__ e,
                                                    const Geo f, const Shift sh) {
    const long long n = (long long)f.NX * f.NY * f.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = blockIdx.y;
    const int x = (int)(i / ((long long)f.NY * f.NZ));
    const int rem = (int)(i - (long long)x * f.NY * f.NZ);
    const int y = rem / f.NZ, z = rem - y * f.NZ;
    e[cell(f, b, x, y, z)] += ec[cell(c, b, x >> sh.x, y >> sh.y, z >> sh.z)];
}

// out = A in on interior cells (A in = factor * in - weighted neighbour sum, Dirichlet ghosts 0).
__global__ void __launch_bounds__(256) k_mg_apply(const float* __restrict__ in, const float* __restrict__ fx,
                                                  const float* __restrict__ fy, const float* __restrict__ fz,
                                                  const float* __restrict__ dv, float* __restrict__ out, const Geo g) {
    const long long n = (long long)g.NX * g.NY * g.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = blockIdx.y;
    const int x = (int)(i / ((long long)g.NY * g.NZ));
    const int rem = (int)(i - (long long)x * g.NY * g.NZ);
    const int y = rem / g.NZ, z = rem - y * g.NZ;
    out[cell(g, b, x, y, z)] = -residual_at(g, b, x, y, z, in, nullptr, fx, fy, fz, dv);
}

// Per padded row (blockIdx.x = row y of plane blockIdx.y = b * NX + x): float64 sums over the
// row's interior cells of a1*b1 and (if a2) a2*b2 -> part[2][B*NX*NY].
__global__ void __launch_bounds__(128) k_mg_dot_rows(const float* __restrict__ a1, const float* __restrict__ b1,
                                                     const float* __restrict__ a2, const float* __restrict__ b2,
                                                     double* __restrict__ part, const Geo g) {
    __shared__ double red[2][4];
    const int y = blockIdx.x;
    const long long bx = blockIdx.y;
    const long long row = bx * g.plane_f + (long long)(y + HY) * g.row_f;
    double s1 = 0.0, s2 = 0.0;
    for (int q = 0; q < 2; ++q) {
        const int nj = half_len(g.NZ, q);
        const long long base = row + q * g.ZH + HJ;
        for (int j = threadIdx.x; j < nj; j += blockDim.x) {
            s1 += (double)a1[base + j] * (double)b1[base + j];
            if (a2) s2 += (double)a2[base + j] * (double)b2[base + j];
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, s);
        s2 += __shfl_xor_sync(0xffffffffu, s2, s);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s1;
        red[1][threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long rows = (long long)g.B * g.NX * g.NY;
        const long long k = bx * g.NY + y;
        part[k] = (red[0][0] + red[0][1]) + (red[0][2] + red[0][3]);
        part[rows + k] = (red[1][0] + red[1][1]) + (red[1][2] + red[1][3]);
    }
}

// One block per volume: out[v][b] = sum of the volume's row partials of product v, fixed order.
__global__ void __launch_bounds__(256) k_mg_dot_sum(const double* __restrict__ part, double* __restrict__ out,
                                                    const Geo g, int nprod) {
    __shared__ double red[2][8];
    const int b = blockIdx.x;
    const long long rows = (long long)g.B * g.NX * g.NY;
    const long long per = (long long)g.NX * g.NY;
    for (int v = 0; v < nprod; ++v) {
        const double* p = part + v * rows + b * per;
        double s = 0.0;
        for (long long k = threadIdx.x; k < per; k += blockDim.x) s += p[k];
        for (int sh = 16; sh > 0; sh >>= 1) s += __shfl_xor_sync(0xffffffffu, s, sh);
        if ((threadIdx.x & 31) == 0) red[v][threadIdx.x >> 5] = s;
    }
    __syncthreads();
    if (threadIdx.x < nprod) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += red[threadIdx.x][w];
        out[threadIdx.x * g.B + b] = s;
    }
}

// per-volume step num/den, 0 when the denominator is not a positive finite number
__device__ __forceinline__ float safe_ratio(double num, double den) {
    return (den > 0.0 && den < 1e300 && num == num) ? (float)(num / den) : 0.0f;
}

// x += alpha p, r -= alpha q with alpha = rz[b] / pq[b]; whole padded volume (float4 groups)
__global__ void __launch_bounds__(256) k_pcg_xr(float4* __restrict__ x, float4* __restrict__ r,
                                                const float4* __restrict__ p, const float4* __restrict__ q,
                                                const double* __restrict__ rz, const double* __restrict__ pq,
                                                long long n4, long long vol4) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n4) return;
    const int b = (int)(i / vol4);
    const float al = safe_ratio(rz[b], pq[b]);
    const float4 pv = p[i], qv = q[i];
    float4 xv = x[i], rv = r[i];
    xv.x += al * pv.x; xv.y += al * pv.y; xv.z += al * pv.z; xv.w += al * pv.w;
    rv.x -= al * qv.x; rv.y -= al * qv.y; rv.z -= al * qv.z; rv.w -= al * qv.w;
    x[i] = xv;
    r[i] = rv;
}

// p = z + beta p with beta = rz_new[b] / rz_old[b]
__global__ void __launch_bounds__(256) k_pcg_p(float4* __restrict__ p, const float4* __restrict__ z,
                                               const double* __restrict__ rz_new, const double* __restrict__ rz_old,
                                               long long n4, long long vol4) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n4) return;
    const int b = (int)(i / vol4);
    const float be = safe_ratio(rz_new[b], rz_old[b]);
    const float4 zv = z[i];
    float4 pv = p[i];
    pv.x = zv.x + be * pv.x; pv.y = zv.y + be * pv.y; pv.z = zv.z + be * pv.z; pv.w = zv.w + be * pv.w;
    p[i] = pv;
}

// the coarse level of `f` along every axis (halved or kept); false if `c` is not one
static bool coarse_of(const tf_geom& f, const tf_geom& c, Shift* sh) {
    auto axis = [](int fn, int cn, int* s) {
        if (cn == fn) *s = 0;
        else if (cn == (fn + 1) / 2) *s = 1;
        else return false;
        return true;
    };
    return f.batch == c.batch && c.halo_y == HY && c.halo_j == HJ && f.halo_y == HY && f.halo_j == HJ &&
           axis(f.nx, c.nx, &sh->x) && axis(f.ny, c.ny, &sh->y) && axis(f.nz, c.nz, &sh->z);
}

static dim3 cell_grid(const tf_geom& g) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    return dim3((unsigned)((n + 255) / 256), g.batch);
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace tf

using namespace tf;

extern "C" {

int tf_mg_coarsen(const tf_geom* fine, const float* fx_dev, const float* fy_dev, const float* fz_dev,
                  const tf_geom* coarse, float* cfx_dev, float* cfy_dev, float* cfz_dev, float* cdiv_dev,
                  int periodic, float scale, void* stream) {
    if (!fine || !coarse || !fx_dev || !fy_dev || !fz_dev || !cfx_dev || !cfy_dev || !cfz_dev || !cdiv_dev)
        return TF_ERR_ARG;
    Shift sh;
    if (!coarse_of(*fine, *coarse, &sh) || !(scale > 0.0f)) return TF_ERR_ARG;
    if ((long long)coarse->batch * coarse->nx > 65535 || coarse->yp > 65535) return TF_ERR_UNSUPPORTED;
    const Geo f = make_geo(*fine), c = make_geo(*coarse);
    dim3 grid((2 * coarse->zh + 127) / 128, coarse->yp, coarse->batch * coarse->nx);
    k_mg_coarsen<<<grid, 128, 0, (cudaStream_t)stream>>>(fx_dev, fy_dev, fz_dev, f, cfx_dev, cfy_dev, cfz_dev,
                                                          cdiv_dev, c, sh, periodic, scale);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_mg_restrict(const tf_geom* fine, const float* e_dev, const float* rhs_dev, const float* fx_dev,
                   const float* fy_dev, const float* fz_dev, const float* div_dev, const tf_geom* coarse,
                   float* rc_dev, void* stream) {
    if (!fine || !coarse || !e_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev || !rc_dev) return TF_ERR_ARG;
    Shift sh;
    if (!coarse_of(*fine, *coarse, &sh) || coarse->batch > 65535) return TF_ERR_ARG;
    const Geo f = make_geo(*fine), c = make_geo(*coarse);
    k_mg_restrict<<<cell_grid(*coarse), 256, 0, (cudaStream_t)stream>>>(e_dev, rhs_dev, fx_dev, fy_dev, fz_dev,
                                                                         div_dev, f, rc_dev, c, sh);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_mg_prolong(const tf_geom* coarse, const float* ec_dev, const tf_geom* fine, float* e_dev, int periodic,
                  void* stream) {
    if (!fine || !coarse || !ec_dev || !e_dev) return TF_ERR_ARG;
    Shift sh;
    if (!coarse_of(*fine, *coarse, &sh) || fine->batch > 65535) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const Geo f = make_geo(*fine), c = make_geo(*coarse);
    k_mg_prolong<<<cell_grid(*fine), 256, 0, st>>>(ec_dev, c, e_dev, f, sh);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    return periodic ? refresh_ghosts(*fine, periodic, e_dev, st) : TF_OK;
}

int tf_mg_apply(const tf_geom* g, const float* in_dev, const float* fx_dev, const float* fy_dev,
                const float* fz_dev, const float* div_dev, float* out_dev, void* stream) {
    if (!g || !in_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev || !out_dev || g->batch > 65535)
        return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    k_mg_apply<<<cell_grid(*g), 256, 0, (cudaStream_t)stream>>>(in_dev, fx_dev, fy_dev, fz_dev, div_dev, out_dev, geo);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_mg_dot(const tf_geom* g, const float* a1_dev, const float* b1_dev, const float* a2_dev, const float* b2_dev,
              double* part_dev, double* out_dev, void* stream) {
    if (!g || !a1_dev || !b1_dev || !part_dev || !out_dev || (!a2_dev) != (!b2_dev)) return TF_ERR_ARG;
    if ((long long)g->batch * g->nx > 65535 || g->ny > 2147483647 / 2) return TF_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    const Geo geo = make_geo(*g);
    dim3 grid(g->ny, g->batch * g->nx);
    k_mg_dot_rows<<<grid, 128, 0, st>>>(a1_dev, b1_dev, a2_dev, b2_dev, part_dev, geo);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    k_mg_dot_sum<<<g->batch, 256, 0, st>>>(part_dev, out_dev, geo, a2_dev ? 2 : 1);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_pcg_update_xr(const tf_geom* g, float* x_dev, float* r_dev, const float* p_dev, const float* q_dev,
                     const double* rz_dev, const double* pq_dev, void* stream) {
    if (!g || !x_dev || !r_dev || !p_dev || !q_dev || !rz_dev || !pq_dev) return TF_ERR_ARG;
    if (!aligned16(x_dev) || !aligned16(r_dev) || !aligned16(p_dev) || !aligned16(q_dev)) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const long long n4 = g->field_elems / 4, vol4 = geo.vol_f / 4;
    k_pcg_xr<<<(unsigned)((n4 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<float4*>(x_dev), reinterpret_cast<float4*>(r_dev), reinterpret_cast<const float4*>(p_dev),
        reinterpret_cast<const float4*>(q_dev), rz_dev, pq_dev, n4, vol4);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_pcg_update_p(const tf_geom* g, float* p_dev, const float* z_dev, const double* rz_new_dev,
                    const double* rz_old_dev, void* stream) {
    if (!g || !p_dev || !z_dev || !rz_new_dev || !rz_old_dev) return TF_ERR_ARG;
    if (!aligned16(p_dev) || !aligned16(z_dev)) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const long long n4 = g->field_elems / 4, vol4 = geo.vol_f / 4;
    k_pcg_p<<<(unsigned)((n4 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<float4*>(p_dev), reinterpret_cast<const float4*>(z_dev), rz_new_dev, rz_old_dev, n4, vol4);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

}  // extern "C"
