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
// k_mg_dot_rows / k_mg_dot_sum   per-volume dot products over interior cells (float32 products of
//                                a float4 group, float64 accumulation), in a fixed order
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
// and factor of the wrapped cell, closed ghost positions 0 (factor inf), as k_kappa_face_pack
// writes them.
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
    // the factor on interior cells and periodic ghost positions (the wrapped cell's)
    float d = kInf;
    {
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

// One thread per interior cell of the coarse level: the sum over the aggregate of the fine
// residual, children in a fixed order.
__global__ void __launch_bounds__(128) k_mg_restrict(const float* __restrict__ e, const float* __restrict__ rhs,
                                                     const float* __restrict__ fx, const float* __restrict__ fy,
                                                     const float* __restrict__ fz, const float* __restrict__ dv,
                                                     const Geo f, float* __restrict__ rc, const Geo c, const Shift sh) {
    // grid (z blocks, y, b * NX + x) of the coarse level: no index division
    const int zc = blockIdx.x * blockDim.x + threadIdx.x;
    if (zc >= c.NZ) return;
    const int yc = blockIdx.y;
    const int xc = blockIdx.z % c.NX, b = blockIdx.z / c.NX;
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
__global__ void __launch_bounds__(128) k_mg_prolong(const float* __restrict__ ec, const Geo c, float* __restrict__ e,
                                                    const Geo f, const Shift sh) {
    // grid (z blocks, y, b * NX + x) of the fine level
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= f.NZ) return;
    const int y = blockIdx.y;
    const int x = blockIdx.z % f.NX, b = blockIdx.z / f.NX;
    e[cell(f, b, x, y, z)] += ec[cell(c, b, x >> sh.x, y >> sh.y, z >> sh.z)];
}

// out = A in on interior cells (A in = factor * in - weighted neighbour sum, Dirichlet ghosts 0):
// one thread per float4 group of a half-row (blockIdx.y: row groups of 8, threadIdx.y the row;
// blockIdx.z = b * NX + x), both half-rows; 0 where the factor is not finite.
__global__ void __launch_bounds__(256) k_mg_apply(const float* __restrict__ in, const float* __restrict__ fx,
                                                  const float* __restrict__ fy, const float* __restrict__ fz,
                                                  const float* __restrict__ dv, float* __restrict__ out, const Geo g) {
    const int gmax = (half_len(g.NZ, 0) + 3) >> 2;
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= gmax || y >= g.NY) return;
    const int bx = blockIdx.z;
    const int x = bx % g.NX, b = bx / g.NX;
    const int j = 4 * gi;
    const long long row = (long long)bx * g.plane_f + (long long)(y + HY) * g.row_f;
    const long long fxr = ((long long)b * (g.NX + 1) + x) * g.plane_f + (long long)(y + HY) * g.row_f;
    for (int q = 0; q < 2; ++q) {
        const int nj = half_len(g.NZ, q);
        if (j >= nj) continue;
        const long long rq = row + q * g.ZH + HJ + j;        // this group
        const long long ro = row + (q ^ 1) * g.ZH + HJ + j;  // the other half-row, same j
        const float4 cc = ld4(in + rq);
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 xp = x + 1 < g.NX ? ld4(in + rq + g.plane_f) : zero4;
        const float4 xm = x > 0 ? ld4(in + rq - g.plane_f) : zero4;
        const float4 yp = ld4(in + rq + g.row_f), ym = ld4(in + rq - g.row_f);
        float4 zp, zm;
        z_neighbours(q, ld4(in + ro), q ? in[ro + 4] : in[ro - 1], zp, zm);
        const long long fq = fxr + q * g.ZH + HJ + j;
        const float4 fxm = ld4(fx + fq), fxp = ld4(fx + fq + g.plane_f);
        const float4 fyp = ld4(fy + rq), fym = ld4(fy + rq - g.row_f);
        const float4 fzp = ld4(fz + rq);
        float4 fzm;  // the face between z - 1 and z, stored at cell z - 1
        if (q) {
            fzm = ld4(fz + ro);
        } else {
            const float4 fo = ld4(fz + ro);
            fzm = make_float4(fz[ro - 1], fo.x, fo.y, fo.z);
        }
        const float4 d = ld4(dv + rq);
        float4 r;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float s = comp(xp, i) * comp(fxp, i) + comp(xm, i) * comp(fxm, i);
            s += comp(yp, i) * comp(fyp, i);
            s += comp(ym, i) * comp(fym, i);
            s += comp(zp, i) * comp(fzp, i);
            s += comp(zm, i) * comp(fzm, i);
            const float di = comp(d, i);
            set_comp(r, i, di < kInf ? di * comp(cc, i) - s : 0.0f);
        }
        float* dst = out + rq;
        if (j + 4 <= nj)
            st4(dst, r);
        else
            for (int i = 0; i < nj - j; ++i) dst[i] = comp(r, i);
    }
}

// Rows of one plane per block of the dot products (the partial sums are per block).
constexpr int kDotRows = 16;

// float64 sums over interior cells of a1*b1 and (if a2) a2*b2 for kDotRows rows (blockIdx.x)
// of the plane blockIdx.y = b * NX + x -> part[2][B*NX*ny_blocks], float4 loads, fixed order.
__global__ void __launch_bounds__(256) k_mg_dot_rows(const float* __restrict__ a1, const float* __restrict__ b1,
                                                     const float* __restrict__ a2, const float* __restrict__ b2,
                                                     double* __restrict__ part, const Geo g) {
    __shared__ double red[2][8];
    const long long bx = blockIdx.y;
    const int y0 = blockIdx.x * kDotRows;
    const int y1 = y0 + kDotRows < g.NY ? y0 + kDotRows : g.NY;
    const int n0 = half_len(g.NZ, 0), n1 = half_len(g.NZ, 1);
    const int g0 = (n0 + 3) >> 2, g1 = (n1 + 3) >> 2;  // float4 groups per half-row
    const int per_row = g0 + g1;
    const long long plane = bx * g.plane_f;
    double s1 = 0.0, s2 = 0.0;
    for (int k = threadIdx.x; k < (y1 - y0) * per_row; k += blockDim.x) {
        const int r = k / per_row, gi = k - r * per_row;
        const int q = gi >= g0 ? 1 : 0;
        const int j = 4 * (q ? gi - g0 : gi);
        const int nj = q ? n1 : n0;
        const long long o = plane + (long long)(y0 + r + HY) * g.row_f + q * g.ZH + HJ + j;
        // a group's four products summed in float32 (relative error ~1e-7, ample for the CG
        // scalars), the groups in float64: one float64 add per group instead of eight float64
        // operations, which would bound the kernel on GB300's FP64 pipe
        const float4 x1 = *reinterpret_cast<const float4*>(a1 + o), w1 = *reinterpret_cast<const float4*>(b1 + o);
        float t1 = x1.x * w1.x;
        if (j + 1 < nj) t1 += x1.y * w1.y;
        if (j + 2 < nj) t1 += x1.z * w1.z;
        if (j + 3 < nj) t1 += x1.w * w1.w;
        s1 += (double)t1;
        if (a2) {
            const float4 x2 = *reinterpret_cast<const float4*>(a2 + o), w2 = *reinterpret_cast<const float4*>(b2 + o);
            float t2 = x2.x * w2.x;
            if (j + 1 < nj) t2 += x2.y * w2.y;
            if (j + 2 < nj) t2 += x2.z * w2.z;
            if (j + 3 < nj) t2 += x2.w * w2.w;
            s2 += (double)t2;
        }
    }
    for (int sh = 16; sh > 0; sh >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, sh);
        s2 += __shfl_xor_sync(0xffffffffu, s2, sh);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s1;
        red[1][threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p1 = 0.0, p2 = 0.0;
        for (int w = 0; w < 8; ++w) {
            p1 += red[0][w];
            p2 += red[1][w];
        }
        const long long nb = (long long)g.B * g.NX * gridDim.x;
        const long long k = bx * gridDim.x + blockIdx.x;
        part[k] = p1;
        part[nb + k] = p2;
    }
}

// One block per volume: out[v][b] = sum of the volume's block partials of product v (nper per
// volume), fixed order.
__global__ void __launch_bounds__(256) k_mg_dot_sum(const double* __restrict__ part, double* __restrict__ out,
                                                    const Geo g, long long nper, int nprod) {
    __shared__ double red[2][8];
    const int b = blockIdx.x;
    const long long nb = (long long)g.B * nper;
    for (int v = 0; v < nprod; ++v) {
        const double* p = part + v * nb + b * nper;
        double s = 0.0;
        for (long long k = threadIdx.x; k < nper; k += blockDim.x) s += p[k];
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

// (z blocks of 128, y, b * nx + x) over the interior cells of a level
static dim3 cell_grid(const tf_geom& g) { return dim3((g.nz + 127) / 128, g.ny, g.batch * g.nx); }
static bool cell_grid_ok(const tf_geom& g) { return (long long)g.batch * g.nx <= 65535 && g.ny <= 65535; }

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
    if (!coarse_of(*fine, *coarse, &sh)) return TF_ERR_ARG;
    if (!cell_grid_ok(*coarse)) return TF_ERR_UNSUPPORTED;
    const Geo f = make_geo(*fine), c = make_geo(*coarse);
    k_mg_restrict<<<cell_grid(*coarse), 128, 0, (cudaStream_t)stream>>>(e_dev, rhs_dev, fx_dev, fy_dev, fz_dev,
                                                                         div_dev, f, rc_dev, c, sh);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_mg_prolong(const tf_geom* coarse, const float* ec_dev, const tf_geom* fine, float* e_dev, int periodic,
                  void* stream) {
    if (!fine || !coarse || !ec_dev || !e_dev) return TF_ERR_ARG;
    Shift sh;
    if (!coarse_of(*fine, *coarse, &sh)) return TF_ERR_ARG;
    if (!cell_grid_ok(*fine)) return TF_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    const Geo f = make_geo(*fine), c = make_geo(*coarse);
    k_mg_prolong<<<cell_grid(*fine), 128, 0, st>>>(ec_dev, c, e_dev, f, sh);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    return periodic ? refresh_ghosts(*fine, periodic, e_dev, st) : TF_OK;
}

int tf_mg_apply(const tf_geom* g, const float* in_dev, const float* fx_dev, const float* fy_dev,
                const float* fz_dev, const float* div_dev, float* out_dev, void* stream) {
    if (!g || !in_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev || !out_dev || g->batch > 65535)
        return TF_ERR_ARG;
    if (!aligned16(in_dev) || !aligned16(fx_dev) || !aligned16(fy_dev) || !aligned16(fz_dev) || !aligned16(div_dev) ||
        !aligned16(out_dev) || (long long)g->batch * g->nx > 65535)
        return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const int gmax = (half_len(g->nz, 0) + 3) >> 2;
    const dim3 bs(32, 8);
    const dim3 grid((gmax + 31) / 32, (g->ny + 7) / 8, g->batch * g->nx);
    k_mg_apply<<<grid, bs, 0, (cudaStream_t)stream>>>(in_dev, fx_dev, fy_dev, fz_dev, div_dev, out_dev, geo);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_mg_dot(const tf_geom* g, const float* a1_dev, const float* b1_dev, const float* a2_dev, const float* b2_dev,
              double* part_dev, double* out_dev, void* stream) {
    if (!g || !a1_dev || !b1_dev || !part_dev || !out_dev || (!a2_dev) != (!b2_dev)) return TF_ERR_ARG;
    if ((long long)g->batch * g->nx > 65535) return TF_ERR_UNSUPPORTED;
    if (!aligned16(a1_dev) || !aligned16(b1_dev) || (a2_dev && (!aligned16(a2_dev) || !aligned16(b2_dev))))
        return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const Geo geo = make_geo(*g);
    const int nyb = (g->ny + kDotRows - 1) / kDotRows;
    dim3 grid(nyb, g->batch * g->nx);
    k_mg_dot_rows<<<grid, 256, 0, st>>>(a1_dev, b1_dev, a2_dev, b2_dev, part_dev, geo);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    k_mg_dot_sum<<<g->batch, 256, 0, st>>>(part_dev, out_dev, geo, (long long)g->nx * nyb, a2_dev ? 2 : 1);
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
