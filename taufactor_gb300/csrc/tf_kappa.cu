// Per-voxel conductivity ("kappa field") operator and its adjoint (sm_103a).
//
// MultiPhaseSolver (taufactor.py:508-620) assigns each label a diffusivity and couples voxels
// through harmonic-mean faces 2ab/(a+b) (:577-596), with the x-ghost planes copying the
// adjacent voxel (:590-592) and the diagonal `factor` summed in a fixed order (:598-603).
// Here the diffusivity is an arbitrary float32 per voxel, kappa, stored in the field's split
// layout (ghost cells 0 on closed faces, wrapped copies on periodic ones). With
// kappa = D[label] every face, factor and update equals MultiPhaseSolver's bit for bit.
//
// k_kappa_sweep      one half-sweep in place (one thread per voxel of one colour), optional RHS
// k_kappa_face_pack  the operator's faces and factor, once per kappa field
// k_kappa_sweep4     one half-sweep in place from the packed faces (float4 groups of one
//                    colour, one division per voxel), optional RHS; the same bits as
//                    k_kappa_sweep
// k_kappa_residual   float64 r = b - A c with an explicit float64 right-hand side or the
//                    Dirichlet terms; per-plane sums of r^2 and b^2
//
// The float64 steps (residual, float64 layer sums, adjoint right-hand side) take their
// coefficients either as the sweeps do (float32 faces and float32 `factor`: the reference's own
// discrete operator) or as float64 faces 2ab/(a+b) of the float32 kappa values with the exact
// float64 diagonal. In the second form D_eff is a smooth function of kappa, which is what
// dD_eff/dkappa and its finite-difference checks need: float32 faces change in steps of one
// rounding, so a central difference of step h carries noise of about 1e-7/h relative.
// k_kappa_layer_sums per-plane float64 sums of face_x * (c[x+1] - c[x]) and of c
// k_kappa_dJdc       adjoint right-hand side dD_eff/dc (float64)
// k_kappa_grad       dD_eff/dkappa per voxel from c and the adjoint lambda (float64)
#include "tf_common.cuh"
#include "tf_internal.h"
#include "tf_update.cuh"

namespace tf {

// harmonic face in the reference's float32 order: ((2a) b) / (a + b), 0 when a + b == 0
__device__ __forceinline__ float hface(float a, float b) {
    const float den = __fadd_rn(a, b);
    return den > 0.0f ? __fdiv_rn(__fmul_rn(__fmul_rn(2.0f, a), b), den) : 0.0f;
}

struct KView {
    Geo g;
    __device__ __forceinline__ long long off(int x, int y, int z) const {
        return (long long)x * g.plane_f + (long long)(y + HY) * g.row_f + (z & 1) * g.ZH + HJ + (z >> 1);
    }
};

// The six faces of voxel (x,y,z) and their neighbour values, in the reference's roles.
struct Faces {
    float xp, xm, yp, ym, zp, zm;   // conductances
    float div;                      // factor (inf if 0)
};

// Neighbour (y, z) index with ghost rows/cells: the split layout already holds periodic copies
// or zeros within one cell of every face, so plain offsets work for y+-1 and z+-1.
__device__ __forceinline__ Faces kappa_faces(const float* kp, const KView& v, int x, int y, int z, float kc) {
    Faces f;
    f.xm = x > 0 ? hface(kc, kp[v.off(x - 1, y, z)]) : hface(kc, kc);
    f.xp = x + 1 < v.g.NX ? hface(kc, kp[v.off(x + 1, y, z)]) : hface(kc, kc);
    f.ym = hface(kc, kp[v.off(x, y - 1, z)]);
    f.yp = hface(kc, kp[v.off(x, y + 1, z)]);
    f.zm = hface(kc, kp[v.off(x, y, z - 1)]);
    f.zp = hface(kc, kp[v.off(x, y, z + 1)]);
    float d = __fadd_rn(f.xm, f.xp);
    d = __fadd_rn(d, f.ym);
    d = __fadd_rn(d, f.yp);
    d = __fadd_rn(d, f.zm);
    d = __fadd_rn(d, f.zp);
    if (x == 0) d = __fadd_rn(d, f.xm);
    if (x == v.g.NX - 1) d = __fadd_rn(d, f.xp);
    f.div = d == 0.0f ? __int_as_float(0x7f800000) : d;
    return f;
}

// float64 face of the float32 values a, b: 2ab/(a+b), 0 when a + b == 0 (hface64(k, k) = k)
__device__ __forceinline__ double hface64(double a, double b) {
    const double den = a + b;
    return den > 0.0 ? 2.0 * a * b / den : 0.0;
}

// The faces and the diagonal in float64; F64C selects float64 coefficients, otherwise the
// float32 ones of kappa_faces widened. `active` = the voxel has a finite diagonal.
struct Faces64 {
    double xp, xm, yp, ym, zp, zm, div;
    bool active;
};

template <bool F64C>
__device__ __forceinline__ Faces64 kappa_faces_fp64(const float* kp, const KView& v, int x, int y, int z, float kc) {
    Faces64 d;
    if (F64C) {
        const double k = kc;
        d.xm = x > 0 ? hface64(k, kp[v.off(x - 1, y, z)]) : k;
        d.xp = x + 1 < v.g.NX ? hface64(k, kp[v.off(x + 1, y, z)]) : k;
        d.ym = hface64(k, kp[v.off(x, y - 1, z)]);
        d.yp = hface64(k, kp[v.off(x, y + 1, z)]);
        d.zm = hface64(k, kp[v.off(x, y, z - 1)]);
        d.zp = hface64(k, kp[v.off(x, y, z + 1)]);
        d.div = d.xm + d.xp + d.ym + d.yp + d.zm + d.zp;
        if (x == 0) d.div += d.xm;
        if (x == v.g.NX - 1) d.div += d.xp;
        d.active = d.div > 0.0;
    } else {
        const Faces f = kappa_faces(kp, v, x, y, z, kc);
        d.xm = f.xm;
        d.xp = f.xp;
        d.ym = f.ym;
        d.yp = f.yp;
        d.zm = f.zm;
        d.zp = f.zp;
        d.div = f.div;
        d.active = f.div < __int_as_float(0x7f800000);
    }
    return d;
}

// One thread per interior voxel of colour `colour`; in place (neighbours have the other colour,
// and periodic ghosts are refreshed after the launch, as for the plain binary sweep).
__global__ void __launch_bounds__(256) k_kappa_sweep(float* __restrict__ c, const float* __restrict__ kp,
                                                     const float* __restrict__ rhs, const SweepArgs a, int colour) {
    const Geo& g = a.g;
    const KView v{g};
    const long long n = (long long)g.NX * g.NY * ((g.NZ + 1) / 2);
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int hz = (g.NZ + 1) / 2;
    const int x = (int)(i / ((long long)g.NY * hz));
    const int rem = (int)(i - (long long)x * g.NY * hz);
    const int y = rem / hz;
    const int zz = rem - y * hz;
    const int z = 2 * zz + ((x + y + colour) & 1);  // the colour-`colour` voxel of this pair
    if (z >= g.NZ) return;
    const long long b0 = (long long)blockIdx.y * g.vol_f;
    float* cb = c + b0;
    const float* kb = kp + b0;
    const long long o = v.off(x, y, z);
    const float kc = kb[o];
    const Faces f = kappa_faces(kb, v, x, y, z, kc);
    const float cxp = x + 1 < g.NX ? cb[v.off(x + 1, y, z)] : a.ghi;
    const float cxm = x > 0 ? cb[v.off(x - 1, y, z)] : a.glo;
    // taufactor.py:607-612: products, then left-to-right sum
    float s = __fadd_rn(__fmul_rn(cxp, f.xp), __fmul_rn(cxm, f.xm));
    s = __fadd_rn(s, __fmul_rn(cb[v.off(x, y + 1, z)], f.yp));
    s = __fadd_rn(s, __fmul_rn(cb[v.off(x, y - 1, z)], f.ym));
    s = __fadd_rn(s, __fmul_rn(cb[v.off(x, y, z + 1)], f.zp));
    s = __fadd_rn(s, __fmul_rn(cb[v.off(x, y, z - 1)], f.zm));
    if (rhs) s = __fadd_rn(s, rhs[b0 + o]);
    cb[o] = sor_finish(cb[o], quotient(s, f.div), a.omega);
}

// Packed faces, in the float32 values the sweeps use. hface(a, b) == hface(b, a) bit for bit
// ((2a) b and (2b) a are the same rounded product), so a face is stored once and read by both
// of its voxels.
//   fx [b][x'][plane], x' = 0..NX: x' = x + 1 holds the face between planes x and x + 1; x' = 0
//      and x' = NX hold the Dirichlet faces hface(k, k) of planes 0 and NX - 1
//   fy [b][x][Y][...]: the face between padded rows Y and Y + 1 (0 past the last padded row)
//   fz [b][x][Y][q][jp]: the face between cell z = 2 (jp - HJ) + q and z + 1 (0 past the row)
//   dv [b][x][Y][q][jp]: the factor of kappa_faces for interior cells and periodic ghost
//      positions (the wrapped cell's), inf elsewhere
__global__ void k_kappa_face_pack(const float* __restrict__ kp, float* __restrict__ fx, float* __restrict__ fy,
                                  float* __restrict__ fz, float* __restrict__ dv, const Geo g, int periodic) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q * ZH + jp
    if (pos >= 2 * g.ZH) return;
    const int Y = blockIdx.y;
    const int bx = blockIdx.z;  // b * NX + x
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = pos >= g.ZH ? 1 : 0;
    const int jp = pos - q * g.ZH;
    const long long o = (long long)bx * g.plane_f + (long long)Y * g.row_f + pos;
    const float kc = kp[o];
    fy[o] = Y + 1 < g.YP ? hface(kc, kp[o + g.row_f]) : 0.0f;
    const long long on = q == 0 ? o + g.ZH : (jp + 1 < g.ZH ? o - g.ZH + 1 : -1);
    fz[o] = on >= 0 ? hface(kc, kp[on]) : 0.0f;
    const long long fxo = ((long long)b * (g.NX + 1) + x) * g.plane_f + (long long)Y * g.row_f + pos;
    fx[fxo + g.plane_f] = x + 1 < g.NX ? hface(kc, kp[o + g.plane_f]) : hface(kc, kc);
    if (x == 0) fx[fxo] = hface(kc, kc);
    // the factor of interior cells, and on periodic ghost positions that of the wrapped cell (a
    // fused sweep updates the ghost copies of its tile's halo like the cells they mirror)
    int y = Y - HY, z = 2 * (jp - HJ) + q;
    bool ok = true;
    if (y < 0 || y >= g.NY) {
        ok = ok && (periodic & TF_PERIODIC_Y);
        y = wrap(y, g.NY);
    }
    if (z < 0 || z >= g.NZ) {
        ok = ok && (periodic & TF_PERIODIC_Z);
        z = wrap(z, g.NZ);
    }
    float d = __int_as_float(0x7f800000);
    if (ok) {
        const KView v{g};
        const float* kb = kp + (long long)b * g.vol_f;
        d = kappa_faces(kb, v, x, y, z, kb[v.off(x, y, z)]).div;
    }
    dv[o] = d;
}

// One half-sweep in place from the packed faces: one thread per float4 group of the colour's
// half-row (the arithmetic of k_kappa_sweep, taufactor.py:607-612).
template <bool RHS>
__global__ void __launch_bounds__(256) k_kappa_sweep4(float* __restrict__ c, const float* __restrict__ fx,
                                                      const float* __restrict__ fy, const float* __restrict__ fz,
                                                      const float* __restrict__ dv, const SweepArgs a, int colour) {
    const Geo& g = a.g;
    const int gmax = (half_len(g.NZ, 0) + 3) >> 2;
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;  // rows of the plane across the block
    if (gi >= gmax || y >= g.NY) return;
    const int bx = blockIdx.z;  // b * NX + x
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = (x + y + colour) & 1;
    const int nj = half_len(g.NZ, q);
    const int j = 4 * gi;
    if (j >= nj) return;
    const long long base = (long long)bx * g.plane_f + (long long)(y + HY) * g.row_f;
    const long long rq = base + q * g.ZH + HJ + j;        // this group
    const long long ro = base + (q ^ 1) * g.ZH + HJ + j;  // the other half-row, same j
    const float4 cc = ld4(c + rq);
    const float4 xp = x + 1 < g.NX ? ld4(c + rq + g.plane_f) : make_float4(a.ghi, a.ghi, a.ghi, a.ghi);
    const float4 xm = x > 0 ? ld4(c + rq - g.plane_f) : make_float4(a.glo, a.glo, a.glo, a.glo);
    const float4 yp = ld4(c + rq + g.row_f);
    const float4 ym = ld4(c + rq - g.row_f);
    float4 zp, zm;
    z_neighbours(q, ld4(c + ro), q ? c[ro + 4] : c[ro - 1], zp, zm);
    const long long fxq = ((long long)b * (g.NX + 1) + x) * g.plane_f + (long long)(y + HY) * g.row_f + q * g.ZH +
                          HJ + j;  // fx plane x: the face between x - 1 and x
    const float4 fxm = ld4(fx + fxq), fxp = ld4(fx + fxq + g.plane_f);
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
    float4 rv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (RHS) rv = ld4(a.rhs + rq);
    float4 nv;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float s = __fadd_rn(__fmul_rn(comp(xp, i), comp(fxp, i)), __fmul_rn(comp(xm, i), comp(fxm, i)));
        s = __fadd_rn(s, __fmul_rn(comp(yp, i), comp(fyp, i)));
        s = __fadd_rn(s, __fmul_rn(comp(ym, i), comp(fym, i)));
        s = __fadd_rn(s, __fmul_rn(comp(zp, i), comp(fzp, i)));
        s = __fadd_rn(s, __fmul_rn(comp(zm, i), comp(fzm, i)));
        if (RHS) s = __fadd_rn(s, comp(rv, i));
        set_comp(nv, i, sor_finish(comp(cc, i), quotient(s, comp(d, i)), a.omega));
    }
    float* dst = c + rq;
    if (j + 4 <= nj)
        st4(dst, nv);
    else
        for (int i = 0; i < nj - j; ++i) dst[i] = comp(nv, i);
}

// float64 residual; bsrc (float64, split layout) replaces the Dirichlet terms when non-null.
template <bool F64C>
__global__ void __launch_bounds__(256) k_kappa_residual(const double* __restrict__ c64, const float* __restrict__ kp,
                                                        const double* __restrict__ bsrc, float* __restrict__ r32,
                                                        double* __restrict__ r2, double* __restrict__ b2, const Geo g,
                                                        float glo, float ghi) {
    __shared__ double red[2][32];
    const KView v{g};
    const int x = blockIdx.x, b = blockIdx.y;
    const long long b0 = (long long)b * g.vol_f;
    const double* cb = c64 + b0;
    const float* kb = kp + b0;
    double rs = 0.0, bs = 0.0;
    for (long long it = threadIdx.x; it < (long long)g.NY * g.NZ; it += blockDim.x) {
        const int y = (int)(it / g.NZ), z = (int)(it - (long long)y * g.NZ);
        const long long o = v.off(x, y, z);
        const Faces64 f = kappa_faces_fp64<F64C>(kb, v, x, y, z, kb[o]);
        double res = 0.0, rhs = 0.0;
        if (f.active) {
            double s = f.yp * cb[v.off(x, y + 1, z)] + f.ym * cb[v.off(x, y - 1, z)] +
                       f.zp * cb[v.off(x, y, z + 1)] + f.zm * cb[v.off(x, y, z - 1)];
            if (x > 0) s += f.xm * cb[v.off(x - 1, y, z)];
            else if (!bsrc) rhs += f.xm * glo;
            if (x + 1 < g.NX) s += f.xp * cb[v.off(x + 1, y, z)];
            else if (!bsrc) rhs += f.xp * ghi;
            if (bsrc) rhs = bsrc[b0 + o];
            res = rhs - (f.div * cb[o] - s);
        }
        r32[b0 + o] = (float)res;
        rs += res * res;
        bs += rhs * rhs;
    }
    for (int s = 16; s > 0; s >>= 1) {
        rs += __shfl_xor_sync(0xffffffffu, rs, s);
        bs += __shfl_xor_sync(0xffffffffu, bs, s);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = rs;
        red[1][threadIdx.x >> 5] = bs;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p = 0.0, q = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            p += red[0][w];
            q += red[1][w];
        }
        r2[(long long)b * g.NX + x] = p;
        b2[(long long)b * g.NX + x] = q;
    }
}

// T = float or double field; F64C (double fields only) = float64 faces
template <typename T, bool F64C>
__global__ void __launch_bounds__(256) k_kappa_layer_sums(const T* __restrict__ c, const float* __restrict__ kp,
                                                          double* __restrict__ flux, double* __restrict__ csum,
                                                          const Geo g) {
    __shared__ double red[2][32];
    const KView v{g};
    const int x = blockIdx.x, b = blockIdx.y;
    const long long b0 = (long long)b * g.vol_f;
    const bool has_flux = x + 1 < g.NX;
    double fs = 0.0, cs = 0.0;
    for (long long it = threadIdx.x; it < (long long)g.NY * g.NZ; it += blockDim.x) {
        const int y = (int)(it / g.NZ), z = (int)(it - (long long)y * g.NZ);
        const long long o = v.off(x, y, z);
        const T a = c[b0 + o];
        cs += (double)a;
        if (has_flux) {
            const long long o1 = v.off(x + 1, y, z);
            if (sizeof(T) == 4) {
                const float face = hface(kp[b0 + o], kp[b0 + o1]);
                fs += (double)__fmul_rn(face, __fsub_rn((float)c[b0 + o1], (float)a));  // :617-619 in float32
            } else {
                const double face = F64C ? hface64(kp[b0 + o], kp[b0 + o1]) : (double)hface(kp[b0 + o], kp[b0 + o1]);
                fs += face * ((double)c[b0 + o1] - (double)a);
            }
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        fs += __shfl_xor_sync(0xffffffffu, fs, s);
        cs += __shfl_xor_sync(0xffffffffu, cs, s);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = fs;
        red[1][threadIdx.x >> 5] = cs;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p = 0.0, q = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            p += red[0][w];
            q += red[1][w];
        }
        if (has_flux) flux[(long long)b * (g.NX - 1) + x] = p;
        csum[(long long)b * g.NX + x] = q;
    }
}

// dJ/dc for J = D_0 * mean_x(layer flux) * Nx / |bc_hi - bc_lo| with layer flux
// (1/(Ny Nz)) sum face_x (c[x+1] - c[x]): dJ/dc[x] = K (face_{x-1|x} - face_{x|x+1}),
// K = D_0 Nx / (|dbc| (Nx-1) Ny Nz). Written for interior voxels (0 elsewhere).
template <bool F64C>
__global__ void k_kappa_dJdc(const float* __restrict__ kp, double* __restrict__ g_out, const Geo g, double K) {
    const KView v{g};
    const long long n = (long long)g.NX * g.NY * g.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i / ((long long)g.NY * g.NZ));
    const int rem = (int)(i - (long long)x * g.NY * g.NZ);
    const int y = rem / g.NZ, z = rem - (rem / g.NZ) * g.NZ;
    const long long b0 = (long long)blockIdx.y * g.vol_f;
    const long long o = v.off(x, y, z);
    const float kc = kp[b0 + o];
    double d = 0.0;
    if (x > 0) {
        const float kw = kp[b0 + v.off(x - 1, y, z)];
        d += F64C ? hface64(kw, kc) : (double)hface(kw, kc);
    }
    if (x + 1 < g.NX) {
        const float kw = kp[b0 + v.off(x + 1, y, z)];
        d -= F64C ? hface64(kc, kw) : (double)hface(kc, kw);
    }
    g_out[b0 + o] = K * d;
}

// d hface(a, b) / d a = 2 b^2 / (a + b)^2 (0 if a + b == 0), in float64
__device__ __forceinline__ double dface_da(double a, double b) {
    const double s = a + b;
    return s > 0.0 ? 2.0 * b * b / (s * s) : 0.0;
}

// dJ/dkappa[u] = sum over u's faces f of dJ/dg_f * dg_f/dkappa_u, with
//   interior face (u,w): dJ/dg = explicit - (lam_u - lam_w)(c_u - c_w),
//                        explicit = K (c[x+1] - c[x]) for x-faces between two interior planes;
//   Dirichlet face of u (x = 0 or Nx-1, conductance hface(k_u, k_u), counted twice in A and b):
//                        dJ/dg = 2 lam_u (bc - c_u), dg/dk_u = d/dk hface(k, k) = 1.
// Out: natural layout [b][x][y][z] float64.
__global__ void k_kappa_grad(const double* __restrict__ c64, const double* __restrict__ lam,
                             const float* __restrict__ kp, double* __restrict__ grad, const Geo g, int periodic,
                             double K, double bc_lo, double bc_hi) {
    const KView v{g};
    const long long n = (long long)g.NX * g.NY * g.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i / ((long long)g.NY * g.NZ));
    const int rem = (int)(i - (long long)x * g.NY * g.NZ);
    const int y = rem / g.NZ, z = rem - y * g.NZ;
    const long long b0 = (long long)blockIdx.y * g.vol_f;
    const long long o = v.off(x, y, z);
    const double ku = kp[b0 + o], cu = c64[b0 + o], lu = lam[b0 + o];
    double gr = 0.0;
    // x faces
    if (x > 0) {
        const long long w = v.off(x - 1, y, z);
        const double kw = kp[b0 + w], cw = c64[b0 + w], lw = lam[b0 + w];
        const double dj = K * (cu - cw) - (lu - lw) * (cu - cw);
        gr += dj * dface_da(ku, kw);
    } else {
        gr += 2.0 * lu * (bc_lo - cu);
    }
    if (x + 1 < g.NX) {
        const long long w = v.off(x + 1, y, z);
        const double kw = kp[b0 + w], cw = c64[b0 + w], lw = lam[b0 + w];
        const double dj = K * (cw - cu) - (lu - lw) * (cu - cw);
        gr += dj * dface_da(ku, kw);
    } else {
        gr += 2.0 * lu * (bc_hi - cu);
    }
    // y and z faces (neighbours outside closed faces have kappa 0 -> face 0, derivative 0)
    const int dy[4] = {1, -1, 0, 0}, dz[4] = {0, 0, 1, -1};
    for (int k = 0; k < 4; ++k) {
        int yy = y + dy[k], zq = z + dz[k];
        if (yy < 0 || yy >= g.NY) {
            if (!(periodic & TF_PERIODIC_Y)) continue;
            yy = wrap(yy, g.NY);
        }
        if (zq < 0 || zq >= g.NZ) {
            if (!(periodic & TF_PERIODIC_Z)) continue;
            zq = wrap(zq, g.NZ);
        }
        const long long w = v.off(x, yy, zq);
        const double kw = kp[b0 + w], cw = c64[b0 + w], lw = lam[b0 + w];
        gr += -(lu - lw) * (cu - cw) * dface_da(ku, kw);
    }
    grad[(long long)blockIdx.y * n + i] = gr;
}

// ---------------------------------------------------------------- packed float64 faces
// The float64 faces of the FP64 steps (coeff_f64 = 1) in the layout of k_kappa_face_pack,
// computed once per kappa field: each face 2ab/(a+b) costs a float64 division, which GB300's
// FP64 pipe makes the bound of every step that recomputes them (six per voxel per residual).
//   fx [b][x'][plane] (x' = 0..NX; x' = 0 and NX: the Dirichlet faces kappa of planes 0, NX-1),
//   fy, fz: the +y / +z face of every padded position; k_kappa_diag64 then writes dv, the
//   diagonal (0 outside the system).
__global__ void k_kappa_face_pack64(const float* __restrict__ kp, double* __restrict__ fx, double* __restrict__ fy,
                                    double* __restrict__ fz, double* __restrict__ dv, const Geo g) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q * ZH + jp
    if (pos >= 2 * g.ZH) return;
    const int Y = blockIdx.y;
    const int bx = blockIdx.z;  // b * NX + x
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = pos >= g.ZH ? 1 : 0;
    const int jp = pos - q * g.ZH;
    const long long o = (long long)bx * g.plane_f + (long long)Y * g.row_f + pos;
    const double k = kp[o];
    fy[o] = Y + 1 < g.YP ? hface64(k, kp[o + g.row_f]) : 0.0;
    const long long on = q == 0 ? o + g.ZH : (jp + 1 < g.ZH ? o - g.ZH + 1 : -1);
    fz[o] = on >= 0 ? hface64(k, kp[on]) : 0.0;
    const long long fxo = ((long long)b * (g.NX + 1) + x) * g.plane_f + (long long)Y * g.row_f + pos;
    fx[fxo + g.plane_f] = x + 1 < g.NX ? hface64(k, kp[o + g.plane_f]) : k;
    if (x == 0) fx[fxo] = k;
}

// The diagonal of the packed float64 faces: the six faces of kappa_faces_fp64<true> read back
// (hface64 is symmetric, so a face packed at the neighbour is the same float64), summed in its
// order, the Dirichlet faces once more; 0 outside the system. One thread per padded position.
__global__ void k_kappa_diag64(const double* __restrict__ fx, const double* __restrict__ fy,
                               const double* __restrict__ fz, double* __restrict__ dv, const Geo g) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q * ZH + jp
    if (pos >= 2 * g.ZH) return;
    const int Y = blockIdx.y;
    const int bx = blockIdx.z;  // b * NX + x
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = pos >= g.ZH ? 1 : 0;
    const int jp = pos - q * g.ZH;
    const long long o = (long long)bx * g.plane_f + (long long)Y * g.row_f + pos;
    const int y = Y - HY, z = 2 * (jp - HJ) + q;
    double d = 0.0;
    if (y >= 0 && y < g.NY && jp >= HJ && z < g.NZ) {
        const long long fxo = ((long long)b * (g.NX + 1) + x) * g.plane_f + (long long)Y * g.row_f + pos;
        const KView v{g};
        const long long b0 = (long long)b * g.vol_f;
        const double xm = fx[fxo], xp = fx[fxo + g.plane_f];
        const double ym = fy[b0 + v.off(x, y - 1, z)], yp = fy[o];
        const double zm = fz[b0 + v.off(x, y, z - 1)], zp = fz[o];
        d = xm + xp + ym + yp + zm + zp;
        if (x == 0) d += xm;
        if (x == g.NX - 1) d += xp;
        if (!(d > 0.0)) d = 0.0;
    }
    dv[o] = d;
}

// k_kappa_residual<true> from the packed float64 faces with fused multiply-adds (the same r to
// a few float64 roundings); 1024 threads per plane.
__global__ void __launch_bounds__(1024, 1) k_kappa_residual_p64(const double* __restrict__ c64,
                                                            const double* __restrict__ fx,
                                                            const double* __restrict__ fy,
                                                            const double* __restrict__ fz,
                                                            const double* __restrict__ dv,
                                                            const double* __restrict__ bsrc, float* __restrict__ r32,
                                                            double* __restrict__ r2, double* __restrict__ b2,
                                                            const Geo g, float glo, float ghi) {
    __shared__ double red[2][32];
    const KView v{g};
    const int x = blockIdx.x, b = blockIdx.y;
    const long long b0 = (long long)b * g.vol_f;
    const long long fx0 = ((long long)b * (g.NX + 1) + x) * g.plane_f - (long long)x * g.plane_f;  // + v.off
    const double* cb = c64 + b0;
    double rs = 0.0, bs = 0.0;
    // warp w takes rows y = w, w + 32, ...; its lanes walk z (no index division)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int y = wid; y < g.NY; y += nw)
        for (int z = lane; z < g.NZ; z += 32) {
            const long long o = v.off(x, y, z);
            const double div = dv[b0 + o];
            double res = 0.0, rhs = 0.0;
            if (div > 0.0) {
                // fused multiply-adds: GB300's FP64 pipe (2 operations per SM per clock) bounds
                // this kernel, and each fma halves the operations of a product and a sum
                const double xm = fx[fx0 + o], xp = fx[fx0 + o + g.plane_f];
                const long long oym = v.off(x, y - 1, z), ozm = v.off(x, y, z - 1);
                double s = fy[b0 + o] * cb[v.off(x, y + 1, z)];
                s = fma(fy[b0 + oym], cb[oym], s);
                s = fma(fz[b0 + o], cb[v.off(x, y, z + 1)], s);
                s = fma(fz[b0 + ozm], cb[ozm], s);
                if (x > 0) s = fma(xm, cb[o - g.plane_f], s);
                else if (!bsrc) rhs = xm * glo;
                if (x + 1 < g.NX) s = fma(xp, cb[o + g.plane_f], s);
                else if (!bsrc) rhs = fma(xp, (double)ghi, rhs);
                if (bsrc) rhs = bsrc[b0 + o];
                res = fma(-div, cb[o], rhs + s);
            }
            r32[b0 + o] = (float)res;
            rs = fma(res, res, rs);
            bs = fma(rhs, rhs, bs);
        }
    for (int s = 16; s > 0; s >>= 1) {
        rs += __shfl_xor_sync(0xffffffffu, rs, s);
        bs += __shfl_xor_sync(0xffffffffu, bs, s);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = rs;
        red[1][threadIdx.x >> 5] = bs;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p = 0.0, q = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            p += red[0][w];
            q += red[1][w];
        }
        r2[(long long)b * g.NX + x] = p;
        b2[(long long)b * g.NX + x] = q;
    }
}

// k_kappa_layer_sums<double, true> from the packed float64 x faces (same bits).
__global__ void __launch_bounds__(1024, 1) k_kappa_layer_sums_p64(const double* __restrict__ c,
                                                              const double* __restrict__ fx,
                                                              double* __restrict__ flux, double* __restrict__ csum,
                                                              const Geo g) {
    __shared__ double red[2][32];
    const KView v{g};
    const int x = blockIdx.x, b = blockIdx.y;
    const long long b0 = (long long)b * g.vol_f;
    const long long fx1 = ((long long)b * (g.NX + 1) + x + 1) * g.plane_f - (long long)x * g.plane_f;  // + v.off
    const bool has_flux = x + 1 < g.NX;
    double fs = 0.0, cs = 0.0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int y = wid; y < g.NY; y += nw)
        for (int z = lane; z < g.NZ; z += 32) {
            const long long o = v.off(x, y, z);
            const double a = c[b0 + o];
            cs += a;
            if (has_flux) fs += fx[fx1 + o] * (c[b0 + o + g.plane_f] - a);
        }
    for (int s = 16; s > 0; s >>= 1) {
        fs += __shfl_xor_sync(0xffffffffu, fs, s);
        cs += __shfl_xor_sync(0xffffffffu, cs, s);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = fs;
        red[1][threadIdx.x >> 5] = cs;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p = 0.0, q = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            p += red[0][w];
            q += red[1][w];
        }
        if (has_flux) flux[(long long)b * (g.NX - 1) + x] = p;
        csum[(long long)b * g.NX + x] = q;
    }
}

// dJ/dkappa per voxel (k_kappa_grad's formula) from the packed float64 faces: d face / d k_u
// = 2 k_w^2 / (k_u + k_w)^2 = face^2 / (2 k_u^2), one division per voxel instead of one per face
// (the original form where k_u = 0). Out: natural layout [b][x][y][z] float64.
__global__ void k_kappa_grad_p64(const double* __restrict__ c64, const double* __restrict__ lam,
                                 const float* __restrict__ kp, const double* __restrict__ fx,
                                 const double* __restrict__ fy, const double* __restrict__ fz,
                                 double* __restrict__ grad, const Geo g, int periodic, double K, double bc_lo,
                                 double bc_hi) {
    const KView v{g};
    const long long n = (long long)g.NX * g.NY * g.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i / ((long long)g.NY * g.NZ));
    const int rem = (int)(i - (long long)x * g.NY * g.NZ);
    const int y = rem / g.NZ, z = rem - y * g.NZ;
    const long long b0 = (long long)blockIdx.y * g.vol_f;
    const long long fxb = ((long long)blockIdx.y * (g.NX + 1)) * g.plane_f;
    const long long o = v.off(x, y, z);
    const double ku = kp[b0 + o], cu = c64[b0 + o], lu = lam[b0 + o];
    const double inv = ku > 0.0 ? 1.0 / (2.0 * ku * ku) : 0.0;
    // d face / d k_u from the face (ku > 0) or from k_w (ku = 0: 2 k_w^2 / k_w^2 = 2 if k_w > 0)
    auto dface = [&](double face, double kw) { return ku > 0.0 ? face * face * inv : dface_da(ku, kw); };
    double gr = 0.0;
    if (x > 0) {
        const long long w = o - g.plane_f;
        const double cw = c64[b0 + w], lw = lam[b0 + w];
        const double dj = K * (cu - cw) - (lu - lw) * (cu - cw);
        gr += dj * dface(fx[fxb + o], kp[b0 + w]);
    } else {
        gr += 2.0 * lu * (bc_lo - cu);
    }
    if (x + 1 < g.NX) {
        const long long w = o + g.plane_f;
        const double cw = c64[b0 + w], lw = lam[b0 + w];
        const double dj = K * (cw - cu) - (lu - lw) * (cu - cw);
        gr += dj * dface(fx[fxb + o + g.plane_f], kp[b0 + w]);
    } else {
        gr += 2.0 * lu * (bc_hi - cu);
    }
    // y and z faces: packed at the lower cell of each pair; ghost positions hold the wrapped
    // faces (periodic) or 0 (closed, derivative 0)
    const int dy[4] = {1, -1, 0, 0}, dz[4] = {0, 0, 1, -1};
    for (int k = 0; k < 4; ++k) {
        int yy = y + dy[k], zq = z + dz[k];
        if (yy < 0 || yy >= g.NY) {
            if (!(periodic & TF_PERIODIC_Y)) continue;
            yy = wrap(yy, g.NY);
        }
        if (zq < 0 || zq >= g.NZ) {
            if (!(periodic & TF_PERIODIC_Z)) continue;
            zq = wrap(zq, g.NZ);
        }
        const double face = k == 0 ? fy[b0 + o] : k == 1 ? fy[b0 + v.off(x, y - 1, z)]
                          : k == 2 ? fz[b0 + o] : fz[b0 + v.off(x, y, z - 1)];
        const long long w = v.off(x, yy, zq);
        const double kw = kp[b0 + w], cw = c64[b0 + w], lw = lam[b0 + w];
        gr += -(lu - lw) * (cu - cw) * dface(face, kw);
    }
    grad[(long long)blockIdx.y * n + i] = gr;
}

}  // namespace tf

// ------------------------------------------------------------------------------ host side
namespace tf {

// kappa natural [b][x][y][z] -> split layout with ghost cells (0 on closed faces, wrapped
// copies on periodic ones); initial field = profile[x] where kappa > 0 (taufactor.py:282-291
// with MultiPhaseSolver's conductive mask, :571-575).
__global__ void k_kappa_pack(const float* __restrict__ kin, const float* __restrict__ profile,
                             float* __restrict__ kout, float* __restrict__ field, const Geo g, int periodic) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;  // q*ZH + jp
    if (pos >= 2 * g.ZH) return;
    const int Y = blockIdx.y, bx = blockIdx.z;
    const int x = bx % g.NX, b = bx / g.NX;
    const int q = pos >= g.ZH ? 1 : 0;
    const int jp = pos - q * g.ZH;
    int y = Y - HY, z = 2 * (jp - HJ) + q;
    float kv = 0.0f, fv = 0.0f;
    bool ok = true;
    if (y < 0 || y >= g.NY) {
        ok = ok && (periodic & TF_PERIODIC_Y);
        y = wrap(y, g.NY);
    }
    if (z < 0 || z >= g.NZ) {
        ok = ok && (periodic & TF_PERIODIC_Z);
        z = wrap(z, g.NZ);
    }
    if (ok) {
        kv = kin[(((long long)b * g.NX + x) * g.NY + y) * g.NZ + z];
        fv = kv > 0.0f ? profile[x] : 0.0f;
    }
    const long long o = ((long long)bx * g.YP + Y) * 2 * g.ZH + pos;
    kout[o] = kv;
    field[o] = fv;
}

// split layout (float64) -> natural [b][x][y][z] (float64)
__global__ void k_split_to_natural(const double* __restrict__ in, double* __restrict__ out, const Geo g) {
    const long long n = (long long)g.NX * g.NY * g.NZ;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i / ((long long)g.NY * g.NZ));
    const int rem = (int)(i - (long long)x * g.NY * g.NZ);
    const int y = rem / g.NZ, z = rem - y * g.NZ;
    const KView v{g};
    out[(long long)blockIdx.y * n + i] = in[(long long)blockIdx.y * g.vol_f + v.off(x, y, z)];
}

}  // namespace tf

using namespace tf;

extern "C" {

int tf_kappa_pack(const tf_geom* g, const tf_operator* op, const float* kappa_dev, const float* profile_dev,
                  float* kappa_split_dev, float* field_dev, void* stream) {
    if (!g || !op || !kappa_dev || !profile_dev || !kappa_split_dev || !field_dev) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    dim3 grid((2 * g->zh + 127) / 128, g->yp, g->batch * g->nx);
    k_kappa_pack<<<grid, 128, 0, (cudaStream_t)stream>>>(kappa_dev, profile_dev, kappa_split_dev, field_dev, geo,
                                                         op->periodic);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_advance(const tf_geom* g, const tf_operator* op, float* field_dev, const float* kappa_split_dev,
                     const float* rhs_dev, int first_colour, int n_half, void* stream) {
    if (!g || !op || !field_dev || !kappa_split_dev || n_half < 0) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const Geo geo = make_geo(*g);
    const long long n = (long long)g->nx * g->ny * ((g->nz + 1) / 2);
    dim3 grid((unsigned)((n + 255) / 256), g->batch);
    int colour = first_colour & 1;
    for (int i = 0; i < n_half; ++i, colour ^= 1) {
        SweepArgs a = make_args(geo, *op, field_dev, colour, 1, nullptr);
        k_kappa_sweep<<<grid, 256, 0, st>>>(field_dev, kappa_split_dev, rhs_dev, a, colour);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
        if (op->periodic) {
            const int rc = refresh_ghosts(*g, op->periodic, field_dev, st);
            if (rc) return rc;
        }
    }
    return TF_OK;
}

int tf_kappa_faces(const tf_geom* g, const float* kappa_split_dev, float* fx_dev, float* fy_dev, float* fz_dev,
                   float* div_dev, int periodic, void* stream) {
    if (!g || !kappa_split_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    dim3 grid((2 * g->zh + 127) / 128, g->yp, g->batch * g->nx);
    k_kappa_face_pack<<<grid, 128, 0, (cudaStream_t)stream>>>(kappa_split_dev, fx_dev, fy_dev, fz_dev, div_dev, geo,
                                                               periodic);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_advance_faces(const tf_geom* g, const tf_operator* op, float* field_dev, const float* fx_dev,
                           const float* fy_dev, const float* fz_dev, const float* div_dev, const float* rhs_dev,
                           int first_colour, int n_half, void* stream) {
    if (!g || !op || !field_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev || n_half < 0) return TF_ERR_ARG;
    const uintptr_t al = reinterpret_cast<uintptr_t>(field_dev) | reinterpret_cast<uintptr_t>(fx_dev) |
                         reinterpret_cast<uintptr_t>(fy_dev) | reinterpret_cast<uintptr_t>(fz_dev) |
                         reinterpret_cast<uintptr_t>(div_dev) | reinterpret_cast<uintptr_t>(rhs_dev);
    if (al & 15) return TF_ERR_ARG;  // float4 loads
    cudaStream_t st = (cudaStream_t)stream;
    const Geo geo = make_geo(*g);
    const int gmax = (half_len(g->nz, 0) + 3) >> 2;
    // a warp per 32 float4 groups of one half-row, 8 rows per block
    const dim3 bs(32, 8);
    dim3 grid((gmax + 31) / 32, (g->ny + 7) / 8, g->batch * g->nx);
    int colour = first_colour & 1;
    for (int i = 0; i < n_half; ++i, colour ^= 1) {
        SweepArgs a = make_args(geo, *op, field_dev, colour, 1, nullptr);
        a.rhs = rhs_dev;
        if (rhs_dev)
            k_kappa_sweep4<true><<<grid, bs, 0, st>>>(field_dev, fx_dev, fy_dev, fz_dev, div_dev, a, colour);
        else
            k_kappa_sweep4<false><<<grid, bs, 0, st>>>(field_dev, fx_dev, fy_dev, fz_dev, div_dev, a, colour);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
        if (op->periodic) {
            const int rc = refresh_ghosts(*g, op->periodic, field_dev, st);
            if (rc) return rc;
        }
    }
    return TF_OK;
}

int tf_kappa_layer_sums(const tf_geom* g, const void* field_dev, int field_is_f64, int coeff_f64,
                        const float* kappa_split_dev, double* flux_sum_dev, double* c_sum_dev, void* stream) {
    if (!g || !field_dev || !kappa_split_dev || !c_sum_dev || (g->nx > 1 && !flux_sum_dev)) return TF_ERR_ARG;
    if (coeff_f64 && !field_is_f64) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    dim3 grid(g->nx, g->batch);
    if (field_is_f64 && coeff_f64)
        k_kappa_layer_sums<double, true><<<grid, 256, 0, (cudaStream_t)stream>>>(
            static_cast<const double*>(field_dev), kappa_split_dev, flux_sum_dev, c_sum_dev, geo);
    else if (field_is_f64)
        k_kappa_layer_sums<double, false><<<grid, 256, 0, (cudaStream_t)stream>>>(
            static_cast<const double*>(field_dev), kappa_split_dev, flux_sum_dev, c_sum_dev, geo);
    else
        k_kappa_layer_sums<float, false><<<grid, 256, 0, (cudaStream_t)stream>>>(
            static_cast<const float*>(field_dev), kappa_split_dev, flux_sum_dev, c_sum_dev, geo);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_residual_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                          const float* kappa_split_dev, const double* b64_dev, int coeff_f64, float* rhs_dev,
                          double* r2_sum_dev, double* b2_sum_dev, void* stream) {
    if (!g || !op || !field64_dev || !kappa_split_dev || !rhs_dev || !r2_sum_dev || !b2_sum_dev) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const dim3 grid(g->nx, g->batch);
    if (coeff_f64)
        k_kappa_residual<true><<<grid, 256, 0, (cudaStream_t)stream>>>(
            field64_dev, kappa_split_dev, b64_dev, rhs_dev, r2_sum_dev, b2_sum_dev, geo, op->ghost_lo, op->ghost_hi);
    else
        k_kappa_residual<false><<<grid, 256, 0, (cudaStream_t)stream>>>(
            field64_dev, kappa_split_dev, b64_dev, rhs_dev, r2_sum_dev, b2_sum_dev, geo, op->ghost_lo, op->ghost_hi);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    return op->periodic ? refresh_ghosts(*g, op->periodic, rhs_dev, (cudaStream_t)stream) : TF_OK;
}

int tf_kappa_adjoint_rhs(const tf_geom* g, const float* kappa_split_dev, double* out64_dev, double scale,
                         int coeff_f64, void* stream) {
    if (!g || !kappa_split_dev || !out64_dev) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const long long n = (long long)g->nx * g->ny * g->nz;
    const dim3 grid((unsigned)((n + 255) / 256), g->batch);
    if (coeff_f64)
        k_kappa_dJdc<true><<<grid, 256, 0, (cudaStream_t)stream>>>(kappa_split_dev, out64_dev, geo, scale);
    else
        k_kappa_dJdc<false><<<grid, 256, 0, (cudaStream_t)stream>>>(kappa_split_dev, out64_dev, geo, scale);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_gradient(const tf_geom* g, const tf_operator* op, const double* field64_dev, const double* lambda64_dev,
                      const float* kappa_split_dev, double* grad_dev, double scale, double bc_lo, double bc_hi,
                      void* stream) {
    if (!g || !op || !field64_dev || !lambda64_dev || !kappa_split_dev || !grad_dev) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const long long n = (long long)g->nx * g->ny * g->nz;
    k_kappa_grad<<<dim3((unsigned)((n + 255) / 256), g->batch), 256, 0, (cudaStream_t)stream>>>(
        field64_dev, lambda64_dev, kappa_split_dev, grad_dev, geo, op->periodic, scale, bc_lo, bc_hi);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_split_to_natural_f64(const tf_geom* g, const double* split_dev, double* natural_dev, void* stream) {
    if (!g || !split_dev || !natural_dev) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const long long n = (long long)g->nx * g->ny * g->nz;
    k_split_to_natural<<<dim3((unsigned)((n + 255) / 256), g->batch), 256, 0, (cudaStream_t)stream>>>(
        split_dev, natural_dev, geo);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_faces_f64(const tf_geom* g, const float* kappa_split_dev, double* fx_dev, double* fy_dev, double* fz_dev,
                       double* div_dev, void* stream) {
    if (!g || !kappa_split_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev) return TF_ERR_ARG;
    if ((long long)g->batch * g->nx > 65535 || g->yp > 65535) return TF_ERR_UNSUPPORTED;
    const Geo geo = make_geo(*g);
    dim3 grid((2 * g->zh + 127) / 128, g->yp, g->batch * g->nx);
    k_kappa_face_pack64<<<grid, 128, 0, (cudaStream_t)stream>>>(kappa_split_dev, fx_dev, fy_dev, fz_dev, div_dev, geo);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    k_kappa_diag64<<<grid, 128, 0, (cudaStream_t)stream>>>(fx_dev, fy_dev, fz_dev, div_dev, geo);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_residual_faces_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                                const double* fx_dev, const double* fy_dev, const double* fz_dev,
                                const double* div_dev, const double* b64_dev, float* rhs_dev, double* r2_sum_dev,
                                double* b2_sum_dev, void* stream) {
    if (!g || !op || !field64_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev || !rhs_dev || !r2_sum_dev ||
        !b2_sum_dev)
        return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    k_kappa_residual_p64<<<dim3(g->nx, g->batch), 1024, 0, (cudaStream_t)stream>>>(
        field64_dev, fx_dev, fy_dev, fz_dev, div_dev, b64_dev, rhs_dev, r2_sum_dev, b2_sum_dev, geo, op->ghost_lo,
        op->ghost_hi);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    return op->periodic ? refresh_ghosts(*g, op->periodic, rhs_dev, (cudaStream_t)stream) : TF_OK;
}

int tf_kappa_layer_sums_faces_f64(const tf_geom* g, const double* field64_dev, const double* fx_dev,
                                  double* flux_sum_dev, double* c_sum_dev, void* stream) {
    if (!g || !field64_dev || !fx_dev || !c_sum_dev || (g->nx > 1 && !flux_sum_dev)) return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    k_kappa_layer_sums_p64<<<dim3(g->nx, g->batch), 1024, 0, (cudaStream_t)stream>>>(field64_dev, fx_dev,
                                                                                     flux_sum_dev, c_sum_dev, geo);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_kappa_gradient_faces_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                                const double* lambda64_dev, const float* kappa_split_dev, const double* fx_dev,
                                const double* fy_dev, const double* fz_dev, double* grad_dev, double scale,
                                double bc_lo, double bc_hi, void* stream) {
    if (!g || !op || !field64_dev || !lambda64_dev || !kappa_split_dev || !fx_dev || !fy_dev || !fz_dev || !grad_dev)
        return TF_ERR_ARG;
    const Geo geo = make_geo(*g);
    const long long n = (long long)g->nx * g->ny * g->nz;
    const dim3 grid((unsigned)((n + 255) / 256), g->batch);
    k_kappa_grad_p64<<<grid, 256, 0, (cudaStream_t)stream>>>(field64_dev, lambda64_dev, kappa_split_dev, fx_dev,
                                                             fy_dev, fz_dev, grad_dev, geo, op->periodic, scale, bc_lo,
                                                             bc_hi);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

}  // extern "C"
