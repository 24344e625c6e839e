// Impedance (tau_e) solve on the device (sm_103a): ImpedanceSolver / PeriodicImpedanceSolver of
// taufactor/electrode.py:160-402.
//
// The field is complex128 in the reference's padded layout [F][nx+2][ny+2][nz+2] (interleaved
// re, im), one slice per frequency, so the Python side hands out the tensor itself. One thread
// updates one voxel of the half-sweep's colour: the six face neighbours summed left to right in
// the reference's order (x+1, x-1, y+1, y-1, z+1, z-1), the complex product with the voxel's
// factor 1 / (nn + i frc nr) from a per-frequency table, minus the voxel, times omega, added
// back; every operation is one IEEE rounding with no contraction (__d*_rn), as the reference's
// vectorised loops do. FP64 work is the bound on GB300 (22 double operations per voxel-update;
// 10 to 32 bytes of memory traffic per update, well below HBM bandwidth at that rate).
#include "tf_common.cuh"
#include "tf_internal.h"

namespace tf {

constexpr int IMP_TABLE = TF_IMP_TABLE;

struct ImpDims {
    int nx, ny, nz;
    long long sy, sx, sf;  // padded strides (z stride 1)
};

__host__ __device__ inline ImpDims imp_dims(int nx, int ny, int nz) {
    ImpDims d;
    d.nx = nx;
    d.ny = ny;
    d.nz = nz;
    d.sy = nz + 2;
    d.sx = (long long)(ny + 2) * (nz + 2);
    d.sf = (long long)(nx + 2) * d.sx;
    return d;
}

// code = 0 outside the conductive phase, else 0x80 | (nn + 8 nr); phase bit 0 = conductive,
// bit 1 = reactive. nn counts the inlet ghost (x = -1) twice and the outlet ghost not at all.
__global__ void k_imp_pack(const uint8_t* __restrict__ phase, ImpDims d, int periodic, uint8_t* __restrict__ code,
                           unsigned long long* __restrict__ counts) {
    const long long n = (long long)d.nx * d.ny * d.nz;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(v % d.nz);
        const int y = (int)((v / d.nz) % d.ny);
        const int x = (int)(v / ((long long)d.nz * d.ny));
        const long long pl = (long long)d.ny * d.nz;
        if (!(phase[v] & 1)) {
            code[v] = 0;
            continue;
        }
        int nn = 0, nr = 0;
        auto add = [&](long long w) {
            const uint8_t p = phase[w];
            nn += p & 1;
            nr += (p >> 1) & 1;
        };
        if (x + 1 < d.nx) add(v + pl);
        if (x > 0) add(v - pl);
        else nn += 2;
        if (y + 1 < d.ny) add(v + d.nz);
        else if (periodic) add(v - (long long)(d.ny - 1) * d.nz);
        if (y > 0) add(v - d.nz);
        else if (periodic) add(v + (long long)(d.ny - 1) * d.nz);
        if (z + 1 < d.nz) add(v + 1);
        else if (periodic) add(v - (d.nz - 1));
        if (z > 0) add(v - 1);
        else if (periodic) add(v + (d.nz - 1));
        code[v] = (uint8_t)(0x80 | (nn + 8 * nr));
        atomicAdd(&counts[2 * x], 1ull);
        if (nr) atomicAdd(&counts[2 * x + 1], (unsigned long long)nr);
    }
}

// electrode.py:214-233: mask * phi[f][x] inside, 2 left_bc on the inlet ghost plane's interior,
// 0 on every other ghost.
__global__ void k_imp_fill(ImpDims d, int F, const uint8_t* __restrict__ code, const double2* __restrict__ phi,
                           double ghost_lo, double2* __restrict__ field) {
    const long long n = (long long)F * d.sf;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(i / d.sf);
        const long long r = i - f * d.sf;
        const int xp = (int)(r / d.sx);
        const int yp = (int)((r / d.sy) % (d.ny + 2));
        const int zp = (int)(r % d.sy);
        double2 v = make_double2(0.0, 0.0);
        const bool yz_in = yp >= 1 && yp <= d.ny && zp >= 1 && zp <= d.nz;
        if (yz_in && xp == 0) {
            v.x = ghost_lo;
        } else if (yz_in && xp >= 1 && xp <= d.nx) {
            const long long vox = ((long long)(xp - 1) * d.ny + (yp - 1)) * d.nz + (zp - 1);
            if (code[vox] & 0x80) v = phi[(long long)f * d.nx + (xp - 1)];
        }
        field[i] = v;
    }
}

// electrode.py:398-402 composed: every y/z ghost cell of every x plane (ghost planes included)
// takes the interior cell it ends up copying, (x, wy(y), wz(z)) with wy(0) = ny, wy(ny+1) = 1.
__global__ void k_imp_ghosts(ImpDims d, int F, double2* __restrict__ field) {
    const int per_plane = 2 * (d.nz + 2) + 2 * d.ny;
    const long long n = (long long)F * (d.nx + 2) * per_plane;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long plane = i / per_plane;  // f * (nx + 2) + xp
        int g = (int)(i - plane * per_plane);
        int y, z;
        if (g < d.nz + 2) {
            y = 0;
            z = g;
        } else if (g < 2 * (d.nz + 2)) {
            y = d.ny + 1;
            z = g - (d.nz + 2);
        } else {
            g -= 2 * (d.nz + 2);
            y = 1 + (g >> 1);
            z = (g & 1) ? d.nz + 1 : 0;
        }
        const int wy = y == 0 ? d.ny : (y == d.ny + 1 ? 1 : y);
        const int wz = z == 0 ? d.nz : (z == d.nz + 1 ? 1 : z);
        const long long base = plane * d.sx;
        field[base + y * d.sy + z] = field[base + wy * d.sy + wz];
    }
}

// One half-sweep of colour `parity` ((x + y + z) % 2 == parity, interior coordinates) for every
// active frequency. Threads cover (zh, y) of a plane with z = 2 zh + ((x + y + parity) & 1);
// blockIdx.z walks the (f, x) planes.
__global__ void __launch_bounds__(256) k_imp_sweep(ImpDims d, int F, int hz, double2* __restrict__ field,
                                                    const uint8_t* __restrict__ code,
                                                    const double2* __restrict__ table,
                                                    const uint8_t* __restrict__ active, int parity, double omega) {
    const int zh = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (zh >= hz || y >= d.ny) return;
    const int planes = F * d.nx;
    for (int fx = blockIdx.z; fx < planes; fx += gridDim.z) {
        const int f = fx / d.nx;
        const int x = fx - f * d.nx;
        if (active && !active[f]) continue;
        const int z = 2 * zh + ((x + y + parity) & 1);
        if (z >= d.nz) continue;
        const long long p = f * d.sf + (x + 1) * d.sx + (y + 1) * d.sy + (z + 1);
        const double2 xp = field[p + d.sx], xm = field[p - d.sx];
        const double2 yp = field[p + d.sy], ym = field[p - d.sy];
        const double2 zp = field[p + 1], zm = field[p - 1];
        double sr = __dadd_rn(xp.x, xm.x), si = __dadd_rn(xp.y, xm.y);
        sr = __dadd_rn(sr, yp.x);
        si = __dadd_rn(si, yp.y);
        sr = __dadd_rn(sr, ym.x);
        si = __dadd_rn(si, ym.y);
        sr = __dadd_rn(sr, zp.x);
        si = __dadd_rn(si, zp.y);
        sr = __dadd_rn(sr, zm.x);
        si = __dadd_rn(si, zm.y);
        const double2 fac = __ldg(&table[f * IMP_TABLE + (code[((long long)x * d.ny + y) * d.nz + z] & 0x7f)]);
        double ir = __dsub_rn(__dmul_rn(sr, fac.x), __dmul_rn(si, fac.y));
        double ii = __dadd_rn(__dmul_rn(sr, fac.y), __dmul_rn(si, fac.x));
        const double2 c = field[p];
        ir = __dmul_rn(__dsub_rn(ir, c.x), omega);
        ii = __dmul_rn(__dsub_rn(ii, c.y), omega);
        field[p] = make_double2(__dadd_rn(c.x, ir), __dadd_rn(c.y, ii));
    }
}

// Per (f, x) plane: sum of |c| over the interior (electrode.py:381), and on plane 0 the sums of
// the inlet flux 2 left_bc - 2 c (0 where c == 0; :326-328); NaN cells per frequency (:293).
__global__ void __launch_bounds__(256) k_imp_metrics(ImpDims d, const double2* __restrict__ field, double left_bc,
                                                      double* __restrict__ abs_sum, double* __restrict__ influx,
                                                      int32_t* __restrict__ nan_count) {
    const int x = blockIdx.x;
    const int f = blockIdx.y;
    const int pl = d.ny * d.nz;
    const double2* base = field + f * d.sf + (x + 1) * d.sx;
    double a = 0.0, qr = 0.0, qi = 0.0;
    int nans = 0;
    for (int k = threadIdx.x; k < pl; k += blockDim.x) {
        const int y = k / d.nz, z = k - (k / d.nz) * d.nz;
        const double2 c = base[(y + 1) * d.sy + (z + 1)];
        a += hypot(c.x, c.y);
        nans += (isnan(c.x) || isnan(c.y)) ? 1 : 0;
        if (x == 0 && !(c.x == 0.0 && c.y == 0.0)) {
            // (2 + 0i) c as a complex product, then (2 left_bc + 0i) minus it
            const double tr = __dsub_rn(__dmul_rn(c.x, 2.0), __dmul_rn(c.y, 0.0));
            const double ti = __dadd_rn(__dmul_rn(c.x, 0.0), __dmul_rn(c.y, 2.0));
            qr += __dsub_rn(2.0 * left_bc, tr);
            qi += __dsub_rn(0.0, ti);
        }
    }
    __shared__ double s_a[8], s_r[8], s_i[8];
    __shared__ int s_n[8];
    for (int o = 16; o; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        qr += __shfl_down_sync(0xffffffffu, qr, o);
        qi += __shfl_down_sync(0xffffffffu, qi, o);
        nans += __shfl_down_sync(0xffffffffu, nans, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_a[w] = a;
        s_r[w] = qr;
        s_i[w] = qi;
        s_n[w] = nans;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        double ta = 0.0, tr = 0.0, ti = 0.0;
        int tn = 0;
        for (int i = 0; i < nw; ++i) {
            ta += s_a[i];
            tr += s_r[i];
            ti += s_i[i];
            tn += s_n[i];
        }
        abs_sum[(long long)f * d.nx + x] = ta;
        if (x == 0) {
            influx[2 * f] = tr;
            influx[2 * f + 1] = ti;
        }
        if (tn) atomicAdd(&nan_count[f], tn);
    }
}

static unsigned grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    const long long cap = (long long)sm_count() * 16;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

static bool dims_ok(int n_freq, int nx, int ny, int nz) {
    if (n_freq < 1 || nx < 1 || ny < 1 || nz < 1 || n_freq > 65535) return false;
    const long long cells = (long long)n_freq * (nx + 2) * (ny + 2) * (nz + 2);
    return cells < (1ll << 40) && (long long)n_freq * nx < (1ll << 31) &&
           (long long)(ny + 2) * (nz + 2) < (1ll << 31) && ny < (1 << 24);
}

}  // namespace tf

using namespace tf;

extern "C" int tf_impedance_pack(int nx, int ny, int nz, int periodic, const uint8_t* phase_dev, uint8_t* code_dev,
                                 uint64_t* plane_counts_dev, void* stream) {
    if (!dims_ok(1, nx, ny, nz) || !phase_dev || !code_dev || !plane_counts_dev) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const ImpDims d = imp_dims(nx, ny, nz);
    if (cudaMemsetAsync(plane_counts_dev, 0, sizeof(uint64_t) * 2 * nx, st) != cudaSuccess) return TF_ERR_CUDA;
    const long long n = (long long)nx * ny * nz;
    k_imp_pack<<<grid_for(n, 256), 256, 0, st>>>(phase_dev, d, periodic ? 1 : 0, code_dev,
                                                 (unsigned long long*)plane_counts_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

extern "C" int tf_impedance_fill(int n_freq, int nx, int ny, int nz, const uint8_t* code_dev, const double* phi_dev,
                                 double ghost_lo, double* field_dev, void* stream) {
    if (!dims_ok(n_freq, nx, ny, nz) || !code_dev || !phi_dev || !field_dev) return TF_ERR_ARG;
    if (((uintptr_t)field_dev | (uintptr_t)phi_dev) & 15) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const ImpDims d = imp_dims(nx, ny, nz);
    k_imp_fill<<<grid_for((long long)n_freq * d.sf, 256), 256, 0, st>>>(d, n_freq, code_dev, (const double2*)phi_dev,
                                                                         ghost_lo, (double2*)field_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

extern "C" int tf_impedance_sweep(int n_freq, int nx, int ny, int nz, int periodic, double* field_dev,
                                  const uint8_t* code_dev, const double* table_dev, const uint8_t* active_dev,
                                  double omega, int first_iter, int n_half, void* stream) {
    if (!dims_ok(n_freq, nx, ny, nz) || !field_dev || !code_dev || !table_dev || n_half < 0 || first_iter < 0)
        return TF_ERR_ARG;
    if (((uintptr_t)field_dev | (uintptr_t)table_dev) & 15) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const ImpDims d = imp_dims(nx, ny, nz);
    const int hz = (nz + 1) / 2;
    int bx = 1;
    while (bx < hz && bx < 64) bx <<= 1;
    const dim3 block(bx, 256 / bx);
    if ((ny + (int)block.y - 1) / (int)block.y > 65535) return TF_ERR_UNSUPPORTED;
    const long long planes = (long long)n_freq * nx;
    const dim3 grid((hz + bx - 1) / bx, (ny + block.y - 1) / block.y, (unsigned)(planes < 65535 ? planes : 65535));
    const int per_plane = 2 * (nz + 2) + 2 * ny;
    const unsigned gg = grid_for((long long)n_freq * (nx + 2) * per_plane, 256);
    for (int s = 0; s < n_half; ++s) {
        if (periodic) {
            k_imp_ghosts<<<gg, 256, 0, st>>>(d, n_freq, (double2*)field_dev);
            note_launch();
        }
        k_imp_sweep<<<grid, block, 0, st>>>(d, n_freq, hz, (double2*)field_dev, code_dev, (const double2*)table_dev,
                                            active_dev, (first_iter + s) & 1, omega);
        note_launch();
    }
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

extern "C" int tf_impedance_metrics(int n_freq, int nx, int ny, int nz, const double* field_dev, double left_bc,
                                    double* abs_sum_dev, double* influx_sum_dev, int32_t* nan_count_dev,
                                    void* stream) {
    if (!dims_ok(n_freq, nx, ny, nz) || !field_dev || !abs_sum_dev || !influx_sum_dev || !nan_count_dev)
        return TF_ERR_ARG;
    if ((uintptr_t)field_dev & 15) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const ImpDims d = imp_dims(nx, ny, nz);
    if (cudaMemsetAsync(nan_count_dev, 0, sizeof(int32_t) * n_freq, st) != cudaSuccess) return TF_ERR_CUDA;
    k_imp_metrics<<<dim3((unsigned)nx, (unsigned)n_freq), 256, 0, st>>>(d, (const double2*)field_dev, left_bc,
                                                                        abs_sum_dev, influx_sum_dev, nan_count_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}
