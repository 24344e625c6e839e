// extern "C" entry points of libtaufactor_gb300 (declared in include/taufactor_gb300.h).
#include <atomic>
#include <cmath>
#include <mutex>

#include "tf_common.cuh"
#include "tf_internal.h"

namespace tf {

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int sm_count() {
    constexpr int MAX_DEVICES = 64;
    static std::atomic<int> cached[MAX_DEVICES];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return 1;
    int n = cached[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 1;
        cached[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

int encode_map_3d(CUtensorMap* map, const void* base, int elem_bytes, long long dim0, long long dim1,
                  long long dim2, long long stride1_bytes, long long stride2_bytes, int box0, int box1) {
    EncodeTiledFn enc = get_encode();
    if (!enc) return TF_ERR_CUDA;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (stride1_bytes & 15) || (stride2_bytes & 15) ||
        ((long long)box0 * elem_bytes) % 16)
        return TF_ERR_ARG;
    const cuuint64_t dims[3] = {(cuuint64_t)dim0, (cuuint64_t)dim1, (cuuint64_t)dim2};
    const cuuint64_t strides[2] = {(cuuint64_t)stride1_bytes, (cuuint64_t)stride2_bytes};
    const cuuint32_t box[3] = {(cuuint32_t)box0, (cuuint32_t)box1, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType dt = elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    const CUresult r = enc(map, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? TF_OK : TF_ERR_CUDA;
}

static bool valid_geom(const tf_geom* g) {
    return g && g->batch > 0 && g->nx > 0 && g->ny > 0 && g->nz > 0 && g->halo_y == HY && g->halo_j == HJ &&
           g->yp == g->ny + 2 * HY && g->zh % 4 == 0 && g->zh >= (g->nz + 1) / 2 + 2 * HJ && g->zhc % 16 == 0 &&
           g->zhc >= g->zh;
}

static bool valid_op(const tf_operator* op) {
    if (!op) return false;
    if (op->kind < TF_KIND_BINARY || op->kind > TF_KIND_ELECTRODE) return false;
    if (op->periodic & ~(TF_PERIODIC_Y | TF_PERIODIC_Z)) return false;
    if (op->kind == TF_KIND_MULTIPHASE && (op->n_phases < 1 || op->n_phases > TF_MAX_PHASES)) return false;
    return std::isfinite(op->omega);
}

}  // namespace tf

using namespace tf;

extern "C" {

const char* tf_version(void) { return "taufactor_gb300 0.1.0 (sm_103a)"; }

const char* tf_status_string(int s) {
    switch (s) {
        case TF_OK: return "ok";
        case TF_ERR_ARG: return "invalid argument";
        case TF_ERR_CUDA: return "CUDA error";
        case TF_ERR_TIMEOUT: return "device wait timed out";
        case TF_ERR_UNSUPPORTED: return "unsupported";
        case TF_ERR_NOTCONV: return "not converged";
    }
    return "unknown status";
}

int64_t tf_launch_count(void) { return g_launches.load(); }

int tf_geometry(int batch, int nx, int ny, int nz, int periodic, tf_geom* out) {
    if (!out || batch <= 0 || nx <= 0 || ny <= 0 || nz <= 0) return TF_ERR_ARG;
    if ((long long)ny + 2 * HY > (1LL << 30) || nz > (1 << 30)) return TF_ERR_ARG;
    tf_geom g{};
    g.batch = batch; g.nx = nx; g.ny = ny; g.nz = nz;
    g.halo_y = HY; g.halo_j = HJ;
    g.yp = ny + 2 * HY;
    g.zh = ((nz + 1) / 2 + 2 * HJ + 3) / 4 * 4;
    g.zhc = (g.zh + 15) / 16 * 16;
    g.field_elems = (long long)batch * nx * g.yp * 2 * g.zh;
    g.code_bytes = (long long)batch * nx * g.yp * 2 * g.zhc;
    // the tiled kernel keeps periodic ghost bands by single-wrap copies of even-sized faces
    bool tiled = true;
    if ((periodic & TF_PERIODIC_Y) && (ny % 2 || ny < 2 * HY)) tiled = false;
    if ((periodic & TF_PERIODIC_Z) && (nz % 2 || nz < 4 * HJ)) tiled = false;
    if ((long long)batch * nx > (1LL << 31) - 1) tiled = false;
    g.tiled = tiled ? 1 : 0;
    *out = g;
    return TF_OK;
}

int tf_pack(const tf_geom* g, const tf_operator* op, const uint8_t* phase_dev, const float* profile_dev,
            uint8_t* code_dev, float* field_dev, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !phase_dev || !profile_dev || !code_dev || !field_dev) return TF_ERR_ARG;
    return pack(*g, *op, phase_dev, profile_dev, code_dev, field_dev, (cudaStream_t)stream);
}

static int advance_impl(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
                        const uint8_t* code_dev, const float* rhs_dev, int first_colour, int n_half, int32_t* err_dev,
                        int* result_in_b, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field_a_dev || !field_b_dev || !code_dev || !result_in_b || n_half < 0 ||
        field_a_dev == field_b_dev)
        return TF_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(field_a_dev) | reinterpret_cast<uintptr_t>(field_b_dev)) & 15)
        return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const bool tiled = g->tiled && !((op->periodic & TF_PERIODIC_Y) && (g->ny % 2 || g->ny < 2 * HY)) &&
                       !((op->periodic & TF_PERIODIC_Z) && (g->nz % 2 || g->nz < 4 * HJ));
    int colour = first_colour & 1;
    if (!tiled) {
        for (int i = 0; i < n_half; ++i, colour ^= 1) {
            const int rc = sweep_plain(*g, *op, field_a_dev, code_dev, rhs_dev, colour, st);
            if (rc) return rc;
        }
        *result_in_b = 0;
        return TF_OK;
    }
    float* in = field_a_dev;
    float* out = field_b_dev;
    int in_b = 0;
    int left = n_half;
    const int kmax = (op->k_max >= 1 && op->k_max <= HY) ? op->k_max : HY;
    while (left > 0) {
        const int nh = left < kmax ? left : kmax;
        const int rc = sweep_tiled(*g, *op, in, out, code_dev, rhs_dev, colour, nh, err_dev, st);
        if (rc) return rc;
        colour ^= (nh & 1);
        left -= nh;
        float* t = in; in = out; out = t;
        in_b ^= 1;
    }
    *result_in_b = in_b;
    return TF_OK;
}

int tf_advance(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
               const uint8_t* code_dev, int first_colour, int n_half, int32_t* err_dev, int* result_in_b,
               void* stream) {
    return advance_impl(g, op, field_a_dev, field_b_dev, code_dev, nullptr, first_colour, n_half, err_dev,
                        result_in_b, stream);
}

int tf_advance_rhs(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
                   const uint8_t* code_dev, const float* rhs_dev, int first_colour, int n_half, int32_t* err_dev,
                   int* result_in_b, void* stream) {
    if (!rhs_dev || (reinterpret_cast<uintptr_t>(rhs_dev) & 15)) return TF_ERR_ARG;
    return advance_impl(g, op, field_a_dev, field_b_dev, code_dev, rhs_dev, first_colour, n_half, err_dev,
                        result_in_b, stream);
}

int tf_widen_f64(const tf_geom* g, const float* field_dev, double* field64_dev, void* stream) {
    if (!valid_geom(g) || !field_dev || !field64_dev) return TF_ERR_ARG;
    return widen(*g, field_dev, field64_dev, (cudaStream_t)stream);
}

int tf_narrow_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev, float* field_dev,
                  void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field_dev || !field64_dev) return TF_ERR_ARG;
    return narrow(*g, *op, field64_dev, field_dev, (cudaStream_t)stream);
}

int tf_axpy_f64(const tf_geom* g, double* field64_dev, const float* e_dev, void* stream) {
    if (!valid_geom(g) || !field64_dev || !e_dev) return TF_ERR_ARG;
    return axpy(*g, field64_dev, e_dev, (cudaStream_t)stream);
}

int tf_residual_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev, const uint8_t* code_dev,
                    float* rhs_dev, double* r2_sum_dev, double* b2_sum_dev, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field64_dev || !code_dev || !rhs_dev || !r2_sum_dev || !b2_sum_dev)
        return TF_ERR_ARG;
    return residual(*g, *op, field64_dev, code_dev, rhs_dev, r2_sum_dev, b2_sum_dev, (cudaStream_t)stream);
}

int tf_layer_sums_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev, const uint8_t* code_dev,
                      double* flux_sum_dev, double* c_sum_dev, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field64_dev || !code_dev || !c_sum_dev || (g->nx > 1 && !flux_sum_dev))
        return TF_ERR_ARG;
    return layer_sums_f64(*g, *op, field64_dev, code_dev, flux_sum_dev, c_sum_dev, (cudaStream_t)stream);
}

int tf_layer_sums(const tf_geom* g, const tf_operator* op, const float* field_dev, const uint8_t* code_dev,
                  double* flux_sum_dev, double* c_sum_dev, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field_dev || !code_dev || !c_sum_dev || (g->nx > 1 && !flux_sum_dev))
        return TF_ERR_ARG;
    return layer_sums(*g, *op, field_dev, code_dev, flux_sum_dev, c_sum_dev, (cudaStream_t)stream);
}

int tf_unpack(const tf_geom* g, const tf_operator* op, const float* field_dev, float* padded_dev, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field_dev || !padded_dev) return TF_ERR_ARG;
    return unpack(*g, *op, field_dev, padded_dev, (cudaStream_t)stream);
}

int tf_repack(const tf_geom* g, const tf_operator* op, const float* padded_dev, float* field_dev, void* stream) {
    if (!valid_geom(g) || !valid_op(op) || !field_dev || !padded_dev) return TF_ERR_ARG;
    return repack(*g, *op, padded_dev, field_dev, (cudaStream_t)stream);
}

int tf_check_small_division(int n, uint64_t* bad_dev, void* stream) {
    if (n < 1 || n > 8 || !bad_dev) return TF_ERR_ARG;
    return check_small_division(n, reinterpret_cast<unsigned long long*>(bad_dev), (cudaStream_t)stream);
}

}  // extern "C"
