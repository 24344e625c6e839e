// Instantiations of the register-streaming sweep (tf_stream.cuh) for KIND_FACES, the operator
// given as packed per-voxel faces and factor (tf_kappa_faces), tile shape 16 rows x 64 z-cells,
// 1..4 half-sweeps per launch, with and without a right-hand side; and its C ABI entry point.
// K fused half-sweeps give the bits of K tf_kappa_advance_faces half-sweeps.
#include "tf_stream.cuh"

namespace tf {

template <int K>
static int launch_faces(const tf_geom& g, const tf_operator& op, const float* in, float* out,
                        const float* const* faces, const float* rhs, int first_colour, int32_t* err, cudaStream_t st) {
    const uint8_t* no_codes = reinterpret_cast<const uint8_t*>(in);  // not read by this kind
    if (rhs)
        return launch_stream<KIND_FACES, 16, 64, K, true>(g, op, in, out, no_codes, rhs, first_colour, err, st, faces);
    return launch_stream<KIND_FACES, 16, 64, K, false>(g, op, in, out, no_codes, nullptr, first_colour, err, st,
                                                       faces);
}

static int sweep_tiled_faces(const tf_geom& g, const tf_operator& op, const float* in, float* out,
                             const float* const* faces, const float* rhs, int first_colour, int n_half, int32_t* err,
                             cudaStream_t st) {
    switch (n_half) {
        case 1: return launch_faces<1>(g, op, in, out, faces, rhs, first_colour, err, st);
        case 2: return launch_faces<2>(g, op, in, out, faces, rhs, first_colour, err, st);
        case 3: return launch_faces<3>(g, op, in, out, faces, rhs, first_colour, err, st);
        case 4: return launch_faces<4>(g, op, in, out, faces, rhs, first_colour, err, st);
    }
    return TF_ERR_ARG;
}

}  // namespace tf

using namespace tf;

extern "C" int tf_kappa_advance_fused(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
                                      const float* fx_dev, const float* fy_dev, const float* fz_dev,
                                      const float* div_dev, const float* rhs_dev, int first_colour, int n_half,
                                      int32_t* err_dev, int* result_in_b, void* stream) {
    if (!g || !op || !field_a_dev || !field_b_dev || !fx_dev || !fy_dev || !fz_dev || !div_dev || !result_in_b ||
        n_half < 0 || field_a_dev == field_b_dev)
        return TF_ERR_ARG;
    const uintptr_t al = reinterpret_cast<uintptr_t>(field_a_dev) | reinterpret_cast<uintptr_t>(field_b_dev) |
                         reinterpret_cast<uintptr_t>(fx_dev) | reinterpret_cast<uintptr_t>(fy_dev) |
                         reinterpret_cast<uintptr_t>(fz_dev) | reinterpret_cast<uintptr_t>(div_dev) |
                         reinterpret_cast<uintptr_t>(rhs_dev);
    if (al & 15) return TF_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    // the shapes the tiled kernel keeps periodic ghost bands for (as tf_advance); otherwise the
    // packed-face half-sweeps in place on field A
    const bool tiled = g->tiled && !((op->periodic & TF_PERIODIC_Y) && (g->ny % 2 || g->ny < 2 * HY)) &&
                       !((op->periodic & TF_PERIODIC_Z) && (g->nz % 2 || g->nz < 4 * HJ));
    if (!tiled) {
        *result_in_b = 0;
        return tf_kappa_advance_faces(g, op, field_a_dev, fx_dev, fy_dev, fz_dev, div_dev, rhs_dev, first_colour,
                                      n_half, stream);
    }
    const float* faces[4] = {fx_dev, fy_dev, fz_dev, div_dev};
    float* in = field_a_dev;
    float* out = field_b_dev;
    int in_b = 0, colour = first_colour & 1, left = n_half;
    const int kmax = (op->k_max >= 1 && op->k_max <= HY) ? op->k_max : HY;
    while (left > 0) {
        const int nh = left < kmax ? left : kmax;
        const int rc = sweep_tiled_faces(*g, *op, in, out, faces, rhs_dev, colour, nh, err_dev, st);
        if (rc) return rc;
        colour ^= (nh & 1);
        left -= nh;
        float* t = in;
        in = out;
        out = t;
        in_b ^= 1;
    }
    *result_in_b = in_b;
    return TF_OK;
}

extern "C" int tf_refresh_ghosts(const tf_geom* g, int periodic, float* field_dev, void* stream) {
    if (!g || !field_dev) return TF_ERR_ARG;
    if ((long long)g->batch * g->nx > 65535 || g->yp > 65535) return TF_ERR_UNSUPPORTED;
    if (!(periodic & (TF_PERIODIC_Y | TF_PERIODIC_Z))) return TF_OK;
    return refresh_ghosts(*g, periodic, field_dev, (cudaStream_t)stream);
}
