// Instantiations of the register-streaming sweep (tf_stream.cuh) for TF_KIND_BINARY, tile shape
// 1 (16 rows x 128 z-cells), 2..4 half-sweeps per launch.
#include "tf_stream.cuh"

namespace tf {

int sweep_tiled_bin_t1(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                       int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    return dispatch_k234<16, 128>(g, op, in, out, code, first_colour, n_half, err, st);
}

}  // namespace tf
