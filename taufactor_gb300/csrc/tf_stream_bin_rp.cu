// Instantiations of the row-pair sweep (tf_stream_rp.cuh) for TF_KIND_BINARY, tile shape 3
// (16 rows x 128 z-cells), 2 or 4 half-sweeps per launch.
#include "tf_stream_rp.cuh"

namespace tf {

int sweep_tiled_bin_rp(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                       int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    switch (n_half) {
        case 2: return launch_stream_rp<16, 128, 2>(g, op, in, out, code, first_colour, err, st);
        case 4: return launch_stream_rp<16, 128, 4>(g, op, in, out, code, first_colour, err, st);
    }
    return TF_ERR_ARG;
}

}  // namespace tf
