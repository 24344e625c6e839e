// Instantiations of the register-streaming sweep (tf_stream.cuh) for TF_KIND_ELECTRODE.
#include "tf_stream.cuh"

namespace tf {

int sweep_tiled_electrode(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                          const float* rhs, int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    return dispatch_kind<TF_KIND_ELECTRODE>(g, op, in, out, code, rhs, first_colour, n_half, err, st);
}

}  // namespace tf
