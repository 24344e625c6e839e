// Instantiations of the register-streaming sweep (tf_stream.cuh) for TF_KIND_BINARY, tile shape
// 0 (16x64; also every single half-sweep and every correction solve), and the dispatch to the
// other shapes' translation units. Shape 3 (row pairs, tf_stream_rp.cuh) fuses an even number of
// half-sweeps; an odd count on it runs on shape 1.
#include "tf_stream.cuh"

namespace tf {

int sweep_tiled_bin_t1(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, int, int, int32_t*,
                       cudaStream_t);
int sweep_tiled_bin_t2(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, int, int, int32_t*,
                       cudaStream_t);
int sweep_tiled_bin_rp(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, int, int, int32_t*,
                       cudaStream_t);

int sweep_tiled_bin(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                    const float* rhs, int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    if (!rhs && op.tile == 3 && (n_half == 2 || n_half == 4))
        return sweep_tiled_bin_rp(g, op, in, out, code, first_colour, n_half, err, st);
    if (!rhs && n_half >= 2 && (op.tile == 1 || op.tile == 3)) return sweep_tiled_bin_t1(g, op, in, out, code, first_colour, n_half, err, st);
    if (!rhs && n_half >= 2 && op.tile == 2) return sweep_tiled_bin_t2(g, op, in, out, code, first_colour, n_half, err, st);
    return dispatch_kind<TF_KIND_BINARY>(g, op, in, out, code, rhs, first_colour, n_half, err, st);
}

}  // namespace tf
