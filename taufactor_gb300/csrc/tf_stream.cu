// Dispatch of the register-streaming sweep to its per-operator translation units.
#include "tf_internal.h"

namespace tf {

int sweep_tiled_bin(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, const float*, int, int,
                    int32_t*, cudaStream_t);
int sweep_tiled_aniso(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, const float*, int, int,
                      int32_t*, cudaStream_t);
int sweep_tiled_mp(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, const float*, int, int,
                   int32_t*, cudaStream_t);
int sweep_tiled_electrode(const tf_geom&, const tf_operator&, const float*, float*, const uint8_t*, const float*, int,
                          int, int32_t*, cudaStream_t);

int sweep_tiled(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                const float* rhs, int first_colour, int n_half, int32_t* err, cudaStream_t st) {
    switch (op.kind) {
        case TF_KIND_BINARY: return sweep_tiled_bin(g, op, in, out, code, rhs, first_colour, n_half, err, st);
        case TF_KIND_ANISOTROPIC: return sweep_tiled_aniso(g, op, in, out, code, rhs, first_colour, n_half, err, st);
        case TF_KIND_MULTIPHASE: return sweep_tiled_mp(g, op, in, out, code, rhs, first_colour, n_half, err, st);
        case TF_KIND_ELECTRODE:
            return sweep_tiled_electrode(g, op, in, out, code, rhs, first_colour, n_half, err, st);
    }
    return TF_ERR_ARG;
}

}  // namespace tf
