// Internal host-side interface between the translation units of libtaufactor_gb300.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/taufactor_gb300.h"

namespace tf {

void note_launch();

// Streaming multiprocessors of the current device (cached per device; 1 if unknown).
int sm_count();

// 3-D tiled tensor map over [dim2][dim1][dim0] with the given byte strides of dims 1 and 2.
int encode_map_3d(CUtensorMap* map, const void* base, int elem_bytes, long long dim0, long long dim1,
                  long long dim2, long long stride1_bytes, long long stride2_bytes, int box0, int box1);

// K = n_half (1..TF_MAX_HALF_SWEEPS) half-sweeps in one register-streaming launch, in -> out.
// rhs: right-hand side of a correction solve A e = r (split layout with ghost copies) or null.
int sweep_tiled(const tf_geom& g, const tf_operator& op, const float* in, float* out, const uint8_t* code,
                const float* rhs, int first_colour, int n_half, int32_t* err, cudaStream_t st);
int sweep_plain(const tf_geom& g, const tf_operator& op, float* f, const uint8_t* code, const float* rhs,
                int colour, cudaStream_t st);
int refresh_ghosts(const tf_geom& g, int periodic, float* f, cudaStream_t st);
int check_small_division(int n, unsigned long long* bad_dev, cudaStream_t st);

int pack(const tf_geom& g, const tf_operator& op, const uint8_t* phase, const float* profile, uint8_t* code,
         float* field, cudaStream_t st);
int unpack(const tf_geom& g, const tf_operator& op, const float* field, float* padded, cudaStream_t st);
int repack(const tf_geom& g, const tf_operator& op, const float* padded, float* field, cudaStream_t st);
int widen(const tf_geom& g, const float* f32, double* f64, cudaStream_t st);
int narrow(const tf_geom& g, const tf_operator& op, const double* f64, float* f32, cudaStream_t st);
int axpy(const tf_geom& g, double* c64, const float* e32, cudaStream_t st);
int residual(const tf_geom& g, const tf_operator& op, const double* c64, const uint8_t* code, float* r32, double* r2,
             double* b2, cudaStream_t st);
int layer_sums_f64(const tf_geom& g, const tf_operator& op, const double* f64, const uint8_t* code, double* flux,
                   double* csum, cudaStream_t st);
int layer_sums(const tf_geom& g, const tf_operator& op, const float* field, const uint8_t* code, double* flux,
               double* csum, cudaStream_t st);

}  // namespace tf
