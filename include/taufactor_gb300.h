/*
 * taufactor_gb300 C ABI: GB300 (sm_103a) kernels for TauFactor's steady-state voxel
 * diffusion solve (red-black over-relaxed Jacobi on the 7-point stencil).
 *
 * The reference (tldr-group/taufactor v1.2.1) is pure Python on torch eager ops and has no FFI;
 * each entry point below replaces one torch op sequence of its solve path, cited per function
 * as taufactor/taufactor.py:<lines>.
 *
 * Conventions
 *  - Every pointer argument named *_dev is device memory owned by the caller (the Python host
 *    uses torch's caching allocator). The library borrows pointers for the call and frees nothing.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default stream. All
 *    launches are asynchronous and stream-ordered; no entry point synchronises the host except
 *    where stated.
 *  - Return value: TF_OK or one of the TF_ERR_* codes; tf_status_string() names them.
 *  - Geometry: volumes of one batch share one shape. Voxel (x, y, z) of volume b lives in the
 *    "z-parity split" layout: row (b, x, y) holds the even-z half-row, then the odd-z half-row,
 *    each with `halo_j` ghost cells on both sides; rows have `halo_y` ghost rows on both y sides.
 *    Ghost cells hold 0 (closed faces) or copies of the wrapped interior (periodic faces).
 *    tf_geometry() computes the pitches and buffer sizes.
 */
#ifndef TAUFACTOR_GB300_H
#define TAUFACTOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TF_OK 0
#define TF_ERR_ARG 1         /* invalid argument (shape, pointer, alignment, sizes)        */
#define TF_ERR_CUDA 2        /* a CUDA runtime call failed                                 */
#define TF_ERR_TIMEOUT 3     /* a bounded device-side wait ran out; kernel returned early   */
#define TF_ERR_UNSUPPORTED 4 /* valid request the library does not handle                   */
#define TF_ERR_NOTCONV 5     /* iteration limit reached before convergence                  */

/* operator kinds */
#define TF_KIND_BINARY 0      /* Solver / PeriodicSolver: divisor = conductive-neighbour count  */
#define TF_KIND_ANISOTROPIC 1 /* AnisotropicSolver: y, z neighbours weighted by ky, kz          */
#define TF_KIND_MULTIPHASE 2  /* MultiPhaseSolver(s): harmonic-mean face conductances          */
#define TF_KIND_ELECTRODE 3   /* ElectrodeSolver(s): binary neighbour sum, divisor nn + k0 * nr  */

/* periodic flags */
#define TF_PERIODIC_Y 1
#define TF_PERIODIC_Z 2

#define TF_MAX_PHASES 31      /* multiphase: phase indices 1..31; index 0 = outside the volume */
#define TF_MAX_HALF_SWEEPS 4  /* half-sweeps fused into one tiled launch (= ghost rows)        */

typedef struct tf_geom {
    int32_t batch, nx, ny, nz; /* interior extents (x = transport axis)                       */
    int32_t halo_y;            /* ghost rows on each y side                                   */
    int32_t halo_j;            /* ghost cells on each side of each z-parity half-row           */
    int32_t yp;                /* rows per x-plane = ny + 2*halo_y                             */
    int32_t zh;                /* floats per half-row (multiple of 4)                          */
    int32_t zhc;               /* bytes per half-row of the code buffer (multiple of 16)       */
    int32_t tiled;             /* 1 if the tiled multi-half-sweep kernel can run this shape    */
    int64_t field_elems;       /* floats in one field buffer (whole batch)                    */
    int64_t code_bytes;        /* bytes in one code buffer (whole batch)                      */
} tf_geom;

typedef struct tf_operator {
    int32_t kind;              /* TF_KIND_*                                                    */
    int32_t periodic;          /* TF_PERIODIC_* bits                                           */
    float omega;               /* float32 over-relaxation factor                               */
    float ghost_lo, ghost_hi;  /* Dirichlet ghost values 2*bc: -1 (x = -1) and +1 (x = nx)     */
    float ky, kz;              /* anisotropic y, z weights (dx/dy)^2, (dx/dz)^2                */
    int32_t n_phases;          /* multiphase: phases 1..n_phases                               */
    int32_t tile;              /* tiled-kernel tile shape: 0 = 16x64, 1 = 16x128, 2 = 32x64,   */
                               /* 3 = 16x128 row pairs (binary; even half-sweeps per launch)    */
    int32_t k_max;             /* half-sweeps per tiled launch, 1..4 (0 = 4)                   */
    float divisor[256];        /* binary/anisotropic: code -> diagonal (inf = frozen voxel)    */
    float face[32 * 32];       /* multiphase: [phase a][phase b] harmonic face conductance     */
    uint8_t conductive[32];    /* multiphase: phase -> D > 0 (mask of the initial field)       */
} tf_operator;

/* Library version string. */
const char* tf_version(void);

/* Human-readable name of a TF_* status code. */
const char* tf_status_string(int status);

/* Number of CUDA kernels this library has launched since load (for launch accounting). */
int64_t tf_launch_count(void);

/* Fill *out with pitches and buffer sizes for a batch of `batch` volumes of nx*ny*nz voxels.
 * Pure host arithmetic. `periodic` selects which shapes the tiled kernel accepts. */
int tf_geometry(int batch, int nx, int ny, int nz, int periodic, tf_geom* out);

/* Per-plane counts of label 1 (uint64 [batch][nx]) and the largest label (int32, one) of a uint8
 * label batch [batch][nx][ny][nz] in device memory, in one pass. Replaces the host-side 0/1 label
 * check of Solver (taufactor.py:387-397) and the conductive fraction vol_x = mean(mask, (2, 3))
 * (:42) for labels that serve as tf_pack phase indices as they are. TF_ERR_UNSUPPORTED if
 * batch * nx > 65535. */
int tf_label_stats(int batch, int nx, int ny, int nz, const uint8_t* labels_dev, uint64_t* plane_counts_dev,
                   int32_t* max_label_dev, void* stream);

/* Per-plane count of kappa > 0 (uint64 [batch][nx]) and float64 sum of kappa ([batch][nx]) of a
 * float32 conductivity field [batch][nx][ny][nz] in device memory, and *bad_dev = 1 if any value
 * is negative, infinite or NaN (else 0). One CTA per plane, fixed summation order. KappaSolver
 * set-up: vol_x, D_mean and the input check without torch reductions. */
int tf_kappa_stats(int batch, int nx, int ny, int nz, const float* kappa_dev, uint64_t* plane_positive_dev,
                   double* plane_sums_dev, int32_t* bad_dev, void* stream);

/* out[i] = table[labels[i]] for n voxels: uint8 labels, a 256-entry float32 table, float32 out,
 * all in device memory (MultiPhaseSolver.phase_gradients: the conductivity field D[label]). */
int tf_label_map(const uint8_t* labels_dev, long long n, const float* table_dev, float* out_dev, void* stream);

/* Per-plane float64 sums of values_dev (float64 [batch][nx][ny][nz]) over the voxels of each label
 * slot: plane_sums_dev[(b * nx + x) * n_slots + s] = sum of the values whose label l has
 * slot_of_dev[l] == s (int32 [256]; -1 = no slot). One CTA per plane in a fixed order
 * (MultiPhaseSolver.phase_gradients: dD_eff/dD_p as the sum of dD_eff/dkappa over label p). */
int tf_label_sums(int batch, int nx, int ny, int nz, const uint8_t* labels_dev, const double* values_dev,
                  const int32_t* slot_of_dev, int n_slots, double* plane_sums_dev, void* stream);

/* Build the code buffer and the initial field from per-voxel phase indices.
 * Replaces ThroughTransportSolver.init_field + _pad (taufactor.py:282-291, :228-238),
 * Solver/PeriodicSolver/AnisotropicSolver.init_conductive_neighbours (:402-410, :493-499,
 * :459-471), the label map of MultiPhaseSolver.init_conductive_neighbours (:585-592) and the
 * chequerboard (:218-225; colour is taken from the voxel index instead).
 *   phase_dev   uint8 [batch][nx][ny][nz] (natural layout). binary/anisotropic: 1 = conductive,
 *               0 = not; multiphase: phase index 1..n_phases; electrode: 1 = conductive,
 *               2 = reactive, 0 = neither.
 *   profile_dev float [nx] initial value of a conductive voxel in plane x.
 *   code_dev    uint8 [code_bytes]: binary = neighbour count (0 = frozen), anisotropic =
 *               neighbour pattern index into op->divisor, multiphase = phase index,
 *               electrode = 1 + nn + 8 nr for conductive voxels (nn conductive neighbours, the
 *               inlet face x = -1 counted twice and the outlet face x = nx closed; nr reactive
 *               neighbours; taufactor/electrode.py:46-62) and 0 otherwise; the divisor of volume
 *               b is nn + nr * op->divisor[b] in float32 (op->divisor[b] = k_0 of volume b,
 *               taufactor.py:47-55), inf where 0.
 *   field_dev   float [field_elems]. Ghost cells are filled too. */
int tf_pack(const tf_geom* g, const tf_operator* op, const uint8_t* phase_dev,
            const float* profile_dev, uint8_t* code_dev, float* field_dev, void* stream);

/* Advance the solve by n_half half-sweeps (one colour each), colour of the first one =
 * first_colour (reference: iter % 2). Replaces the loop body of SORSolver.solve
 * (taufactor.py:174-182) with sum_weighted_neighbours (:95-103, :473-478, :606-613) and the
 * periodic ghost copies (:501-505, :652-656), repeated n_half times.
 * Fields ping-pong between field_a_dev and field_b_dev; *result_in_b is set to 1 when the
 * result is in field_b_dev, 0 when in field_a_dev (the input must be in field_a_dev).
 * err_dev (int32, may be NULL) receives TF_ERR_TIMEOUT if a bounded device wait ran out. */
int tf_advance(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
               const uint8_t* code_dev, int first_colour, int n_half, int32_t* err_dev,
               int* result_in_b, void* stream);

/* tf_advance for a correction solve A e = r: every update adds rhs_dev (float [field_elems],
 * split layout with periodic ghost copies, as written by tf_residual_f64) to the neighbour sum.
 * Use an operator whose ghost_lo/ghost_hi are 0 (homogeneous Dirichlet faces). No reference
 * counterpart: the reference iterates in float32 only (taufactor.py:172-182). */
int tf_advance_rhs(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
                   const uint8_t* code_dev, const float* rhs_dev, int first_colour, int n_half,
                   int32_t* err_dev, int* result_in_b, void* stream);

/* float32 field -> float64 field (same split layout, double [field_elems]). */
int tf_widen_f64(const tf_geom* g, const float* field_dev, double* field64_dev, void* stream);

/* float64 field -> float32 field; periodic ghost cells are rebuilt. */
int tf_narrow_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev, float* field_dev,
                  void* stream);

/* field64 += e (float32), every element. */
int tf_axpy_f64(const tf_geom* g, double* field64_dev, const float* e_dev, void* stream);

/* float64 residual r = b - A c of the operator the reference's iteration converges to
 * (A c = d c - weighted in-volume neighbour sum, b = Dirichlet ghost terms; taufactor.py:95-103,
 * :176-181, :598-613). Writes r as float32 into rhs_dev (split layout, periodic ghost copies)
 * and per-plane float64 sums of r^2 and b^2 into r2_sum_dev / b2_sum_dev [batch][nx].
 * TF_KIND_ELECTRODE: d = the sweep's float32 nn + nr * k_0 (taufactor.py:47-55), b = the inlet
 * ghost term; the closed outlet adds nothing. */
int tf_residual_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                    const uint8_t* code_dev, float* rhs_dev, double* r2_sum_dev, double* b2_sum_dev,
                    void* stream);

/* tf_layer_sums on a float64 field (differences and products in float64); for
 * TF_KIND_ELECTRODE the [batch][nx] plane fluxes of ElectrodeSolver, as tf_layer_sums. */
int tf_layer_sums_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                      const uint8_t* code_dev, double* flux_sum_dev, double* c_sum_dev, void* stream);

/* Per-layer float64 sums (not means) for the convergence metrics. Replaces
 * Solver.vertical_flux / MultiPhaseSolver.vertical_flux (taufactor.py:412-419, :615-620) with
 * torch.mean(..., (2, 3)) (:296) and the c_x mean (:307).
 *   flux_sum_dev double [batch][nx-1]: sum over (y, z) of the x-flux through face x|x+1
 *   c_sum_dev    double [batch][nx]:   sum over (y, z) of the field in plane x
 * TF_KIND_ELECTRODE: flux_sum_dev holds [batch][nx] sums of ElectrodeSolver's fluxes
 * (taufactor/electrode.py:70-74): plane 0 (left_bc - c) / 0.5 with left_bc = ghost_lo / 2,
 * plane x > 0 c[x-1] - c[x], each 0 where c or its x-1 neighbour is 0. */
int tf_layer_sums(const tf_geom* g, const tf_operator* op, const float* field_dev,
                  const uint8_t* code_dev, double* flux_sum_dev, double* c_sum_dev, void* stream);

/* Write the reference's padded field layout float [batch][nx+2][ny+2][nz+2]
 * (SORSolver.field, taufactor.py:43, padding :228-238): interior from field_dev, x ghost planes
 * 2*bc, y/z ghosts 0 or (periodic) the wrapped interior. */
int tf_unpack(const tf_geom* g, const tf_operator* op, const float* field_dev, float* padded_dev,
              void* stream);

/* Inverse of tf_unpack for the interior: load a padded reference-layout field into field_dev
 * (ghost cells are rebuilt). Used to resume from a user-supplied field. */
int tf_repack(const tf_geom* g, const tf_operator* op, const float* padded_dev, float* field_dev,
              void* stream);

/* Self-check of the binary sweep's division: for divisor n in 1..8, count the float32 inputs s
 * (all finite bit patterns) where the exact division by n (one multiply and two FMAs with
 * RN(1/n)) differs bitwise from IEEE division s / n, where the sweeps' select-free form differs
 * other than in the sign of a zero quotient, and where the SOR step c + w (q - c) with c = s
 * differs between q = +0 and q = -0. Adds the count to *bad_dev (uint64).
 * No reference counterpart: it guards the bitwise parity of the update `sum / nn`
 * (taufactor.py:177). */
int tf_check_small_division(int n, uint64_t* bad_dev, void* stream);

/* ---------------------------------------------------------------- batched uneven solves
 * Many binary volumes (Solver / PeriodicSolver operators) of different shapes advance in the
 * same launches; each volume keeps its own buffers (tf_geometry with batch = 1) and its own
 * convergence state, evaluated on the device with the reference's rule (taufactor.py:109-153).
 * No reference counterpart as an API: the reference batches only same-shape volumes, which
 * converge together (taufactor.py:30-31, :143). */
#define TF_BATCH_ACTIVE 0
#define TF_BATCH_CONVERGED 1
#define TF_BATCH_NEEDS_HOST 2 /* a layer flux is 0 and percolation is unknown: host decides */

typedef struct tf_batch_state { /* device arrays of n_vol entries unless noted */
    int32_t* status;            /* TF_BATCH_*                                                 */
    int32_t* perc;              /* 0 unknown, 1 spanning path, 2 none (set by the host)       */
    int32_t* conv_iter;         /* half-sweeps at convergence (or at the pause)               */
    int32_t* conv_parity;       /* 1 if the volume's final field is in its buffer B           */
    double* old_tau;            /* tau of the previous check (starts at 0)                    */
    double* tau;                /* last tau, relative flux spread and D_rel                   */
    double* rel;
    double* d_rel;
    int32_t* iter_base;         /* one int: half-sweeps completed before the current graph    */
} tf_batch_state;

/* Bytes of the device descriptor table for n_vol volumes. */
size_t tf_batch_desc_bytes(int n_vol);

/* Tile shape of tile class 0 (class 1: tile_z = 128; class 2: tile_y = 32) and half-sweeps per
 * launch of the batched sweep. */
void tf_batch_tile(int* tile_y, int* tile_z, int* half_sweeps);

/* Fill the descriptor table (device memory, tf_batch_desc_bytes) from per-volume geometry,
 * operator, buffers (field A holds the current field), layer-sum offsets (flux arena offset of
 * plane 0; csum arena likewise) and mean conductive fraction d_mean (tau = d_mean / D_rel).
 * ops[v].tile picks the volume's tile class (rows x z-cells): 1 = 16 x 128, 2 = 32 x 64,
 * otherwise 16 x 64; a volume's work items go to the launches of its class. Synchronous (copies the table to the
 * device). */
int tf_batch_describe(int n_vol, const tf_geom* geoms, const tf_operator* ops, float* const* field_a,
                      float* const* field_b, const uint8_t* const* codes, const int64_t* flux_off,
                      const int64_t* csum_off, const double* d_mean, int32_t* err_dev, void* desc_dev);

/* Descriptor table for batched FP64 defect correction (no reference counterpart): the sweeps
 * solve A e = r per volume with Dirichlet ghosts 0, rhs[v] = float32 right-hand side of volume v
 * (16-byte aligned, field layout), e ping-ponging between field_a[v] and field_b[v]. Synchronous. */
int tf_batch_describe_rhs(int n_vol, const tf_geom* geoms, const tf_operator* ops, float* const* field_a,
                          float* const* field_b, const uint8_t* const* codes, const float* const* rhs,
                          int32_t* err_dev, void* desc_dev);

/* Launch number `launch` (0, 1, ...) of a batched correction solve on a tf_batch_describe_rhs
 * table: volume v takes part while launch < launches_dev[v] (int32 per volume; give an even
 * count so that its result ends in field A). Launch parity selects A -> B or B -> A. */
int tf_batch_advance_rhs(const void* desc_dev, const int32_t* work_dev, int n_work, const int32_t* launches_dev,
                         int launch, void* stream);
/* The same for the work items of tile class `tile` (0..2); tf_batch_advance_rhs is class 0. */
int tf_batch_advance_rhs_tile(const void* desc_dev, const int32_t* work_dev, int n_work,
                              const int32_t* launches_dev, int launch, int tile, void* stream);

/* Advance every active volume by the batch's half-sweeps per launch (colour 0 first, so the
 * completed half-sweeps must stay a multiple of it). work_dev: int32 quads (volume, tile, x0, x1)
 * with tile = ty * tiles_z + tz: the CTA writes planes [x0, x1) of that tile column (items of
 * one column must cover [0, nx) without overlap). parity 0 reads buffers A and writes B, 1 the
 * reverse. */
int tf_batch_advance(const void* desc_dev, const int32_t* work_dev, int n_work, const int32_t* status_dev,
                     int parity, void* stream);
/* The same for the work items of tile class `tile` (0..2); tf_batch_advance is class 0. Items
 * of volumes of the other class return at once. The two classes' volumes are independent, so
 * their launches may run on different streams between two layer-sum / check steps. */
int tf_batch_advance_tile(const void* desc_dev, const int32_t* work_dev, int n_work, const int32_t* status_dev,
                          int parity, int tile, void* stream);

/* Per-plane float64 flux / field sums of every active volume (tf_layer_sums per volume) into
 * the arenas; planes_dev: int32 pairs (volume, x). cur_in_b: the current fields are in B. */
int tf_batch_layer_sums(const void* desc_dev, const int32_t* planes_dev, int n_planes,
                        const int32_t* status_dev, int cur_in_b, double* flux_dev, double* csum_dev,
                        void* stream);

/* The reference's convergence decision for every active volume from its layer fluxes; the
 * current iteration is *iter_base + 100 * (interval + 1). */
int tf_batch_check(const void* desc_dev, int n_vol, const double* flux_dev, tf_batch_state state,
                   double conv_crit, int interval, int cur_in_b, void* stream);

/* *iter_base_dev += half_sweeps (stream-ordered). */
int tf_batch_tick(int32_t* iter_base_dev, int half_sweeps, void* stream);

/* tf_batch_layer_sums followed by tf_batch_check, for callers that cannot give the library any
 * device memory beyond their own buffers (a host whose GPU memory another framework has
 * reserved in full, or a binding that never links the CUDA allocator). The per-plane sums go to
 * a static array inside the library instead of caller arenas; only `state` is written, so the
 * per-layer sums themselves are not returned. No counterpart in the reference.
 *   Limit: flux_len and csum_len (the arena lengths the descriptor's offsets were built for:
 *   sum of nx-1, resp. nx, over the volumes) must each be <= 65536, else TF_ERR_UNSUPPORTED.
 *   desc_dev must be a table that tf_batch_describe built on the current device, with n_vol at
 *   most its volumes and every offset it was given ending within flux_len / csum_len; anything
 *   else is TF_ERR_ARG, before any launch. Plane items outside the table's volumes are skipped.
 *   Allocates nothing (no cudaMalloc/cudaFree). The first call on a device looks up the device
 *   address of the static array for that device (make it before any stream capture), and looks
 *   it up again if the device's context has changed since (cudaDeviceReset); the array is shared
 *   by every call in the process and keeps the last call's contents, so calls whose work
 *   overlaps on the GPU race. It holds 1 MiB on every GPU that loads the library. */
int tf_batch_converge_static(const void* desc_dev, const int32_t* planes_dev, int n_planes, int n_vol,
                             int64_t flux_len, int64_t csum_len, tf_batch_state state, double conv_crit,
                             int interval, int cur_in_b, void* stream);

/* ---------------------------------------------------------------- per-voxel conductivity
 * MultiPhaseSolver's operator (taufactor.py:508-620) with the diffusivity given per voxel as a
 * float32 field kappa >= 0 instead of per label, plus its adjoint. With kappa = D[label] the
 * faces, factor and half-sweeps equal MultiPhaseSolver's bit for bit. kappa_split_dev is a
 * float [field_elems] buffer in the field layout written by tf_kappa_pack. No reference
 * counterpart for the adjoint: the reference solve runs under no_grad (taufactor.py:172). */

/* kappa_dev float [batch][nx][ny][nz] -> kappa_split_dev (ghost cells 0 / wrapped copies) and
 * the initial field (profile[x] where kappa > 0; taufactor.py:282-291, :571-575). */
int tf_kappa_pack(const tf_geom* g, const tf_operator* op, const float* kappa_dev, const float* profile_dev,
                  float* kappa_split_dev, float* field_dev, void* stream);

/* n_half half-sweeps in place (taufactor.py:174-182 with :606-613 on per-voxel faces); rhs_dev
 * (float [field_elems], may be NULL) is added to the neighbour sum for correction solves. */
int tf_kappa_advance(const tf_geom* g, const tf_operator* op, float* field_dev, const float* kappa_split_dev,
                     const float* rhs_dev, int first_colour, int n_half, void* stream);

/* Spanning-path test of the zero-flux branch of the convergence check (taufactor.py:318-327,
 * extract_through_feature(mask, 1, 'x'), taufactor/metrics/connectivity.py:138-213): for every
 * volume, whether a face-connected cluster of conductive voxels (conductive[phase] != 0, host
 * table of 256 entries; no periodic wrap) touches both x = 0 and x = nx - 1.
 *   phase_dev  uint8 [batch][nx][ny][nz]; labels_dev int32 scratch of the same size
 *   spans_dev  int32 [batch]: 1 / 0.  err_dev: TF_ERR_TIMEOUT if a bounded loop ran out.
 * batch * nx * ny * nz must stay below 2^31. */
int tf_spans_x(int batch, int nx, int ny, int nz, const uint8_t* phase_dev, const uint8_t* conductive,
               int32_t* labels_dev, int32_t* spans_dev, int32_t* err_dev, void* stream);

/* Phase indices of the anchored system (no reference counterpart; the system the FP64 oracle
 * solves): out_phase_dev[v] = phase_dev[v] where v belongs to a face-connected cluster of
 * conductive voxels (conductive[phase] != 0, host table of 256 entries; wrapping in y / z for
 * the TF_PERIODIC_* bits of `periodic`) that touches x = 0 or x = nx - 1, else 0. Clusters that
 * touch neither face carry no flux; with a rounded float32 diagonal their block of the operator
 * is nearly singular, and the FP64 refinement packs its codes from this map so that they stay out
 * of its residual. labels_dev int32 and flags_dev uint8 are scratch of batch*nx*ny*nz entries;
 * err_dev: TF_ERR_TIMEOUT if a bounded loop ran out. batch * nx * ny * nz must stay below 2^31. */
int tf_anchored_phase(int batch, int nx, int ny, int nz, int periodic, const uint8_t* phase_dev,
                      const uint8_t* conductive, int32_t* labels_dev, uint8_t* flags_dev, uint8_t* out_phase_dev,
                      int32_t* err_dev, void* stream);

/* The operator's faces for tf_kappa_advance_faces, computed once per kappa field (float32, the
 * values the sweeps use; taufactor.py:586-603 with a per-voxel diffusivity): fx_dev holds
 * batch * (nx + 1) planes of field_elems / (batch * nx) floats each (plane x + 1 = the face
 * between x and x + 1, planes 0 and nx the Dirichlet faces of planes 0 and nx - 1), fy_dev,
 * fz_dev and div_dev field_elems floats each (the +y and +z faces of every cell and the factor;
 * the factor also on periodic ghost positions, those of the TF_PERIODIC_* bits of `periodic`). */
int tf_kappa_faces(const tf_geom* g, const float* kappa_split_dev, float* fx_dev, float* fy_dev, float* fz_dev,
                   float* div_dev, int periodic, void* stream);

/* tf_kappa_advance from the packed faces: the same half-sweeps bit for bit, one division per
 * voxel instead of six, float4 groups (every pointer 16-byte aligned). */
int tf_kappa_advance_faces(const tf_geom* g, const tf_operator* op, float* field_dev, const float* fx_dev,
                           const float* fy_dev, const float* fz_dev, const float* div_dev, const float* rhs_dev,
                           int first_colour, int n_half, void* stream);

/* tf_kappa_advance_faces fused: K <= op->k_max (0 = 4) half-sweeps per register-streaming launch
 * (the TMA wavefront of tf_advance; faces and factor read per group from the packed arrays), the
 * same half-sweeps bit for bit. field_a_dev -> field_b_dev -> ... like tf_advance: *result_in_b
 * says which buffer holds the result. Shapes the tiled kernel cannot keep periodic ghost bands
 * for (g->tiled = 0) run tf_kappa_advance_faces in place on field_a_dev. The faces must come from
 * tf_kappa_faces with the operator's periodic bits (the factor on periodic ghost positions), and
 * a periodic rhs_dev must carry its ghost copies (tf_refresh_ghosts): a fused launch updates the
 * ghost rows of its tiles like the cells they mirror. err_dev: TF_ERR_TIMEOUT if a bounded wait
 * ran out. Every pointer 16-byte aligned. */
int tf_kappa_advance_fused(const tf_geom* g, const tf_operator* op, float* field_a_dev, float* field_b_dev,
                           const float* fx_dev, const float* fy_dev, const float* fz_dev, const float* div_dev,
                           const float* rhs_dev, int first_colour, int n_half, int32_t* err_dev, int* result_in_b,
                           void* stream);

/* Periodic ghost copies of a float field in the split layout, rebuilt from the interior for the
 * TF_PERIODIC_* bits of `periodic` (taufactor.py:501-505); nothing for 0. */
int tf_refresh_ghosts(const tf_geom* g, int periodic, float* field_dev, void* stream);

/* Coefficients of the float64 steps below (coeff_f64): 0 = the sweeps' own float32 faces and
 * float32 diagonal (the reference's discrete operator, taufactor.py:577-603); 1 = float64 faces
 * 2ab/(a+b) of the float32 kappa values and the exact float64 diagonal, under which D_eff is a
 * smooth function of kappa (the form that gradients and their finite-difference checks need). */

/* per-plane float64 sums of face * (c[x+1] - c[x]) and of c (taufactor.py:615-620, :296, :307);
 * field_dev is float (field_is_f64 = 0, float32 faces; coeff_f64 must be 0) or double (1). */
int tf_kappa_layer_sums(const tf_geom* g, const void* field_dev, int field_is_f64, int coeff_f64,
                        const float* kappa_split_dev, double* flux_sum_dev, double* c_sum_dev, void* stream);

/* float64 residual r = b - A c; b = the Dirichlet terms of op (b64_dev NULL) or b64_dev
 * (double [field_elems]). r -> rhs_dev (float, periodic ghosts rebuilt); per-plane sums of r^2
 * and b^2 -> r2_sum_dev / b2_sum_dev [batch][nx]. */
int tf_kappa_residual_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                          const float* kappa_split_dev, const double* b64_dev, int coeff_f64, float* rhs_dev,
                          double* r2_sum_dev, double* b2_sum_dev, void* stream);

/* Adjoint right-hand side dD_eff/dc = scale * (face_{x-1|x} - face_{x|x+1}) per voxel
 * (double [field_elems]); scale = D_0 nx / (|bc_hi - bc_lo| (nx-1) ny nz). */
int tf_kappa_adjoint_rhs(const tf_geom* g, const float* kappa_split_dev, double* out64_dev, double scale,
                         int coeff_f64, void* stream);

/* dD_eff/dkappa per voxel, double [batch][nx][ny][nz], from the float64 field c and the adjoint
 * lambda (A lambda = dD_eff/dc): interior faces -(lam_u - lam_w)(c_u - c_w) (+ scale *
 * (c[x+1]-c[x]) on x-faces) times 2 k_w^2/(k_u+k_w)^2, Dirichlet faces 2 lam_u (bc - c_u). */
int tf_kappa_gradient(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                      const double* lambda64_dev, const float* kappa_split_dev, double* grad_dev, double scale,
                      double bc_lo, double bc_hi, void* stream);

/* double field layout -> natural [batch][nx][ny][nz]. */
int tf_split_to_natural_f64(const tf_geom* g, const double* split_dev, double* natural_dev, void* stream);

/* The float64 coefficients (coeff_f64 = 1) packed once per kappa field, in the layout of
 * tf_kappa_faces but double: fx_dev batch * (nx + 1) planes (planes 0 and nx: the Dirichlet faces
 * kappa), fy_dev / fz_dev the +y / +z face of every cell, div_dev the diagonal (0 for a voxel
 * outside the system). Each face costs a float64 division; the three functions below read them
 * instead (no reference counterpart: the float64 steps of the FP64 correction and adjoint). */
int tf_kappa_faces_f64(const tf_geom* g, const float* kappa_split_dev, double* fx_dev, double* fy_dev, double* fz_dev,
                       double* div_dev, void* stream);
/* tf_kappa_residual_f64 with coeff_f64 = 1 from the packed faces (float64 fused multiply-adds:
 * the same r to a few float64 roundings). */
int tf_kappa_residual_faces_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                                const double* fx_dev, const double* fy_dev, const double* fz_dev,
                                const double* div_dev, const double* b64_dev, float* rhs_dev, double* r2_sum_dev,
                                double* b2_sum_dev, void* stream);
/* tf_kappa_layer_sums on a double field with coeff_f64 = 1, from the packed x faces. */
int tf_kappa_layer_sums_faces_f64(const tf_geom* g, const double* field64_dev, const double* fx_dev,
                                  double* flux_sum_dev, double* c_sum_dev, void* stream);
/* tf_kappa_gradient from the packed faces: d face / d kappa_u = face^2 / (2 kappa_u^2). */
int tf_kappa_gradient_faces_f64(const tf_geom* g, const tf_operator* op, const double* field64_dev,
                                const double* lambda64_dev, const float* kappa_split_dev, const double* fx_dev,
                                const double* fy_dev, const double* fz_dev, double* grad_dev, double scale,
                                double bc_lo, double bc_hi, void* stream);

/* ---- Multigrid-preconditioned conjugate gradients for the correction solve A e = r ---------
 * No reference counterpart: the reference solves only by red-black SOR (taufactor.py:156-191).
 * These serve the float32 inner solve of the FP64 defect correction (KappaSolver). A level is a
 * tf_geom of dims (nx, ny, nz), the next one of dims ((nx+1)/2, (ny+1)/2, (nz+1)/2) and the same
 * batch, each with packed faces in the tf_kappa_faces layout; its smoother is
 * tf_kappa_advance_faces with omega 1 and ghost values 0. Dirichlet x ghosts are 0 throughout. */

/* Coarse faces and factor: `scale` times the sum of the fine faces across each coarse interface
 * (aggregates of 2 cells per axis, 1 at the end of an odd extent), the factor their sum in the
 * order of tf_kappa_faces with the Dirichlet x faces counted twice; periodic ghost positions hold
 * the wrapped cell's faces (TF_PERIODIC_* bits of `periodic`), closed ones 0 (factor inf). */
int tf_mg_coarsen(const tf_geom* fine, const float* fx_dev, const float* fy_dev, const float* fz_dev,
                  const tf_geom* coarse, float* cfx_dev, float* cfy_dev, float* cfz_dev, float* cdiv_dev,
                  int periodic, float scale, void* stream);

/* Coarse right-hand side rc = sum over each aggregate of (rhs - A e) on the fine level (rhs_dev
 * may be NULL); writes the coarse interior cells only. */
int tf_mg_restrict(const tf_geom* fine, const float* e_dev, const float* rhs_dev, const float* fx_dev,
                   const float* fy_dev, const float* fz_dev, const float* div_dev, const tf_geom* coarse,
                   float* rc_dev, void* stream);

/* e += the coarse value of its aggregate on every fine interior cell; periodic ghosts rebuilt. */
int tf_mg_prolong(const tf_geom* coarse, const float* ec_dev, const tf_geom* fine, float* e_dev, int periodic,
                  void* stream);

/* out = A in on interior cells (0 where the factor is not finite); other cells untouched. The
 * ghost cells of in_dev must be current (periodic copies or 0). */
int tf_mg_apply(const tf_geom* g, const float* in_dev, const float* fx_dev, const float* fy_dev,
                const float* fz_dev, const float* div_dev, float* out_dev, void* stream);

/* Per-volume dot products over interior cells (a float4 group's products summed in float32, the
 * groups accumulated in float64), in a fixed order: out[b] = sum a1*b1 and,
 * when a2_dev/b2_dev are given, out[batch + b] = sum a2*b2. part_dev: double [2 * batch*nx*ny]. */
int tf_mg_dot(const tf_geom* g, const float* a1_dev, const float* b1_dev, const float* a2_dev, const float* b2_dev,
              double* part_dev, double* out_dev, void* stream);

/* Conjugate-gradient updates over whole volumes with per-volume steps (0 where a denominator is
 * not a positive finite number): x += a p, r -= a q with a = rz[b] / pq[b]; p = z + c p with
 * c = rz_new[b] / rz_old[b]. Pointers 16-byte aligned. */
int tf_pcg_update_xr(const tf_geom* g, float* x_dev, float* r_dev, const float* p_dev, const float* q_dev,
                     const double* rz_dev, const double* pq_dev, void* stream);
int tf_pcg_update_p(const tf_geom* g, float* p_dev, const float* z_dev, const double* rz_new_dev,
                    const double* rz_old_dev, void* stream);

/* ---- Impedance (tau_e) solve: ImpedanceSolver / PeriodicImpedanceSolver ----------------------
 * (taufactor/electrode.py:160-402). One volume; n_freq frequencies solved side by side. The field
 * is complex128 in the reference's padded layout [n_freq][nx+2][ny+2][nz+2], interleaved
 * (re, im) doubles, 16-byte aligned. A voxel's code is 0 outside the conductive phase, else
 * 0x80 | (nn + 8 nr) with nn its conductive face neighbours (the inlet ghost x = -1 counted 2)
 * and nr its reactive ones; the factor table holds 1 / (nn + i frc nr) per frequency at index
 * nn + 8 nr (entry 0 = 0), TF_IMP_TABLE complex entries per frequency. */
#define TF_IMP_TABLE 56

/* Codes and per-plane counts (conductive voxels, reactive faces) as uint64 [nx][2] from phase
 * bits (bit 0 conductive, bit 1 reactive) of uint8 [nx][ny][nz]; periodic in y and z if set.
 * Replaces ImpedanceSolver.count_neighbours (electrode.py:235-264), the periodic variant
 * (:373-396) and the vol_x / a_x sums of __init__ (:186-187). */
int tf_impedance_pack(int nx, int ny, int nz, int periodic, const uint8_t* phase_dev, uint8_t* code_dev,
                      uint64_t* plane_counts_dev, void* stream);

/* Initial field: phi[f][x] (complex, [n_freq][nx] interleaved) on conductive voxels, 0 elsewhere,
 * ghost_lo on the inlet ghost plane's interior, 0 on every other ghost. Replaces
 * ImpedanceSolver.init_field_internal (electrode.py:214-233), phi computed by the caller. */
int tf_impedance_fill(int n_freq, int nx, int ny, int nz, const uint8_t* code_dev, const double* phi_dev,
                      double ghost_lo, double* field_dev, void* stream);

/* n_half half-sweeps; half-sweep s updates colour (first_iter + s) % 2 of every frequency whose
 * active_dev byte is non-zero (active_dev NULL: all), after the periodic ghost copy if periodic.
 * Replaces the loop body of ImpedanceSolver.solve (electrode.py:302-309) with
 * PeriodicImpedanceSolver.apply_boundary_conditions (:398-402). */
int tf_impedance_sweep(int n_freq, int nx, int ny, int nz, int periodic, double* field_dev,
                       const uint8_t* code_dev, const double* table_dev, const uint8_t* active_dev,
                       double omega, int first_iter, int n_half, void* stream);

/* Per-plane sums of |c| (double [n_freq][nx]), sums of the inlet flux 2 left_bc - 2 c over plane
 * 0 where c != 0 (double [n_freq][2]: re, im) and the NaN cells per frequency (int32 [n_freq]).
 * Replaces the reductions of ImpedanceSolver.compute_metrics (electrode.py:379-392),
 * calc_input_impedance (:324-330) and the NaN test of solve (:293). */
int tf_impedance_metrics(int n_freq, int nx, int ny, int nz, const double* field_dev, double left_bc,
                         double* abs_sum_dev, double* influx_sum_dev, int32_t* nan_count_dev, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TAUFACTOR_GB300_H */
