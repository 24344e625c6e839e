// Batched solve of many volumes of uneven shapes (sm_103a).
//
// Every volume keeps its own split-layout buffers and geometry; a descriptor table in device
// memory holds, per volume, the TMA tensor maps of its two field buffers and its codes, the
// sweep arguments for both ping-pong directions and the offsets of its layer sums. One
// k_stream_multi launch advances every still-active volume by K half-sweeps: CTA w takes work
// item (volume, tile, x0, x1) from a table and runs the same per-tile body as the single-volume
// kernel on planes [x0, x1) of that tile column (x-chunks keep the items of large and small
// volumes about equally long); CTAs of volumes whose status is not "active" return at once.
// Volumes come in three tile classes (rows x z-cells: 0 = 16 x 64, 1 = 16 x 128, 2 = 32 x 64),
// each with its own kernel instantiation and work list; the class is the volume's
// tf_operator.tile.
// k_layer_sums_multi and
// k_batch_check then evaluate the reference's convergence rule (taufactor.py:109-153,
// :293-331) per volume on the device and set its status, so a whole check interval -- sweeps,
// layer sums, decision -- runs without the host and can be captured in a CUDA graph.
//
// FP64 defect correction of the whole batch uses a second table whose sweeps solve the
// correction equation A e = r (homogeneous Dirichlet ghosts, float32 right-hand side r per
// volume): k_stream_multi_rhs runs every volume's inner half-sweeps in the same launches, each
// volume for its own number of launches.
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "tf_layers.cuh"
#include "tf_stream.cuh"

namespace tf {

constexpr int BTY = 16, BTZ = 64, BK = 4;  // tile (class 0) and fused depth of the batched sweep
constexpr int BTZ1 = 128;                  // z-cells of a class-1 tile (16 rows)
constexpr int BTY2 = 32;                   // rows of a class-2 tile (64 z-cells)
using BShape = StreamShape<BTY, BTZ, BK>;
using BShape1 = StreamShape<BTY, BTZ1, BK>;
using BShape2 = StreamShape<BTY2, BTZ, BK>;

struct alignas(64) VolDesc {
    CUtensorMap map_a, map_b, map_c;  // field A, field B, codes (boxes of the volume's tile class)
    SweepArgs ab, ba;                 // A -> B and B -> A
    const uint8_t* code;
    int tiles_z, tiles_y;
    int tile_y, tile_z;               // rows and z-cells of the volume's tiles (its class)
    long long flux_off, csum_off;  // offsets into the layer-sum arenas
    double d_mean;                 // mean conductive fraction (tau = d_mean / D_rel)
    double inv_area;               // 1 / (ny * nz)
};

// Work items of volumes of another tile class (a caller's mix-up) return without touching them.
template <int TY, int TZ>
__global__ void __launch_bounds__(StreamShape<TY, TZ, BK>::NT, StreamShape<TY, TZ, BK>::NT <= 256 ? 2 : 1)
    k_stream_multi(const VolDesc* __restrict__ desc, const int4* __restrict__ work,
                   const int32_t* __restrict__ status, int parity) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int4 item = work[blockIdx.x];
    const int v = item.x;
    if (status[v] != TF_BATCH_ACTIVE) return;
    const VolDesc* d = desc + v;
    if (d->tile_y != TY || d->tile_z != TZ) return;
    const int tz = item.y % d->tiles_z, ty = item.y / d->tiles_z;
    const SweepArgs a = parity ? d->ba : d->ab;
    stream_tile<TF_KIND_BINARY, TY, TZ, BK, false>(parity ? &d->map_b : &d->map_a, &d->map_c, a, nullptr,
                                                   tz * (TZ / 2), ty * TY, 0, item.z, item.w, smem);
}

// Correction sweeps: launch `launch` of an inner solve; volume v takes part while
// launch < launches[v] (an even count, so each volume's result ends in buffer A).
template <int TY, int TZ>
__global__ void __launch_bounds__(StreamShape<TY, TZ, BK>::NT, StreamShape<TY, TZ, BK>::NT <= 256 ? 2 : 1)
    k_stream_multi_rhs(const VolDesc* __restrict__ desc, const int4* __restrict__ work,
                       const int32_t* __restrict__ launches, int launch) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int4 item = work[blockIdx.x];
    const int v = item.x;
    if (launch >= launches[v]) return;
    const VolDesc* d = desc + v;
    if (d->tile_y != TY || d->tile_z != TZ) return;
    const int tz = item.y % d->tiles_z, ty = item.y / d->tiles_z;
    const int parity = launch & 1;
    const SweepArgs a = parity ? d->ba : d->ab;
    stream_tile<TF_KIND_BINARY, TY, TZ, BK, true>(parity ? &d->map_b : &d->map_a, &d->map_c, a, nullptr,
                                                  tz * (TZ / 2), ty * TY, 0, item.z, item.w, smem);
}

// One CTA per (volume, plane): float64 sums of the masked x-flux through face x|x+1 and of the
// field in plane x (taufactor.py:294-296, :307, :412-419), exactly as the single-volume
// k_layer_sums sums them. Binary operators only.
// GUARDED (the static-scratch path): items naming a volume >= n_desc or a plane outside the
// volume are skipped, and so is any sum whose index would reach past flux_cap / csum_cap.
template <bool GUARDED>
__global__ void __launch_bounds__(256) k_layer_sums_multi(const VolDesc* __restrict__ desc,
                                                          const int2* __restrict__ planes,
                                                          const int32_t* __restrict__ status, int cur_in_b,
                                                          double* __restrict__ flux, double* __restrict__ csum,
                                                          int n_desc = 0, long long flux_cap = 0,
                                                          long long csum_cap = 0) {
    const int2 item = planes[blockIdx.x];
    const int v = item.x, x = item.y;
    if (GUARDED && (v < 0 || v >= n_desc)) return;
    if (status[v] != TF_BATCH_ACTIVE) return;
    const VolDesc* d = desc + v;
    const Geo g = d->ab.g;
    if (GUARDED && (x < 0 || x >= g.NX)) return;
    const float* field = cur_in_b ? d->ab.out : d->ba.out;  // ab.out is buffer B
    const bool has_flux = x + 1 < g.NX;
    double fs = 0.0, cs = 0.0;
    plane_partials<TF_KIND_BINARY>(field + (long long)x * g.plane_f, d->code + (long long)x * g.plane_c, g, has_flux,
                                   nullptr, fs, cs);
    block_sum_pair(fs, cs);
    if (threadIdx.x == 0) {
        const long long fi = d->flux_off + x, ci = d->csum_off + x;
        if (has_flux && (!GUARDED || (fi >= 0 && fi < flux_cap))) flux[fi] = fs;
        if (!GUARDED || (ci >= 0 && ci < csum_cap)) csum[ci] = cs;
    }
}

// One CTA (one warp) per volume: the reference's convergence rule on its layer fluxes.
//   rel = (max - min) / max of the layer-mean fluxes (NaN if max == 0); D_rel = mean * Nx;
//   tau = d_mean / D_rel (NaN if D_rel == 0). Converged iff rel < conv_crit and
//   |tau - old_tau| < 2e-3; otherwise old_tau = tau. A zero layer flux pauses the volume
//   (status "needs host") until its percolation is known: non-percolating volumes converge
//   with tau = 0 (reported as inf), percolating ones continue. A NaN mean converges.
__global__ void k_batch_check(const VolDesc* __restrict__ desc, int n_vol, const double* __restrict__ flux,
                              tf_batch_state st, double conv_crit, int interval, int cur_in_b) {
    const int v = blockIdx.x;
    if (v >= n_vol || st.status[v] != TF_BATCH_ACTIVE) return;
    const VolDesc* d = desc + v;
    const int nx = d->ab.g.NX;
    const int nf = nx - 1;
    double mx = -INFINITY, mn = INFINITY, sum = 0.0;
    for (int i = threadIdx.x; i < nf; i += 32) {
        const double f = flux[d->flux_off + i] * d->inv_area;
        mx = fmax(mx, f);
        mn = fmin(mn, f);
        sum += f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    if (threadIdx.x != 0) return;
    const double mean = sum / nf;
    const int iter = *st.iter_base + 100 * (interval + 1);
    double rel = mx != 0.0 ? (mx - mn) / mx : NAN;
    double d_rel = mean * nx;
    double tau = d_rel != 0.0 ? d->d_mean / d_rel : NAN;
    if (mn == 0.0 || mx == 0.0 || mean == 0.0) {
        if (st.perc[v] == 0) {  // percolation unknown: let the host decide
            st.status[v] = TF_BATCH_NEEDS_HOST;
            st.conv_iter[v] = iter;
            st.conv_parity[v] = cur_in_b;
            return;
        }
        if (st.perc[v] == 2) {  // no spanning path: converged, tau reported as inf
            rel = 0.0;
            d_rel = 0.0;
            tau = 0.0;
        }
    }
    if (isnan(mean)) rel = 0.0;
    st.tau[v] = tau;
    st.rel[v] = rel;
    st.d_rel[v] = d_rel;
    if (rel < conv_crit && fabs(tau - st.old_tau[v]) < 2e-3) {
        st.status[v] = TF_BATCH_CONVERGED;
        st.conv_iter[v] = iter;
        st.conv_parity[v] = cur_in_b;
    } else {
        st.old_tau[v] = tau;
    }
}

__global__ void k_batch_tick(int32_t* iter_base, int step) { *iter_base += step; }

}  // namespace tf

using namespace tf;

extern "C" {

size_t tf_batch_desc_bytes(int n_vol) { return n_vol > 0 ? (size_t)n_vol * sizeof(VolDesc) : 0; }

void tf_batch_tile(int* tile_y, int* tile_z, int* half_sweeps) {
    if (tile_y) *tile_y = BTY;
    if (tile_z) *tile_z = BTZ;
    if (half_sweeps) *half_sweeps = BK;
}

}  // extern "C"

namespace tf {

// What tf_batch_describe built at a descriptor address (per device): the number of volumes and
// the end of the layer-sum offsets, max over v of flux_off + nx - 1 and csum_off + nx (-1 for a
// correction-solve table, which has no layer sums). tf_batch_converge_static checks its
// arguments against it before writing sums into its fixed array.
struct DescExtent {
    int n_vol;
    long long flux_end, csum_end;
};
static std::mutex g_extent_mu;
static std::map<std::pair<int, const void*>, DescExtent> g_extent;

static void record_extent(const void* desc_dev, const DescExtent& e) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lock(g_extent_mu);
    g_extent[{dev, desc_dev}] = e;
}

static bool find_extent(const void* desc_dev, DescExtent* e) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lock(g_extent_mu);
    const auto it = g_extent.find({dev, desc_dev});
    if (it == g_extent.end()) return false;
    *e = it->second;
    return true;
}

// Descriptor table of the plain solve (rhs == nullptr) or of the correction solve (rhs[v] = the
// float32 right-hand side of volume v; Dirichlet ghosts 0; layer-sum fields unused).
static int describe(int n_vol, const tf_geom* geoms, const tf_operator* ops, float* const* field_a,
                    float* const* field_b, const uint8_t* const* codes, const float* const* rhs,
                    const int64_t* flux_off, const int64_t* csum_off, const double* d_mean, int32_t* err_dev,
                    void* desc_dev) {
    std::vector<VolDesc> h(n_vol);
    DescExtent ext{n_vol, rhs ? -1 : 0, rhs ? -1 : 0};
    for (int v = 0; v < n_vol; ++v) {
        const tf_geom& gg = geoms[v];
        tf_operator op = ops[v];
        if (gg.batch != 1 || !gg.tiled || op.kind != TF_KIND_BINARY) return TF_ERR_UNSUPPORTED;
        if ((flux_off && flux_off[v] < 0) || (csum_off && csum_off[v] < 0)) return TF_ERR_ARG;
        if (!rhs) {
            const long long fe = (flux_off ? flux_off[v] : 0) + gg.nx - 1, ce = (csum_off ? csum_off[v] : 0) + gg.nx;
            ext.flux_end = fe > ext.flux_end ? fe : ext.flux_end;
            ext.csum_end = ce > ext.csum_end ? ce : ext.csum_end;
        }
        if (rhs && (!rhs[v] || (reinterpret_cast<uintptr_t>(rhs[v]) & 15))) return TF_ERR_ARG;
        if (rhs) op.ghost_lo = op.ghost_hi = 0.0f;
        VolDesc& d = h[v];
        std::memset(&d, 0, sizeof(VolDesc));
        const long long planes = (long long)gg.nx;
        const int cls = op.tile == 1 || op.tile == 2 ? op.tile : 0;
        const int wj = cls == 1 ? BShape1::WJ : (cls == 2 ? BShape2::WJ : BShape::WJ);
        const int wjc = cls == 1 ? BShape1::WJC : (cls == 2 ? BShape2::WJC : BShape::WJC);
        const int rows = cls == 1 ? BShape1::ROWS : (cls == 2 ? BShape2::ROWS : BShape::ROWS);
        int rc = encode_map_3d(&d.map_a, field_a[v], 4, gg.zh, 2 * gg.yp, planes, (long long)gg.zh * 4,
                               (long long)gg.zh * 4 * 2 * gg.yp, wj, 2 * rows);
        if (!rc)
            rc = encode_map_3d(&d.map_b, field_b[v], 4, gg.zh, 2 * gg.yp, planes, (long long)gg.zh * 4,
                               (long long)gg.zh * 4 * 2 * gg.yp, wj, 2 * rows);
        if (!rc)
            rc = encode_map_3d(&d.map_c, codes[v], 1, gg.zhc, 2 * gg.yp, planes, gg.zhc,
                               (long long)gg.zhc * 2 * gg.yp, wjc, 2 * rows);
        if (rc) return rc;
        d.tile_y = cls == 2 ? BTY2 : BTY;
        d.tile_z = cls == 1 ? BTZ1 : BTZ;
        const Geo g = make_geo(gg);
        d.ab = make_args(g, op, field_b[v], 0, BK, err_dev);
        d.ba = make_args(g, op, field_a[v], 0, BK, err_dev);
        if (rhs) d.ab.rhs = d.ba.rhs = rhs[v];
        d.code = codes[v];
        d.tiles_z = (gg.nz + d.tile_z - 1) / d.tile_z;
        d.tiles_y = (gg.ny + d.tile_y - 1) / d.tile_y;
        d.flux_off = flux_off ? flux_off[v] : 0;
        d.csum_off = csum_off ? csum_off[v] : 0;
        d.d_mean = d_mean ? d_mean[v] : 0.0;
        d.inv_area = 1.0 / ((double)gg.ny * gg.nz);
    }
    // kernel attributes are set here, outside any stream capture
    const cudaFuncAttribute smem_attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const bool ok = rhs ? cudaFuncSetAttribute(k_stream_multi_rhs<BTY, BTZ>, smem_attr, BShape::SMEM) == cudaSuccess &&
                              cudaFuncSetAttribute(k_stream_multi_rhs<BTY, BTZ1>, smem_attr, BShape1::SMEM) ==
                                  cudaSuccess &&
                              cudaFuncSetAttribute(k_stream_multi_rhs<BTY2, BTZ>, smem_attr, BShape2::SMEM) ==
                                  cudaSuccess
                        : cudaFuncSetAttribute(k_stream_multi<BTY, BTZ>, smem_attr, BShape::SMEM) == cudaSuccess &&
                              cudaFuncSetAttribute(k_stream_multi<BTY, BTZ1>, smem_attr, BShape1::SMEM) ==
                                  cudaSuccess &&
                              cudaFuncSetAttribute(k_stream_multi<BTY2, BTZ>, smem_attr, BShape2::SMEM) == cudaSuccess;
    if (!ok) return TF_ERR_CUDA;
    if (cudaMemcpy(desc_dev, h.data(), sizeof(VolDesc) * n_vol, cudaMemcpyHostToDevice) != cudaSuccess)
        return TF_ERR_CUDA;
    record_extent(desc_dev, ext);
    return TF_OK;
}

}  // namespace tf

extern "C" {

int tf_batch_describe(int n_vol, const tf_geom* geoms, const tf_operator* ops, float* const* field_a,
                      float* const* field_b, const uint8_t* const* codes, const int64_t* flux_off,
                      const int64_t* csum_off, const double* d_mean, int32_t* err_dev, void* desc_dev) {
    if (n_vol <= 0 || !geoms || !ops || !field_a || !field_b || !codes || !flux_off || !csum_off || !d_mean ||
        !desc_dev)
        return TF_ERR_ARG;
    return describe(n_vol, geoms, ops, field_a, field_b, codes, nullptr, flux_off, csum_off, d_mean, err_dev,
                    desc_dev);
}

int tf_batch_describe_rhs(int n_vol, const tf_geom* geoms, const tf_operator* ops, float* const* field_a,
                          float* const* field_b, const uint8_t* const* codes, const float* const* rhs,
                          int32_t* err_dev, void* desc_dev) {
    if (n_vol <= 0 || !geoms || !ops || !field_a || !field_b || !codes || !rhs || !desc_dev) return TF_ERR_ARG;
    return describe(n_vol, geoms, ops, field_a, field_b, codes, rhs, nullptr, nullptr, nullptr, err_dev, desc_dev);
}

int tf_batch_advance_rhs_tile(const void* desc_dev, const int32_t* work_dev, int n_work,
                              const int32_t* launches_dev, int launch, int tile, void* stream) {
    if (!desc_dev || !work_dev || n_work <= 0 || !launches_dev || launch < 0 || tile < 0 || tile > 2)
        return TF_ERR_ARG;
    const VolDesc* d = static_cast<const VolDesc*>(desc_dev);
    const int4* w = reinterpret_cast<const int4*>(work_dev);
    cudaStream_t st = (cudaStream_t)stream;
    if (tile == 1)
        k_stream_multi_rhs<BTY, BTZ1><<<n_work, BShape1::NT, BShape1::SMEM, st>>>(d, w, launches_dev, launch);
    else if (tile == 2)
        k_stream_multi_rhs<BTY2, BTZ><<<n_work, BShape2::NT, BShape2::SMEM, st>>>(d, w, launches_dev, launch);
    else
        k_stream_multi_rhs<BTY, BTZ><<<n_work, BShape::NT, BShape::SMEM, st>>>(d, w, launches_dev, launch);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_batch_advance_rhs(const void* desc_dev, const int32_t* work_dev, int n_work, const int32_t* launches_dev,
                         int launch, void* stream) {
    return tf_batch_advance_rhs_tile(desc_dev, work_dev, n_work, launches_dev, launch, 0, stream);
}

int tf_batch_advance_tile(const void* desc_dev, const int32_t* work_dev, int n_work, const int32_t* status_dev,
                          int parity, int tile, void* stream) {
    if (!desc_dev || !work_dev || n_work <= 0 || !status_dev || tile < 0 || tile > 2) return TF_ERR_ARG;
    const VolDesc* d = static_cast<const VolDesc*>(desc_dev);
    const int4* w = reinterpret_cast<const int4*>(work_dev);
    cudaStream_t st = (cudaStream_t)stream;
    if (tile == 1)
        k_stream_multi<BTY, BTZ1><<<n_work, BShape1::NT, BShape1::SMEM, st>>>(d, w, status_dev, parity & 1);
    else if (tile == 2)
        k_stream_multi<BTY2, BTZ><<<n_work, BShape2::NT, BShape2::SMEM, st>>>(d, w, status_dev, parity & 1);
    else
        k_stream_multi<BTY, BTZ><<<n_work, BShape::NT, BShape::SMEM, st>>>(d, w, status_dev, parity & 1);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_batch_advance(const void* desc_dev, const int32_t* work_dev, int n_work, const int32_t* status_dev,
                     int parity, void* stream) {
    return tf_batch_advance_tile(desc_dev, work_dev, n_work, status_dev, parity, 0, stream);
}

int tf_batch_layer_sums(const void* desc_dev, const int32_t* planes_dev, int n_planes, const int32_t* status_dev,
                        int cur_in_b, double* flux_dev, double* csum_dev, void* stream) {
    if (!desc_dev || !planes_dev || n_planes <= 0 || !status_dev || !flux_dev || !csum_dev) return TF_ERR_ARG;
    k_layer_sums_multi<false><<<n_planes, 256, 0, (cudaStream_t)stream>>>(static_cast<const VolDesc*>(desc_dev),
                                                                    reinterpret_cast<const int2*>(planes_dev),
                                                                    status_dev, cur_in_b & 1, flux_dev, csum_dev);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_batch_check(const void* desc_dev, int n_vol, const double* flux_dev, tf_batch_state state, double conv_crit,
                   int interval, int cur_in_b, void* stream) {
    if (!desc_dev || n_vol <= 0 || !flux_dev || !state.status || !state.perc || !state.conv_iter ||
        !state.conv_parity || !state.old_tau || !state.tau || !state.rel || !state.d_rel || !state.iter_base)
        return TF_ERR_ARG;
    k_batch_check<<<n_vol, 32, 0, (cudaStream_t)stream>>>(static_cast<const VolDesc*>(desc_dev), n_vol, flux_dev,
                                                          state, conv_crit, interval, cur_in_b & 1);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

int tf_batch_tick(int32_t* iter_base_dev, int half_sweeps, void* stream) {
    if (!iter_base_dev) return TF_ERR_ARG;
    k_batch_tick<<<1, 1, 0, (cudaStream_t)stream>>>(iter_base_dev, half_sweeps);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

}  // extern "C"

// ------------------------------------------------------------------------------ allocation-free
// check step. Some callers cannot hand the library any device memory beyond their own inputs
// and outputs: a host whose device memory is fully reserved up front by another framework's
// pool, or a language binding that never links the CUDA allocator and only passes buffers it
// already owns. For them, tf_batch_converge_static runs the batched convergence step (the
// per-plane layer sums that tf_batch_layer_sums writes into caller arenas, then the decision of
// tf_batch_check) with the per-plane sums kept in this library's own statically sized device
// array. The array lives in every GPU that loads the library until the process exits.
namespace tf {

constexpr long long STATIC_PLANES = 1 << 16;  // capacity of each half of the static scratch

// [0, STATIC_PLANES): per-plane flux sums; [STATIC_PLANES, 2*STATIC_PLANES): field sums.
static __device__ __align__(256) double g_static_sums[2 * STATIC_PLANES];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// The calling thread's current CUDA context (null if none yet or if the lookup fails).
static CUcontext current_context() {
    static CtxGetCurrentFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(p);
    });
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// Device address of g_static_sums on the current device, resolved with that device current the
// first time and again whenever the device's context has changed (after a cudaDeviceReset the
// module, and with it the array, is loaded anew).
static double* static_sums_address() {
    constexpr int MAX_DEVICES = 64;
    static double* addr[MAX_DEVICES] = {nullptr};
    static CUcontext ctx[MAX_DEVICES] = {nullptr};
    static std::mutex mu;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    const CUcontext now = current_context();
    if (!addr[dev] || !now || now != ctx[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_sums) != cudaSuccess) return nullptr;
        addr[dev] = static_cast<double*>(p);
        ctx[dev] = current_context();
    }
    return addr[dev];
}

}  // namespace tf

extern "C" int tf_batch_converge_static(const void* desc_dev, const int32_t* planes_dev, int n_planes, int n_vol,
                                        int64_t flux_len, int64_t csum_len, tf_batch_state state,
                                        double conv_crit, int interval, int cur_in_b, void* stream) {
    if (!desc_dev || !planes_dev || n_planes <= 0 || n_vol <= 0 || !state.status || !state.perc ||
        !state.conv_iter || !state.conv_parity || !state.old_tau || !state.tau || !state.rel || !state.d_rel ||
        !state.iter_base)
        return TF_ERR_ARG;
    // the descriptor's layer-sum offsets must fit the static array: flux_len / csum_len are the
    // arena lengths the descriptor was built for (sum of nx-1, resp. nx, over the volumes)
    if (flux_len <= 0 || csum_len <= 0 || flux_len > STATIC_PLANES || csum_len > STATIC_PLANES)
        return TF_ERR_UNSUPPORTED;
    // and they must be what tf_batch_describe actually built at desc_dev on this device: the
    // offsets it wrote end within flux_len / csum_len, and n_vol does not exceed its volumes
    DescExtent ext;
    if (!find_extent(desc_dev, &ext) || ext.flux_end < 0 || n_vol > ext.n_vol || ext.flux_end > flux_len ||
        ext.csum_end > csum_len)
        return TF_ERR_ARG;
    double* sums = static_sums_address();
    if (!sums) return TF_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // every sum the decision reads is written by the layer-sum launch of this same call, so
    // nothing in the shared array has to start at zero; the guarded kernel also skips plane items
    // outside the descriptor's volumes and any index past the array
    k_layer_sums_multi<true><<<n_planes, 256, 0, st>>>(static_cast<const VolDesc*>(desc_dev),
                                                        reinterpret_cast<const int2*>(planes_dev), state.status,
                                                        cur_in_b & 1, sums, sums + STATIC_PLANES, ext.n_vol,
                                                        STATIC_PLANES, STATIC_PLANES);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return TF_ERR_CUDA;
    k_batch_check<<<n_vol, 32, 0, st>>>(static_cast<const VolDesc*>(desc_dev), n_vol, sums, state, conv_crit,
                                        interval, cur_in_b & 1);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}
