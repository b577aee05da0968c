// Stencil skeletons of libmsl_gb300.so with the built-in functors of
// msl_gb300.h: plain Jacobi (fixed boundary), heat2D, box mean/sum at any
// radius, Game of Life (DM), heat3D and 3-D box sum/mean (DC).
//
// Reference: DM::mapStencil (src/dm.cpp:1535-1591) and DC::mapStencil
// (src/dc.cpp:559-592); functors examples/heatdiffusion.cpp:55-76,
// examples/gameoflife.cpp:22-42, examples/meanblur2.cpp:46-57.
#include <cmath>

#include "../include/detail/msl_stencil3d_tb.cuh"
#include "stencil_functors.cuh"

using namespace msl;
using namespace msl::gpu;
using msl::rt::ctx;

namespace {

using namespace msl::builtin;

// ---- dispatch -----------------------------------------------------------------------
struct Sweep {
    unsigned long long *resid;  // nullptr: no residual
    bool tma;
};

// 3-D kernel choice of msl_set_stencil3d_persistent (-1 = default).
std::atomic<int> g_persistent3d{-1};
// Sweeps per launch of msl_stencil3d_iterate where the z-marching kernel
// applies (1 or 2). Two is the default: on heat3D 512^3 the two-sweep kernel
// (half the HBM traffic per sweep, bound by instruction issue) runs 1.5x the
// one-sweep kernel, which is itself at the HBM roofline.
std::atomic<int> g_depth3d{2};
// z planes per CTA of the z-marching kernel (0: chosen per grid).
std::atomic<int> g_zchunk3d{0};

template <typename S>
cudaError_t sweep2d(int kind, const S *in, S *out, int rows, int cols, int r, double neutral_d, const Sweep &sw) {
    using T = typename Compute<S>::type;
    auto &c = ctx();
    const T neutral = (T)neutral_d;
    switch (kind) {
        case MSL_ST2_JACOBI5:
            return launch_stencil2d<S>(in, out, rows, cols, r, neutral, StJacobi5<T>{}, sw.resid, c.err_word, c.stream,
                                       sw.tma);
        case MSL_ST2_HEAT5:
            return launch_stencil2d<S>(in, out, rows, cols, r, neutral, StHeat5<T>{}, sw.resid, c.err_word, c.stream,
                                       sw.tma);
        case MSL_ST2_BOXMEAN:
        case MSL_ST2_BOXSUM: {
            const bool mean = kind == MSL_ST2_BOXMEAN;
            if constexpr (std::is_same<S, float>::value) {
                switch (r) {
                    case 1: return box_fixed_f32<1>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                    case 2: return box_fixed_f32<2>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                    case 3: return box_fixed_f32<3>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                    case 4: return box_fixed_f32<4>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                    case 6: return box_fixed_f32<6>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                    case 8: return box_fixed_f32<8>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                    case 10: return box_fixed_f32<10>(in, out, rows, cols, neutral, mean, sw.resid, sw.tma);
                }
            }
            return launch_stencil2d<S>(in, out, rows, cols, r, neutral, StBoxAny<T>{r, mean}, sw.resid, c.err_word,
                                       c.stream, sw.tma);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t sweep2d_life(const int32_t *in, int32_t *out, int rows, int cols, int r, double neutral, const Sweep &sw) {
    auto &c = ctx();
    return launch_stencil2d<int32_t>(in, out, rows, cols, r, (int32_t)(long long)neutral, StLife{}, sw.resid,
                                     c.err_word, c.stream, sw.tma);
}

template <typename S>
cudaError_t sweep3d(int kind, const S *in, S *out, int depth, int rows, int cols, int r, double neutral_d,
                    const Sweep &sw) {
    using T = typename Compute<S>::type;
    auto &c = ctx();
    const T neutral = (T)neutral_d;
    const int pers = g_persistent3d.load(std::memory_order_relaxed);
    if (kind == MSL_ST3_HEAT7)
        return launch_stencil3d<S>(in, out, depth, rows, cols, r, neutral, StHeat7<T>{}, sw.resid, c.err_word, c.stream,
                                   c.sm_count, sw.tma, pers);
    return launch_stencil3d<S>(in, out, depth, rows, cols, r, neutral, StBox3<T>{r, kind == MSL_ST3_BOXMEAN}, sw.resid,
                               c.err_word, c.stream, c.sm_count, sw.tma, pers);
}

bool kind2_ok(int dtype, int kind) {
    if (dtype == MSL_I32) return kind == MSL_ST2_LIFE;
    if (dtype == MSL_BF16) return kind == MSL_ST2_JACOBI5 || kind == MSL_ST2_HEAT5;
    if (dtype == MSL_F32 || dtype == MSL_F64) return kind >= MSL_ST2_JACOBI5 && kind <= MSL_ST2_BOXSUM;
    return false;
}

int check2d(const char *what, int dtype, int kind, const void *a, const void *b, int rows, int cols, int r) {
    if (rows <= 0 || cols <= 0) return rt::fail(MSL_ERR_SIZE_MISMATCH, "%s: empty grid %d x %d", what, rows, cols);
    if ((long long)rows * cols > (1LL << 31) - 1) return rt::fail(MSL_ERR_SIZE_MISMATCH, "%s: grid too large", what);
    if (r < 0 || r > 64) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: radius %d outside 0..64", what, r);
    if (!a || !b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: NULL pointer", what);
    if (a == b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: input and output must differ", what);
    if (!kind2_ok(dtype, kind))
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: stencil kind %d not available for dtype %d", what, kind, dtype);
    if (stencil2d_smem<float>(r) > kMaxStencilSmem)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: radius %d needs too much shared memory", what, r);
    return MSL_OK;
}

int check3d(const char *what, int dtype, int kind, const void *a, const void *b, int depth, int rows, int cols, int r) {
    if (depth <= 0 || rows <= 0 || cols <= 0) return rt::fail(MSL_ERR_SIZE_MISMATCH, "%s: empty cube", what);
    if ((long long)depth * rows * cols > (1LL << 31) - 1) return rt::fail(MSL_ERR_SIZE_MISMATCH, "%s: cube too large", what);
    if (r < 0 || r > 7) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: radius %d outside 0..7", what, r);
    if (!a || !b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: NULL pointer", what);
    if (a == b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: input and output must differ", what);
    if ((dtype != MSL_F32 && dtype != MSL_F64) || kind < MSL_ST3_HEAT7 || kind > MSL_ST3_BOXMEAN)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: stencil kind %d not available for dtype %d", what, kind, dtype);
    if (stencil3d_smem<double>(r) > kMaxStencilSmem)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: radius %d needs too much shared memory", what, r);
    return MSL_OK;
}

cudaError_t dispatch2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int r, double neutral,
                       const Sweep &sw) {
    switch (dtype) {
        case MSL_F32: return sweep2d<float>(kind, (const float *)in, (float *)out, rows, cols, r, neutral, sw);
        case MSL_F64: return sweep2d<double>(kind, (const double *)in, (double *)out, rows, cols, r, neutral, sw);
        case MSL_BF16: return sweep2d<bf16s>(kind, (const bf16s *)in, (bf16s *)out, rows, cols, r, neutral, sw);
        case MSL_I32: return sweep2d_life((const int32_t *)in, (int32_t *)out, rows, cols, r, neutral, sw);
    }
    return cudaErrorInvalidValue;
}

cudaError_t dispatch3d(int dtype, int kind, const void *in, void *out, int d, int rows, int cols, int r, double neutral,
                       const Sweep &sw) {
    if (dtype == MSL_F32) return sweep3d<float>(kind, (const float *)in, (float *)out, d, rows, cols, r, neutral, sw);
    return sweep3d<double>(kind, (const double *)in, (double *)out, d, rows, cols, r, neutral, sw);
}

// Read the fused residual slot (synchronises).
int read_residual(double *residual, const char *what) {
    auto &c = ctx();
    MSL_TRY_CUDA(cudaMemcpyAsync(c.host_result, c.resid, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c.stream),
                 what);
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), what);
    unsigned long long bits = *(volatile unsigned long long *)c.host_result;
    memcpy(residual, &bits, sizeof bits);
    return MSL_OK;
}

std::atomic<int> g_tma_enabled{1};
bool tma_enabled() { return g_tma_enabled.load(std::memory_order_relaxed) != 0; }

// `iters` ping-pong sweeps a -> b -> a ..., `depth` sweeps per launch (the
// first launch runs `first` sweeps when that is > 0; the last launch takes the
// remainder). The residual is fused into the last sweep.
template <class Launch>
int iterate(const char *what, void *a, void *b, int iters, int depth, double *residual, int *result_in_b,
            Launch launch, int first = 0) {
    auto &c = ctx();
    Sweep sw{nullptr, tma_enabled()};
    if (residual) MSL_TRY_CUDA(cudaMemsetAsync(c.resid, 0, sizeof(unsigned long long), c.stream), what);
    void *p = a, *q = b;
    for (int i = 0; i < iters;) {
        const int k = std::min(std::max(i == 0 && first > 0 ? first : depth, 1), iters - i);
        sw.resid = (residual && i + k == iters) ? c.resid : nullptr;
        cudaError_t e = launch(p, q, k, sw);
        if (e != cudaSuccess) return rt::cuda_fail(e, what);
        rt::count_launch();
        void *t = p;
        p = q;
        q = t;
        i += k;
    }
    if (result_in_b) *result_in_b = (p == b);
    if (residual) {
        if (int e = read_residual(residual, what)) return e;
        return rt::check_device_errors(what);
    }
    return MSL_OK;
}

std::atomic<int> g_temporal_depth{0};
std::atomic<int> g_tile_rows{0};

// Tile height of the temporal-blocking kernel: the fixed setting, or (0) the
// autotuner's record, else 32.
int tile_rows_for(int dtype, int kind, int rows, int cols, int r) {
    const int t = g_tile_rows.load(std::memory_order_relaxed);
    if (t > 0) return t;
    return msl::rt::tuned_tile_rows(dtype, kind, rows, cols, r);
}

// Sweeps per launch for a 2-D iteration: the fixed setting, or (0) the
// autotuner's choice recorded for this grid, else 1.
int depth_for(int dtype, int kind, int rows, int cols, int r) {
    if (!tb_supported_2d(dtype, kind)) return 1;
    int d = g_temporal_depth.load(std::memory_order_relaxed);
    if (d > 0) return d;
    return msl::rt::tuned_depth(dtype, kind, rows, cols, r);
}

}  // namespace

namespace msl {
namespace rt {
int temporal_depth_setting() { return g_temporal_depth.load(std::memory_order_relaxed); }
int tile_rows_setting() { return g_tile_rows.load(std::memory_order_relaxed); }
int stencil3d_pair_sweeps() { return g_depth3d.load(std::memory_order_relaxed) == 2; }
int stencil3d_zchunk() { return g_zchunk3d.load(std::memory_order_relaxed); }
}  // namespace rt
}  // namespace msl

extern "C" {

int msl_set_tma(int enabled) {
    g_tma_enabled.store(enabled ? 1 : 0);
    return MSL_OK;
}

int msl_set_stencil3d_depth(int sweeps) {
    if (sweeps < 1 || sweeps > 2) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_stencil3d_depth: %d not 1 or 2", sweeps);
    g_depth3d.store(sweeps);
    return MSL_OK;
}

int msl_set_stencil3d_zchunk(int planes) {
    if (planes < 0 || planes > 1024)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_stencil3d_zchunk: %d not in 0..1024", planes);
    g_zchunk3d.store(planes);
    return MSL_OK;
}

int msl_set_stencil3d_persistent(int mode) {
    if (mode < -1 || mode > 1) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_stencil3d_persistent: %d not in -1..1", mode);
    g_persistent3d.store(mode);
    return MSL_OK;
}

int msl_set_tile_rows(int rows) {
    if (rows != 0 && !valid_tile_rows(rows))
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_tile_rows: %d not 0, 16, 32 or 64", rows);
    g_tile_rows.store(rows);
    return MSL_OK;
}

int msl_set_temporal_depth(int depth) {
    if (depth < 0 || depth > 32) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_temporal_depth: %d not in 0..32", depth);
    g_temporal_depth.store(depth);
    return MSL_OK;
}

int msl_stencil2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int radius, double neutral) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check2d("msl_stencil2d", dtype, kind, in, out, rows, cols, radius)) return e;
    cudaError_t e = dispatch2d(dtype, kind, in, out, rows, cols, radius, neutral, Sweep{nullptr, tma_enabled()});
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_stencil2d");
    rt::count_launch();
    return MSL_OK;
}

int msl_stencil2d_iterate(int dtype, int kind, void *a, void *b, int rows, int cols, int radius, double neutral,
                          int iters, double *residual, int *result_in_b) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check2d("msl_stencil2d_iterate", dtype, kind, a, b, rows, cols, radius)) return e;
    if (iters < 1) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_stencil2d_iterate: iters must be >= 1");
    const int depth = depth_for(dtype, kind, rows, cols, radius);
    const int tile_rows = tile_rows_for(dtype, kind, rows, cols, radius);
    // Life: every launch after the first reads the output of a Life launch,
    // whose cells are all 0 or 1, and may take the bit-packed kernel. The first
    // launch then runs a single generation (the cell-by-cell kernel at full
    // memory speed) and every later one `depth` packed generations; only a
    // last launch with a residual runs several generations cell by cell.
    const bool life_packed = dtype == MSL_I32 && kind == MSL_ST2_LIFE && radius == 1 && neutral == 0.0 &&
                             depth <= builtin::kLifePackedMaxDepth;
    const int first = life_packed ? 1 : 0;
    const bool generic_tb = depth > 1 && (!life_packed || residual);
    if (generic_tb && stencil2d_tb_smem<double>(radius, depth, tile_rows) > kMaxStencilSmem)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_stencil2d_iterate: temporal depth %d too deep for radius %d",
                        depth, radius);
    int launch_no = 0;
    return iterate("msl_stencil2d_iterate", a, b, iters, depth, residual, result_in_b,
                   [&](void *p, void *q, int k, const Sweep &sw) {
                       const bool binary_in = launch_no++ > 0;
                       if (life_packed && binary_in && !sw.resid) {
                           cudaError_t e = life_packed_2d(p, q, rows, cols, k);
                           if (e != cudaErrorNotSupported) return e;
                       }
                       if (k > 1)
                           return tb_sweeps_2d(dtype, kind, p, q, rows, cols, radius, k, neutral, sw.resid, sw.tma,
                                               tile_rows);
                       return dispatch2d(dtype, kind, p, q, rows, cols, radius, neutral, sw);
                   },
                   first);
}

int msl_stencil3d(int dtype, int kind, const void *in, void *out, int depth, int rows, int cols, int radius,
                  double neutral) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check3d("msl_stencil3d", dtype, kind, in, out, depth, rows, cols, radius)) return e;
    cudaError_t e = dispatch3d(dtype, kind, in, out, depth, rows, cols, radius, neutral, Sweep{nullptr, tma_enabled()});
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_stencil3d");
    rt::count_launch();
    return MSL_OK;
}

int msl_stencil3d_iterate(int dtype, int kind, void *a, void *b, int depth, int rows, int cols, int radius,
                          double neutral, int iters, double *residual, int *result_in_b) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check3d("msl_stencil3d_iterate", dtype, kind, a, b, depth, rows, cols, radius)) return e;
    if (iters < 1) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_stencil3d_iterate: iters must be >= 1");
    // heat3D (FP32, radius 1, neutral +0) on grids TMA can address: two
    // sweeps per launch by z-marching
    const bool ztb = dtype == MSL_F32 && kind == MSL_ST3_HEAT7 && radius == 1 && neutral == 0.0 &&
                     !std::signbit(neutral) && g_depth3d.load(std::memory_order_relaxed) == 2 && tma_enabled() &&
                     stencil_tma_ok<float>(a, cols, kZtbPitch, kZtbRows) &&
                     stencil_tma_ok<float>(b, cols, kZtbPitch, kZtbRows);
    return iterate("msl_stencil3d_iterate", a, b, iters, ztb ? 2 : 1, residual, result_in_b,
                   [&](void *p, void *q, int k, const Sweep &sw) {
                       if (k == 2)
                           return launch_stencil3d_ztb((const float *)p, (float *)q, depth, rows, cols,
                                                       StHeat7<float>{}, sw.resid, ctx().err_word, ctx().stream,
                                                       g_zchunk3d.load(std::memory_order_relaxed));
                       return dispatch3d(dtype, kind, p, q, depth, rows, cols, radius, neutral, sw);
                   });
}

}  // extern "C"
