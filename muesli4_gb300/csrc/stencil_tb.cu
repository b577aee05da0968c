// Temporally blocked 2-D sweeps (several sweeps per launch) for the built-in
// Jacobi, heat2D and Life functors; see stencil2d_tb_kernel.
#include "../include/detail/msl_life.cuh"
#include "stencil_functors.cuh"

namespace msl {
namespace builtin {

bool tb_supported_2d(int dtype, int kind) {
    if (dtype == MSL_I32) return kind == MSL_ST2_LIFE;
    if (dtype == MSL_F32 || dtype == MSL_F64 || dtype == MSL_BF16)
        return kind == MSL_ST2_JACOBI5 || kind == MSL_ST2_HEAT5;
    return false;
}

template <typename S>
cudaError_t tb_float(int kind, const S *in, S *out, int rows, int cols, int r, int depth, double neutral,
                     unsigned long long *resid, bool tma, int tile_rows) {
    using T = typename Compute<S>::type;
    auto &c = rt::ctx();
    if (kind == MSL_ST2_JACOBI5)
        return launch_stencil2d_tb<S>(in, out, rows, cols, r, depth, (T)neutral, StJacobi5<T>{}, resid, c.err_word,
                                      c.stream, tma, tile_rows);
    return launch_stencil2d_tb<S>(in, out, rows, cols, r, depth, (T)neutral, StHeat5<T>{}, resid, c.err_word, c.stream,
                                  tma, tile_rows);
}

cudaError_t tb_sweeps_2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int r, int depth,
                         double neutral, unsigned long long *resid, bool tma, int tile_rows) {
    auto &c = rt::ctx();
    switch (dtype) {
        case MSL_F32:
            return tb_float<float>(kind, (const float *)in, (float *)out, rows, cols, r, depth, neutral, resid, tma,
                                   tile_rows);
        case MSL_F64:
            return tb_float<double>(kind, (const double *)in, (double *)out, rows, cols, r, depth, neutral, resid, tma,
                                    tile_rows);
        case MSL_BF16:
            return tb_float<bf16s>(kind, (const bf16s *)in, (bf16s *)out, rows, cols, r, depth, neutral, resid, tma,
                                   tile_rows);
        case MSL_I32:
            return launch_stencil2d_tb_rows<int32_t, StLife, kSt2BY>((const int32_t *)in, (int32_t *)out, rows, cols, r,
                                                                     depth, (int32_t)(long long)neutral, StLife{}, resid,
                                                                     c.err_word, c.stream, tma);
    }
    return cudaErrorInvalidValue;
}

static_assert(kLifePackedMaxDepth == gpu::kLifeMaxDepth, "Life kernel depth limit");

cudaError_t life_packed_2d(const void *in, void *out, int rows, int cols, int depth) {
    auto &c = rt::ctx();
    return launch_life_packed((const int32_t *)in, (int32_t *)out, rows, cols, depth, c.stream);
}

}  // namespace builtin
}  // namespace msl
