// Fixed-radius box stencils (F32), split across files so they compile in parallel.
#include "../include/detail/msl_box2d.cuh"
#include "stencil_functors.cuh"

namespace msl {
namespace builtin {

template <int R>
cudaError_t box_fixed_f32(const float *in, float *out, int rows, int cols, float neutral, bool mean,
                          unsigned long long *resid, bool tma) {
    auto &c = rt::ctx();
    // two columns per thread with packed additions where it applies
    const cudaError_t e = mean ? launch_box2d_pair<R, true>(in, out, rows, cols, neutral, resid, c.err_word, c.stream, tma)
                               : launch_box2d_pair<R, false>(in, out, rows, cols, neutral, resid, c.err_word, c.stream, tma);
    if (e != cudaErrorNotSupported) return e;
    if (mean)
        return launch_stencil2d<float>(in, out, rows, cols, R, neutral, StBoxFixed<float, R, true>{}, resid, c.err_word,
                                       c.stream, tma);
    return launch_stencil2d<float>(in, out, rows, cols, R, neutral, StBoxFixed<float, R, false>{}, resid, c.err_word,
                                   c.stream, tma);
}

template cudaError_t box_fixed_f32<8>(const float *, float *, int, int, float, bool, unsigned long long *, bool);

}  // namespace builtin
}  // namespace msl
