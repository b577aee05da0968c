// Fold skeleton of libmsl_gb300.so with the built-in functors (sum, max, min)
// and the fused FP64 residual max|a - b|.
//
// Reference: DS::fold (src/ds.cpp:741-912) / foldCPU (:924-954), foldKernel +
// reduce() (src/fold_kernels.cu:51-129, 298-403); the residual of
// examples/jacobisolver.cpp:127-140 (zip with |x - y|, then fold with max).
#include "../include/detail/msl_fold.cuh"
#include "msl_internal.h"

using namespace msl;
using namespace msl::gpu;
using msl::rt::ctx;

namespace {

template <typename T, int OP> struct FoldOp {
    __device__ __forceinline__ T operator()(T a, T b) const {
        if constexpr (OP == MSL_FOLD_SUM) return Arith<T>::add(a, b);
        else if constexpr (OP == MSL_FOLD_MAX) return a > b ? a : b;
        else return a < b ? a : b;
    }
};
struct MaxNan {  // max that keeps a NaN (a residual must not hide one)
    __device__ __forceinline__ double operator()(double a, double b) const { return (b > a || b != b) ? b : a; }
};

// The fold kernel writes (value, present) straight into a mapped pinned
// host slot (the value at offset 0, the flag at 64): the result reaches the
// host with the kernel, without a copy after it.
FoldScratch mapped_result_scratch() {
    auto &c = ctx();
    FoldScratch s = c.fold;
    s.result = c.host_fold_dev;
    s.result_have = (int *)((char *)c.host_fold_dev + 64);
    return s;
}

template <typename R> int finish_fold(void *result, const char *what) {
    auto &c = ctx();
    rt::count_launch();
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), what);
    const char *h = (const char *)c.host_fold;
    if (!*(volatile const int *)(h + 64)) return rt::fail(MSL_ERR_CUDA, "%s: the fold produced no value", what);
    memcpy(result, h, sizeof(R));
    return MSL_OK;
}

template <typename T, int OP> int fold_op(const void *in, size_t n, void *result) {
    auto &c = ctx();
    constexpr int V = vec_width1<T>();
    cudaError_t e = launch_fold<FoldSrcArray, T>(n, FoldOp<T, OP>{}, mapped_result_scratch(), c.stream, c.sm_count,
                                                 aligned_to(in, V * sizeof(T)), (const T *)in);
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_fold");
    return finish_fold<T>(result, "msl_fold");
}

template <typename T> int fold_t(int op, const void *in, size_t n, void *result) {
    switch (op) {
        case MSL_FOLD_SUM: return fold_op<T, MSL_FOLD_SUM>(in, n, result);
        case MSL_FOLD_MAX: return fold_op<T, MSL_FOLD_MAX>(in, n, result);
        case MSL_FOLD_MIN: return fold_op<T, MSL_FOLD_MIN>(in, n, result);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold: unknown op %d", op);
}

template <typename T> int absdiff_t(const void *a, const void *b, size_t n, double *result) {
    auto &c = ctx();
    constexpr int V = vec_width1<T>();
    const bool vec = aligned_to(a, V * sizeof(T)) && aligned_to(b, V * sizeof(T));
    cudaError_t e = launch_fold<FoldSrcAbsDiff, T>(n, MaxNan{}, mapped_result_scratch(), c.stream, c.sm_count, vec, (const T *)a,
                                                   (const T *)b);
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_fold_absdiff_max");
    return finish_fold<double>(result, "msl_fold_absdiff_max");
}

}  // namespace

extern "C" {

int msl_fold(int dtype, int op, const void *in, size_t n, void *result) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (n == 0) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold: empty input has no fold (no identity element)");
    if (!in || !result) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold: NULL pointer");
    switch (dtype) {
        case MSL_F32: return fold_t<float>(op, in, n, result);
        case MSL_F64: return fold_t<double>(op, in, n, result);
        case MSL_I32: return fold_t<int32_t>(op, in, n, result);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold: unsupported dtype %d", dtype);
}

int msl_fold_absdiff_max(int dtype, const void *a, const void *b, size_t n, double *result) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (n == 0) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_absdiff_max: empty input");
    if (!a || !b || !result) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_absdiff_max: NULL pointer");
    switch (dtype) {
        case MSL_F32: return absdiff_t<float>(a, b, n, result);
        case MSL_F64: return absdiff_t<double>(a, b, n, result);
        case MSL_I32: return absdiff_t<int32_t>(a, b, n, result);
        case MSL_BF16: return absdiff_t<bf16s>(a, b, n, result);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_absdiff_max: unsupported dtype %d", dtype);
}

}  // extern "C"
