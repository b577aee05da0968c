// Row/column skeletons of DM with built-in functors: row folds, column folds,
// row/column rotations, setColumn and the matrix-by-row-vector broadcast zip.
//
// Reference: DM::reduceRows (src/dm.cpp:1596-1707, foldRowsKernel
// src/fold_kernels.cu:215-294), DM::rotateRows (src/dm.cpp:1345-1475),
// DM::rotateCols (src/dm.cpp:1483-1533), DM::setColumn (src/dm.cpp:1856-1879),
// the DM x DA zips (src/dm.cpp:1757-1853, src/zip_kernels.cu:45-71).
#include "../include/detail/msl_matrix.cuh"
#include "msl_internal.h"

using namespace msl;
using namespace msl::gpu;
using msl::rt::ctx;

namespace {

template <typename T> using A = Arith<T>;

template <typename T, int OP> struct RowFoldOp {
    __device__ __forceinline__ T operator()(T a, T b) const {
        if constexpr (OP == MSL_FOLD_SUM) return A<T>::add(a, b);
        else if constexpr (OP == MSL_FOLD_MAX) return a > b ? a : b;
        else return a < b ? a : b;
    }
};

template <typename T, int OP> struct RowZipOp {
    __device__ __forceinline__ T operator()(T a, T b) const {
        if constexpr (OP == MSL_ZIP_ADD) return A<T>::add(a, b);
        else if constexpr (OP == MSL_ZIP_SUB) return A<T>::sub(a, b);
        else if constexpr (OP == MSL_ZIP_MUL) return A<T>::mul(a, b);
        else if constexpr (OP == MSL_ZIP_MULADD) return A<T>::add(A<T>::mul(a, b), a);
        else if constexpr (OP == MSL_ZIP_ABSDIFF) {
            T d = A<T>::sub(a, b);
            return d < T(0) ? A<T>::sub(T(0), d) : d;
        } else if constexpr (OP == MSL_ZIP_MAX) return a > b ? a : b;
        else return a < b ? a : b;
    }
};

int done(cudaError_t e, const char *what, unsigned launches = 1) {
    if (e != cudaSuccess) return rt::cuda_fail(e, what);
    rt::count_launch(launches);
    return MSL_OK;
}

template <typename T, int OP> int fold_rows_op(const void *in, void *out, long long rows, long long cols, int tpb) {
    auto &c = ctx();
    return done(launch_fold_rows((const T *)in, (T *)out, rows, cols, tpb, RowFoldOp<T, OP>{}, c.stream, c.sm_count),
                "msl_fold_rows");
}
template <typename T, int OP> int fold_cols_op(const void *in, void *out, long long rows, long long cols) {
    auto &c = ctx();
    return done(launch_fold_cols((const T *)in, (T *)out, rows, cols, RowFoldOp<T, OP>{}, c.stream, c.sm_count),
                "msl_fold_cols");
}

template <typename T> int fold_rows_t(int op, const void *in, void *out, long long rows, long long cols, int tpb) {
    switch (op) {
        case MSL_FOLD_SUM: return fold_rows_op<T, MSL_FOLD_SUM>(in, out, rows, cols, tpb);
        case MSL_FOLD_MAX: return fold_rows_op<T, MSL_FOLD_MAX>(in, out, rows, cols, tpb);
        case MSL_FOLD_MIN: return fold_rows_op<T, MSL_FOLD_MIN>(in, out, rows, cols, tpb);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_rows: unknown op %d", op);
}
template <typename T> int fold_cols_t(int op, const void *in, void *out, long long rows, long long cols) {
    switch (op) {
        case MSL_FOLD_SUM: return fold_cols_op<T, MSL_FOLD_SUM>(in, out, rows, cols);
        case MSL_FOLD_MAX: return fold_cols_op<T, MSL_FOLD_MAX>(in, out, rows, cols);
        case MSL_FOLD_MIN: return fold_cols_op<T, MSL_FOLD_MIN>(in, out, rows, cols);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_cols: unknown op %d", op);
}

template <typename T, int OP>
int zip_rows_op(const void *m, const void *v, void *out, long long rows, long long cols) {
    auto &c = ctx();
    ZipRowsOp<T, RowZipOp<T, OP>> op{(const T *)m, (const T *)v, (T *)out, cols, {}};
    return done(launch_row_cells(rows, cols, op, c.stream, c.sm_count), "msl_zip_rows");
}
template <typename T> int zip_rows_t(int op, const void *m, const void *v, void *out, long long rows, long long cols) {
    switch (op) {
        case MSL_ZIP_ADD: return zip_rows_op<T, MSL_ZIP_ADD>(m, v, out, rows, cols);
        case MSL_ZIP_SUB: return zip_rows_op<T, MSL_ZIP_SUB>(m, v, out, rows, cols);
        case MSL_ZIP_MUL: return zip_rows_op<T, MSL_ZIP_MUL>(m, v, out, rows, cols);
        case MSL_ZIP_MULADD: return zip_rows_op<T, MSL_ZIP_MULADD>(m, v, out, rows, cols);
        case MSL_ZIP_ABSDIFF: return zip_rows_op<T, MSL_ZIP_ABSDIFF>(m, v, out, rows, cols);
        case MSL_ZIP_MAX: return zip_rows_op<T, MSL_ZIP_MAX>(m, v, out, rows, cols);
        case MSL_ZIP_MIN: return zip_rows_op<T, MSL_ZIP_MIN>(m, v, out, rows, cols);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip_rows: unknown op %d", op);
}

// Copies move raw elements: one instantiation per element size.
template <typename W> int rotate_rows_w(const void *in, void *out, long long rows, long long cols, long long a) {
    auto &c = ctx();
    return done(launch_row_cells(rows, cols, RotateRowsOp<W>{(const W *)in, (W *)out, rows, cols, a}, c.stream,
                                 c.sm_count),
                "msl_rotate_rows");
}
template <typename W> int rotate_cols_w(const void *in, void *out, long long rows, long long cols, long long a) {
    auto &c = ctx();
    return done(launch_row_cells(rows, cols, RotateColsOp<W>{(const W *)in, (W *)out, cols, a}, c.stream, c.sm_count),
                "msl_rotate_cols");
}
template <typename W> int set_column_w(void *dm, const void *da, long long rows, long long cols, long long col) {
    auto &c = ctx();
    set_column_kernel<<<rows_blocks(rows, kRowThreads, c.sm_count), kRowThreads, 0, c.stream>>>(
        (W *)dm, (const W *)da, rows, cols, col);
    return done(cudaGetLastError(), "msl_set_column");
}

int check_shape(const char *what, long long rows, long long cols) {
    if (rows <= 0 || cols <= 0) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: empty matrix %lld x %lld", what, rows, cols);
    if (rows > (1LL << 40) / cols) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: matrix too large", what);
    return MSL_OK;
}

int element_bytes(int dtype) {
    switch (dtype) {
        case MSL_F32:
        case MSL_I32: return 4;
        case MSL_F64: return 8;
        case MSL_BF16: return 2;
    }
    return 0;
}

// Copy dispatch by element size.
#define MSL_BY_SIZE(fn, bytes, ...)                                  \
    ((bytes) == 4   ? fn<uint32_t>(__VA_ARGS__)                       \
     : (bytes) == 8 ? fn<unsigned long long>(__VA_ARGS__)             \
                    : fn<uint16_t>(__VA_ARGS__))

}  // namespace

extern "C" {

int msl_fold_rows(int dtype, int op, const void *in, long long rows, long long cols, int threads_per_block,
                  void *out) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_shape("msl_fold_rows", rows, cols)) return e;
    if (!in || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_rows: NULL pointer");
    if (threads_per_block < 1 || threads_per_block > 1024 || (threads_per_block & (threads_per_block - 1)))
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_rows: threads_per_block %d is not a power of two in [1, 1024]",
                        threads_per_block);
    switch (dtype) {
        case MSL_F32: return fold_rows_t<float>(op, in, out, rows, cols, threads_per_block);
        case MSL_F64: return fold_rows_t<double>(op, in, out, rows, cols, threads_per_block);
        case MSL_I32: return fold_rows_t<int32_t>(op, in, out, rows, cols, threads_per_block);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_rows: unsupported dtype %d", dtype);
}

int msl_fold_cols(int dtype, int op, const void *in, long long rows, long long cols, void *out) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_shape("msl_fold_cols", rows, cols)) return e;
    if (!in || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_cols: NULL pointer");
    switch (dtype) {
        case MSL_F32: return fold_cols_t<float>(op, in, out, rows, cols);
        case MSL_F64: return fold_cols_t<double>(op, in, out, rows, cols);
        case MSL_I32: return fold_cols_t<int32_t>(op, in, out, rows, cols);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_cols: unsupported dtype %d", dtype);
}

int msl_zip_rows(int dtype, int op, const void *m, const void *v, void *out, long long rows, long long cols) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_shape("msl_zip_rows", rows, cols)) return e;
    if (!m || !v || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip_rows: NULL pointer");
    switch (dtype) {
        case MSL_F32: return zip_rows_t<float>(op, m, v, out, rows, cols);
        case MSL_F64: return zip_rows_t<double>(op, m, v, out, rows, cols);
        case MSL_I32: return zip_rows_t<int32_t>(op, m, v, out, rows, cols);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip_rows: unsupported dtype %d", dtype);
}

int msl_rotate_rows(int dtype, const void *in, void *out, long long rows, long long cols, long long a) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_shape("msl_rotate_rows", rows, cols)) return e;
    const int bytes = element_bytes(dtype);
    if (!bytes) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_rotate_rows: unsupported dtype %d", dtype);
    if (!in || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_rotate_rows: NULL pointer");
    if (in == out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_rotate_rows: in and out must differ");
    const long long howmuch = a < 0 ? -a : a;
    if (howmuch > rows)  // RotateRowManyNotImplementedException (src/dm.cpp:1363-1368)
        return rt::fail(MSL_ERR_NOT_IMPLEMENTED, "msl_rotate_rows: |%lld| rows exceed the %lld rows", a, rows);
    long long s = a % rows;
    if (s < 0) s += rows;
    return MSL_BY_SIZE(rotate_rows_w, bytes, in, out, rows, cols, s);
}

int msl_rotate_cols(int dtype, const void *in, void *out, long long rows, long long cols, long long a) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_shape("msl_rotate_cols", rows, cols)) return e;
    const int bytes = element_bytes(dtype);
    if (!bytes) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_rotate_cols: unsupported dtype %d", dtype);
    if (!in || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_rotate_cols: NULL pointer");
    if (in == out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_rotate_cols: in and out must differ");
    long long s = a % cols;
    if (s < 0) s += cols;
    return MSL_BY_SIZE(rotate_cols_w, bytes, in, out, rows, cols, s);
}

int msl_set_column(int dtype, void *dm, const void *da, long long rows, long long cols, long long col) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_shape("msl_set_column", rows, cols)) return e;
    const int bytes = element_bytes(dtype);
    if (!bytes) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_column: unsupported dtype %d", dtype);
    if (!dm || !da) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_column: NULL pointer");
    if (col < 0 || col >= cols)  // IndexOutOfBoundsException (src/dm.cpp:1858-1860)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_set_column: column %lld outside [0, %lld)", col, cols);
    return MSL_BY_SIZE(set_column_w, bytes, dm, da, rows, cols, col);
}

}  // extern "C"
