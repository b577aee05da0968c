// Element-wise skeletons of libmsl_gb300.so with the built-in functors of
// msl_gb300.h: map / mapInPlace, zip / zipInPlace, zipInPlace3, and the index
// map/zip of DA, DM and DC.
//
// Reference: DS::map/mapInPlace/zip/zipInPlace (src/ds.cpp:614-727);
// DA::mapIndex*/zipIndex*/zipInPlace3 (src/da.cpp:232-459);
// DM::mapIndex*/zipIndex* (src/dm.cpp:372-501); DC::mapIndex*/zipIndex*
// (src/dc.cpp:387-550); kernels src/map_kernels.cu:36-101, src/zip_kernels.cu:37-148.
#include "../include/detail/msl_elementwise.cuh"
#include "msl_internal.h"

using namespace msl;
using namespace msl::gpu;
using msl::rt::ctx;

namespace {

template <typename T> using A = Arith<T>;

// ---- built-in map / zip functors (the coordinate argument is ignored) --------------
template <typename T> struct MapAffine {
    T a, b;
    template <class S> __device__ __forceinline__ T operator()(S, T x) const { return A<T>::add(A<T>::mul(a, x), b); }
};
template <typename T> struct MapAbs {
    template <class S> __device__ __forceinline__ T operator()(S, T x) const { return x < T(0) ? A<T>::sub(T(0), x) : x; }
};
template <typename T> struct MapSquare {
    template <class S> __device__ __forceinline__ T operator()(S, T x) const { return A<T>::mul(x, x); }
};
template <typename T, int OP> struct ZipOp {
    template <class S> __device__ __forceinline__ T operator()(S, T a, T b) const {
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
template <typename T, int OP> struct Zip3Op {
    template <class S> __device__ __forceinline__ T operator()(S, T a, T b, T c) const {
        if constexpr (OP == MSL_ZIP3_MULADD) return A<T>::add(A<T>::mul(a, b), c);
        else return A<T>::add(A<T>::add(a, b), c);
    }
};

// ---- built-in index functors ------------------------------------------------------
// Coordinates in the reference's argument order.
__device__ __forceinline__ long long coord(const IdxFlat::S &s, int) { return s.i; }
__device__ __forceinline__ long long coord(const IdxRowCol::S &s, int k) { return k == 0 ? s.row : s.col; }
__device__ __forceinline__ long long coord(const IdxXYZ::S &s, int k) { return k == 0 ? s.x : (k == 1 ? s.y : s.z); }

template <typename T> __device__ __forceinline__ T from_coord(long long c) { return (T)c; }

template <typename T, int ND> struct IdxLinear {
    T p[ND + 2];
    template <class S> __device__ __forceinline__ T lin(const S &s) const {
        T acc = A<T>::mul(p[0], from_coord<T>(coord(s, 0)));
#pragma unroll
        for (int k = 1; k < ND; k++) acc = A<T>::add(acc, A<T>::mul(p[k], from_coord<T>(coord(s, k))));
        return acc;
    }
    template <class S> __device__ __forceinline__ T operator()(S s, T v) const {
        return A<T>::add(lin(s), A<T>::mul(p[ND], v));
    }
    template <class S> __device__ __forceinline__ T operator()(S s, T v, T w) const {
        return A<T>::add(A<T>::add(lin(s), A<T>::mul(p[ND], v)), A<T>::mul(p[ND + 1], w));
    }
};
template <typename T, int ND> struct IdxProduct {
    template <class S> __device__ __forceinline__ T prod(const S &s) const {
        T acc = from_coord<T>(coord(s, 0));
#pragma unroll
        for (int k = 1; k < ND; k++) acc = A<T>::mul(acc, from_coord<T>(coord(s, k)));
        return acc;
    }
    template <class S> __device__ __forceinline__ T operator()(S s, T v) const { return A<T>::mul(prod(s), v); }
    template <class S> __device__ __forceinline__ T operator()(S s, T v, T w) const {
        return A<T>::mul(A<T>::mul(prod(s), v), w);
    }
};
struct IdxXorMask {  // DA<int>: v ^ (i & mask)
    int32_t mask;
    __device__ __forceinline__ int32_t operator()(IdxFlat::S s, int32_t v) const {
        return v ^ (int32_t)((uint32_t)s.i & (uint32_t)mask);
    }
};
template <typename T, int ND> struct IdxBorder {
    T top, edge;
    long long d0, d1, d2;  // dims as passed: DA (n), DM (rows, cols), DC (depth, rows, cols)
    template <class S> __device__ __forceinline__ T operator()(S s, T v) const {
        bool is_top, is_edge;
        if constexpr (ND == 1) {
            is_top = coord(s, 0) == 0;
            is_edge = coord(s, 0) == d0 - 1;
        } else if constexpr (ND == 2) {
            is_top = coord(s, 0) == 0;
            is_edge = coord(s, 0) == d0 - 1 || coord(s, 1) == 0 || coord(s, 1) == d1 - 1;
        } else {
            is_top = coord(s, 1) == 0;
            is_edge = coord(s, 0) == 0 || coord(s, 0) == d2 - 1 || coord(s, 1) == d1 - 1 || coord(s, 2) == 0 ||
                      coord(s, 2) == d0 - 1;
        }
        return is_top ? top : (is_edge ? edge : v);
    }
};

template <typename T> T param(const double *p, int k) { return p ? (T)p[k] : T(0); }
template <> int32_t param<int32_t>(const double *p, int k) { return p ? (int32_t)(long long)p[k] : 0; }

int ew_status(cudaError_t e, const char *what) {
    if (e != cudaSuccess) return rt::cuda_fail(e, what);
    rt::count_launch();
    return MSL_OK;
}

template <typename T> int map_t(int op, const void *in, void *out, size_t n, const double *p) {
    auto &c = ctx();
    const T *a = (const T *)in;
    T *o = (T *)out;
    switch (op) {
        case MSL_MAP_AFFINE:
            return ew_status(launch_map(o, a, n, IdxNone{}, MapAffine<T>{param<T>(p, 0), param<T>(p, 1)}, c.stream, c.sm_count),
                             "msl_map");
        case MSL_MAP_ABS:
            return ew_status(launch_map(o, a, n, IdxNone{}, MapAbs<T>{}, c.stream, c.sm_count), "msl_map");
        case MSL_MAP_SQUARE:
            return ew_status(launch_map(o, a, n, IdxNone{}, MapSquare<T>{}, c.stream, c.sm_count), "msl_map");
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_map: unknown op %d", op);
}

template <typename T, int OP> int zip_op(const void *a, const void *b, void *out, size_t n) {
    auto &c = ctx();
    return ew_status(launch_zip((T *)out, (const T *)a, (const T *)b, n, IdxNone{}, ZipOp<T, OP>{}, c.stream, c.sm_count),
                     "msl_zip");
}
template <typename T> int zip_t(int op, const void *a, const void *b, void *out, size_t n) {
    switch (op) {
        case MSL_ZIP_ADD: return zip_op<T, MSL_ZIP_ADD>(a, b, out, n);
        case MSL_ZIP_SUB: return zip_op<T, MSL_ZIP_SUB>(a, b, out, n);
        case MSL_ZIP_MUL: return zip_op<T, MSL_ZIP_MUL>(a, b, out, n);
        case MSL_ZIP_MULADD: return zip_op<T, MSL_ZIP_MULADD>(a, b, out, n);
        case MSL_ZIP_ABSDIFF: return zip_op<T, MSL_ZIP_ABSDIFF>(a, b, out, n);
        case MSL_ZIP_MAX: return zip_op<T, MSL_ZIP_MAX>(a, b, out, n);
        case MSL_ZIP_MIN: return zip_op<T, MSL_ZIP_MIN>(a, b, out, n);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip: unknown op %d", op);
}
template <typename T> int zip3_t(int op, const void *a, const void *b, const void *cc, void *out, size_t n) {
    auto &c = ctx();
    if (op == MSL_ZIP3_MULADD)
        return ew_status(launch_zip3((T *)out, (const T *)a, (const T *)b, (const T *)cc, n, IdxNone{},
                                     Zip3Op<T, MSL_ZIP3_MULADD>{}, c.stream, c.sm_count),
                         "msl_zip3");
    if (op == MSL_ZIP3_SUM)
        return ew_status(launch_zip3((T *)out, (const T *)a, (const T *)b, (const T *)cc, n, IdxNone{},
                                     Zip3Op<T, MSL_ZIP3_SUM>{}, c.stream, c.sm_count),
                         "msl_zip3");
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip3: unknown op %d", op);
}

// Index skeletons: pick the coordinate generator from ndim, then the functor.
template <typename T, int ND, class Ix>
int index_nd(int op, const void *a, const void *b, void *out, size_t n, Ix ix, const long long *dims, const double *p) {
    auto &c = ctx();
    const T *x = (const T *)a;
    const T *y = (const T *)b;
    T *o = (T *)out;
    const char *what = b ? "msl_zip_index" : "msl_map_index";
    if (op == MSL_IDX_LINEAR) {
        IdxLinear<T, ND> f;
        for (int k = 0; k < ND + 2; k++) f.p[k] = param<T>(p, k);
        return ew_status(b ? launch_zip(o, x, y, n, ix, f, c.stream, c.sm_count) : launch_map(o, x, n, ix, f, c.stream, c.sm_count),
                         what);
    }
    if (op == MSL_IDX_PRODUCT) {
        IdxProduct<T, ND> f;
        return ew_status(b ? launch_zip(o, x, y, n, ix, f, c.stream, c.sm_count) : launch_map(o, x, n, ix, f, c.stream, c.sm_count),
                         what);
    }
    if (op == MSL_IDX_BORDER && !b) {
        IdxBorder<T, ND> f{param<T>(p, 0), param<T>(p, 1), dims[0], ND > 1 ? dims[1] : 0, ND > 2 ? dims[2] : 0};
        return ew_status(launch_map(o, x, n, ix, f, c.stream, c.sm_count), what);
    }
    if constexpr (ND == 1 && std::is_same<T, int32_t>::value) {
        if (op == MSL_IDX_XOR_MASK && !b)
            return ew_status(launch_map(o, x, n, ix, IdxXorMask{param<int32_t>(p, 0)}, c.stream, c.sm_count), what);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: op %d is not available for this element type / rank", what, op);
}

template <typename T>
int index_t(int op, const void *a, const void *b, void *out, int ndim, const long long *dims, const double *p) {
    if (ndim == 1) return index_nd<T, 1>(op, a, b, out, (size_t)dims[0], IdxFlat{0}, dims, p);
    if (ndim == 2) return index_nd<T, 2>(op, a, b, out, (size_t)(dims[0] * dims[1]), IdxRowCol{dims[1]}, dims, p);
    return index_nd<T, 3>(op, a, b, out, (size_t)(dims[0] * dims[1] * dims[2]), IdxXYZ{dims[2], dims[1]}, dims, p);
}

int check_index_args(const char *what, const void *a, const void *out, int ndim, const long long *dims) {
    if (ndim < 1 || ndim > 3 || !dims) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: ndim must be 1..3", what);
    long long n = 1;
    for (int k = 0; k < ndim; k++) {
        if (dims[k] < 0 || dims[k] > (1LL << 31) - 1)
            return rt::fail(MSL_ERR_SIZE_MISMATCH, "%s: dimension %d = %lld out of range", what, k, dims[k]);
        n *= dims[k];
    }
    if (n > 0 && (!a || !out)) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "%s: NULL pointer", what);
    return MSL_OK;
}

}  // namespace

extern "C" {

int msl_map(int dtype, int op, const void *in, void *out, size_t n, const double *params) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (n == 0) return MSL_OK;
    if (!in || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_map: NULL pointer");
    switch (dtype) {
        case MSL_F32: return map_t<float>(op, in, out, n, params);
        case MSL_F64: return map_t<double>(op, in, out, n, params);
        case MSL_I32: return map_t<int32_t>(op, in, out, n, params);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_map: unsupported dtype %d", dtype);
}

int msl_zip(int dtype, int op, const void *a, const void *b, void *out, size_t n) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (n == 0) return MSL_OK;
    if (!a || !b || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip: NULL pointer");
    switch (dtype) {
        case MSL_F32: return zip_t<float>(op, a, b, out, n);
        case MSL_F64: return zip_t<double>(op, a, b, out, n);
        case MSL_I32: return zip_t<int32_t>(op, a, b, out, n);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip: unsupported dtype %d", dtype);
}

int msl_zip3(int dtype, int op, const void *a, const void *b, const void *c, void *out, size_t n) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (n == 0) return MSL_OK;
    if (!a || !b || !c || !out) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip3: NULL pointer");
    switch (dtype) {
        case MSL_F32: return zip3_t<float>(op, a, b, c, out, n);
        case MSL_F64: return zip3_t<double>(op, a, b, c, out, n);
        case MSL_I32: return zip3_t<int32_t>(op, a, b, c, out, n);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip3: unsupported dtype %d", dtype);
}

int msl_map_index(int dtype, int op, const void *in, void *out, int ndim, const long long *dims, const double *params) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_index_args("msl_map_index", in, out, ndim, dims)) return e;
    switch (dtype) {
        case MSL_F32: return index_t<float>(op, in, nullptr, out, ndim, dims, params);
        case MSL_F64: return index_t<double>(op, in, nullptr, out, ndim, dims, params);
        case MSL_I32: return index_t<int32_t>(op, in, nullptr, out, ndim, dims, params);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_map_index: unsupported dtype %d", dtype);
}

int msl_zip_index(int dtype, int op, const void *a, const void *b, void *out, int ndim, const long long *dims,
                  const double *params) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (int e = rt::require_init()) return e;
    if (int e = check_index_args("msl_zip_index", a, out, ndim, dims)) return e;
    if (!b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip_index: NULL second input");
    if (op != MSL_IDX_LINEAR && op != MSL_IDX_PRODUCT)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip_index: op %d is not a zip-index functor", op);
    switch (dtype) {
        case MSL_F32: return index_t<float>(op, a, b, out, ndim, dims, params);
        case MSL_F64: return index_t<double>(op, a, b, out, ndim, dims, params);
        case MSL_I32: return index_t<int32_t>(op, a, b, out, ndim, dims, params);
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_zip_index: unsupported dtype %d", dtype);
}

}  // extern "C"
