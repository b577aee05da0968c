// Row/column skeletons of DM<T> and the DM x DA broadcast zips.
//
// Reference: DM::reduceRows (src/dm.cpp:1596-1707, foldRowsKernel
// src/fold_kernels.cu:215-294), DM::rotateRows / rotateCols
// (src/dm.cpp:1345-1533), DM::setColumn (src/dm.cpp:1856-1879), the DM x DA
// zips zipIndexInPlaceMA / A / AAA (src/dm.cpp:1757-1853, kernels
// src/zip_kernels.cu:45-71), DA::mapIndexInPlaceDMRows / zipIndexInPlaceDMRows
// (src/da.cpp:256-324, kernels src/map_kernels.cu:80-86,
// src/zip_kernels.cu:73-78).
//
// Layout: every kernel walks the matrix row by row. A row is given a segment
// of `seg` threads (a power of two <= the CTA size): a CTA covers
// blockDim.x / seg rows per pass and each segment thread strides over the
// row's columns, so row and column are known without a per-element division
// and the accesses of a warp stay on consecutive addresses.
//
// Row folds follow the reference's foldRowsKernel order exactly: with L lanes
// per row (a power of two, row_fold_lanes), lane t folds row[t], row[t + L],
// ... left to right, then the lane values are combined by the halving tree
// v[t] = f(v[t], v[t + h]) for h = L/2, ..., 1. The tree runs in shared
// memory down to 32 lanes and in warp shuffles below, which performs the
// same f calls on the same operands. Column folds run top to bottom,
// element-seeded, one thread per column.
#pragma once

#include "msl_elementwise.cuh"
#include "msl_fold.cuh"

namespace msl {
namespace gpu {

constexpr int kRowThreads = 256;

// Threads given to one row: the next power of two >= cols, at most the CTA.
inline int row_segment(long long cols) {
    int s = 1;
    while (s < cols && s < kRowThreads) s <<= 1;
    return s;
}

// Lanes per row of the reference's row fold: nextPow2((cols + 1) / 2) while
// cols < threads_per_block, else threads_per_block (src/dm.cpp:1679-1680).
inline int row_fold_lanes(long long cols, int threads_per_block) {
    if (cols >= threads_per_block) return threads_per_block;
    const long long half = (cols + 1) / 2;
    int p = 1;
    while (p < half) p <<= 1;
    return p;
}

inline unsigned rows_blocks(long long rows, int rows_per_block, int sms) {
    long long b = (rows + rows_per_block - 1) / rows_per_block;
    const long long cap = (long long)(sms > 0 ? sms : 152) * 16;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// Row fold with lanes <= 32: 32 / lanes rows per warp.
template <typename T, class F>
__global__ void fold_rows_warp_kernel(const T *in, T *out, long long rows, long long cols, int lanes, F f) {
    const int lane = threadIdx.x & 31, per_warp = 32 / lanes, g = lane / lanes, t = lane - g * lanes;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long base = warp * per_warp; base < rows; base += nwarps * per_warp) {  // warp-uniform
        const long long r = base + g;
        const bool live = r < rows;
        T acc{};
        if (live) {
            const T *row = in + r * cols;
            acc = row[t];  // lanes <= cols: every lane has a first element
            for (long long c = t + lanes; c < cols; c += lanes) acc = f(acc, row[c]);
        }
        for (int h = lanes >> 1; h > 0; h >>= 1) {
            const T o = shfl_down(acc, h, lanes);
            if (live && t < h) acc = f(acc, o);
        }
        if (live && t == 0) out[r] = acc;
    }
}

// Row fold with lanes in [64, 1024]: one CTA of `lanes` threads per row,
// dynamic shared memory of lanes * sizeof(T).
template <typename T, class F>
__global__ void fold_rows_block_kernel(const T *in, T *out, long long rows, long long cols, F f) {
    extern __shared__ __align__(16) unsigned char fold_rows_raw[];
    T *s = reinterpret_cast<T *>(fold_rows_raw);
    const int t = threadIdx.x, lanes = blockDim.x;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const T *row = in + r * cols;
        T acc = row[t];
        for (long long c = t + lanes; c < cols; c += lanes) acc = f(acc, row[c]);
        s[t] = acc;
        __syncthreads();
        for (int h = lanes >> 1; h >= 32; h >>= 1) {
            if (t < h) s[t] = f(s[t], s[t + h]);
            __syncthreads();
        }
        if (t < 32) {  // warp 0, all lanes present
            acc = s[t];
            for (int h = 16; h > 0; h >>= 1) {
                const T o = shfl_down(acc, h);
                if (t < h) acc = f(acc, o);
            }
            if (t == 0) out[r] = acc;
        }
        __syncthreads();  // s is reused by the next row
    }
}

// out[c] = f(...f(f(in[0][c], in[1][c]), in[2][c])..., in[rows-1][c]).
template <typename T, class F>
__global__ void fold_cols_kernel(const T *in, T *out, long long rows, long long cols, F f) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += stride) {
        T acc = in[c];
        for (long long r = 1; r < rows; r++) acc = f(acc, in[r * cols + c]);
        out[c] = acc;
    }
}

// Calls op(op.row(r), r, c) for every cell, `seg` threads per row. op.row(r)
// is evaluated once per row and thread (row base pointers, broadcast values).
template <class Op>
__global__ void __launch_bounds__(kRowThreads) row_cells_kernel(long long rows, long long cols, int seg, Op op) {
    const int per = blockDim.x / seg, g = threadIdx.x / seg, t = threadIdx.x - g * seg;
    for (long long r = (long long)blockIdx.x * per + g; r < rows; r += (long long)gridDim.x * per) {
        const auto row = op.row(r);
        for (long long c = t; c < cols; c += seg) op(row, r, c);
    }
}

template <class Op> cudaError_t launch_row_cells(long long rows, long long cols, Op op, cudaStream_t s, int sms) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    const int seg = row_segment(cols);
    row_cells_kernel<<<rows_blocks(rows, kRowThreads / seg, sms), kRowThreads, 0, s>>>(rows, cols, seg, op);
    return cudaGetLastError();
}

// out row k = in row (k - a) mod rows: positive a moves rows down
// (src/dm.cpp:1376-1475, with the wrap-around rows taken from the other end).
template <typename T> struct RotateRowsOp {
    const T *in;
    T *out;
    long long rows, cols, a;  // 0 <= a < rows
    struct Row { const T *src; T *dst; };
    __device__ __forceinline__ Row row(long long r) const {
        long long s = r - a;
        if (s < 0) s += rows;
        return Row{in + s * cols, out + r * cols};
    }
    __device__ __forceinline__ void operator()(const Row &w, long long, long long c) const { w.dst[c] = w.src[c]; }
};

// out column j = in column (j + a) mod cols (src/dm.cpp:1503-1527).
template <typename T> struct RotateColsOp {
    const T *in;
    T *out;
    long long cols, a;  // 0 <= a < cols
    __device__ __forceinline__ long long row(long long r) const { return r * cols; }
    __device__ __forceinline__ void operator()(long long base, long long, long long c) const {
        long long s = c + a;
        if (s >= cols) s -= cols;
        out[base + c] = in[base + s];
    }
};

// Broadcast zip out[r][c] = f(m[r][c], v[r]) of a matrix with a per-row vector.
template <typename T, class F> struct ZipRowsOp {
    const T *m, *v;
    T *out;
    long long cols;
    F f;
    struct Row { long long base; T x; };
    __device__ __forceinline__ Row row(long long r) const { return Row{r * cols, v[r]}; }
    __device__ __forceinline__ void operator()(const Row &w, long long, long long c) const {
        out[w.base + c] = f(m[w.base + c], w.x);
    }
};

// dm[r][col] = da[r] (src/dm.cpp:1856-1879, kernel detail::setColumn).
template <typename T> __global__ void set_column_kernel(T *dm, const T *da, long long rows, long long cols, long long col) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += stride) dm[r * cols + col] = da[r];
}

// Calls f(k) for every k in [0, n) (the DA-sized skeletons that pass a row of
// a DM by pointer).
template <class F> __global__ void for_each_index_kernel(long long n, F f) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) f(k);
}

template <class F> cudaError_t launch_for_each_index(long long n, F f, cudaStream_t s, int sms) {
    if (n <= 0) return cudaSuccess;
    for_each_index_kernel<<<rows_blocks(n, kRowThreads, sms), kRowThreads, 0, s>>>(n, f);
    return cudaGetLastError();
}

// Row fold launch: out[r] = fold of row r with threads_per_block as the
// reference's lane count (a power of two in [1, 1024]).
template <typename T, class F>
cudaError_t launch_fold_rows(const T *in, T *out, long long rows, long long cols, int threads_per_block, F f,
                             cudaStream_t s, int sms) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    const int lanes = row_fold_lanes(cols, threads_per_block);
    if (lanes <= 32) {
        const int rows_per_block = (kRowThreads / 32) * (32 / lanes);
        fold_rows_warp_kernel<<<rows_blocks(rows, rows_per_block, sms), kRowThreads, 0, s>>>(in, out, rows, cols,
                                                                                           lanes, f);
    } else {
        const unsigned blocks = rows_blocks(rows, 1, sms * 2);
        fold_rows_block_kernel<<<blocks, lanes, (size_t)lanes * sizeof(T), s>>>(in, out, rows, cols, f);
    }
    return cudaGetLastError();
}

template <typename T, class F>
cudaError_t launch_fold_cols(const T *in, T *out, long long rows, long long cols, F f, cudaStream_t s, int sms) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    fold_cols_kernel<<<rows_blocks(cols, kRowThreads, sms), kRowThreads, 0, s>>>(in, out, rows, cols, f);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
