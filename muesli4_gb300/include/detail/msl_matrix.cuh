// Row/column skeletons of DM<T> and the DM x DA broadcast zips.
//
// Reference: DM::reduceRows (src/dm.cpp:1593-1725, foldRows/foldCols kernels
// src/fold_kernels.cu:131-296), DM::rotateRows / rotateCols
// (src/dm.cpp:1345-1533), DM::setColumn (src/dm.cpp:1856-1879), the DM x DA
// zips zipIndexInPlaceMA / A / AAA (src/dm.cpp:1757-1853, kernels
// src/zip_kernels.cu:45-71) and DA::mapIndexInPlaceDMRows /
// zipIndexInPlaceDMRows (src/da.cpp:256-324).
//
// Row folds: one warp per row, each lane folding a strided part of the row,
// then the element-seeded warp fold of msl_fold.cuh (the reference's
// foldRowsKernel is a shared-memory tree, also element-seeded). Column folds:
// one thread per column walking down the rows (coalesced across the warp).
// Rotations and setColumn are index-remapping copies.
#pragma once

#include "msl_elementwise.cuh"
#include "msl_fold.cuh"

namespace msl {
namespace gpu {

template <typename T, class F>
__global__ void fold_rows_kernel(const T *in, T *out, long long rows, long long cols, F f) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += warps) {
        const T *row = in + r * cols;
        T acc{};
        bool have = false;
        for (long long c = lane; c < cols; c += 32) fold_in(acc, have, row[c], true, f);
        warp_fold(acc, have, f);
        if (lane == 0 && have) out[r] = acc;
    }
}

template <typename T, class F>
__global__ void fold_cols_kernel(const T *in, T *out, long long rows, long long cols, F f) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += stride) {
        T acc = in[c];
        for (long long r = 1; r < rows; r++) acc = f(acc, in[r * cols + c]);
        out[c] = acc;
    }
}

// out row k = in row (k - a) mod rows (positive a rotates downwards).
template <typename T> __global__ void rotate_rows_kernel(const T *in, T *out, long long rows, long long cols, long long a) {
    const long long n = rows * cols, stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long long k = i / cols, c = i - k * cols;
        long long src = (k - a) % rows;
        if (src < 0) src += rows;
        out[i] = in[src * cols + c];
    }
}

// out column j = in column (j + a) mod cols (src/dm.cpp:1516-1527).
template <typename T> __global__ void rotate_cols_kernel(const T *in, T *out, long long rows, long long cols, long long a) {
    const long long n = rows * cols, stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long long k = i / cols, j = i - k * cols;
        long long src = (j + a) % cols;
        if (src < 0) src += cols;
        out[i] = in[k * cols + src];
    }
}

template <typename T> __global__ void set_column_kernel(T *dm, const T *da, long long rows, long long cols, long long col) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += stride) dm[r * cols + col] = da[r];
}

// Calls f(k) for every k in [0, n): the body of the DM x DA broadcast zips,
// whose operands are captured in f.
template <class F> __global__ void for_each_index_kernel(long long n, F f) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) f(k);
}

inline unsigned rows_blocks(long long units, int per_block, int sms) {
    long long b = (units + per_block - 1) / per_block;
    const long long cap = (long long)(sms > 0 ? sms : 152) * 8;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace gpu
}  // namespace msl
