// plmatrix.h -- the legacy 2-D stencil view of DM::mapStencilMM (drop-in for
// include/plmatrix.h:49-181): get(row, col) returns the input cell, or, for a
// cell outside the matrix, the neutral value -- a scalar, or the value a
// neutral-value functor gives for that (row, col). On GB300 it is a thin
// wrapper over the NPLMatrix tile view, so mapStencilMM runs on the same
// TMA-staged kernel as mapStencil (no padded copy of the matrix, no per-call
// allocation).
#pragma once
#include "detail/msl_stencil.cuh"

namespace msl {

// The cells within `r` of a rows x cols matrix that lie outside it, as one
// array: the top band (rows -r..-1, cols -r..cols+r-1), the bottom band
// (rows rows..rows+r-1, same columns), then per matrix row its r cells on the
// left and r cells on the right.
struct HaloRing {
    int rows, cols, r;
    __host__ __device__ __forceinline__ long long band() const { return (long long)cols + 2 * r; }
    __host__ __device__ __forceinline__ long long size() const { return 2LL * r * band() + 2LL * r * rows; }
    // Index of (row, col), or -1 when the cell is inside the matrix or
    // farther than r from it.
    __host__ __device__ __forceinline__ long long index(int row, int col) const {
        if (row < -r || row >= rows + r || col < -r || col >= cols + r) return -1;
        if (row < 0) return (long long)(row + r) * band() + (col + r);
        if (row >= rows) return (long long)r * band() + (long long)(row - rows) * band() + (col + r);
        if (col >= 0 && col < cols) return -1;
        return 2LL * r * band() + (long long)row * 2 * r + (col < 0 ? col + r : r + (col - cols));
    }
    // (row, col) of element k (0 <= k < size()).
    __host__ __device__ __forceinline__ void cell(long long k, int &row, int &col) const {
        const long long top = (long long)r * band();
        if (k < top) {
            row = (int)(k / band()) - r;
            col = (int)(k % band()) - r;
        } else if (k < 2 * top) {
            k -= top;
            row = rows + (int)(k / band());
            col = (int)(k % band()) - r;
        } else {
            k -= 2 * top;
            row = (int)(k / (2 * r));
            const int j = (int)(k % (2 * r));
            col = j < r ? j - r : cols + (j - r);
        }
    }
};

template <typename T> class PLMatrix {
   public:
    __host__ __device__ __forceinline__ explicit PLMatrix(const NPLMatrix<T> &view) : view_(view) {}
    // With a halo: cells outside the matrix within the ring's radius read the
    // neutral-value functor's values stored in `halo` (HaloRing order).
    __host__ __device__ __forceinline__ PLMatrix(const NPLMatrix<T> &view, const T *halo, int r)
        : view_(view), halo_(halo), r_(r) {}
    __host__ __device__ __forceinline__ T get(int row, int col) const {
        // Interior tiles (check_ false) never read outside the matrix.
        if (halo_ && view_.check_ && ((unsigned)row >= (unsigned)view_.height || (unsigned)col >= (unsigned)view_.width)) {
            const long long k = HaloRing{view_.height, view_.width, r_}.index(row, col);
            return k >= 0 ? halo_[k] : view_.neutralValue;
        }
        return view_(col, row);
    }
    __host__ __device__ __forceinline__ int getRows() const { return view_.height; }
    __host__ __device__ __forceinline__ int getCols() const { return view_.width; }

   private:
    const NPLMatrix<T> &view_;
    const T *halo_ = nullptr;
    int r_ = 0;
};

}  // namespace msl
