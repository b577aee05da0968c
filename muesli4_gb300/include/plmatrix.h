// plmatrix.h -- the legacy 2-D stencil view of DM::mapStencilMM (drop-in for
// include/plmatrix.h:49-181): get(row, col) returns the input cell, or the
// neutral value outside the matrix. On GB300 it is a thin wrapper over the
// NPLMatrix tile view, so mapStencilMM runs on the same TMA-staged kernel as
// mapStencil (no padded copy of the matrix, no per-call allocation).
#pragma once
#include "detail/msl_stencil.cuh"

namespace msl {

template <typename T> class PLMatrix {
   public:
    __host__ __device__ __forceinline__ explicit PLMatrix(const NPLMatrix<T> &view) : view_(view) {}
    __host__ __device__ __forceinline__ T get(int row, int col) const { return view_(col, row); }
    __host__ __device__ __forceinline__ int getRows() const { return view_.height; }
    __host__ __device__ __forceinline__ int getCols() const { return view_.width; }

   private:
    const NPLMatrix<T> &view_;
};

}  // namespace msl
