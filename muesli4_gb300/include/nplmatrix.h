// nplmatrix.h -- the 2-D stencil view (drop-in for include/nplmatrix.h).
// msl::NPLMatrix<T> is defined with the stencil kernels: public width,
// height, stencilSize, neutralValue and operator()(x, y), which returns
// neutralValue outside the grid and otherwise the input cell, read from the
// tile staged in shared memory.
#pragma once
#include "detail/msl_stencil.cuh"
