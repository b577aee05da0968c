// plcube.h -- the 3-D stencil view (drop-in for include/plcube.h).
// msl::PLCube<T> is defined with the stencil kernels: public width, height,
// depth, stencilSize, neutralValue and operator()(x, y, z), which returns
// neutralValue outside the cube and otherwise the input cell, read from the
// ring of z-planes staged in shared memory.
#pragma once
#include "detail/msl_stencil.cuh"
