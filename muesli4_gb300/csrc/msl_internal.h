// Internal host-side state shared by the translation units of libmsl_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstddef>
#include <mutex>

#include "../../include/msl_gb300.h"
#include "../include/detail/msl_fold.cuh"

namespace msl {
namespace rt {

// One process-wide context for the device bound by msl_init (the reference
// keeps the same kind of state in the static Muesli class, include/muesli.h:149-181).
struct Context {
    bool initialised = false;
    int device = -1;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;     // own_stream or a caller's stream
    void *scratch = nullptr;           // device: fold scratch | error word | residual slot
    gpu::FoldScratch fold;             // carved from scratch
    unsigned *err_word = nullptr;      // device error bits (gpu::kErrBarrierTimeout ...)
    unsigned long long *resid = nullptr;  // device residual slot (double bits)
    void *host_result = nullptr;       // pinned host slot for fold/residual results
    void *host_fold = nullptr;         // mapped pinned slot the fold kernel writes its result to
    void *host_fold_dev = nullptr;     // its device address
    std::atomic<unsigned long long> launches{0};
    std::recursive_mutex mu;           // serialises the ABI per context
};

Context &ctx();

// Record an error for msl_last_error_string() and return `code`.
int fail(int code, const char *fmt, ...);
// Map a CUDA error to MSL_ERR_CUDA (or OUT_OF_MEMORY) with a message.
int cuda_fail(cudaError_t e, const char *what);
// Common entry check: initialised, returns 0 or an error code.
int require_init();
// Read and clear the device error word (synchronises the stream).
int check_device_errors(const char *what);
inline void count_launch(unsigned n = 1) { ctx().launches.fetch_add(n, std::memory_order_relaxed); }

size_t dtype_size(int dtype);

// Host-side allocation fault injection (msl_debug_fail_allocs): true when the
// allocation about to be made must fail as out of memory. Consumes one
// allowed allocation otherwise.
bool alloc_fault();

// Autotuner table (autotune.cu): sweeps per launch recorded for a 2-D stencil
// of this element type, functor, radius and grid size; 1 when none is recorded.
int tuned_depth(int dtype, int kind, int rows, int cols, int radius);
// Tile height (16, 32 or 64 rows of 64 columns) recorded with that depth; 32
// when none is recorded.
int tuned_tile_rows(int dtype, int kind, int rows, int cols, int radius);

// msl_set_temporal_depth / msl_set_tile_rows as last set (0: automatic).
int temporal_depth_setting();
int tile_rows_setting();
// heat3D sweeps per launch (msl_set_stencil3d_depth, stencil.cu): nonzero when
// pairs of sweeps run on the z-marching kernel; its z planes per CTA (0: chosen
// per grid).
int stencil3d_pair_sweeps();
int stencil3d_zchunk();

}  // namespace rt
}  // namespace msl

#define MSL_TRY_CUDA(call, what)                                  \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return ::msl::rt::cuda_fail(_e, what); \
    } while (0)
