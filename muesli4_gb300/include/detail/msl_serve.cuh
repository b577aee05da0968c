// Device side of the stencil-solve server: the 3-D counterpart of the batched
// 2-D rounds (msl_batch.cuh). Every active heat3D request's cube is cut into
// 64 x 16 x 8 blocks; a persistent kernel takes (request, block) items
// round-robin and advances each block one sweep (buf[cur] -> buf[cur ^ 1]);
// the last CTA of each launch then advances the sweep counts and, on check
// sweeps, takes the per-request FP64 residuals. 2-D Jacobi requests use
// batch_round_kernel (same fused finalize) and, when both iterates fit in
// shared memory, batch_resident_kernel (one launch per check interval).
#pragma once

#include "msl_batch.cuh"
#include "msl_stencil3d_tb.cuh"

namespace msl {
namespace gpu {

struct ServeCube {
    void *buf[2];
    int depth, rows, cols;
    int cur, done;
    long long iters;
    double residual;
    unsigned long long resid_bits;
    long long first_block;  // prefix of block counts over the active list
};

// heat3D (examples/heatdiffusion.cpp:55-65), Dirichlet 0 outside the cube.
struct Heat7Fn {
    static constexpr bool kStar7 = true;
    static constexpr bool kSum7Div6 = true;
    __device__ __forceinline__ float sum7(float w, float e, float n, float s, float b, float f) const {
        float v = 0.0f;
        v = __fadd_rn(v, w);
        v = __fadd_rn(v, e);
        v = __fadd_rn(v, n);
        v = __fadd_rn(v, s);
        v = __fadd_rn(v, b);
        return __fadd_rn(v, f);
    }
    __device__ __forceinline__ float star7(float w, float e, float n, float s, float b, float f) const {
        return div6_rn(sum7(w, e, n, s, b, f));
    }
    template <class V> __device__ __forceinline__ float operator()(const V &c, int x, int y, int z) const {
        return star7(c(x - 1, y, z), c(x + 1, y, z), c(x, y - 1, z), c(x, y + 1, z), c(x, y, z - 1), c(x, y, z + 1));
    }
};

// After a sweep: advance the sweep counts and, on a check sweep, take the
// residuals and retire converged cubes. Run by one whole CTA.
MSL_DEV void serve3d_finalize_body(ServeCube *cubes, const int *list, int nlist, int check, double tol,
                                   long long max_iters) {
    for (int i = threadIdx.x; i < nlist; i += blockDim.x) {
        ServeCube &cb = cubes[list[i]];
        if (cb.done) continue;
        cb.iters += 1;
        cb.cur ^= 1;
        if (check) {
            const double r = __longlong_as_double((long long)cb.resid_bits);
            cb.residual = r;
            cb.resid_bits = 0ull;
            if (!(r > tol)) cb.done = 1;
        }
        if (cb.iters >= max_iters) cb.done = 1;
    }
}

static __global__ void __launch_bounds__(kT3Threads, 3)
    serve3d_round_kernel(ServeCube *cubes, const int *list, const int *block_cube, long long total_blocks, int check,
                         unsigned *ticket, int nlist, double tol, long long max_iters) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *box = reinterpret_cast<float *>(smem_raw + kStHeader);
    const int r = 1, hx = halo_x<float>(1);
    const int pitch = kT3BX + 2 * hx, th = kT3BY + 2 * r, tz = kT3BZ + 2 * r;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Heat7Fn fn;
    for (long long item = blockIdx.x; item < total_blocks; item += gridDim.x) {
        ServeCube &cb = cubes[list[block_cube[item]]];  // block_cube: list position of the block's cube
        if (cb.done) continue;  // uniform for the CTA
        const int depth = cb.depth, rows = cb.rows, cols = cb.cols;
        const int bx = (cols + kT3BX - 1) / kT3BX, by = (rows + kT3BY - 1) / kT3BY;
        const unsigned b = (unsigned)(item - cb.first_block);  // < 2^31 cells / 8192 per block
        const unsigned bxy = (unsigned)bx * (unsigned)by, bz = b / bxy, rem = b - bz * bxy, byy = rem / (unsigned)bx;
        const int x0 = (int)(rem - byy * (unsigned)bx) * kT3BX, y0 = (int)byy * kT3BY, z0 = (int)bz * kT3BZ;
        const float *in = (const float *)cb.buf[cb.cur];
        float *out = (float *)cb.buf[cb.cur ^ 1];
        const int wx0 = x0 - hx, wy0 = y0 - r, wz0 = z0 - r;
        __syncthreads();  // the previous item's readers are done with the box
        stage_window<float>(box, in, pitch, th, th * tz, wx0, wy0, wz0, depth, rows, cols);
        __syncthreads();
        // The staged box holds zeros outside the cube (Dirichlet 0), so every
        // block runs the 7-point register path; boundary blocks mask stores.
        const int x = x0 + (warp % (kT3BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kT3BX / 32)) * kT3RPT;
        const bool interior = wx0 >= 0 && wy0 >= 0 && wz0 >= 0 && wx0 + pitch <= cols && wy0 + th <= rows &&
                              wz0 + tz <= depth;
        double dmax = 0.0;
        if (interior)
            star7_block<float, true>(fn, box, pitch, pitch * th, x - wx0, ys - wy0, z0 - wz0, x, ys, z0, depth, rows,
                                     cols, out, check != 0, dmax);
        else
            star7_block<float, false>(fn, box, pitch, pitch * th, x - wx0, ys - wy0, z0 - wz0, x, ys, z0, depth, rows,
                                      cols, out, check != 0, dmax);
        if (check) {
            dmax = block_max(dmax);
            if (threadIdx.x == 0) atomic_max_nonneg(&cb.resid_bits, dmax);
        }
    }
    // The last CTA to finish advances the counts (one launch per sweep).
    if (last_cta_arrives(ticket)) serve3d_finalize_body(cubes, list, nlist, check, tol, max_iters);
}

inline size_t serve3d_smem() {
    return (size_t)kStHeader + (size_t)(kT3BX + 2 * halo_x<float>(1)) * (kT3BY + 2) * (kT3BZ + 2) * sizeof(float);
}

}  // namespace gpu
}  // namespace msl
