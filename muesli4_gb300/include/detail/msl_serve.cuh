// Device side of the stencil-solve server: the 3-D counterpart of the batched
// 2-D rounds (msl_batch.cuh). Every active heat3D request's cube is cut into
// 64 x 16 x 8 blocks; a persistent kernel takes (request, block) items
// round-robin and advances each block one sweep (buf[cur] -> buf[cur ^ 1]);
// serve3d_finalize then advances the sweep counts and, on check sweeps, takes
// the per-request FP64 residuals. 2-D Jacobi requests use batch_round_kernel.
#pragma once

#include "msl_batch.cuh"

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
    template <class V> __device__ __forceinline__ float operator()(const V &c, int x, int y, int z) const {
        float v = 0.0f;
        v = __fadd_rn(v, c(x - 1, y, z));
        v = __fadd_rn(v, c(x + 1, y, z));
        v = __fadd_rn(v, c(x, y - 1, z));
        v = __fadd_rn(v, c(x, y + 1, z));
        v = __fadd_rn(v, c(x, y, z - 1));
        v = __fadd_rn(v, c(x, y, z + 1));
        return div6_rn(v);
    }
};

static __global__ void __launch_bounds__(kT3Threads, 3)
    serve3d_round_kernel(ServeCube *cubes, const int *list, const int *block_cube, long long total_blocks, int check) {
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
        const long long b = item - cb.first_block;
        const int x0 = (int)(b % bx) * kT3BX, y0 = (int)((b / bx) % by) * kT3BY, z0 = (int)(b / ((long long)bx * by)) * kT3BZ;
        const float *in = (const float *)cb.buf[cb.cur];
        float *out = (float *)cb.buf[cb.cur ^ 1];
        const int wx0 = x0 - hx, wy0 = y0 - r, wz0 = z0 - r;
        __syncthreads();  // the previous item's readers are done with the box
        for (int i = threadIdx.x; i < pitch * th * tz; i += blockDim.x) {
            const int zz = i / (pitch * th), rem = i - zz * pitch * th, yy = rem / pitch, xx = rem - yy * pitch;
            const int gx = wx0 + xx, gy = wy0 + yy, gz = wz0 + zz;
            box[i] = (gx >= 0 && gx < cols && gy >= 0 && gy < rows && gz >= 0 && gz < depth)
                         ? in[((size_t)gz * rows + gy) * cols + gx]
                         : 0.0f;
        }
        __syncthreads();
        PLCube<float> c;
        c.width = cols;
        c.height = rows;
        c.depth = depth;
        c.stencilSize = r;
        c.neutralValue = 0.0f;
        c.ring_ = box;
        c.global_ = in;
        c.ox_ = wx0;
        c.oy_ = wy0;
        c.oz_ = wz0;
        c.pitch_ = pitch;
        c.tile_h_ = th;
        c.plane_ = pitch * th;
        c.mask_ = -1;
        c.zlo_ = wz0;
        c.zhi_ = wz0 + tz - 1;
        c.check_ = true;
        const int x = x0 + (warp % (kT3BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kT3BX / 32)) * kT3RPT;
        double dmax = 0.0;
        stencil3d_block<float, false>(fn, c, x, ys, z0, depth, rows, cols, out, check != 0, dmax);
        if (check) {
            dmax = block_max(dmax);
            if (threadIdx.x == 0) atomic_max_nonneg(&cb.resid_bits, dmax);
        }
    }
}

static __global__ void serve3d_finalize_kernel(ServeCube *cubes, const int *list, int nlist, int check, double tol,
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

inline size_t serve3d_smem() {
    return (size_t)kStHeader + (size_t)(kT3BX + 2 * halo_x<float>(1)) * (kT3BY + 2) * (kT3BZ + 2) * sizeof(float);
}

}  // namespace gpu
}  // namespace msl
