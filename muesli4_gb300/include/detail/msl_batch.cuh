// Batched plain-Jacobi solves: many independent grids of uneven size advance
// together until each reaches its residual tolerance.
//
// The reference has no batching: each DM::mapStencil call sweeps one grid
// (src/dm.cpp:1535-1591) and examples/jacobisolver.cpp:127-140 checks the
// residual with a separate zip + fold every 50 sweeps. Here:
//  * grids small enough to sit in one CTA's shared memory (both iterates) are
//    solved by batch_resident_kernel: one CTA per grid iterates in shared
//    memory and touches HBM only to load the grid and store the result;
//  * the other grids share one tile work-list: batch_round_kernel is a
//    persistent kernel whose CTAs take (grid, 64x32 tile) items round-robin and
//    advance each tile `depth` sweeps with temporal blocking; batch_finalize
//    then updates every grid's sweep count, residual and convergence. A host
//    loop of (round, finalize) pairs is captured once in a CUDA graph and
//    replayed until every grid has converged.
// Every grid is iterated exactly as msl_stencil2d_iterate would iterate it
// alone (same functor, same sweeps, residual = max |last - previous| in FP64
// every `check_every` sweeps), so results are bit-identical to the
// one-grid-at-a-time path and do not depend on what else is in the batch.
#pragma once

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

struct BatchGrid {
    void *buf[2];           // the two iterates (storage type)
    int rows, cols;
    int cur;                // which buffer holds the latest iterate
    int done;               // converged or out of sweeps
    long long iters;        // sweeps performed
    double residual;        // FP64 max |last - previous| at the last check
    unsigned long long resid_bits;  // per-round residual slot (atomic max of double bits)
    long long first_tile;   // prefix of tile counts (work-list grids only)
};

// True in every thread of the CTA that finishes last among the launch's CTAs
// (a ticket taken after a fence, so the other CTAs' writes are visible to
// it); that CTA resets the ticket for the next launch.
MSL_DEV bool last_cta_arrives(unsigned *ticket) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        if (threadIdx.x == 0) *ticket = 0u;
    }
    return s_last != 0;
}

// After a round: advance the sweep counts and, on a check round, take the
// residuals and retire converged grids (and grids out of sweeps). Counts the
// grids still running into *active. Run by one whole CTA.
MSL_DEV void batch_finalize_body(BatchGrid *grids, const int *list, int nlist, int depth, int check, double tol,
                                 long long max_iters, int *active) {
    __shared__ int s_active;
    if (threadIdx.x == 0) s_active = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nlist; i += blockDim.x) {
        BatchGrid &g = grids[list[i]];
        if (g.done) continue;
        g.iters += depth;
        g.cur ^= 1;
        if (check) {
            double r = __longlong_as_double((long long)g.resid_bits);
            g.residual = r;
            g.resid_bits = 0ull;
            if (!(r > tol)) g.done = 1;
        }
        if (g.iters >= max_iters) g.done = 1;
        if (!g.done) atomicAdd(&s_active, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) *active = s_active;
}

// The plain-Jacobi functor: boundary cells keep their value, inside cells
// take (((0 + W) + E) + N) + S times 0.25 (heatdiffusion order; x*0.25 == x/4).
struct JacobiFn {
    static constexpr bool kStrip2 = true;
    template <class V, typename T> __device__ __forceinline__ void strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) const {
        heat5_strip<true>(m, x, y0, out);
    }
    template <class V> __device__ __forceinline__ auto operator()(const V &m, int x, int y) const -> decltype(m(x, y)) {
        using T = decltype(m(x, y));
        if (x == 0 || y == 0 || x == m.width - 1 || y == m.height - 1) return m(x, y);
        T v = T(0);
        v = Arith<T>::add(v, m(x - 1, y));
        v = Arith<T>::add(v, m(x + 1, y));
        v = Arith<T>::add(v, m(x, y - 1));
        v = Arith<T>::add(v, m(x, y + 1));
        return Arith<T>::mul(v, T(0.25));
    }
};

constexpr int kBatchResidentThreads = 512;

// One CTA per grid in `list`: load the latest iterate into shared memory,
// sweep until the residual check passes, max_iters sweeps are done or this
// launch's max_sweeps have run (a multiple of check_every), store the result
// into buf[0].
template <typename S>
__global__ void __launch_bounds__(kBatchResidentThreads)
    batch_resident_kernel(BatchGrid *grids, const int *list, double tol, long long max_iters, int check_every,
                          long long max_sweeps) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    BatchGrid &g = grids[list[blockIdx.x]];
    if (g.done) return;  // converged or out of sweeps in an earlier solve
    const int rows = g.rows, cols = g.cols, n = rows * cols;
    const int n_pad = (n * (int)sizeof(S) + 127) / 128 * 128 / (int)sizeof(S);
    S *bufs[2] = {reinterpret_cast<S *>(smem_raw), reinterpret_cast<S *>(smem_raw) + n_pad};
    const S *src_g = (const S *)g.buf[g.cur];
    for (int i = threadIdx.x; i < n; i += blockDim.x) bufs[0][i] = src_g[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    NPLMatrix<T, S> m;
    m.width = cols;
    m.height = rows;
    m.stencilSize = 1;
    m.neutralValue = T(0);
    m.global_ = nullptr;
    m.ox_ = 0;
    m.oy_ = 0;
    m.pitch_ = cols;
    m.tile_h_ = rows;
    m.check_ = false;  // the Jacobi functor reads neighbours of inside cells only
    JacobiFn fn;
    int c = 0;
    long long it = g.iters;  // a multiple of check_every: checks stay on the same sweeps
    const long long it_end = max_sweeps < max_iters - it ? it + max_sweeps : max_iters;  // this launch's sweeps
    double res = g.residual;
    bool converged = false;
    __shared__ int s_stop;
    while (it < it_end) {
        const long long k = min((long long)check_every, it_end - it);
        double dmax = 0.0;
        for (long long s = 0; s < k; s++) {
            m.tile_ = bufs[c];
            S *dst = bufs[c ^ 1];
            const bool last = s == k - 1;
            for (int y = warp; y < rows; y += nwarps)
                for (int x = lane; x < cols; x += 32) {
                    const S v = narrow<S>(fn(m, x, y));
                    dst[y * cols + x] = v;
                    if (last) {
                        const double d = fabs(stored_f64(v) - stored_f64(bufs[c][y * cols + x]));
                        if (d > dmax || d != d) dmax = d;
                    }
                }
            __syncthreads();
            c ^= 1;
        }
        it += k;
        dmax = block_max(dmax);
        if (threadIdx.x == 0) {
            res = dmax;
            s_stop = !(dmax > tol);  // NaN keeps iterating until max_iters
        }
        __syncthreads();
        if (s_stop) {
            converged = true;
            break;
        }
    }
    S *dst_g = (S *)g.buf[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst_g[i] = bufs[c][i];
    if (threadIdx.x == 0) {
        g.cur = 0;
        g.iters = it;
        g.residual = res;
        g.done = converged || it >= max_iters;
    }
}

// One round of the work-list grids: every tile of every unfinished grid does
// `depth` sweeps from buf[cur] to buf[cur ^ 1] (each grid's own direction, so
// grids that joined at different times can share a round). Plain coalesced loads
// stage the windows (grids differ in pointer and shape). `check` marks the
// round whose last sweep ends a residual-check chunk.
template <typename S>
__global__ void __launch_bounds__(kSt2Threads)
    batch_round_kernel(BatchGrid *grids, const int *list, const int *tile_grid, long long total_tiles, int depth,
                       int check, unsigned *ticket, int nlist, double tol, long long max_iters, int *active) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int r = 1;
    const int hx = halo_x<S>(depth * r);
    const int pitch = kSt2BX + 2 * hx, th = kSt2BY + 2 * depth * r;
    const int buf_elems = (pitch * th * (int)sizeof(S) + 127) / 128 * 128 / (int)sizeof(S);
    S *buf0 = reinterpret_cast<S *>(smem_raw + kStHeader);
    S *buf1 = buf0 + buf_elems;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    JacobiFn fn;
    for (long long item = blockIdx.x; item < total_tiles; item += gridDim.x) {
        BatchGrid &g = grids[list[tile_grid[item]]];  // tile_grid: work-list position of the tile's grid
        if (g.done) continue;  // uniform for the CTA
        const int rows = g.rows, cols = g.cols;
        const int tiles_x = (cols + kSt2BX - 1) / kSt2BX;
        const unsigned t = (unsigned)(item - g.first_tile);  // < 2^30 cells / 2048 per tile
        const int x0 = (int)(t % (unsigned)tiles_x) * kSt2BX, y0 = (int)(t / (unsigned)tiles_x) * kSt2BY;
        const S *in = (const S *)g.buf[g.cur];
        S *out = (S *)g.buf[g.cur ^ 1];
        const int wx0 = x0 - hx, wy0 = y0 - depth * r;
        __syncthreads();  // previous item's readers are done with the buffers
        stage_window<S>(buf0, in, pitch, th, th, wx0, wy0, 0, 1, rows, cols);
        __syncthreads();
        NPLMatrix<T, S> m;
        m.width = cols;
        m.height = rows;
        m.stencilSize = r;
        m.neutralValue = T(0);
        m.tile_ = buf0;
        m.global_ = in;
        m.ox_ = wx0;
        m.oy_ = wy0;
        m.pitch_ = pitch;
        m.tile_h_ = th;
        tb_inner_sweeps<S>(fn, m, buf0, buf1, x0, y0, rows, cols, r, depth, pitch, wx0, wy0);
        const int x = x0 + (warp % (kSt2BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kSt2BX / 32)) * kSt2RPT;
        double dmax = 0.0;
        if (x0 - r >= 0 && y0 - r >= 0 && x0 + kSt2BX + r <= cols && y0 + kSt2BY + r <= rows) {
            m.check_ = false;
            stencil2d_strip<S, true>(fn, m, x, ys, rows, cols, out, check != 0, dmax);
        } else {
            m.check_ = true;
            stencil2d_strip<S, false>(fn, m, x, ys, rows, cols, out, check != 0, dmax);
        }
        if (check) {
            dmax = block_max(dmax);
            if (threadIdx.x == 0) atomic_max_nonneg(&g.resid_bits, dmax);
        }
    }
    // With a ticket the last CTA to finish also does batch_finalize's work
    // (one launch per round instead of two).
    if (ticket && last_cta_arrives(ticket)) batch_finalize_body(grids, list, nlist, depth, check, tol, max_iters, active);
}

static __global__ void batch_finalize_kernel(BatchGrid *grids, const int *list, int nlist, int depth,
                                      int check, double tol, long long max_iters, int *active) {
    batch_finalize_body(grids, list, nlist, depth, check, tol, max_iters, active);
}

}  // namespace gpu
}  // namespace msl
