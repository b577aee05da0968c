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
    void *buf[2];           // the two iterates (storage type); defect correction: the two corrections (BF16)
    int rows, cols;
    int cur;                // which buffer holds the latest iterate
    int done;               // converged or out of sweeps
    long long iters;        // sweeps performed
    double residual;        // FP64 max |last - previous| at the last check
    unsigned long long resid_bits;  // per-round residual slot (atomic max of double bits)
    long long first_tile;   // prefix of tile counts (work-list grids only)
    // Defect correction only: the FP32 solution (two buffers, ucur the
    // latest) and the BF16 defect of the last cycle.
    void *u[2];
    void *rhs;
    int ucur;
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
    static constexpr bool kStripAnyTile = true;  // strip() reads the window only and handles the edges
    static constexpr bool kPairStrip = true;     // FP32 grids: packed pairs (jacobi_pair_strip)
    template <class V, typename T> __device__ __forceinline__ void strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) const {
        jacobi_strip_window(m, x, y0, out);
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

// Defect correction (FP32 solution u, BF16-stored correction d and defect
// r): a cycle of L sweeps first applies the previous cycle's correction,
// u <- u + d, and takes the FP64 defect r = J(u) - u of the result (its
// max-norm is the residual checked against the tolerance); then it solves the
// correction equation d = A d + r (A: the Jacobi average of the four
// neighbours, zero on the boundary) by L - 1 sweeps from d = r. In exact
// arithmetic u + d then equals u after L Jacobi sweeps; the BF16 rounding of
// d and r is relative to the correction, which shrinks as u converges, so u
// converges to FP32 accuracy although the sweeps move 16-bit values.
//
// The correction sweep: boundary cells stay 0, inside cells take
// heat5(W, E, N, S) + r, both in FP32.
struct DefectFn {
    static constexpr bool kStrip2 = true;
    static constexpr bool kStripAnyTile = true;  // strip() reads the window (and r) only and handles the edges
    const bf16s *rhs;
    int cols;
    template <class V> __device__ __forceinline__ auto operator()(const V &m, int x, int y) const -> decltype(m(x, y)) {
        using T = decltype(m(x, y));
        if (x == 0 || y == 0 || x == m.width - 1 || y == m.height - 1) return T(0);
        const T v = heat5_value<T>(m(x - 1, y), m(x + 1, y), m(x, y - 1), m(x, y + 1));
        return Arith<T>::add(v, bf16_to_f(rhs[(size_t)y * cols + x]));
    }
    // kSt2RPT cells of column x from row y0, as operator() computes them.
    template <class V, typename T> __device__ __forceinline__ void strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) const {
        const auto *p = m.window_at(x, y0 - 1);
        const int pitch = m.pitch_;
        T c[kSt2RPT + 2];
#pragma unroll
        for (int k = 0; k < kSt2RPT + 2; k++) c[k] = gpu::widen(p[k * pitch]);
        const bool xb = x <= 0 || x >= m.width - 1;
#pragma unroll
        for (int j = 0; j < kSt2RPT; j++) {
            const int y = y0 + j;
            out[j] = T(0);
            if (!(xb || y <= 0 || y >= m.height - 1)) {
                const auto *q = p + (j + 1) * pitch;
                const T v = heat5_value<T>(gpu::widen(q[-1]), gpu::widen(q[1]), c[j], c[j + 2]);
                out[j] = Arith<T>::add(v, bf16_to_f(rhs[(size_t)y * cols + x]));
            }
        }
    }
};
// The defect of one inside cell of the corrected solution v (FP32 values):
// (((W + E) + N) + S) * 0.25 - v in FP64.
MSL_DEV double defect_f64(float w, float e, float n, float s, float c) {
    double j = __dadd_rn((double)w, (double)e);
    j = __dadd_rn(j, (double)n);
    j = __dadd_rn(j, (double)s);
    return __dsub_rn(__dmul_rn(j, 0.25), (double)c);
}

// The functor a round kernel applies to a grid.
struct JacobiSel {
    static MSL_DEV JacobiFn make(const BatchGrid &) { return JacobiFn{}; }
};
struct DefectSel {
    static MSL_DEV DefectFn make(const BatchGrid &g) { return DefectFn{(const bf16s *)g.rhs, g.cols}; }
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

// Tile height of the work-list rounds: FP32 Jacobi rounds (packed-pair
// strips) take 64 x 64 tiles -- less halo recomputed per useful update, and
// the strips of a sweep fill the CTA's passes better -- the others 64 x 32.
template <typename S, class Sel> constexpr int batch_tile_rows() {
    return std::is_same<S, float>::value && std::is_same<Sel, JacobiSel>::value ? 64 : kSt2BY;
}

// One round of the work-list grids: every tile of every unfinished grid does
// `depth` sweeps from buf[cur] to buf[cur ^ 1] (each grid's own direction, so
// grids that joined at different times can share a round). Plain coalesced loads
// stage the windows (grids differ in pointer and shape). `check` marks the
// round whose last sweep ends a residual-check chunk.
template <typename S, class Sel = JacobiSel>
__global__ void __launch_bounds__(kSt2Threads)
    batch_round_kernel(BatchGrid *grids, const int *list, const int *tile_grid, long long total_tiles, int depth,
                       int check, unsigned *ticket, int nlist, double tol, long long max_iters, int *active) {
    using T = typename Compute<S>::type;
    constexpr int BY = batch_tile_rows<S, Sel>();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int r = 1;
    const int hx = halo_x<S>(depth * r);
    const int pitch = kSt2BX + 2 * hx, th = BY + 2 * depth * r;
    const int buf_elems = (pitch * th * (int)sizeof(S) + 127) / 128 * 128 / (int)sizeof(S);
    S *buf0 = reinterpret_cast<S *>(smem_raw + kStHeader);
    S *buf1 = buf0 + buf_elems;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long item = blockIdx.x; item < total_tiles; item += gridDim.x) {
        BatchGrid &g = grids[list[tile_grid[item]]];  // tile_grid: work-list position of the tile's grid
        if (g.done) continue;  // uniform for the CTA
        const auto fn = Sel::make(g);
        const int rows = g.rows, cols = g.cols;
        const int tiles_x = (cols + kSt2BX - 1) / kSt2BX;
        const unsigned t = (unsigned)(item - g.first_tile);  // < 2^30 cells / 2048 per tile
        const int x0 = (int)(t % (unsigned)tiles_x) * kSt2BX, y0 = (int)(t / (unsigned)tiles_x) * BY;
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
        tb_inner_sweeps<S, BY>(fn, m, buf0, buf1, x0, y0, rows, cols, r, depth, pitch, wx0, wy0);
        const int x = x0 + (warp % (kSt2BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kSt2BX / 32)) * kSt2RPT;
        double dmax = 0.0;
        if constexpr (has_pair_strip<std::remove_cv_t<decltype(fn)>>::value && std::is_same<S, float>::value) {
            jacobi_pair_block(reinterpret_cast<const float *>(m.tile_), pitch, wx0, wy0, x0, y0, rows, cols,
                              reinterpret_cast<float *>(out), check != 0, dmax, BY);
        } else if (x0 - r >= 0 && y0 - r >= 0 && x0 + kSt2BX + r <= cols && y0 + BY + r <= rows) {
            m.check_ = false;
            stencil2d_strip<S, true>(fn, m, x, ys, rows, cols, out, check != 0, dmax);
        } else {
            m.check_ = !has_any_tile_strip<std::remove_cv_t<decltype(fn)>>::value;
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

// ---- defect correction ------------------------------------------------------------

// The step that opens a cycle, for every tile of every unfinished work-list
// grid: v = u + d over the tile and a one-cell halo (FP32), written to the
// other solution buffer; r = J(v) - v in FP64 for the tile's inside cells,
// stored as BF16 both as the defect and as the first correction d = r; the
// tile's max |r| into the grid's residual slot.
static __global__ void __launch_bounds__(kSt2Threads)
    batch_defect_kernel(BatchGrid *grids, const int *list, const int *tile_grid, long long total_tiles) {
    constexpr int hu = 4, hd = 8;  // x halos of the two windows, 16-byte multiples
    constexpr int pu = kSt2BX + 2 * hu, pd = kSt2BX + 2 * hd, th = kSt2BY + 2;
    __shared__ __align__(16) float su[th * pu];
    __shared__ __align__(16) bf16s sd[th * pd];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long item = blockIdx.x; item < total_tiles; item += gridDim.x) {
        BatchGrid &g = grids[list[tile_grid[item]]];
        if (g.done) continue;
        const int rows = g.rows, cols = g.cols;
        const int tiles_x = (cols + kSt2BX - 1) / kSt2BX;
        const unsigned t = (unsigned)(item - g.first_tile);
        const int x0 = (int)(t % (unsigned)tiles_x) * kSt2BX, y0 = (int)(t / (unsigned)tiles_x) * kSt2BY;
        const float *u = (const float *)g.u[g.ucur];
        float *u_out = (float *)g.u[g.ucur ^ 1];
        const bf16s *d = (const bf16s *)g.buf[g.cur];
        bf16s *d_out = (bf16s *)g.buf[g.cur ^ 1];  // neighbouring tiles still read d
        bf16s *rhs = (bf16s *)g.rhs;
        __syncthreads();
        stage_window<float>(su, u, pu, th, th, x0 - hu, y0 - 1, 0, 1, rows, cols);
        stage_window<bf16s>(sd, d, pd, th, th, x0 - hd, y0 - 1, 0, 1, rows, cols);
        __syncthreads();
        for (int k = threadIdx.x; k < th * pu; k += blockDim.x) {  // v = u + d (zero outside the grid)
            const int yy = k / pu, xx = k - yy * pu;
            su[k] = __fadd_rn(su[k], bf16_to_f(sd[yy * pd + xx - hu + hd]));
        }
        __syncthreads();
        double dmax = 0.0;
        const int x = x0 + (warp % (kSt2BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kSt2BX / 32)) * kSt2RPT;
        if (x < cols) {
#pragma unroll
            for (int j = 0; j < kSt2RPT; j++) {
                const int y = ys + j;
                if (y >= rows) break;
                const float *c = su + (y - y0 + 1) * pu + (x - x0 + hu);
                double dd = 0.0;
                if (x > 0 && y > 0 && x < cols - 1 && y < rows - 1) {
                    dd = defect_f64(c[-1], c[1], c[-pu], c[pu], c[0]);
                    if (fabs(dd) > dmax || dd != dd) dmax = fabs(dd);
                }
                const size_t o = (size_t)y * cols + x;
                const bf16s rb = f_to_bf16(__double2float_rn(dd));
                u_out[o] = c[0];
                rhs[o] = rb;
                d_out[o] = rb;
            }
        }
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(&g.resid_bits, dmax);
    }
}

// After the cycle-opening step: switch to the corrected solution and check
// the residual; a grid that goes on counts the sweep that produced d = r.
static __global__ void batch_defect_finalize_kernel(BatchGrid *grids, const int *list, int nlist, double tol,
                                                    long long max_iters, int *active) {
    __shared__ int s_active;
    if (threadIdx.x == 0) s_active = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nlist; i += blockDim.x) {
        BatchGrid &g = grids[list[i]];
        if (g.done) continue;
        g.ucur ^= 1;
        g.cur ^= 1;
        const double r = __longlong_as_double((long long)g.resid_bits);
        g.residual = r;
        g.resid_bits = 0ull;
        if (!(r > tol) || g.iters >= max_iters) g.done = 1;
        else g.iters += 1;
        if (!g.done) atomicAdd(&s_active, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) *active = s_active;
}
// After a correction round of `depth` sweeps.
static __global__ void batch_defect_round_finalize_kernel(BatchGrid *grids, const int *list, int nlist, int depth) {
    for (int i = threadIdx.x; i < nlist; i += blockDim.x) {
        BatchGrid &g = grids[list[i]];
        if (g.done) continue;
        g.iters += depth;
        g.cur ^= 1;
    }
}

constexpr int kBatchDefectMaxCycle = 64;

// Resident grids under defect correction: one CTA per grid holds u (FP32),
// both corrections and the defect (BF16) in shared memory and runs whole
// cycles until the residual check passes or max_iters sweeps are done; the
// solution is stored into u[0].
static __global__ void __launch_bounds__(kBatchResidentThreads)
    batch_resident_defect_kernel(BatchGrid *grids, const int *list, double tol, long long max_iters, int cycle) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    BatchGrid &g = grids[list[blockIdx.x]];
    if (g.done) return;
    const int rows = g.rows, cols = g.cols, n = rows * cols;
    const int nf = (n * 4 + 127) / 128 * 32, nb = (n * 2 + 127) / 128 * 64;
    float *su = reinterpret_cast<float *>(smem_raw);
    bf16s *sd[2] = {reinterpret_cast<bf16s *>(su + nf), reinterpret_cast<bf16s *>(su + nf) + nb};
    bf16s *sr = sd[1] + nb;
    const float *ug = (const float *)g.u[g.ucur];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        su[i] = ug[i];
        sd[0][i] = bf16s{0};  // no pending correction at the start of a solve
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    NPLMatrix<float, bf16s> m;
    m.width = cols;
    m.height = rows;
    m.stencilSize = 1;
    m.neutralValue = 0.0f;
    m.global_ = nullptr;
    m.ox_ = 0;
    m.oy_ = 0;
    m.pitch_ = cols;
    m.tile_h_ = rows;
    m.check_ = false;  // the functor reads neighbours of inside cells only
    const DefectFn fn{sr, cols};
    long long it = g.iters;
    double res = g.residual;
    __shared__ int s_stop;
    for (;;) {
        // open a cycle: u <- u + d, r = J(u) - u, d = r
        for (int i = threadIdx.x; i < n; i += blockDim.x) su[i] = __fadd_rn(su[i], bf16_to_f(sd[0][i]));
        __syncthreads();
        double dmax = 0.0;
        for (int y = warp; y < rows; y += nwarps)
            for (int x = lane; x < cols; x += 32) {
                const int k = y * cols + x;
                double dd = 0.0;
                if (x > 0 && y > 0 && x < cols - 1 && y < rows - 1) {
                    dd = defect_f64(su[k - 1], su[k + 1], su[k - cols], su[k + cols], su[k]);
                    if (fabs(dd) > dmax || dd != dd) dmax = fabs(dd);
                }
                const bf16s rb = f_to_bf16(__double2float_rn(dd));
                sr[k] = rb;
                sd[0][k] = rb;
            }
        dmax = block_max(dmax);
        if (threadIdx.x == 0) {
            res = dmax;
            s_stop = !(dmax > tol) || it >= max_iters;
        }
        __syncthreads();
        if (s_stop) break;
        it += 1;
        int c = 0;
        for (int s = 1; s < cycle; s++) {
            m.tile_ = sd[c];
            bf16s *dst = sd[c ^ 1];
            for (int y = warp; y < rows; y += nwarps)
                for (int x = lane; x < cols; x += 32) dst[y * cols + x] = narrow<bf16s>(fn(m, x, y));
            __syncthreads();
            c ^= 1;
        }
        it += cycle - 1;
        if (c) {  // keep the correction in sd[0]
            for (int i = threadIdx.x; i < n; i += blockDim.x) sd[0][i] = sd[1][i];
            __syncthreads();
        }
    }
    float *dst_g = (float *)g.u[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst_g[i] = su[i];
    if (threadIdx.x == 0) {
        g.ucur = 0;
        g.iters = it;
        g.residual = res;
        g.done = 1;
    }
}

}  // namespace gpu
}  // namespace msl
