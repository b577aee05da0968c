// Stencil skeletons: DM::mapStencil (2-D) and DC::mapStencil (3-D).
//
// Reference (include/detail/map_kernels.cuh:140-168, src/dm.cpp:1535-1591,
// src/dc.cpp:559-592): one thread per cell in a 1-D grid; every neighbour
// read goes through NPLMatrix/PLCube::operator(), a branchy bounds check plus
// a global load (include/nplmatrix.h:123-139, include/plcube.h:105-119).
//
// Here the halo handling becomes a tile staged in shared memory:
//  * 2-D: each CTA owns a 64 x 32 block of outputs; one TMA 2-D load
//    (cp.async.bulk.tensor.2d, completion on an mbarrier) brings the block
//    plus its halo into shared memory; each thread evaluates the functor for a
//    vertical strip of 8 cells of one column (a warp covers 32 consecutive
//    columns, so shared-memory reads are conflict-free and global stores are
//    coalesced).
//  * 3-D: each CTA owns a 64 x 32 column of the cube for a chunk of planes and
//    marches along z with a ring of shared-memory planes (2r+1 in use, one in
//    flight), one TMA 3-D load per plane.
// The functor sees the same view type the reference passes (NPLMatrix /
// PLCube): public width/height[/depth], neutralValue, stencilSize and
// operator()(x, y[, z]) that returns neutralValue outside the grid and reads
// every other cell from shared memory. As in the reference -- whose halo
// buffers hold exactly stencilSize rows/planes (include/dm.h:224-291) -- a
// functor must read only within the radius it declares; defining
// MSL_STENCIL_CHECK_RADIUS makes the view test that and serve reads beyond the
// staged window from global memory instead. Tiles whose staged window lies
// inside the grid run the functor with the bounds test compiled out, so an
// interior read is one shared-memory load at an offset the compiler can fold
// and reuse across the vertically adjacent cells a thread computes. Where TMA
// cannot address the grid (row pitch not a multiple of 16
// bytes, misaligned base, oversized halo) the same kernel stages the window
// with plain coalesced loads.
//
// Optional fused residual: max |new - old| over the sweep, in FP64, reduced in
// the CTA and folded into one device word with an atomic max (non-negative
// doubles order like their bit patterns).
#pragma once

#include <cuda.h>

#include <algorithm>
#include <type_traits>

#include "msl_device.cuh"

namespace msl {

// ---- views (the types user stencil functors receive) ---------------------------
// T is the arithmetic type the functor sees, S the storage type (S == T except
// for bfloat16 storage, where T is float).
template <typename T, typename S = T> class NPLMatrix {
   public:
    int width = 0, height = 0;
    int stencilSize = 0;
    T neutralValue{};
    // staging window: tile_[ty * pitch_ + tx] holds cell (ox_ + tx, oy_ + ty)
    const S *tile_ = nullptr;
    const S *global_ = nullptr;
    int ox_ = 0, oy_ = 0, pitch_ = 0, tile_h_ = 0;
    bool check_ = true;

    __host__ __device__ __forceinline__ T operator()(int x, int y) const {
#ifdef MSL_STENCIL_CHECK_RADIUS
        const unsigned tx = (unsigned)(x - ox_), ty = (unsigned)(y - oy_);
        if (!(tx < (unsigned)pitch_ && ty < (unsigned)tile_h_)) {  // beyond the declared radius
            if ((unsigned)x < (unsigned)width && (unsigned)y < (unsigned)height)
                return gpu::widen<S>(global_[(size_t)y * width + x]);
            return neutralValue;
        }
#endif
        if (check_ && ((unsigned)x >= (unsigned)width || (unsigned)y >= (unsigned)height)) return neutralValue;
        return gpu::widen<S>(tile_[(y - oy_) * pitch_ + (x - ox_)]);
    }
    // Unchecked access for strip functors (valid while check_ is false: the
    // staged window then holds every cell the functor reads): the window
    // address of cell (x, y); rows are pitch_ apart.
    __host__ __device__ __forceinline__ const S *window_at(int x, int y) const {
        return tile_ + (y - oy_) * pitch_ + (x - ox_);
    }
};

template <typename T, typename S = T> class PLCube {
   public:
    int width = 0, height = 0, depth = 0;
    int stencilSize = 0;
    T neutralValue{};
    // ring of planes: plane z lives in slot (z & mask_) - oz_ while zlo_ <= z <= zhi_
    const S *ring_ = nullptr;
    const S *global_ = nullptr;
    int ox_ = 0, oy_ = 0, pitch_ = 0, tile_h_ = 0, plane_ = 0, mask_ = 0, zlo_ = 0, zhi_ = -1;
    int oz_ = 0;  // plane index of slot 0 when the planes form a linear box (mask_ = -1)
    bool check_ = true;

    __host__ __device__ __forceinline__ T operator()(int x, int y, int z) const {
#ifdef MSL_STENCIL_CHECK_RADIUS
        const unsigned tx = (unsigned)(x - ox_), ty = (unsigned)(y - oy_);
        if (!(tx < (unsigned)pitch_ && ty < (unsigned)tile_h_ && z >= zlo_ && z <= zhi_)) {
            if ((unsigned)x < (unsigned)width && (unsigned)y < (unsigned)height && (unsigned)z < (unsigned)depth)
                return gpu::widen<S>(global_[((size_t)z * height + y) * width + x]);
            return neutralValue;
        }
#endif
        if (check_ && ((unsigned)x >= (unsigned)width || (unsigned)y >= (unsigned)height || (unsigned)z >= (unsigned)depth))
            return neutralValue;
        return gpu::widen<S>(ring_[((z & mask_) - oz_) * plane_ + (y - oy_) * pitch_ + (x - ox_)]);
    }
};

namespace gpu {

constexpr int kSt2BX = 64, kSt2BY = 32, kSt2RPT = 8, kSt2Threads = 256;
constexpr int kSt3BX = 64, kSt3BY = 32, kSt3RPT = 8, kSt3Threads = 256;
constexpr int kStHeader = 128;  // mbarriers live in the first 128 bytes of dynamic smem

// Halo in x, rounded up to 16 bytes so that a TMA box starting at x0 - hx keeps
// its innermost coordinate 16-byte aligned (x0 is a multiple of 64).
template <typename S> MSL_HD int halo_x(int r) {
    const int q = (int)(16 / sizeof(S));
    return (r + q - 1) / q * q;
}

// Stage a window of `nrows` rows (pitch elements each) with plain coalesced
// loads: window row k is grid row (wy0 + k % th) of plane (wz0 + k / th); the
// elements outside the grid become zero. Each warp takes kStageRows rows at a
// time and every lane issues all of its loads for them (up to kStageRows x
// kStageCols) before the first store, so the loads' latencies overlap instead
// of adding up row after row. Windows wider than 32 * kStageCols take a
// row-at-a-time loop.
constexpr int kStageRows = 4, kStageCols = 4;

template <typename S>
MSL_DEV void stage_window(S *dst, const S *in, int pitch, int th, int nrows, int wx0, int wy0, int wz0, int depth,
                          int rows, int cols) {
    // A single-plane window inside the grid whose rows start 16-byte aligned
    // in global and shared memory: 16-byte copies without per-element tests,
    // four loads in flight per thread. (dst is 16-byte aligned.)
    constexpr int kV = 16 / (int)sizeof(S);
    if (nrows == th && wz0 == 0 && depth == 1 && wx0 >= 0 && wy0 >= 0 && wx0 + pitch <= cols &&
        wy0 + nrows <= rows && (wx0 % kV) == 0 && (pitch % kV) == 0 && (cols % kV) == 0 &&
        ((uintptr_t)in % 16) == 0) {
        const int vpr = pitch / kV, total = nrows * vpr;  // 16-byte vectors per row, in the window
        const int q = (int)blockDim.x / vpr, rq = (int)blockDim.x - q * vpr;
        int k = (int)threadIdx.x / vpr, v = (int)threadIdx.x - k * vpr;  // row and vector of item threadIdx.x
        for (int i = threadIdx.x; i < total; i += 4 * (int)blockDim.x) {
            uint4 val[4];
            int kk[4], vv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                kk[u] = k;
                vv[u] = v;
                if (i + u * (int)blockDim.x < total)
                    val[u] = *reinterpret_cast<const uint4 *>(in + (size_t)(wy0 + k) * cols + wx0 + v * kV);
                k += q;  // next item: i + blockDim.x
                v += rq;
                if (v >= vpr) {
                    v -= vpr;
                    k++;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (i + u * (int)blockDim.x < total) reinterpret_cast<uint4 *>(dst + kk[u] * pitch)[vv[u]] = val[u];
        }
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    auto row_src = [&](int k, bool &row_in) {
        const int zz = k / th, gy = wy0 + (k - zz * th), gz = wz0 + zz;
        row_in = gy >= 0 && gy < rows && gz >= 0 && gz < depth;
        return in + ((size_t)(row_in ? gz : 0) * rows + (row_in ? gy : 0)) * cols;
    };
    if (pitch > 32 * kStageCols) {
        for (int k = warp; k < nrows; k += nwarps) {
            bool row_in;
            const S *src = row_src(k, row_in);
            S *d = dst + (size_t)k * pitch;
            for (int xx = lane; xx < pitch; xx += 32) {
                const int gx = wx0 + xx;
                d[xx] = (row_in && gx >= 0 && gx < cols) ? src[gx] : S{};
            }
        }
        return;
    }
    for (int k0 = warp * kStageRows; k0 < nrows; k0 += nwarps * kStageRows) {
        S v[kStageRows][kStageCols];
#pragma unroll
        for (int u = 0; u < kStageRows; u++) {
            bool row_in = false;
            const S *src = k0 + u < nrows ? row_src(k0 + u, row_in) : in;
#pragma unroll
            for (int q = 0; q < kStageCols; q++) {
                const int xx = lane + 32 * q, gx = wx0 + xx;
                v[u][q] = (row_in && xx < pitch && gx >= 0 && gx < cols) ? src[gx] : S{};
            }
        }
#pragma unroll
        for (int u = 0; u < kStageRows; u++) {
            if (k0 + u >= nrows) break;
            S *d = dst + (size_t)(k0 + u) * pitch;
#pragma unroll
            for (int q = 0; q < kStageCols; q++)
                if (lane + 32 * q < pitch) d[lane + 32 * q] = v[u][q];
        }
    }
}

// heat2D of one cell from its four neighbours: (((0 + W) + E) + N) + S, then
// times 0.25 (== / 4 for every value: both round the same real number once).
template <typename T> MSL_DEV T heat5_value(T w, T e, T n, T s) {
    T v = T(0);
    v = Arith<T>::add(v, w);
    v = Arith<T>::add(v, e);
    v = Arith<T>::add(v, n);
    v = Arith<T>::add(v, s);
    return Arith<T>::mul(v, T(0.25));
}

// kSt2RPT cells of column x from row y0 of the 5-point heat2D stencil
// (JACOBI: boundary cells of the grid keep their value): the column's
// kSt2RPT + 2 values are read once and serve as N, S and centre of the cells.
template <bool JACOBI, class V, typename T>
MSL_DEV void heat5_strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) {
    if (!m.check_) {
        // the window holds every cell read: address it directly (one pointer,
        // row offsets by pitch) instead of through the view's checks
        const auto *p = m.window_at(x, y0 - 1);
        const int pitch = m.pitch_;
        T c[kSt2RPT + 2];
#pragma unroll
        for (int k = 0; k < kSt2RPT + 2; k++) c[k] = gpu::widen(p[k * pitch]);
        const bool edge = JACOBI && (x == 0 || x == m.width - 1 || y0 == 0 || y0 + kSt2RPT >= m.height);
        if (!edge) {
#pragma unroll
            for (int j = 0; j < kSt2RPT; j++) {
                const auto *q = p + (j + 1) * pitch;
                out[j] = heat5_value<T>(gpu::widen(q[-1]), gpu::widen(q[1]), c[j], c[j + 2]);
            }
            return;
        }
    }
    T c[kSt2RPT + 2];
#pragma unroll
    for (int k = 0; k < kSt2RPT + 2; k++) c[k] = m(x, y0 - 1 + k);
    const bool xb = JACOBI && (x == 0 || x == m.width - 1);
#pragma unroll
    for (int j = 0; j < kSt2RPT; j++) {
        const int y = y0 + j;
        if (JACOBI && (xb || y == 0 || y == m.height - 1)) out[j] = c[j + 1];
        else out[j] = heat5_value<T>(m(x - 1, y), m(x + 1, y), c[j], c[j + 2]);
    }
}

// Functors may provide strip(view, x, y0, vals) computing kSt2RPT vertically
// adjacent cells at once (register reuse); others are called per cell.
template <class F, class = void> struct has_strip2 : std::false_type {};
template <class F> struct has_strip2<F, decltype((void)F::kStrip2, void())> : std::true_type {};
// Functors whose strip() reads only the staged window and handles the grid's
// edges itself (kStripAnyTile): boundary tiles then take the strip path too,
// with the view's bounds test off. The window must hold finite values
// wherever it lies outside the grid (staging writes zeros there).
template <class F, class = void> struct has_any_tile_strip : std::false_type {};
template <class F>
struct has_any_tile_strip<F, std::void_t<decltype(F::kStripAnyTile)>> : std::bool_constant<F::kStripAnyTile> {};

// Plain Jacobi for kSt2RPT cells of column x from row y0, read from the
// window only: every cell takes heat2D of its window neighbours, then cells on
// the grid's edge keep their value (cells outside the grid get their window
// value and are never stored). Inside cells read only cells of the grid, so
// the result is that of the checked path.
template <class V, typename T> MSL_DEV void jacobi_strip_window(const V &m, int x, int y0, T (&out)[kSt2RPT]) {
    const auto *p = m.window_at(x, y0 - 1);
    const int pitch = m.pitch_;
    T c[kSt2RPT + 2];
#pragma unroll
    for (int k = 0; k < kSt2RPT + 2; k++) c[k] = gpu::widen(p[k * pitch]);
    const bool xb = x <= 0 || x >= m.width - 1;
#pragma unroll
    for (int j = 0; j < kSt2RPT; j++) {
        const auto *q = p + (j + 1) * pitch;
        const T v = heat5_value<T>(gpu::widen(q[-1]), gpu::widen(q[1]), c[j], c[j + 2]);
        const int y = y0 + j;
        out[j] = (xb || y <= 0 || y >= m.height - 1) ? c[j + 1] : v;
    }
}

// Functors that are plain Jacobi on FP32 cells may declare kPairStrip: the
// temporal-blocking sweeps then run jacobi_pair_strip on packed pairs of
// columns instead of strip() column by column (same values, bit for bit).
template <class F, class = void> struct has_pair_strip : std::false_type {};
template <class F>
struct has_pair_strip<F, std::void_t<decltype(F::kPairStrip)>> : std::bool_constant<F::kPairStrip> {};
constexpr int kPairRows = 4;

// Plain Jacobi for the cells (x, y0 + k) and (x + 1, y0 + k), k < kPairRows,
// read from the window only (p: the window address of (x, y0), 8-byte
// aligned; rows pitch apart): heat2D of the four neighbours, (((0 + W) + E) +
// N) + S times 0.25, two cells per add.rn/fma.rn.f32x2, computed as
// fma(((W + E) + N) + S, 0.25, +0): the sums differ only when all four terms
// are -0 (-0 against +0), and adding +0 after the exact product turns that -0
// into +0 without changing any other result; then cells on the
// grid's edge -- and cells outside the grid, which are never stored -- keep
// their value, as jacobi_strip_window computes them one by one. c returns the
// cells' previous values. no_edge: the caller knows that no cell of the strip
// lies on or beyond the grid's edge (the edge test is skipped).
MSL_DEV void jacobi_pair_strip(const float *p, int pitch, int x, int y0, int cols, int rows,
                               f32x2 (&c)[kPairRows], f32x2 (&v)[kPairRows], bool no_edge = false) {
    const f32x2 n = ld_pair(p - pitch), s = ld_pair(p + kPairRows * pitch);
#pragma unroll
    for (int k = 0; k < kPairRows; k++) c[k] = ld_pair(p + k * pitch);
#pragma unroll
    for (int k = 0; k < kPairRows; k++) {
        const f32x2 w = pk2(p[k * pitch - 1], lo2(c[k]));
        const f32x2 e = pk2(hi2(c[k]), p[k * pitch + 2]);
        f32x2 t = add2(w, e);
        t = add2(t, k == 0 ? n : c[k - 1]);
        t = add2(t, k == kPairRows - 1 ? s : c[k + 1]);
        v[k] = fma2(t, pk2(0.25f, 0.25f), pk2(0.0f, 0.0f));
    }
    if (no_edge || (x >= 1 && x + 2 <= cols - 1 && y0 >= 1 && y0 + kPairRows <= rows - 1)) return;  // no edge cell
    const bool xb0 = x <= 0 || x >= cols - 1, xb1 = x + 1 <= 0 || x + 1 >= cols - 1;
#pragma unroll
    for (int k = 0; k < kPairRows; k++) {
        const int y = y0 + k;
        const bool yb = y <= 0 || y >= rows - 1;
        v[k] = pk2((xb0 || yb) ? lo2(c[k]) : lo2(v[k]), (xb1 || yb) ? hi2(c[k]) : hi2(v[k]));
    }
}

// The sweep of a 64 x by block to global memory on packed pairs: lane l of
// warp w owns columns x0 + 2 l and the next of the strips of rows y0 +
// kPairRows (w + k nwarps). win: the window holding the sweep's input (origin
// wx0, wy0). With want, the FP64 max |new - old| of the stored cells into
// dmax.
MSL_DEV void jacobi_pair_block(const float *win, int pitch, int wx0, int wy0, int x0, int y0, int rows, int cols,
                               float *out, bool want, double &dmax, int by) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int x = x0 + 2 * lane;
    const bool pairs = (cols & 1) == 0 && ((uintptr_t)out & 7) == 0 && x + 1 < cols;
    for (int sidx = warp; sidx < by / kPairRows; sidx += nwarps) {
        const int y = y0 + kPairRows * sidx;
        f32x2 c[kPairRows], v[kPairRows];
        jacobi_pair_strip(win + (y - wy0) * pitch + (x - wx0), pitch, x, y, cols, rows, c, v);
#pragma unroll
        for (int k = 0; k < kPairRows; k++) {
            if (y + k >= rows || x >= cols) break;
            float *o = out + (size_t)(y + k) * cols + x;
            if (want) {
                const double d0 = fabs((double)lo2(v[k]) - (double)lo2(c[k]));
                if (d0 > dmax || d0 != d0) dmax = d0;
                if (x + 1 < cols) {
                    const double d1 = fabs((double)hi2(v[k]) - (double)hi2(c[k]));
                    if (d1 > dmax || d1 != d1) dmax = d1;
                }
            }
            if (pairs) {
                st_pair(o, v[k]);
            } else {
                o[0] = lo2(v[k]);
                if (x + 1 < cols) o[1] = hi2(v[k]);
            }
        }
    }
}

MSL_DEV void atomic_max_nonneg(unsigned long long *slot, double v) {
    atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}
MSL_DEV double block_max(double v) {
    __shared__ double s[32];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, v, d);
        v = (o > v || o != o) ? o : v;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s[warp] = v;
    __syncthreads();
    v = 0.0;
    if (warp == 0) {
        if (lane < (int)(blockDim.x >> 5)) v = s[lane];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            double o = __shfl_down_sync(0xffffffffu, v, d);
            v = (o > v || o != o) ? o : v;
        }
    }
    return v;
}
template <typename S> MSL_DEV double stored_f64(S s) { return (double)s; }
template <> MSL_DEV double stored_f64<bf16s>(bf16s s) { return (double)bf16_to_f(s); }

// The kSt2RPT vertically adjacent outputs of one thread. All values are
// computed before any is stored: the stores go to global memory, which the
// compiler cannot prove disjoint from the staged tile, so computing first lets
// it share the tile loads of neighbouring outputs. FULL: the whole strip lies
// inside the grid (interior tiles), so no row/column guards are needed.
template <typename S, bool FULL, class Fn, class View>
MSL_DEV void stencil2d_strip(const Fn &fn, const View &m, int x, int ys, int rows, int cols, S *out, bool want,
                             double &dmax) {
    using T = typename Compute<S>::type;
    if (!FULL && x >= cols) return;
    T vals[kSt2RPT];
    if constexpr (has_strip2<Fn>::value) {
        fn.strip(m, x, ys, vals);
    } else {
#pragma unroll
        for (int j = 0; j < kSt2RPT; j++)
            if (FULL || ys + j < rows) vals[j] = fn(m, x, ys + j);
    }
    if (want) {
#pragma unroll
        for (int j = 0; j < kSt2RPT; j++)
            if (FULL || ys + j < rows) {
                const double d = fabs(stored_f64(narrow<S>(vals[j])) - (double)m(x, ys + j));
                if (d > dmax || d != d) dmax = d;
            }
    }
    S *o = out + (size_t)ys * cols + x;
#pragma unroll
    for (int j = 0; j < kSt2RPT; j++)
        if (FULL || ys + j < rows) o[(size_t)j * cols] = narrow<S>(vals[j]);
}

// Sweeps 1 .. depth-1 of a temporally blocked 64 x 32 tile whose window
// (pitch wide, origin (wx0, wy0)) is staged in buf0: sweep s computes the
// block grown by (depth - s) * r on every side into the other buffer, so the
// last sweep (left to the caller) has all the cells it reads. On return
// m.tile_ points at the buffer holding sweep depth-1 (buf0 when depth == 1).
template <typename S, int BY = kSt2BY, class Fn>
MSL_DEV void tb_inner_sweeps(const Fn &fn, NPLMatrix<typename Compute<S>::type, S> &m, S *buf0, S *buf1, int x0,
                             int y0, int rows, int cols, int r, int depth, int pitch, int wx0, int wy0) {
    using T = typename Compute<S>::type;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    S *dst = buf1;
    for (int s = 1; s < depth; s++) {
        const int ext = (depth - s) * r;  // halo the remaining sweeps still need
        const int W = kSt2BX + 2 * ext, H = BY + 2 * ext;
        const int gx0 = x0 - ext, gy0 = y0 - ext;
        const bool interior = gx0 - r >= 0 && gy0 - r >= 0 && gx0 + W + r <= cols && gy0 + H + r <= rows;
        // Every cell of the region, one at a time; cells outside the grid are
        // left alone (the next sweep's view gives them the neutral value
        // without reading them).
        auto sweep_cells = [&](const NPLMatrix<T, S> &v) {
            for (int row = warp; row < H; row += nwarps) {
                const int gy = gy0 + row;
                if ((unsigned)gy >= (unsigned)rows) continue;
                for (int col = lane; col < W; col += 32) {
                    const int gx = gx0 + col;
                    if ((unsigned)gx < (unsigned)cols) dst[(gy - wy0) * pitch + (gx - wx0)] = narrow<S>(fn(v, gx, gy));
                }
            }
        };
        if constexpr (has_pair_strip<Fn>::value && std::is_same<S, float>::value) {
            // Packed pairs (FP32 Jacobi): the region as a list of 2-column x
            // kPairRows-row strips at even window columns (hx is a multiple of
            // 4, so the pair accesses are 8-byte aligned); the strips start
            // every kPairRows rows, the last one moved up to end at row H (two
            // threads then write the same values). A side range of odd width
            // takes one more column outside the region, whose value no cell
            // that a later sweep needs reads; its reads stay inside the buffer.
            const int ext_e = (ext + 1) & ~1;
            const int npairs = kSt2BX / 2 + ext_e, ns = (H + kPairRows - 1) / kPairRows;
            const int wc0 = x0 - wx0 - ext_e, wr0 = gy0 - wy0;
            const float *src = reinterpret_cast<const float *>(m.tile_);
            float *d = reinterpret_cast<float *>(dst);
            // it / npairs as (it * inv) >> 20 with inv = ceil(2^20 / npairs):
            // exact while it * (inv * npairs - 2^20) < 2^20; here npairs <=
            // 64 (halo <= 31 at depth 32) and it < 2048 (64-row tiles), so the
            // product stays below 2^17
            const unsigned inv = ((1u << 20) + (unsigned)npairs - 1) / (unsigned)npairs;
            // no strip cell within one cell of the grid's edge: the window
            // (which holds every strip cell) lies inside the grid's interior
            const bool no_edge =
                wx0 >= 1 && wy0 >= 1 && wx0 + pitch <= cols - 1 && wy0 + BY + 2 * depth * r <= rows - 1;
            for (int it = threadIdx.x; it < ns * npairs; it += blockDim.x) {
                const int sr = (int)(((unsigned)it * inv) >> 20), pc = it - sr * npairs;
                const int wc = wc0 + 2 * pc, wr = wr0 + min(sr * kPairRows, H - kPairRows);
                f32x2 c[kPairRows], v[kPairRows];
                jacobi_pair_strip(src + wr * pitch + wc, pitch, wx0 + wc, wy0 + wr, cols, rows, c, v, no_edge);
#pragma unroll
                for (int k = 0; k < kPairRows; k++) st_pair(d + (wr + k) * pitch + wc, v[k]);
            }
        } else if (interior || has_any_tile_strip<Fn>::value) {
            m.check_ = false;
            if constexpr (has_strip2<Fn>::value) {
                // Whole kSt2RPT-row strips through the functor's strip(): the
                // strips start every kSt2RPT rows and the last one is moved
                // up to end at row H (it recomputes a few rows of the one
                // before; both write the same values, as every cell is a
                // function of the source buffer alone). The block's own 64
                // columns take two full warps per strip row; the ext-wide
                // side columns one thread per strip, from the last threads
                // of the CTA (whose warps have fewer central strips).
                const int ns = (H + kSt2RPT - 1) / kSt2RPT;
                auto strip_at = [&](int col, int sidx) {
                    const int row0 = min(sidx * kSt2RPT, H - kSt2RPT);
                    T vals[kSt2RPT];
                    const int gx = gx0 + col, gy = gy0 + row0;
                    fn.strip(m, gx, gy, vals);
                    S *d = dst + (gy - wy0) * pitch + (gx - wx0);
#pragma unroll
                    for (int j = 0; j < kSt2RPT; j++) d[j * pitch] = narrow<S>(vals[j]);
                };
                for (int item = warp; item < 2 * ns; item += nwarps) strip_at(ext + (item & 1) * 32 + lane, item >> 1);
                const int side = 2 * ext;
                for (int t = (int)blockDim.x - 1 - (int)threadIdx.x; t < side * ns; t += blockDim.x) {
                    const int sidx = t / side, c = t - sidx * side;
                    strip_at(c < ext ? c : kSt2BX + c, sidx);
                }
            } else {
                sweep_cells(m);
            }
        } else {
            m.check_ = true;
            sweep_cells(m);
        }
        __syncthreads();
        m.tile_ = dst;
        dst = (dst == buf1) ? buf0 : buf1;
    }
}

// One CTA = one 64 x 32 output block. Dynamic smem: [0,128) mbarrier, then the
// (32 + 2r) x (64 + 2hx) window.
template <typename S, class Fn, bool TMA>
__global__ void __launch_bounds__(kSt2Threads)
    stencil2d_kernel(const __grid_constant__ CUtensorMap tmap, const S *in, S *out, int rows, int cols, int r,
                     int hx, typename Compute<S>::type neutral, Fn fn, unsigned long long *resid,
                     unsigned *err) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    S *tile = reinterpret_cast<S *>(smem_raw + kStHeader);
    const int pitch = kSt2BX + 2 * hx, th = kSt2BY + 2 * r;
    const int x0 = blockIdx.x * kSt2BX, y0 = blockIdx.y * kSt2BY;
    const int wx0 = x0 - hx, wy0 = y0 - r;
    bool ok = true;
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_barrier_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(bar, (uint32_t)(pitch * th * sizeof(S)));
            tma_load_2d(tile, &tmap, bar, wx0, wy0);
        }
        ok = mbar_wait_bounded(bar, 0, err);
    } else {
        stage_window<S>(tile, in, pitch, th, th, wx0, wy0, 0, 1, rows, cols);
    }
    ok = __syncthreads_and(ok);
    if (!ok) return;

    NPLMatrix<T, S> m;
    m.width = cols;
    m.height = rows;
    m.stencilSize = r;
    m.neutralValue = neutral;
    m.tile_ = tile;
    m.global_ = in;
    m.ox_ = wx0;
    m.oy_ = wy0;
    m.pitch_ = pitch;
    m.tile_h_ = th;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = x0 + (warp % (kSt2BX / 32)) * 32 + lane;
    const int ys = y0 + (warp / (kSt2BX / 32)) * kSt2RPT;
    const bool interior = wx0 >= 0 && wy0 >= 0 && wx0 + pitch <= cols && wy0 + th <= rows;
    const bool want = resid != nullptr;
    double dmax = 0.0;
    if constexpr (has_pair_strip<Fn>::value && std::is_same<S, float>::value) {
        static_assert(kSt2Threads == 32 * (kSt2BY / kPairRows), "one pair strip per thread");
        jacobi_pair_block(reinterpret_cast<const float *>(tile), pitch, wx0, wy0, x0, y0, rows, cols,
                          reinterpret_cast<float *>(out), want, dmax, kSt2BY);
    } else if (interior) {
        m.check_ = false;
        stencil2d_strip<S, true>(fn, m, x, ys, rows, cols, out, want, dmax);
    } else {
        m.check_ = !has_any_tile_strip<Fn>::value;
        stencil2d_strip<S, false>(fn, m, x, ys, rows, cols, out, want, dmax);
    }
    if (want) {
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// Temporal blocking: `depth` sweeps of the same functor in one launch. The
// CTA stages its 64 x 32 output block plus a halo of depth*r cells, runs
// depth-1 sweeps in shared memory on shrinking regions (ping-pong between two
// buffers) and writes the last one to global memory. Cells outside the grid
// are never computed: the view returns the neutral value for them, exactly as
// it does between separate launches, so the result is bit-identical to
// `depth` single sweeps while HBM sees one read and one write per `depth`
// sweeps.
template <typename S, class Fn, bool TMA, int BY = kSt2BY>
__global__ void __launch_bounds__(BY * 8)
    stencil2d_tb_kernel(const __grid_constant__ CUtensorMap tmap, const S *in, S *out, int rows, int cols, int r,
                        int depth, int hx, typename Compute<S>::type neutral, Fn fn, unsigned long long *resid,
                        unsigned *err) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    const int pitch = kSt2BX + 2 * hx, th = BY + 2 * depth * r;
    const int buf_elems = (pitch * th * (int)sizeof(S) + 127) / 128 * 128 / (int)sizeof(S);
    S *buf0 = reinterpret_cast<S *>(smem_raw + kStHeader);
    S *buf1 = buf0 + buf_elems;
    const int x0 = blockIdx.x * kSt2BX, y0 = blockIdx.y * BY;
    const int wx0 = x0 - hx, wy0 = y0 - depth * r;
    bool ok = true;
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_barrier_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(bar, (uint32_t)(pitch * th * sizeof(S)));
            tma_load_2d(buf0, &tmap, bar, wx0, wy0);
        }
        ok = mbar_wait_bounded(bar, 0, err);
    } else {
        stage_window<S>(buf0, in, pitch, th, th, wx0, wy0, 0, 1, rows, cols);
    }
    ok = __syncthreads_and(ok);
    if (!ok) return;

    NPLMatrix<T, S> m;
    m.width = cols;
    m.height = rows;
    m.stencilSize = r;
    m.neutralValue = neutral;
    m.tile_ = buf0;
    m.global_ = in;
    m.ox_ = wx0;
    m.oy_ = wy0;
    m.pitch_ = pitch;
    m.tile_h_ = th;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    tb_inner_sweeps<S, BY>(fn, m, buf0, buf1, x0, y0, rows, cols, r, depth, pitch, wx0, wy0);
    const int x = x0 + (warp % (kSt2BX / 32)) * 32 + lane;
    const int ys = y0 + (warp / (kSt2BX / 32)) * kSt2RPT;
    const bool interior = x0 - r >= 0 && y0 - r >= 0 && x0 + kSt2BX + r <= cols && y0 + BY + r <= rows;
    const bool want = resid != nullptr;
    double dmax = 0.0;
    if constexpr (has_pair_strip<Fn>::value && std::is_same<S, float>::value) {
        static_assert(BY * 8 == 32 * (BY / kPairRows), "one pair strip per thread");
        jacobi_pair_block(reinterpret_cast<const float *>(m.tile_), pitch, wx0, wy0, x0, y0, rows, cols,
                          reinterpret_cast<float *>(out), want, dmax, BY);
    } else if (interior) {
        m.check_ = false;
        stencil2d_strip<S, true>(fn, m, x, ys, rows, cols, out, want, dmax);
    } else {
        m.check_ = !has_any_tile_strip<Fn>::value;
        stencil2d_strip<S, false>(fn, m, x, ys, rows, cols, out, want, dmax);
    }
    if (want) {
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// kSt3RPT vertically adjacent outputs of plane z; computed before stored (see stencil2d_strip).
template <typename S, bool FULL, class Fn, class View>
MSL_DEV void stencil3d_strip(const Fn &fn, const View &c, int x, int ys, int z, int rows, int cols, S *out, bool want,
                             double &dmax) {
    using T = typename Compute<S>::type;
    if (!FULL && x >= cols) return;
    T vals[kSt3RPT];
#pragma unroll
    for (int j = 0; j < kSt3RPT; j++)
        if (FULL || ys + j < rows) vals[j] = fn(c, x, ys + j, z);
    if (want) {
#pragma unroll
        for (int j = 0; j < kSt3RPT; j++)
            if (FULL || ys + j < rows) {
                const double d = fabs(stored_f64(narrow<S>(vals[j])) - (double)c(x, ys + j, z));
                if (d > dmax || d != d) dmax = d;
            }
    }
    S *o = out + ((size_t)z * rows + ys) * cols + x;
#pragma unroll
    for (int j = 0; j < kSt3RPT; j++)
        if (FULL || ys + j < rows) o[(size_t)j * cols] = narrow<S>(vals[j]);
}

// 3-D kernel. The cube is cut into 64 x 32 (x, y) tiles and each tile's
// depth into z-chunks; one CTA per (tile, chunk), sized so that all CTAs are
// resident together. Each CTA's work is a z-march with a ring of
// NS = 2^k >= 2r+2 shared-memory planes, one TMA 3-D load per plane issued one
// plane ahead, one mbarrier per slot (its phase tracked in a bit mask). Only
// the first 2r planes of a chunk are re-read halo.
template <typename S, class Fn, bool TMA>
__global__ void __launch_bounds__(kSt3Threads, 5)
    stencil3d_kernel(const __grid_constant__ CUtensorMap tmap, const S *in, S *out, int depth, int rows, int cols,
                     int r, int hx, int ns_log2, int zchunk, typename Compute<S>::type neutral, Fn fn,
                     unsigned long long *resid, unsigned *err) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);  // up to 16 slots
    S *ring = reinterpret_cast<S *>(smem_raw + kStHeader);
    const int NS = 1 << ns_log2, mask = NS - 1;
    const int pitch = kSt3BX + 2 * hx, th = kSt3BY + 2 * r;
    const int plane = (pitch * th + 31) / 32 * 32;  // keeps every slot 128-byte aligned
    const uint32_t plane_bytes = (uint32_t)(pitch * th * sizeof(S));
    const int tiles_x = (cols + kSt3BX - 1) / kSt3BX, tiles_y = (rows + kSt3BY - 1) / kSt3BY;
    // CTA b marches tile (b mod tiles) through z-chunk (b / tiles): adjacent
    // tiles run side by side at the same depth, so the halo lines one CTA
    // fetches are still in L2 when its neighbours need them.
    const int tiles = tiles_x * tiles_y;
    const int tile0 = (int)(blockIdx.x % tiles), zc = (int)(blockIdx.x / tiles);
    const int zlo = zc * zchunk, zhi = min(depth, zlo + zchunk);
    const long long begin = (long long)tile0 * depth + zlo, end = (long long)tile0 * depth + max(zlo, zhi);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool want = resid != nullptr;
    double dmax = 0.0;
    unsigned phase = 0;  // bit s: parity of the next completion of slot s

    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            for (int s = 0; s < NS; s++) mbar_init(&bars[s], 1);
            fence_barrier_init();
        }
    }
    bool ok = true;
    for (long long pos = begin; pos < end && ok;) {
        const int tile = (int)(pos / depth);
        const int zb = (int)(pos % depth);
        const int ze = (int)min((long long)depth, zb + (end - pos));
        pos += ze - zb;
        const int x0 = (tile % tiles_x) * kSt3BX, y0 = (tile / tiles_x) * kSt3BY;
        const int wx0 = x0 - hx, wy0 = y0 - r;

        auto issue = [&](int p) {  // thread 0 only (TMA) / all threads (plain loads)
            S *dst = ring + (p & mask) * plane;
            if constexpr (TMA) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bars[p & mask], plane_bytes);
                tma_load_3d(dst, &tmap, &bars[p & mask], wx0, wy0, p);
            } else {
                stage_window<S>(dst, in, pitch, th, th, wx0, wy0, p, depth, rows, cols);
            }
        };
        auto wait = [&](int p) {
            const int sl = p & mask;
            const bool done = mbar_wait_bounded(&bars[sl], (phase >> sl) & 1u, err);
            phase ^= 1u << sl;
            return done;
        };

        __syncthreads();  // the previous segment's readers are done with the ring
        if constexpr (TMA) {
            if (threadIdx.x == 0)
                for (int p = zb - r; p <= zb + r; p++) issue(p);  // 2r+1 distinct slots
            for (int p = zb - r; p < zb + r; p++) ok = wait(p) && ok;
        } else {
            for (int p = zb - r; p < zb + r; p++) issue(p);
        }

        PLCube<T, S> c;
        c.width = cols;
        c.height = rows;
        c.depth = depth;
        c.stencilSize = r;
        c.neutralValue = neutral;
        c.ring_ = ring;
        c.global_ = in;
        c.ox_ = wx0;
        c.oy_ = wy0;
        c.pitch_ = pitch;
        c.tile_h_ = th;
        c.plane_ = plane;
        c.mask_ = mask;
        const int x = x0 + (warp % (kSt3BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kSt3BX / 32)) * kSt3RPT;
        const bool xy_inside = wx0 >= 0 && wy0 >= 0 && wx0 + pitch <= cols && wy0 + th <= rows;

        for (int z = zb; z < ze; z++) {
            __syncthreads();  // every thread is done with plane z-r-1's slot
            if constexpr (TMA) {
                if (threadIdx.x == 0 && z + r + 1 <= ze - 1 + r) issue(z + r + 1);
                ok = wait(z + r) && ok;
            } else {
                issue(z + r);
                __syncthreads();
            }
            if (!__syncthreads_and(ok)) {
                if constexpr (TMA) {  // let the plane issued ahead land before the CTA exits
                    if (threadIdx.x == 0 && z + r + 1 <= ze - 1 + r) {
                        const int sl = (z + r + 1) & mask;
                        mbar_poll(&bars[sl], (phase >> sl) & 1u, kMaxWaitPolls);
                    }
                }
                ok = false;
                break;
            }
            c.zlo_ = z - r;
            c.zhi_ = z + r;
            if (xy_inside && z - r >= 0 && z + r < depth) {
                c.check_ = false;
                stencil3d_strip<S, true>(fn, c, x, ys, z, rows, cols, out, want, dmax);
            } else {
                c.check_ = true;
                stencil3d_strip<S, false>(fn, c, x, ys, z, rows, cols, out, want, dmax);
            }
        }
    }
    if (want) {
        __syncthreads();
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// 3-D tile kernel: one CTA per 64 x 16 x 8 block of outputs, staged with a
// single TMA 3-D load of the block plus its halo (the same design as the 2-D
// kernel: no per-plane synchronisation, many CTAs in flight, neighbouring
// blocks launched next to each other so halos are served from L2). Each
// thread computes a 4-row x 8-plane strip of one column, all values before any
// store. Used for radius <= kT3MaxR; larger radii use the z-march kernel.
constexpr int kT3BX = 64, kT3BY = 16, kT3BZ = 8, kT3RPT = 4, kT3Threads = 256, kT3MaxR = 3;
constexpr size_t kT3PipeSmemMax = 112 * 1024;  // two CTAs per SM

// Functors that are a 7-point star -- a function of the six face neighbours
// only -- may declare `static constexpr bool kStar7 = true` and provide
// star7(W, E, N, S, B, F) (x-1, x+1, y-1, y+1, z-1, z+1), returning exactly
// what operator() returns. Interior blocks then run star7_block: each window
// value is read from shared memory once into a register and reused by every
// cell of the strip that needs it, with the index arithmetic hoisted.
template <class Fn, class = void> struct IsStar7 : std::false_type {};
template <class Fn> struct IsStar7<Fn, std::void_t<decltype(Fn::kStar7)>> : std::bool_constant<Fn::kStar7> {};

// One kT3RPT-row x kT3BZ-plane strip of an interior block. `box` holds the
// block with halo (pitch x th x tz); (xl, yl, zl) is the box position of the
// strip's first cell.
template <typename S, bool FULL, class Fn>
MSL_DEV void star7_block(const Fn &fn, const S *box, int pitch, int plane, int xl, int yl, int zl, int x, int ys,
                         int z0, int depth, int rows, int cols, S *out, bool want, double &dmax) {
    using T = typename Compute<S>::type;
    const S *p = box + zl * plane + yl * pitch + xl;
    T cm[kT3RPT], c0[kT3RPT], cp[kT3RPT];
#pragma unroll
    for (int j = 0; j < kT3RPT; j++) {
        cm[j] = widen<S>(p[j * pitch - plane]);
        c0[j] = widen<S>(p[j * pitch]);
    }
    S *o = out + ((size_t)z0 * rows + ys) * cols + x;
    const size_t oplane = (size_t)rows * cols;
#pragma unroll
    for (int k = 0; k < kT3BZ; k++) {
        const S *q = p + k * plane;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) cp[j] = widen<S>(q[j * pitch + plane]);
        const T n = widen<S>(q[-pitch]), sth = widen<S>(q[kT3RPT * pitch]);
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            const T w = widen<S>(q[j * pitch - 1]), e = widen<S>(q[j * pitch + 1]);
            const T v = fn.star7(w, e, j == 0 ? n : c0[j - 1], j == kT3RPT - 1 ? sth : c0[j + 1], cm[j], cp[j]);
            const S sv = narrow<S>(v);
            if (FULL || (x < cols && ys + j < rows && z0 + k < depth)) {
                if (want) {
                    const double d = fabs(stored_f64(sv) - (double)c0[j]);
                    if (d > dmax || d != d) dmax = d;
                }
                o[(size_t)j * cols] = sv;
            }
        }
        o += oplane;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            cm[j] = c0[j];
            c0[j] = cp[j];
        }
    }
}

// Interior blocks of the persistent kernel: every value of the strip is
// computed before the first store, so no store separates the shared-memory
// reads of neighbouring planes and rows and the compiler can keep each window
// value in a register for all the cells that read it.
template <typename S, bool FULL, class Fn, class View>
MSL_DEV void stencil3d_block_regs(const Fn &fn, const View &c, int x, int ys, int z0, int depth, int rows, int cols,
                                  S *out, bool want, double &dmax) {
    using T = typename Compute<S>::type;
    T vals[kT3BZ][kT3RPT];
#pragma unroll
    for (int k = 0; k < kT3BZ; k++)
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) vals[k][j] = fn(c, x, ys + j, z0 + k);
#pragma unroll
    for (int k = 0; k < kT3BZ; k++) {
        S *o = out + ((size_t)(z0 + k) * rows + ys) * cols + x;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            if (!FULL && !(x < cols && ys + j < rows && z0 + k < depth)) continue;
            if (want) {
                const double d = fabs(stored_f64(narrow<S>(vals[k][j])) - (double)c(x, ys + j, z0 + k));
                if (d > dmax || d != d) dmax = d;
            }
            o[(size_t)j * cols] = narrow<S>(vals[k][j]);
        }
    }
}

template <typename S, bool FULL, class Fn, class View>
MSL_DEV void stencil3d_block(const Fn &fn, const View &c, int x, int ys, int z0, int depth, int rows, int cols, S *out,
                             bool want, double &dmax) {
    using T = typename Compute<S>::type;
    if (!FULL && x >= cols) return;
#pragma unroll
    for (int k = 0; k < kT3BZ; k++) {
        const int z = z0 + k;
        if (!FULL && z >= depth) break;
        T vals[kT3RPT];
#pragma unroll
        for (int j = 0; j < kT3RPT; j++)
            if (FULL || ys + j < rows) vals[j] = fn(c, x, ys + j, z);
        if (want) {
#pragma unroll
            for (int j = 0; j < kT3RPT; j++)
                if (FULL || ys + j < rows) {
                    const double d = fabs(stored_f64(narrow<S>(vals[j])) - (double)c(x, ys + j, z));
                    if (d > dmax || d != d) dmax = d;
                }
        }
        S *o = out + ((size_t)z * rows + ys) * cols + x;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++)
            if (FULL || ys + j < rows) o[(size_t)j * cols] = narrow<S>(vals[j]);
    }
}

template <typename S, class Fn, bool TMA>
__global__ void __launch_bounds__(kT3Threads, 3)
    stencil3d_tile_kernel(const __grid_constant__ CUtensorMap tmap, const S *in, S *out, int depth, int rows,
                          int cols, int r, int hx, typename Compute<S>::type neutral, Fn fn,
                          unsigned long long *resid, unsigned *err) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    S *box = reinterpret_cast<S *>(smem_raw + kStHeader);
    const int pitch = kT3BX + 2 * hx, th = kT3BY + 2 * r, tz = kT3BZ + 2 * r;
    const int x0 = blockIdx.x * kT3BX, y0 = blockIdx.y * kT3BY, z0 = blockIdx.z * kT3BZ;
    const int wx0 = x0 - hx, wy0 = y0 - r, wz0 = z0 - r;
    bool ok = true;
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_barrier_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(bar, (uint32_t)(pitch * th * tz * sizeof(S)));
            tma_load_3d(box, &tmap, bar, wx0, wy0, wz0);
        }
        ok = mbar_wait_bounded(bar, 0, err);
    } else {
        stage_window<S>(box, in, pitch, th, th * tz, wx0, wy0, wz0, depth, rows, cols);
    }
    ok = __syncthreads_and(ok);
    if (!ok) return;

    PLCube<T, S> c;
    c.width = cols;
    c.height = rows;
    c.depth = depth;
    c.stencilSize = r;
    c.neutralValue = neutral;
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
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = x0 + (warp % (kT3BX / 32)) * 32 + lane;
    const int ys = y0 + (warp / (kT3BX / 32)) * kT3RPT;
    const bool interior = wx0 >= 0 && wy0 >= 0 && wz0 >= 0 && wx0 + pitch <= cols && wy0 + th <= rows &&
                          wz0 + tz <= depth;
    const bool want = resid != nullptr;
    // Outside the grid the staged box holds zeros (TMA fill, or the plain
    // loads below): with a +0 neutral value the view needs no bounds test.
    const bool zero_fill = is_positive_zero(neutral);
    double dmax = 0.0;
    if constexpr (IsStar7<Fn>::value) {
        if (interior || zero_fill) {
            const int xl = x - wx0, yl = ys - wy0, zl = z0 - wz0;
            if (interior)
                star7_block<S, true>(fn, box, pitch, pitch * th, xl, yl, zl, x, ys, z0, depth, rows, cols, out, want,
                                     dmax);
            else
                star7_block<S, false>(fn, box, pitch, pitch * th, xl, yl, zl, x, ys, z0, depth, rows, cols, out, want,
                                      dmax);
            if (want) {
                dmax = block_max(dmax);
                if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
            }
            return;
        }
    }
    if (interior) {
        c.check_ = false;
        stencil3d_block<S, true>(fn, c, x, ys, z0, depth, rows, cols, out, want, dmax);
    } else {
        c.check_ = !zero_fill;
        stencil3d_block<S, false>(fn, c, x, ys, z0, depth, rows, cols, out, want, dmax);
    }
    if (want) {
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// Persistent, double-buffered form of the 3-D tile kernel (TMA only). Each
// CTA walks the blocks blockIdx.x, blockIdx.x + gridDim.x, ... (x fastest,
// then y, then z); the TMA load of its next block runs while it computes the
// current one, so the load latency no longer serialises with the arithmetic.
// Two CTAs per SM; results and residual are those of stencil3d_tile_kernel.
template <typename S> MSL_HD size_t t3_box_bytes(int r, int hx) {
    return ((size_t)(kT3BX + 2 * hx) * (kT3BY + 2 * r) * (kT3BZ + 2 * r) * sizeof(S) + 127) / 128 * 128;
}

template <typename S, class Fn>
__global__ void __launch_bounds__(kT3Threads, 2)
    stencil3d_pipe_kernel(const __grid_constant__ CUtensorMap tmap, const S *in, S *out, int depth, int rows,
                          int cols, int r, int hx, typename Compute<S>::type neutral, Fn fn,
                          unsigned long long *resid, unsigned *err) {
    using T = typename Compute<S>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);  // one mbarrier per buffer
    const unsigned box_bytes = (unsigned)t3_box_bytes<S>(r, hx);
    // buffer k at smem_raw + kStHeader + k * box_bytes (computed from smem_raw
    // each time, so the compiler keeps shared-memory addressing)
    auto buffer = [&](int k) { return reinterpret_cast<S *>(smem_raw + kStHeader + k * box_bytes); };
    const int pitch = kT3BX + 2 * hx, th = kT3BY + 2 * r, tz = kT3BZ + 2 * r;
    const uint32_t tx_bytes = (uint32_t)(pitch * th * tz * sizeof(S));
    const unsigned nbx = (cols + kT3BX - 1) / kT3BX, nbxy = nbx * ((rows + kT3BY - 1) / kT3BY);
    const unsigned nblocks = nbxy * ((depth + kT3BZ - 1) / kT3BZ);  // < 2^31 (checked by the launcher)
    unsigned b = blockIdx.x;
    if (b >= nblocks) return;
    auto origin = [&](unsigned blk, int &x0, int &y0, int &z0) {
        const unsigned bz = blk / nbxy, rem = blk - bz * nbxy, by = rem / nbx;
        x0 = (int)(rem - by * nbx) * kT3BX;
        y0 = (int)by * kT3BY;
        z0 = (int)bz * kT3BZ;
    };
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
        int x0, y0, z0;
        origin(b, x0, y0, z0);
        mbar_arrive_expect_tx(&bar[0], tx_bytes);
        tma_load_3d(buffer(0), &tmap, &bar[0], x0 - hx, y0 - r, z0 - r);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool want = resid != nullptr;
    const bool zero_fill = is_positive_zero(neutral);
    double dmax = 0.0;
    PLCube<T, S> c;
    c.width = cols;
    c.height = rows;
    c.depth = depth;
    c.stencilSize = r;
    c.neutralValue = neutral;
    c.global_ = in;
    c.pitch_ = pitch;
    c.tile_h_ = th;
    c.plane_ = pitch * th;
    c.mask_ = -1;
    for (int i = 0; b < nblocks; b += gridDim.x, i++) {
        const unsigned nb = b + gridDim.x;
        if (threadIdx.x == 0 && nb < nblocks) {  // prefetch the next block into the other buffer
            int x0, y0, z0;
            origin(nb, x0, y0, z0);
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[(i + 1) & 1], tx_bytes);
            tma_load_3d(buffer((i + 1) & 1), &tmap, &bar[(i + 1) & 1], x0 - hx, y0 - r, z0 - r);
        }
        bool ok = mbar_wait_bounded(&bar[i & 1], (uint32_t)(i >> 1) & 1u, err);
        ok = __syncthreads_and(ok);
        if (!ok) {  // let the prefetch land before the CTA gives up its shared memory
            if (threadIdx.x == 0 && nb < nblocks) mbar_poll(&bar[(i + 1) & 1], (uint32_t)((i + 1) >> 1) & 1u, kMaxWaitPolls);
            __syncthreads();
            return;
        }
        int x0, y0, z0;
        origin(b, x0, y0, z0);
        const int wx0 = x0 - hx, wy0 = y0 - r, wz0 = z0 - r;
        S *box = buffer(i & 1);
        c.ring_ = box;
        c.ox_ = wx0;
        c.oy_ = wy0;
        c.oz_ = wz0;
        c.zlo_ = wz0;
        c.zhi_ = wz0 + tz - 1;
        const int x = x0 + (warp % (kT3BX / 32)) * 32 + lane;
        const int ys = y0 + (warp / (kT3BX / 32)) * kT3RPT;
        const bool interior = wx0 >= 0 && wy0 >= 0 && wz0 >= 0 && wx0 + pitch <= cols && wy0 + th <= rows &&
                              wz0 + tz <= depth;
        if (interior || zero_fill) {
            // The box holds the neutral value wherever it lies outside the
            // grid (TMA fills those elements with zeros), so the view needs
            // no bounds test; boundary blocks only mask their stores.
            c.check_ = false;
            const int xl = x - wx0, yl = ys - wy0, zl = z0 - wz0;
            if constexpr (IsStar7<Fn>::value) {
                if (interior)
                    star7_block<S, true>(fn, box, pitch, pitch * th, xl, yl, zl, x, ys, z0, depth, rows, cols,
                                         out, want, dmax);
                else
                    star7_block<S, false>(fn, box, pitch, pitch * th, xl, yl, zl, x, ys, z0, depth, rows, cols,
                                          out, want, dmax);
            } else {
                if (interior)
                    stencil3d_block_regs<S, true>(fn, c, x, ys, z0, depth, rows, cols, out, want, dmax);
                else
                    stencil3d_block_regs<S, false>(fn, c, x, ys, z0, depth, rows, cols, out, want, dmax);
            }
        } else {
            c.check_ = true;
            stencil3d_block<S, false>(fn, c, x, ys, z0, depth, rows, cols, out, want, dmax);
        }
        __syncthreads();  // every read of this buffer is done before it is loaded again
    }
    if (want) {
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// ---- host side --------------------------------------------------------------------
using TensorMapEncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                        const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                        CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                        CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
inline TensorMapEncodeFn tensor_map_encoder() {
    static TensorMapEncodeFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<TensorMapEncodeFn>(p);
    }();
    return fn;
}

template <typename S> constexpr CUtensorMapDataType tmap_dtype() {
    if constexpr (sizeof(S) == 8) return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    else if constexpr (sizeof(S) == 2) return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    else return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;  // 4-byte elements (float and int32 move alike)
}

inline int st3_ns_log2(int r) {
    int ns = 1, l = 0;
    while (ns < 2 * r + 2) ns <<= 1, l++;
    return l;
}
template <typename S> inline size_t stencil2d_smem(int r) {
    return (size_t)kStHeader + (size_t)(kSt2BX + 2 * halo_x<S>(r)) * (kSt2BY + 2 * r) * sizeof(S);
}
template <typename S> inline size_t stencil3d_smem(int r) {
    const int pitch = kSt3BX + 2 * halo_x<S>(r), th = kSt3BY + 2 * r;
    const size_t plane = (size_t)(pitch * th + 31) / 32 * 32;
    return (size_t)kStHeader + ((size_t)1 << st3_ns_log2(r)) * plane * sizeof(S);
}
constexpr size_t kMaxStencilSmem = 227 * 1024;

// Whether the TMA path can address this grid: 16-byte aligned base and row
// pitch, box dimensions <= 256.
template <typename S> inline bool stencil_tma_ok(const void *in, long long cols, int pitch, int th) {
    return tensor_map_encoder() != nullptr && ((uintptr_t)in % 16) == 0 && (cols * (long long)sizeof(S)) % 16 == 0 &&
           pitch <= 256 && th <= 256;
}

template <typename S, class Fn>
cudaError_t launch_stencil2d(const S *in, S *out, int rows, int cols, int r, typename Compute<S>::type neutral,
                             Fn fn, unsigned long long *resid, unsigned *err, cudaStream_t st, bool allow_tma = true) {
    const int hx = halo_x<S>(r);
    const int pitch = kSt2BX + 2 * hx, th = kSt2BY + 2 * r;
    const size_t smem = stencil2d_smem<S>(r);
    if (smem > kMaxStencilSmem) return cudaErrorInvalidValue;
    dim3 grid((cols + kSt2BX - 1) / kSt2BX, (rows + kSt2BY - 1) / kSt2BY);
    CUtensorMap map{};
    const bool tma = allow_tma && stencil_tma_ok<S>(in, cols, pitch, th);
    if (tma) {
        cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
        cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(S)};
        cuuint32_t box[2] = {(cuuint32_t)pitch, (cuuint32_t)th};
        cuuint32_t estr[2] = {1, 1};
        if (tensor_map_encoder()(&map, tmap_dtype<S>(), 2, const_cast<S *>(in), dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
        auto k = stencil2d_kernel<S, Fn, true>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, kSt2Threads, smem, st>>>(map, in, out, rows, cols, r, hx, neutral, fn, resid, err);
    } else {
        auto k = stencil2d_kernel<S, Fn, false>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, kSt2Threads, smem, st>>>(map, in, out, rows, cols, r, hx, neutral, fn, resid, err);
    }
    return cudaGetLastError();
}

// Tile heights of the temporal-blocking kernel: 64 x BY outputs per CTA of
// BY * 8 threads (each thread a kSt2RPT-row strip of one column).
inline bool valid_tile_rows(int by) { return by == 16 || by == 32 || by == 64; }

template <typename S> inline size_t stencil2d_tb_smem(int r, int depth, int by = kSt2BY) {
    const int pitch = kSt2BX + 2 * halo_x<S>(depth * r), th = by + 2 * depth * r;
    const size_t buf = ((size_t)pitch * th * sizeof(S) + 127) / 128 * 128;
    return (size_t)kStHeader + 2 * buf;
}

template <typename S, class Fn, int BY>
cudaError_t launch_stencil2d_tb_rows(const S *in, S *out, int rows, int cols, int r, int depth,
                                     typename Compute<S>::type neutral, Fn fn, unsigned long long *resid,
                                     unsigned *err, cudaStream_t st, bool allow_tma) {
    const int hx = halo_x<S>(depth * r);
    const int pitch = kSt2BX + 2 * hx, th = BY + 2 * depth * r;
    const size_t smem = stencil2d_tb_smem<S>(r, depth, BY);
    if (smem > kMaxStencilSmem) return cudaErrorInvalidValue;
    dim3 grid((cols + kSt2BX - 1) / kSt2BX, (rows + BY - 1) / BY);
    CUtensorMap map{};
    const bool tma = allow_tma && stencil_tma_ok<S>(in, cols, pitch, th);
    if (tma) {
        cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
        cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(S)};
        cuuint32_t box[2] = {(cuuint32_t)pitch, (cuuint32_t)th};
        cuuint32_t estr[2] = {1, 1};
        if (tensor_map_encoder()(&map, tmap_dtype<S>(), 2, const_cast<S *>(in), dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
        auto k = stencil2d_tb_kernel<S, Fn, true, BY>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, BY * 8, smem, st>>>(map, in, out, rows, cols, r, depth, hx, neutral, fn, resid, err);
    } else {
        auto k = stencil2d_tb_kernel<S, Fn, false, BY>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, BY * 8, smem, st>>>(map, in, out, rows, cols, r, depth, hx, neutral, fn, resid, err);
    }
    return cudaGetLastError();
}

// `depth` fused sweeps in -> out (depth >= 2; depth 1 is launch_stencil2d), on
// 64 x tile_rows tiles (16, 32 or 64 rows: 128, 256 or 512 threads per CTA).
template <typename S, class Fn>
cudaError_t launch_stencil2d_tb(const S *in, S *out, int rows, int cols, int r, int depth,
                                typename Compute<S>::type neutral, Fn fn, unsigned long long *resid, unsigned *err,
                                cudaStream_t st, bool allow_tma = true, int tile_rows = kSt2BY) {
    switch (tile_rows) {
        case 16:
            return launch_stencil2d_tb_rows<S, Fn, 16>(in, out, rows, cols, r, depth, neutral, fn, resid, err, st,
                                                       allow_tma);
        case 64:
            return launch_stencil2d_tb_rows<S, Fn, 64>(in, out, rows, cols, r, depth, neutral, fn, resid, err, st,
                                                       allow_tma);
        default:
            return launch_stencil2d_tb_rows<S, Fn, 32>(in, out, rows, cols, r, depth, neutral, fn, resid, err, st,
                                                       allow_tma);
    }
}

template <typename S> inline size_t stencil3d_tile_smem(int r) {
    return (size_t)kStHeader +
           (size_t)(kT3BX + 2 * halo_x<S>(r)) * (kT3BY + 2 * r) * (kT3BZ + 2 * r) * sizeof(S);
}

// persistent: 1 = the persistent double-buffered kernel where it applies,
// 0 or -1 (the default) = one CTA per block. On GB300 the one-CTA-per-block
// kernel runs four CTAs per SM and overlaps loads and arithmetic across them;
// it measured faster than the two-CTA persistent kernel on heat3D 512^3.
template <typename S, class Fn>
cudaError_t launch_stencil3d_tile(const S *in, S *out, int depth, int rows, int cols, int r,
                                  typename Compute<S>::type neutral, Fn fn, unsigned long long *resid, unsigned *err,
                                  cudaStream_t st, bool allow_tma, int persistent = -1) {
    const int hx = halo_x<S>(r);
    const int pitch = kT3BX + 2 * hx, th = kT3BY + 2 * r, tz = kT3BZ + 2 * r;
    const size_t smem = stencil3d_tile_smem<S>(r);
    dim3 grid((cols + kT3BX - 1) / kT3BX, (rows + kT3BY - 1) / kT3BY, (depth + kT3BZ - 1) / kT3BZ);
    CUtensorMap map{};
    const bool tma = allow_tma && stencil_tma_ok<S>(in, cols, pitch, th) && tz <= 256;
    // Double buffering when two CTAs of two boxes each fit an SM.
    const size_t pipe_smem = (size_t)kStHeader + 2 * t3_box_bytes<S>(r, hx);
    const bool pipe = persistent == 1 && sizeof(S) <= 4 && tma && pipe_smem <= kT3PipeSmemMax &&
                      (long long)grid.x * grid.y * grid.z < (1LL << 31);
    auto k = tma ? stencil3d_tile_kernel<S, Fn, true> : stencil3d_tile_kernel<S, Fn, false>;
    if (!pipe && smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (tma) {
        cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)depth};
        cuuint64_t strides[2] = {(cuuint64_t)cols * sizeof(S), (cuuint64_t)cols * rows * sizeof(S)};
        cuuint32_t box[3] = {(cuuint32_t)pitch, (cuuint32_t)th, (cuuint32_t)tz};
        cuuint32_t estr[3] = {1, 1, 1};
        if (tensor_map_encoder()(&map, tmap_dtype<S>(), 3, const_cast<S *>(in), dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    if constexpr (sizeof(S) <= 4) {
        if (pipe) {
            auto kp = stencil3d_pipe_kernel<S, Fn>;
            cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pipe_smem);
            const long long nblocks = (long long)grid.x * grid.y * grid.z;
            int sms = 0, dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            const long long ctas = std::min<long long>(nblocks, 2LL * (sms > 0 ? sms : 152));
            kp<<<(unsigned)ctas, kT3Threads, pipe_smem, st>>>(map, in, out, depth, rows, cols, r, hx, neutral, fn,
                                                              resid, err);
            return cudaGetLastError();
        }
    }
    k<<<grid, kT3Threads, smem, st>>>(map, in, out, depth, rows, cols, r, hx, neutral, fn, resid, err);
    return cudaGetLastError();
}

template <typename S, class Fn>
cudaError_t launch_stencil3d(const S *in, S *out, int depth, int rows, int cols, int r,
                             typename Compute<S>::type neutral, Fn fn, unsigned long long *resid, unsigned *err,
                             cudaStream_t st, int sm_count, bool allow_tma = true, int persistent = -1) {
    if (r <= kT3MaxR && stencil3d_tile_smem<S>(r) <= 120 * 1024)
        return launch_stencil3d_tile<S>(in, out, depth, rows, cols, r, neutral, fn, resid, err, st, allow_tma,
                                        persistent);
    const int hx = halo_x<S>(r);
    const int pitch = kSt3BX + 2 * hx, th = kSt3BY + 2 * r;
    const int ns_log2 = st3_ns_log2(r);
    if ((1 << ns_log2) > kStHeader / 8) return cudaErrorInvalidValue;  // mbarrier slots
    const size_t smem = stencil3d_smem<S>(r);
    if (smem > kMaxStencilSmem) return cudaErrorInvalidValue;
    const long long total = (long long)((cols + kSt3BX - 1) / kSt3BX) * ((rows + kSt3BY - 1) / kSt3BY) * depth;
    CUtensorMap map{};
    const bool tma = allow_tma && stencil_tma_ok<S>(in, cols, pitch, th);
    auto k = tma ? stencil3d_kernel<S, Fn, true> : stencil3d_kernel<S, Fn, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // One wave of resident CTAs, each with at least 8 tile-planes of work.
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kSt3Threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    // As many z-chunks per tile as the resident CTA slots allow (chunks of at
    // least 8 planes); one chunk per tile when the cross-section alone fills the GPU.
    const long long tiles = total / depth;
    const long long slots = (long long)per_sm * (sm_count > 0 ? sm_count : 152);
    long long nz = slots / tiles;
    if (nz > depth / 8) nz = depth / 8;
    if (nz < 1) nz = 1;
    const int zchunk = (int)((depth + nz - 1) / nz);
    nz = (depth + zchunk - 1) / zchunk;
    const long long grid = tiles * nz;
    if (tma) {
        cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)depth};
        cuuint64_t strides[2] = {(cuuint64_t)cols * sizeof(S), (cuuint64_t)cols * rows * sizeof(S)};
        cuuint32_t box[3] = {(cuuint32_t)pitch, (cuuint32_t)th, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        if (tensor_map_encoder()(&map, tmap_dtype<S>(), 3, const_cast<S *>(in), dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    k<<<(unsigned)grid, kSt3Threads, smem, st>>>(map, in, out, depth, rows, cols, r, hx, ns_log2, zchunk, neutral, fn,
                                                 resid, err);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
