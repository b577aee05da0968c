// Game of Life on a grid whose cells are all 0 or 1, several generations per
// launch, four cells packed into each 32-bit word of shared memory.
//
// The reference's rule (examples/gameoflife.cpp:22-42) on int32 cells: a cell
// becomes 1 when alive == 1 and its eight neighbours sum to 2 or 3, or when
// alive == 0 and they sum to 3; otherwise 0. Every output of the rule is 0 or
// 1, so from the second generation of an iteration on, every input is too.
// For 0/1 cells the rule is `(sum | alive) == 3`, and sums of up to nine 0/1
// cells fit in a byte: with one cell per byte, ordinary 32-bit additions add
// four cells at once (no byte ever carries), `__byte_perm` forms the words of
// the left and right neighbours, and a per-byte zero test evaluates the rule
// for four cells -- about four integer instructions per cell update instead of
// eight neighbour loads and additions. Results are identical to the
// cell-by-cell functor for 0/1 inputs, which the caller guarantees (this
// kernel is used only on the outputs of Life sweeps).
//
// One CTA computes a 128 x 64 block D generations ahead. It reads the block
// and its halo with coalesced 16-byte loads (zeros outside the grid), packs
// the cells into bytes as it stores them to shared memory, runs the
// generations between two packed buffers and writes the last one as int32.
// Cells outside the grid are kept at 0 after every generation, as the dead
// border of the reference's neutral value 0. D is a template parameter, so
// every loop bound and index division is a compile-time constant.
//
// Rows: generation s is computed on rows [s, TH - s), exactly the rows the
// next one reads, so a D-row halo suffices. Columns: each generation computes
// the window's words 1 .. NW-2 only. The edge words of the second buffer are
// zeroed once and those of the first keep the staged cells, so every word
// read holds 0/1 bytes (no byte of a sum can carry into its neighbour); the
// edge words are stale after the first generation, and every generation after
// it spreads that one cell further in (cells < s + 3 from a window edge are
// wrong after generation s). The column halo is therefore D + 3 cells,
// rounded up to whole words.
#pragma once

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

constexpr int kLifeBX = 128, kLifeBY = 64;  // output block, cells
constexpr int kLifeThreads = 256;
constexpr int kLifeStrip = 6;      // word rows per thread task (vertical reuse of the row sums)
constexpr int kLifeMaxDepth = 16;  // generations per launch handled by this kernel

template <int D>
struct LifeWindow {
    static constexpr int kHX = (D + 3 + 3) / 4 * 4;  // column halo, cells (whole words)
    static constexpr int kP = kLifeBX + 2 * kHX;     // window width, cells
    static constexpr int kNW = kP / 4;               // words per window row
    static constexpr int kTH = kLifeBY + 2 * D;      // window height, rows
    static constexpr int kWords = kNW * kTH;
    static_assert(kHX >= D + 3 && kHX % 4 == 0, "column halo");
};

// Bytes equal to 3 -> 1, others -> 0, for bytes <= 15 (a per-byte zero test
// of x ^ 3: adding 0x7F to a byte <= 15 sets its top bit exactly when it is
// not 0 and never carries into the next byte).
MSL_DEV uint32_t life_rule4(uint32_t sum, uint32_t alive) {
    const uint32_t u = ((sum | alive) ^ 0x03030303u) + 0x7F7F7F7Fu;
    return (~u >> 7) & 0x01010101u;
}

// Row sums of three horizontally adjacent cells for the four cells of word
// `c`, given the words to its left and right.
MSL_DEV uint32_t life_hsum(uint32_t l, uint32_t c, uint32_t r) {
    return __byte_perm(l, c, 0x6543) + c + __byte_perm(c, r, 0x4321);
}

// Bytes of word `w` (cells wx0 + 4w .. + 3) that lie in [0, cols): the word
// is wholly inside or outside, since wx0 and cols are multiples of 4.
MSL_DEV uint32_t life_colmask(int wx0, int w, int cols) {
    const int gx = wx0 + 4 * w;
    return (gx >= 0 && gx < cols) ? 0xFFFFFFFFu : 0u;
}

// Generation s: dst = rule(src) on rows [s, TH - s), words 1 .. NW-2.
// MASK (blocks whose window leaves the grid) clears the cells outside it.
template <int D, bool MASK>
MSL_DEV void life_generation(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, int s, int wx0, int cols,
                             int row_lo, int row_hi) {
    using Wd = LifeWindow<D>;
    constexpr int ncw = Wd::kNW - 2;
    const int nrows = Wd::kTH - 2 * s, ns = (nrows + kLifeStrip - 1) / kLifeStrip;
    for (int t = threadIdx.x; t < ncw * ns; t += kLifeThreads) {
        const int sidx = t / ncw, w = 1 + (t - sidx * ncw);
        const int r0 = s + min(sidx * kLifeStrip, nrows - kLifeStrip);  // the last strip ends at the last row
        uint32_t h[kLifeStrip + 2], c[kLifeStrip + 2];
#pragma unroll
        for (int k = 0; k < kLifeStrip + 2; k++) {
            const uint32_t *row = src + (r0 - 1 + k) * Wd::kNW + w;
            c[k] = row[0];
            h[k] = life_hsum(row[-1], c[k], row[1]);
        }
        const uint32_t colmask = MASK ? life_colmask(wx0, w, cols) : 0u;
#pragma unroll
        for (int k = 0; k < kLifeStrip; k++) {
            const uint32_t sum = h[k] + h[k + 1] + h[k + 2] - c[k + 1];  // the eight neighbours
            uint32_t v = life_rule4(sum, c[k + 1]);
            if (MASK) v = (r0 + k >= row_lo && r0 + k < row_hi) ? (v & colmask) : 0u;
            dst[(r0 + k) * Wd::kNW + w] = v;
        }
    }
}

template <int D>
__global__ void __launch_bounds__(kLifeThreads)
    life_packed_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int rows, int cols) {
    using Wd = LifeWindow<D>;
    __shared__ uint32_t buf[2][Wd::kWords];
    const int x0 = blockIdx.x * kLifeBX, y0 = blockIdx.y * kLifeBY;
    const int wx0 = x0 - Wd::kHX, wy0 = y0 - D;
    // stage: 16-byte loads, four at a time in flight per thread; byte i of
    // word w = cell 4w + i
    constexpr int kIter = (Wd::kWords + kLifeThreads - 1) / kLifeThreads;
#pragma unroll
    for (int j0 = 0; j0 < kIter; j0 += 4) {
        int4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = threadIdx.x + (j0 + u) * kLifeThreads;
            v[u] = make_int4(0, 0, 0, 0);
            if (j0 + u < kIter && i < Wd::kWords) {
                const int r = i / Wd::kNW, w = i - r * Wd::kNW;
                const int gy = wy0 + r, gx = wx0 + 4 * w;
                if (gy >= 0 && gy < rows && gx >= 0 && gx < cols)
                    v[u] = __ldg(reinterpret_cast<const int4 *>(in + (size_t)gy * cols + gx));
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = threadIdx.x + (j0 + u) * kLifeThreads;
            if (j0 + u < kIter && i < Wd::kWords)
                buf[0][i] = __byte_perm(__byte_perm(v[u].x, v[u].y, 0x0040), __byte_perm(v[u].z, v[u].w, 0x0040), 0x5410);
        }
    }
    // the edge words of the second buffer are never computed: keep them 0
    for (int i = threadIdx.x; i < 2 * Wd::kTH; i += kLifeThreads)
        buf[1][(i >> 1) * Wd::kNW + ((i & 1) ? Wd::kNW - 1 : 0)] = 0u;
    __syncthreads();
    const bool interior = wx0 >= 0 && wy0 >= 0 && wx0 + Wd::kP <= cols && wy0 + Wd::kTH <= rows;
    const int row_lo = -wy0, row_hi = rows - wy0;  // window rows inside the grid
#pragma unroll
    for (int s = 1; s <= D; s++) {
        const uint32_t *src = buf[(s - 1) & 1];
        uint32_t *dst = buf[s & 1];
        if (interior) life_generation<D, false>(src, dst, s, wx0, cols, row_lo, row_hi);
        else life_generation<D, true>(src, dst, s, wx0, cols, row_lo, row_hi);
        __syncthreads();
    }
    // write the block as int32: a warp stores one 128-cell row
    const uint32_t *res = buf[D & 1];
    constexpr int kBW = kLifeBX / 4, wb = Wd::kHX / 4;  // words per block row, first word of the block
#pragma unroll
    for (int j = 0; j < kLifeBX * kLifeBY / 4 / kLifeThreads; j++) {
        const int t = threadIdx.x + j * kLifeThreads;
        const int ry = t / kBW, wx = t - ry * kBW;
        const int gy = y0 + ry, gx = x0 + 4 * wx;
        if (gy < rows && gx < cols) {
            const uint32_t v = res[(D + ry) * Wd::kNW + wb + wx];
            *reinterpret_cast<int4 *>(out + (size_t)gy * cols + gx) =
                make_int4(__byte_perm(v, 0, 0x4440), __byte_perm(v, 0, 0x4441), __byte_perm(v, 0, 0x4442),
                          __byte_perm(v, 0, 0x4443));
        }
    }
}

template <int D>
inline cudaError_t launch_life_packed_d(const int32_t *in, int32_t *out, int rows, int cols, cudaStream_t st) {
    dim3 grid((cols + kLifeBX - 1) / kLifeBX, (rows + kLifeBY - 1) / kLifeBY);
    life_packed_kernel<D><<<grid, kLifeThreads, 0, st>>>(in, out, rows, cols);
    return cudaGetLastError();
}

// `depth` Life generations from `in` (every cell 0 or 1) to `out`, neutral 0.
// Needs whole 16-byte words per row (cols a multiple of 4, both buffers
// 16-byte aligned), distinct buffers and 1 <= depth <= kLifeMaxDepth; returns
// cudaErrorNotSupported otherwise (the caller then runs the cell-by-cell
// kernels).
inline cudaError_t launch_life_packed(const int32_t *in, int32_t *out, int rows, int cols, int depth,
                                      cudaStream_t st) {
    if (depth < 1 || depth > kLifeMaxDepth || (cols & 3) || ((uintptr_t)in & 15) || ((uintptr_t)out & 15) ||
        in == out || (rows + kLifeBY - 1) / kLifeBY > 65535)
        return cudaErrorNotSupported;
    switch (depth) {
        case 1: return launch_life_packed_d<1>(in, out, rows, cols, st);
        case 2: return launch_life_packed_d<2>(in, out, rows, cols, st);
        case 3: return launch_life_packed_d<3>(in, out, rows, cols, st);
        case 4: return launch_life_packed_d<4>(in, out, rows, cols, st);
        case 5: return launch_life_packed_d<5>(in, out, rows, cols, st);
        case 6: return launch_life_packed_d<6>(in, out, rows, cols, st);
        case 7: return launch_life_packed_d<7>(in, out, rows, cols, st);
        case 8: return launch_life_packed_d<8>(in, out, rows, cols, st);
        case 9: return launch_life_packed_d<9>(in, out, rows, cols, st);
        case 10: return launch_life_packed_d<10>(in, out, rows, cols, st);
        case 11: return launch_life_packed_d<11>(in, out, rows, cols, st);
        case 12: return launch_life_packed_d<12>(in, out, rows, cols, st);
        case 13: return launch_life_packed_d<13>(in, out, rows, cols, st);
        case 14: return launch_life_packed_d<14>(in, out, rows, cols, st);
        case 15: return launch_life_packed_d<15>(in, out, rows, cols, st);
        default: return launch_life_packed_d<16>(in, out, rows, cols, st);
    }
}

}  // namespace gpu
}  // namespace msl
