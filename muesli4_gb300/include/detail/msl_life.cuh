// Game of Life on a grid whose cells are all 0 or 1, several generations per
// launch, one bit per cell in shared memory (32 cells per word).
//
// The reference's rule (examples/gameoflife.cpp:22-42) on int32 cells: a cell
// becomes 1 when alive == 1 and its eight neighbours sum to 2 or 3, or when
// alive == 0 and they sum to 3; otherwise 0. Every output of the rule is 0 or
// 1, so from the second generation of an iteration on, every input is too.
// For 0/1 cells the neighbour count fits in bit-sliced adders: with bit i of a
// word holding cell 32w + i, the words of left and right neighbours are
// funnel shifts of the row's words, full adders (XOR3 and majority, one
// three-input logic instruction each) sum a row's three cells, and the count
// bits c0, c1, c2 (mod 8; a count of 8 reads as 0, which the rule treats like
// 8) give the rule as `c1 & ~c2 & (c0 | alive)` -- about 20 instructions per
// 32 cell updates. Results are identical to the cell-by-cell functor for 0/1
// inputs, which the caller guarantees (this kernel is used only on the
// outputs of Life sweeps).
//
// One CTA computes a 960 x 128 block `depth` generations ahead (depth <= 32).
// Its window is 32 words (1024 cells) wide -- one word per lane, one word of
// halo either side -- and 128 + 2 depth rows high. Staging: each warp reads
// whole window rows with coalesced 4-byte loads (zeros outside the grid) and
// packs 32 cells into a word with one ballot. Generations ping-pong between
// two bit buffers; a warp computes a strip of 8 rows for all 32 words of the
// window (lane = word), reusing each row's three-cell sums for the rows above
// and below it. Cells outside the grid are kept at 0 after every generation,
// as the dead border of the reference's neutral value 0.
//
// Rows: generation s is computed on rows [s, TH - s), exactly the rows the
// next one reads, so a depth-row halo suffices. Columns: the words beyond the
// window are zero pads, so the window's outermost cells see dead neighbours
// there; the error spreads one cell per generation, so after `depth`
// generations cells < depth from a window edge may be wrong and the block,
// one word (32 cells) in from either edge, is exact for depth <= 32.
#pragma once

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

constexpr int kLifeWords = 32;                  // words per window row, one per lane
constexpr int kLifePitch = kLifeWords + 2;      // plus a zero pad either side
constexpr int kLifeBW = kLifeWords - 2;         // words per block row
constexpr int kLifeBX = kLifeBW * 32;           // 960 cells
constexpr int kLifeBY = 128;                    // block rows (taller blocks recompute less halo per generation)
constexpr int kLifeWarps = 8, kLifeThreads = 32 * kLifeWarps;
constexpr int kLifeStrip = 8;                   // rows per warp task (vertical reuse of the row sums)
constexpr int kLifeMaxDepth = 32;               // generations per launch (the block's column halo)
constexpr int kLifeLoadBatch = 8;               // loads in flight per lane while staging

inline size_t life_bits_smem(int depth) {
    return 2 * (size_t)(kLifeBY + 2 * depth) * kLifePitch * sizeof(uint32_t);
}

MSL_DEV uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) { return a ^ b ^ c; }
MSL_DEV uint32_t maj3(uint32_t a, uint32_t b, uint32_t c) { return (a & b) | (c & (a | b)); }

// One warp, one strip: rows [r0, r0 + kLifeStrip) of every window word
// (lane = word). MASK clears cells outside the grid: `colmask` holds the
// lane's in-grid bits, [row_lo, row_hi) the in-grid window rows.
template <bool MASK>
MSL_DEV void life_bits_strip(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, int r0, int lane,
                             uint32_t colmask, int row_lo, int row_hi) {
    uint32_t fs[kLifeStrip + 2], fc[kLifeStrip + 2], hs[kLifeStrip + 2], hc[kLifeStrip + 2], alive[kLifeStrip + 2];
#pragma unroll
    for (int k = 0; k < kLifeStrip + 2; k++) {
        const uint32_t *row = src + (r0 - 1 + k) * kLifePitch + 1 + lane;
        const uint32_t l = row[-1], c = row[0], r = row[1];
        const uint32_t lv = __funnelshift_l(l, c, 1);  // bit i: cell to the left of cell i
        const uint32_t rv = __funnelshift_r(c, r, 1);  // bit i: cell to the right
        fs[k] = xor3(lv, c, rv);                       // three-cell row sum, ones
        fc[k] = maj3(lv, c, rv);                       // and twos
        hs[k] = lv ^ rv;                               // left + right only
        hc[k] = lv & rv;
        alive[k] = c;
    }
#pragma unroll
    for (int k = 1; k <= kLifeStrip; k++) {
        // count = (fs[k-1] + hs[k] + fs[k+1]) + 2 (fc[k-1] + hc[k] + fc[k+1])
        const uint32_t c0 = xor3(fs[k - 1], hs[k], fs[k + 1]);
        const uint32_t k1 = maj3(fs[k - 1], hs[k], fs[k + 1]);
        const uint32_t t = xor3(fc[k - 1], hc[k], fc[k + 1]);
        const uint32_t u = maj3(fc[k - 1], hc[k], fc[k + 1]);
        const uint32_t c1 = t ^ k1, c2 = u ^ (t & k1);
        uint32_t v = c1 & ~c2 & (c0 | alive[k]);
        const int rr = r0 + k - 1;
        if (MASK) v = (rr >= row_lo && rr < row_hi) ? (v & colmask) : 0u;
        dst[rr * kLifePitch + 1 + lane] = v;
    }
}

// One window row: `row` points at the lane's cell of word 0, `gx` is its
// column; CHECK loads only cells inside [0, cols).
template <bool CHECK>
MSL_DEV void life_stage_row(const int32_t *__restrict__ row, uint32_t *words, int lane, int gx, int cols) {
#pragma unroll
    for (int j0 = 0; j0 < kLifeWords; j0 += kLifeLoadBatch) {
        int v[kLifeLoadBatch];
#pragma unroll
        for (int u = 0; u < kLifeLoadBatch; u++) {
            const int x = gx + 32 * (j0 + u);
            v[u] = (!CHECK || (x >= 0 && x < cols)) ? __ldg(row + 32 * (j0 + u)) : 0;
        }
#pragma unroll
        for (int u = 0; u < kLifeLoadBatch; u++) {
            const uint32_t b = __ballot_sync(0xFFFFFFFFu, v[u] != 0);
            if (lane == 0) words[j0 + u] = b;
        }
    }
}

// Bits of the lane's window word (cells gx0 .. gx0 + 31) that lie in [0, cols).
MSL_DEV uint32_t life_colmask(int gx0, int cols) {
    const int lo = max(0, -gx0), hi = min(32, cols - gx0);
    if (hi <= lo) return 0u;
    return hi - lo == 32 ? 0xFFFFFFFFu : ((1u << (hi - lo)) - 1u) << lo;
}

static __global__ void __launch_bounds__(kLifeThreads, 4)
    life_bits_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int rows, int cols, int depth) {
    extern __shared__ uint32_t life_smem[];
    const int th = kLifeBY + 2 * depth;  // window rows
    uint32_t *src = life_smem, *dst = life_smem + th * kLifePitch;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * kLifeBX, y0 = blockIdx.y * kLifeBY;
    const int wx0 = x0 - 32, wy0 = y0 - depth;  // window origin: one word, `depth` rows of halo
    const bool cols_in = wx0 >= 0 && wx0 + 32 * kLifeWords <= cols;
    // zero pads either side of every row of both buffers
    for (int i = threadIdx.x; i < 2 * th; i += kLifeThreads) {
        const int at = (i >> 1) * kLifePitch + ((i & 1) ? kLifePitch - 1 : 0);
        src[at] = 0u;
        dst[at] = 0u;
    }
    // stage: a warp packs whole window rows; word j of a row is the ballot of
    // cells 32 j .. 32 j + 31, stored by lane 0 (rows and words outside the
    // grid are 0). Rows [kLifeBY, th) of this window are rows [0, 2 depth) of
    // the window below: taking them in the order 0, kLifeBY, 1, kLifeBY + 1,
    // ... makes both CTAs read each shared row at about the same time, so the
    // second read finds it in L2.
    for (int i = warp; i < th; i += kLifeWarps) {
        const int r = i < 4 * depth ? (i >> 1) + ((i & 1) ? kLifeBY : 0) : i - 2 * depth;
        const int gy = wy0 + r;
        uint32_t *words = src + r * kLifePitch + 1;
        if (gy < 0 || gy >= rows) {
            words[lane] = 0u;
            continue;
        }
        const int32_t *row = in + (size_t)gy * cols + wx0 + lane;
        if (cols_in) life_stage_row<false>(row, words, lane, 0, 0);
        else life_stage_row<true>(row, words, lane, wx0 + lane, cols);
    }
    __syncthreads();
    const bool interior = cols_in && wy0 >= 0 && wy0 + th <= rows;
    const int row_lo = -wy0, row_hi = rows - wy0;  // window rows inside the grid
    const uint32_t colmask = interior ? 0xFFFFFFFFu : life_colmask(wx0 + 32 * lane, cols);
    for (int s = 1; s <= depth; s++) {
        // generation s: rows [s, th - s); the last strip ends at the last row
        const int nrows = th - 2 * s, ns = (nrows + kLifeStrip - 1) / kLifeStrip;
        for (int sidx = warp; sidx < ns; sidx += kLifeWarps) {
            const int r0 = s + min(sidx * kLifeStrip, nrows - kLifeStrip);
            if (interior) life_bits_strip<false>(src, dst, r0, lane, 0u, 0, 0);
            else life_bits_strip<true>(src, dst, r0, lane, colmask, row_lo, row_hi);
        }
        __syncthreads();
        uint32_t *t = src;
        src = dst;
        dst = t;
    }
    // write the block as int32: lane = cell within a word, 128-byte stores
    const bool block_in = x0 + kLifeBX <= cols;
    for (int ry = warp; ry < kLifeBY && y0 + ry < rows; ry += kLifeWarps) {
        const uint32_t *words = src + (depth + ry) * kLifePitch + 2;  // window word 1 = block word 0
        int32_t *o = out + (size_t)(y0 + ry) * cols + x0 + lane;
        const int jn = block_in ? kLifeBW : min(kLifeBW, (cols - x0 - lane + 31) / 32);  // words with this lane's cell inside
#pragma unroll 5
        for (int j = 0; j < jn; j++) o[32 * j] = (int32_t)((words[j] >> lane) & 1u);
    }
}

// `depth` Life generations from `in` (every cell 0 or 1) to `out`, neutral 0,
// for 1 <= depth <= kLifeMaxDepth and distinct buffers; returns
// cudaErrorNotSupported otherwise (the caller then runs the cell-by-cell
// kernels).
inline cudaError_t launch_life_packed(const int32_t *in, int32_t *out, int rows, int cols, int depth,
                                      cudaStream_t st) {
    const int gy = (rows + kLifeBY - 1) / kLifeBY;
    if (depth < 1 || depth > kLifeMaxDepth || in == out || gy > 65535) return cudaErrorNotSupported;
    const size_t smem = life_bits_smem(depth);  // <= 52224 bytes
    if (smem > 48 * 1024) cudaFuncSetAttribute(life_bits_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((cols + kLifeBX - 1) / kLifeBX, gy);
    life_bits_kernel<<<grid, kLifeThreads, smem, st>>>(in, out, rows, cols, depth);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
