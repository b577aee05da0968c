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
// the left and right neighbours, and an exact per-byte zero test evaluates
// the rule for four cells -- a handful of integer instructions per four cell
// updates instead of eight neighbour loads and additions per cell. Results
// are identical to the cell-by-cell functor for 0/1 inputs, which the caller
// guarantees (this kernel is used only on the outputs of Life sweeps).
//
// One CTA computes a 64 x 32 block `depth` generations ahead: it stages the
// block with a halo by one TMA load (zeros outside the grid), packs it into
// bytes, runs the generations between two packed buffers and writes the last
// one as int32. Cells outside the grid are kept at 0 after every generation,
// as the dead border of the reference's neutral value 0. Rows: generation s
// is computed on rows [s, th - s), exactly the rows the next one reads, so a
// `depth`-row halo suffices. Columns: each generation computes the window's
// words 1 .. nw-2 only, so the edge words hold stale values and every
// generation after the first spreads them one cell further in (cells < s + 3
// from a window edge are wrong after generation s); the column halo is
// therefore depth + 3 cells, rounded up to whole words.
#pragma once

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

constexpr int kLifeStrip = 4;  // word rows per thread task (vertical reuse of the row sums)

// Bytes of `x` equal to 3 -> 1, others -> 0 (exact per-byte zero test of x ^ 3).
MSL_DEV uint32_t life_rule4(uint32_t sum, uint32_t alive) {
    const uint32_t y = (sum | alive) ^ 0x03030303u;
    const uint32_t z = ~(((y & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | y) & 0x80808080u;
    return z >> 7;
}

// Row sums of three horizontally adjacent cells for the four cells of word
// `c`, given the words to its left and right.
MSL_DEV uint32_t life_hsum(uint32_t l, uint32_t c, uint32_t r) {
    return __byte_perm(l, c, 0x6543) + c + __byte_perm(c, r, 0x4321);
}

// Word-rows [r0, r0 + kLifeStrip) of word column w: dst = rule(src).
// `mask` (boundary blocks) clears the bytes of cells outside the grid.
template <bool MASK>
MSL_DEV void life_strip(const uint32_t *src, uint32_t *dst, int nw, int w, int r0, uint32_t colmask, int row_lo,
                        int row_hi) {
    uint32_t h[kLifeStrip + 2], c[kLifeStrip + 2];
#pragma unroll
    for (int k = 0; k < kLifeStrip + 2; k++) {
        const uint32_t *row = src + (r0 - 1 + k) * nw + w;
        c[k] = row[0];
        h[k] = life_hsum(row[-1], c[k], row[1]);
    }
#pragma unroll
    for (int k = 0; k < kLifeStrip; k++) {
        const uint32_t sum = h[k] + h[k + 1] + h[k + 2] - c[k + 1];  // the eight neighbours
        uint32_t v = life_rule4(sum, c[k + 1]);
        if (MASK) v = (r0 + k >= row_lo && r0 + k < row_hi) ? (v & colmask) : 0u;
        dst[(r0 + k) * nw + w] = v;
    }
}

// Bytes of word `w` (cells wx0 + 4w .. + 3) that lie in [0, cols).
MSL_DEV uint32_t life_colmask(int wx0, int w, int cols) {
    uint32_t m = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gx = wx0 + 4 * w + i;
        if (gx >= 0 && gx < cols) m |= 0xFFu << (8 * i);
    }
    return m;
}

static __global__ void __launch_bounds__(256)
    life_packed_kernel(const __grid_constant__ CUtensorMap tmap, int32_t *out, int rows, int cols, int depth, int hx,
                       unsigned *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    const int pitch = kSt2BX + 2 * hx, th = kSt2BY + 2 * depth;  // staged window, cells
    const int nw = pitch / 4;                                      // words per row
    int32_t *tile = reinterpret_cast<int32_t *>(smem_raw + kStHeader);
    uint32_t *buf0 = reinterpret_cast<uint32_t *>(tile + pitch * th);
    uint32_t *buf1 = buf0 + nw * th;
    const int x0 = blockIdx.x * kSt2BX, y0 = blockIdx.y * kSt2BY;
    const int wx0 = x0 - hx, wy0 = y0 - depth;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, (uint32_t)(pitch * th * sizeof(int32_t)));
        tma_load_2d(tile, &tmap, bar, wx0, wy0);
    }
    const bool ok = __syncthreads_and(mbar_wait_bounded(bar, 0, err));
    if (!ok) return;
    // pack: byte i of word w = cell 4w + i (0 or 1)
    for (int i = threadIdx.x; i < nw * th; i += blockDim.x) {
        const int4 v = reinterpret_cast<const int4 *>(tile)[i];  // pitch is a multiple of 4
        buf0[i] = (uint32_t)v.x | ((uint32_t)v.y << 8) | ((uint32_t)v.z << 16) | ((uint32_t)v.w << 24);
    }
    __syncthreads();
    const bool interior = wx0 >= 0 && wy0 >= 0 && wx0 + pitch <= cols && wy0 + th <= rows;
    const int row_lo = -wy0, row_hi = rows - wy0;  // window rows inside the grid
    const uint32_t *src = buf0;
    uint32_t *dst = buf1;
    for (int s = 1; s <= depth; s++) {
        // generation s: rows [s, th - s), words 1 .. nw-2
        const int r_lo = s, nrows = th - 2 * s, ns = (nrows + kLifeStrip - 1) / kLifeStrip, ncw = nw - 2;
        for (int t = threadIdx.x; t < ncw * ns; t += blockDim.x) {
            const int sidx = t / ncw, w = 1 + (t - sidx * ncw);
            const int r0 = r_lo + min(sidx * kLifeStrip, nrows - kLifeStrip);  // last strip ends at the last row
            if (interior) life_strip<false>(src, dst, nw, w, r0, 0u, 0, 0);
            else life_strip<true>(src, dst, nw, w, r0, life_colmask(wx0, w, cols), row_lo, row_hi);
        }
        __syncthreads();
        uint32_t *done = dst;
        dst = const_cast<uint32_t *>(src);
        src = done;
    }
    // write the block: 64 x 32 cells, four per thread task, as int32
    const uint32_t *res = src;
    const int wb = hx / 4;  // first word of the block
    for (int t = threadIdx.x; t < (kSt2BX / 4) * kSt2BY; t += blockDim.x) {
        const int ry = t / (kSt2BX / 4), wx = t - ry * (kSt2BX / 4);
        const uint32_t v = res[(depth + ry) * nw + wb + wx];
        const int gy = y0 + ry, gx = x0 + 4 * wx;
        if (gy >= rows) continue;
        int32_t *o = out + (size_t)gy * cols + gx;
        if (gx + 4 <= cols) {
            *reinterpret_cast<int4 *>(o) = make_int4(v & 0xFF, (v >> 8) & 0xFF, (v >> 16) & 0xFF, v >> 24);
        } else {
            for (int i = 0; i < 4 && gx + i < cols; i++) o[i] = (v >> (8 * i)) & 0xFF;
        }
    }
}

inline int life_packed_halo(int depth) { return halo_x<int32_t>(depth + 3); }

inline size_t life_packed_smem(int depth) {
    const int hx = life_packed_halo(depth);
    const size_t cells = (size_t)(kSt2BX + 2 * hx) * (kSt2BY + 2 * depth);
    return (size_t)kStHeader + cells * sizeof(int32_t) + 2 * cells;  // staged int32 window + two packed buffers
}

// `depth` Life generations from `in` (every cell 0 or 1) to `out`, neutral 0.
// Needs the grid to be addressable by TMA; returns cudaErrorNotSupported
// otherwise (the caller then runs the cell-by-cell kernel).
inline cudaError_t launch_life_packed(const int32_t *in, int32_t *out, int rows, int cols, int depth, unsigned *err,
                                      cudaStream_t st) {
    const int hx = life_packed_halo(depth);
    const int pitch = kSt2BX + 2 * hx, th = kSt2BY + 2 * depth;
    if (depth < 1 || th > 256 || !stencil_tma_ok<int32_t>(in, cols, pitch, th) || ((uintptr_t)out & 15) || (cols & 3))
        return cudaErrorNotSupported;
    const size_t smem = life_packed_smem(depth);
    if (smem > kMaxStencilSmem) return cudaErrorNotSupported;
    CUtensorMap map{};
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(int32_t)};
    cuuint32_t box[2] = {(cuuint32_t)pitch, (cuuint32_t)th};
    cuuint32_t estr[2] = {1, 1};
    if (tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, const_cast<int32_t *>(in), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorNotSupported;
    if (smem > 48 * 1024) cudaFuncSetAttribute(life_packed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((cols + kSt2BX - 1) / kSt2BX, (rows + kSt2BY - 1) / kSt2BY);
    life_packed_kernel<<<grid, 256, smem, st>>>(map, out, rows, cols, depth, hx, err);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
