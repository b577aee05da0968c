// 2-D box sum / mean over (2R+1)^2 FP32 cells, two columns per thread with
// packed FP32 additions.
//
// The reference's box (examples/meanblur2.cpp:46-57, restated in 2-D) adds
// the window's cells one at a time, dx outer and dy inner, starting from 0.
// Bit-exact results need exactly that chain of (2R+1)^2 rounded additions per
// cell, so the kernel is bound by FP32 additions at large R. With one column
// per thread the additions alone fill every issue slot and the shared-memory
// loads have to share them; `add.rn.f32x2` adds two independent lanes (two
// horizontally adjacent cells, each in its own reference order) in one
// issued instruction, which leaves issue slots for the loads and lets the
// FP32 pipe run full.
//
// One CTA of four warps computes a 64 x 32 block: lane p owns columns 2p and
// 2p + 1, warp w rows 8w .. 8w + 7 (eight rows share each column pair's
// loads, which keeps shared-memory traffic below the additions' rate). The window (block plus an R-cell halo, zeros outside the
// grid) is staged by one TMA load or by coalesced plain loads, then copied
// once shifted by one cell, so that every column pair -- starting at an even
// or an odd window column -- is one aligned 8-byte shared-memory load.
// Requirements (checked by the launcher): neutral value +0 (the zero fill),
// no residual.
#pragma once

#include <cstring>

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

constexpr int kBoxRows = 8;                      // rows per thread
constexpr int kBoxThreads = 32 * kSt2BY / kBoxRows;  // 32 column pairs x 4 warps x 8 rows = the 64 x 32 block

MSL_DEV unsigned long long add_f32x2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

inline size_t box2d_pair_smem(int r) {
    const int pitch = kSt2BX + 2 * halo_x<float>(r), th = kSt2BY + 2 * r;
    const size_t buf = ((size_t)pitch * th * sizeof(float) + 127) / 128 * 128;
    return (size_t)kStHeader + 2 * buf;  // the window and its copy shifted by one cell
}

template <int R, bool MEAN, bool TMA>
__global__ void __launch_bounds__(kBoxThreads)
    box2d_pair_kernel(const __grid_constant__ CUtensorMap tmap, const float *in, float *out, int rows, int cols,
                      unsigned *err) {
    constexpr int HX = (R + 3) / 4 * 4;  // halo_x<float>(R)
    constexpr int P = kSt2BX + 2 * HX, TH = kSt2BY + 2 * R;
    constexpr int BUF = (P * TH * 4 + 127) / 128 * 128 / 4;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    float *win = reinterpret_cast<float *>(smem_raw + kStHeader);
    float *shifted = win + BUF;  // shifted[i] = win[i + 1]
    const int x0 = blockIdx.x * kSt2BX, y0 = blockIdx.y * kSt2BY;
    const int wx0 = x0 - HX, wy0 = y0 - R;
    bool ok = true;
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_barrier_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(bar, (uint32_t)(P * TH * sizeof(float)));
            tma_load_2d(win, &tmap, bar, wx0, wy0);
        }
        ok = mbar_wait_bounded(bar, 0, err);
    } else {
        stage_window<float>(win, in, P, TH, TH, wx0, wy0, 0, 1, rows, cols);
    }
    ok = __syncthreads_and(ok);
    if (!ok) return;
    for (int i = threadIdx.x; i < P * TH - 1; i += kBoxThreads) shifted[i] = win[i + 1];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wc = HX + 2 * lane;           // window column of the pair's first cell
    const int wr = R + kBoxRows * warp;     // window row of the thread's first cell
    unsigned long long s[kBoxRows];
#pragma unroll
    for (int j = 0; j < kBoxRows; j++) s[j] = 0ull;  // two +0.0f
#pragma unroll 1
    for (int dx = -R; dx <= R; dx++) {
        const int c = wc + dx;
        const float *base = ((c & 1) ? shifted + (c - 1) : win + c) + (wr - R) * P;
        unsigned long long v[kBoxRows + 2 * R];
#pragma unroll
        for (int k = 0; k < kBoxRows + 2 * R; k++) v[k] = *reinterpret_cast<const unsigned long long *>(base + k * P);
#pragma unroll
        for (int j = 0; j < kBoxRows; j++)
#pragma unroll
            for (int dy = 0; dy <= 2 * R; dy++) s[j] = add_f32x2(s[j], v[j + dy]);
    }
    const int x = x0 + 2 * lane;
    if (x >= cols) return;
#pragma unroll
    for (int j = 0; j < kBoxRows; j++) {
        const int y = y0 + kBoxRows * warp + j;
        if (y >= rows) break;
        float2 r2 = *reinterpret_cast<float2 *>(&s[j]);
        if (MEAN) {
            r2.x = __fdiv_rn(r2.x, float((2 * R + 1) * (2 * R + 1)));  // IEEE division, as the reference
            r2.y = __fdiv_rn(r2.y, float((2 * R + 1) * (2 * R + 1)));
        }
        float *o = out + (size_t)y * cols + x;
        if (x + 1 < cols && (cols & 1) == 0) {
            *reinterpret_cast<float2 *>(o) = r2;
        } else {
            o[0] = r2.x;
            if (x + 1 < cols) o[1] = r2.y;
        }
    }
}

// One box sweep in -> out with neutral +0 and no residual; returns
// cudaErrorNotSupported when that does not apply (the caller then runs the
// one-column-per-thread kernel).
template <int R, bool MEAN>
cudaError_t launch_box2d_pair(const float *in, float *out, int rows, int cols, float neutral, unsigned long long *resid,
                              unsigned *err, cudaStream_t st, bool allow_tma) {
    uint32_t nbits;
    memcpy(&nbits, &neutral, sizeof nbits);
    if (resid || nbits != 0u || ((uintptr_t)out & 7)) return cudaErrorNotSupported;
    constexpr int HX = (R + 3) / 4 * 4;
    const int pitch = kSt2BX + 2 * HX, th = kSt2BY + 2 * R;
    const size_t smem = box2d_pair_smem(R);
    if (smem > kMaxStencilSmem) return cudaErrorNotSupported;
    dim3 grid((cols + kSt2BX - 1) / kSt2BX, (rows + kSt2BY - 1) / kSt2BY);
    CUtensorMap map{};
    const bool tma = allow_tma && stencil_tma_ok<float>(in, cols, pitch, th);
    if (tma) {
        cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
        cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(float)};
        cuuint32_t box[2] = {(cuuint32_t)pitch, (cuuint32_t)th};
        cuuint32_t estr[2] = {1, 1};
        if (tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(in), dims, strides, box,
                                 estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorNotSupported;
        auto k = box2d_pair_kernel<R, MEAN, true>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, kBoxThreads, smem, st>>>(map, in, out, rows, cols, err);
    } else {
        auto k = box2d_pair_kernel<R, MEAN, false>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, kBoxThreads, smem, st>>>(map, in, out, rows, cols, err);
    }
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
