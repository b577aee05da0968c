// Two sweeps per launch of a 7-point 3-D stencil (heat3D) by z-marching:
// temporal blocking without the z halo of a block.
//
// One CTA owns a 64 x 16 column of cells and marches through a chunk of z
// planes. Each step stages an input plane (window 72 x 20: the column plus
// two cells on every side in x and y) with one TMA load into a ring of six
// planes (loads run two steps ahead), computes the first sweep
// ("intermediate") on the column plus a one-cell margin (66 x 18 cells) into
// a ring of three planes, and the second sweep on the column from the
// intermediate planes, straight to HBM. The z
// halo costs two intermediate planes per chunk instead of two per block;
// the x/y margin costs 16 % more first-sweep cells. Every thread owns four
// vertically adjacent cells of the column and keeps their input and
// intermediate values for three consecutive planes in registers (centre, B
// and F of both sweeps); W, E, N and S come from shared memory. One barrier
// per plane.
//
// Requirements (checked by the launcher): FP32 cells, a functor with
// kStar7 (the six face neighbours; heat3D), neutral value +0 -- outside the
// grid both the staged input (TMA zero fill) and the intermediate sweep (set
// explicitly) hold 0, which is exactly the view's neutral value -- and a grid
// TMA can address. Results are bit-identical to two launches of the one-sweep
// kernel: every cell of every sweep is computed by the same functor from the
// same operands; only where the operands live differs.
#pragma once

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

constexpr int kZtbChunk = 32;                    // z planes per CTA
constexpr int kZtbPitch = kT3BX + 8;              // 72: x window (2-cell halo rounded up to 16 bytes)
constexpr int kZtbRows = kT3BY + 4;               // 20: y window
constexpr int kZtbPlane = kZtbPitch * kZtbRows;   // floats per staged plane
constexpr int kZtbIn = 6, kZtbMid = 3;            // ring planes: input (two planes of look-ahead), intermediate

inline size_t stencil3d_ztb_smem() {
    return (size_t)kStHeader + (size_t)(kZtbIn + kZtbMid) * kZtbPlane * sizeof(float);
}

template <class Fn, class = void> struct IsSum7Div6 : std::false_type {};
template <class Fn> struct IsSum7Div6<Fn, std::void_t<decltype(Fn::kSum7Div6)>> : std::bool_constant<Fn::kSum7Div6> {};

// One cell of a sweep. A functor whose value is sum7 / 6 (heat3D) takes the
// division's fast path here; `ok` is cleared when a live cell's sum lies
// outside that path's range, and ztb_fixup redoes those cells.
template <class Fn>
MSL_DEV float ztb_cell(const Fn &fn, float w, float e, float n, float s, float b, float f, bool live, float &sum,
                       bool &ok) {
    if constexpr (IsSum7Div6<Fn>::value) {
        sum = fn.sum7(w, e, n, s, b, f);
        ok = ok && (!live || div6_in_range(sum));
        return div6_core(sum);
    } else {
        return fn.star7(w, e, n, s, b, f);
    }
}

// One vote per warp and sweep: if any lane holds a sum outside the fast
// division's range, those cells take IEEE division.
template <class Fn, int N>
MSL_DEV void ztb_fixup(const Fn &, bool ok, const bool (&live)[N], const float (&sum)[N], float (&v)[N]) {
    if constexpr (IsSum7Div6<Fn>::value) {
        if (__all_sync(0xFFFFFFFFu, ok)) return;
#pragma unroll
        for (int j = 0; j < N; j++)
            if (live[j] && !div6_in_range(sum[j])) v[j] = __fdiv_rn(sum[j], 6.0f);
    }
}

template <class Fn>
__global__ void __launch_bounds__(kT3Threads, 4)
    stencil3d_ztb_kernel(const __grid_constant__ CUtensorMap tmap, float *out, int depth, int rows, int cols, Fn fn,
                         unsigned long long *resid, unsigned *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);  // one mbarrier per input slot
    float *in_ring = reinterpret_cast<float *>(smem_raw + kStHeader);
    float *mid_ring = in_ring + kZtbIn * kZtbPlane;
    const int x0 = blockIdx.x * kT3BX, y0 = blockIdx.y * kT3BY, zb = blockIdx.z * kZtbChunk;
    const int ze = min(zb + kZtbChunk, depth);
    const int wx0 = x0 - 4, wy0 = y0 - 2;  // window origin (x halo 4 for 16-byte TMA alignment)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // this thread's four cells: window column cx, rows cy .. cy+3
    const int cx = 4 + (warp & 1) * 32 + lane, cy = 2 + (warp >> 1) * kT3RPT;
    const int gx = wx0 + cx, gy0 = wy0 + cy;
    const bool x_in = gx < cols;
    const bool xy_in = x0 + kT3BX <= cols && y0 + kT3BY <= rows;  // every thread's own cells lie in the grid
    // margin cell of the first sweep (threads 0 .. 163): window columns 3 and
    // 68 for rows 1..18, and rows 1 and 18 for columns 4..67
    int mx = -1, my = -1;
    {
        const int t = threadIdx.x;
        if (t < 36) {
            mx = t < 18 ? 3 : 4 + kT3BX;
            my = 1 + (t < 18 ? t : t - 18);
        } else if (t < 36 + 2 * kT3BX) {
            const int u = t - 36;
            mx = 4 + (u % kT3BX);
            my = u < kT3BX ? 1 : 2 + kT3BY;
        }
    }
    const bool has_margin = mx >= 0;
    const int mgx = wx0 + mx, mgy = wy0 + my;
    const bool m_in = has_margin && mgx >= 0 && mgx < cols && mgy >= 0 && mgy < rows;

    // ring slots: input plane p in slot (p + 2) % kZtbIn, intermediate plane
    // p in slot (p + 1) % kZtbMid; slot indices are advanced step by step
    auto in_at = [&](int k) { return in_ring + k * kZtbPlane; };
    auto mid_at = [&](int k) { return mid_ring + k * kZtbPlane; };
    auto next_in = [](int k) { return k == kZtbIn - 1 ? 0 : k + 1; };
    auto next_mid = [](int k) { return k == kZtbMid - 1 ? 0 : k + 1; };
    auto in_slot = [&](int p) { return (p - zb + 2) % kZtbIn; };  // p >= zb - 2; used outside the loop
    uint32_t pending = 0;  // thread 0: bit k = a load into slot k not yet waited for
    auto issue = [&](int p) {  // thread 0: TMA load of input plane p (zeros outside the grid)
        const int k = in_slot(p);
        pending |= 1u << k;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[k], (uint32_t)(kZtbPlane * sizeof(float)));
        tma_load_3d(in_at(k), &tmap, &bar[k], wx0, wy0, p);
    };
    // Only thread 0 waits for a plane (the other warps sleep at the barrier
    // that follows instead of polling); the barrier then makes the plane
    // visible to every thread.
    uint32_t phase = 0;  // thread 0: bit k = parity of the next completion of slot k
    auto wait_slot = [&](int k) {
        if (threadIdx.x != 0) return true;
        const bool ok = mbar_wait_bounded(&bar[k], (phase >> k) & 1u, err);  // the load has landed either way
        phase ^= 1u << k;
        pending &= ~(1u << k);
        return ok;
    };

    if (threadIdx.x == 0) {
        for (int k = 0; k < kZtbIn; k++) mbar_init(&bar[k], 1);
        fence_barrier_init();
    }
    __syncthreads();
    // prologue loads: input planes zb-2 .. zb+kZtbIn-3 (each plane zb-2 .. ze+1
    // is loaded once and waited for once)
    if (threadIdx.x == 0)
        for (int p = zb - 2; p <= min(zb + kZtbIn - 3, ze + 1); p++) issue(p);

    using Col = float[kT3RPT];
    auto load_col = [&](Col &dst, const float *plane) {
        const float *q = plane + cy * kZtbPitch + cx;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) dst[j] = q[j * kZtbPitch];
    };
    // First sweep at plane p for this thread's cells and margin cell from
    // input planes pb = p-1, pc = p, pf = p+1 (staged; the own column's values
    // in registers cb, cc, cf). Writes the intermediate plane (0 outside the
    // grid) to `m` and this thread's values to `res`. FULL: plane p and the
    // thread's own cells lie inside the grid (no per-cell tests).
    auto first_sweep = [&](auto full_tag, int p, const float *pb, const float *pc, const float *pf, const Col &cb,
                           const Col &cc, const Col &cf, float *m, Col &res) {
        constexpr bool FULL = decltype(full_tag)::value;
        const bool p_in = FULL || (p >= 0 && p < depth);
        const float *q = pc + cy * kZtbPitch + cx;
        const float n = q[-kZtbPitch], s = q[kT3RPT * kZtbPitch];
        float sum[kT3RPT + 1], v[kT3RPT + 1];
        bool live[kT3RPT + 1];
        bool ok = true;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            live[j] = FULL || (p_in && x_in && gy0 + j < rows);
            v[j] = ztb_cell(fn, q[j * kZtbPitch - 1], q[j * kZtbPitch + 1], j == 0 ? n : cc[j - 1],
                            j == kT3RPT - 1 ? s : cc[j + 1], cb[j], cf[j], live[j], sum[j], ok);
        }
        const int o = has_margin ? my * kZtbPitch + mx : 0;
        live[kT3RPT] = has_margin && p_in && m_in;
        v[kT3RPT] = 0.0f;
        sum[kT3RPT] = 0.0f;
        if (has_margin)
            v[kT3RPT] = ztb_cell(fn, pc[o - 1], pc[o + 1], pc[o - kZtbPitch], pc[o + kZtbPitch], pb[o], pf[o],
                                 live[kT3RPT], sum[kT3RPT], ok);
        ztb_fixup(fn, ok, live, sum, v);
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            const float x = live[j] ? v[j] : 0.0f;
            res[j] = x;
            m[(cy + j) * kZtbPitch + cx] = x;
        }
        if (has_margin) m[o] = live[kT3RPT] ? v[kT3RPT] : 0.0f;
    };

    // Registers: three input columns and three intermediate columns whose
    // roles rotate with the plane (the loop below is unrolled three times so
    // that every role is a fixed register array: no copies between steps).
    Col ca, cb, cc;  // input columns
    Col ma, mb, mc;  // intermediate columns
    bool ok = true;
    int kin = 0, kmid = 0;  // slot of input plane t-1 and of intermediate plane t-1 at step t
    // prologue: intermediate planes zb-1 and zb, from input planes zb-2 .. zb+1
    {
        const int k0 = 0, k1 = 1, k2 = 2, k3 = 3;  // slots of input planes zb-2 .. zb+1
        ok = wait_slot(k0) && wait_slot(k1) && wait_slot(k2);
        ok = __syncthreads_and(ok);
        if (ok) {
            load_col(ca, in_at(k0));
            load_col(cb, in_at(k1));
            load_col(cc, in_at(k2));
            first_sweep(std::false_type{}, zb - 1, in_at(k0), in_at(k1), in_at(k2), ca, cb, cc, mid_at(0), mb);
            ok = wait_slot(k3);
        }
        ok = __syncthreads_and(ok);
        if (ok) {
            load_col(ca, in_at(k3));  // plane zb+1 takes the place of zb-2
            first_sweep(std::false_type{}, zb, in_at(k1), in_at(k2), in_at(k3), cb, cc, ca, mid_at(1), mc);
            ok = wait_slot(4);  // input plane zb+2, read by step zb
        }
        ok = __syncthreads_and(ok);  // intermediate planes zb-1 and zb visible
        kin = k1;                    // input plane zb-1
        kmid = 0;                    // intermediate plane zb-1
    }
    // now: cb = input zb-1, cc = input zb, ca = input zb+1; mb = intermediate
    // zb-1, mc = intermediate zb; ma is free

    double dmax = 0.0;
    const bool want = resid != nullptr;
    // Step t (final plane t; input plane t+2 is staged and visible). Input
    // roles: xb = plane t, xc = t+1, xf gets t+2; intermediate roles: yb =
    // t-1, yc = t, yf gets t+1.
    auto step = [&](int t, Col &xb, Col &xc, Col &xf, Col &yb, Col &yc, Col &yf) {
        const int s0 = next_in(kin), s1 = next_in(s0), s2 = next_in(s1);  // input planes t, t+1, t+2
        const int m1 = next_mid(kmid), m2 = next_mid(m1);                 // intermediate planes t, t+1
        // the slot of plane t-2 is free since step t-2: load plane t+4 into it
        if (threadIdx.x == 0 && t + kZtbIn - 2 <= ze + 1) issue(t + kZtbIn - 2);
        load_col(xf, in_at(s2));
        if (xy_in && t + 1 < depth)
            first_sweep(std::true_type{}, t + 1, in_at(s0), in_at(s1), in_at(s2), xb, xc, xf, mid_at(m2), yf);
        else
            first_sweep(std::false_type{}, t + 1, in_at(s0), in_at(s1), in_at(s2), xb, xc, xf, mid_at(m2), yf);
        // second sweep at plane t from intermediate planes t-1, t, t+1
        const float *q = mid_at(m1) + cy * kZtbPitch + cx;
        const float n = q[-kZtbPitch], s = q[kT3RPT * kZtbPitch];
        float sum[kT3RPT], v[kT3RPT];
        bool live[kT3RPT];
        bool ok2 = true;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            live[j] = xy_in || (x_in && gy0 + j < rows);
            v[j] = ztb_cell(fn, q[j * kZtbPitch - 1], q[j * kZtbPitch + 1], j == 0 ? n : yc[j - 1],
                            j == kT3RPT - 1 ? s : yc[j + 1], yb[j], yf[j], live[j], sum[j], ok2);
        }
        ztb_fixup(fn, ok2, live, sum, v);
        float *o = out + ((size_t)t * rows + gy0) * cols + gx;
#pragma unroll
        for (int j = 0; j < kT3RPT; j++) {
            if (live[j]) {
                if (want) {
                    const double d = fabs((double)v[j] - (double)yc[j]);
                    if (d > dmax || d != d) dmax = d;
                }
                o[(size_t)j * cols] = v[j];
            }
        }
        const bool good = __syncthreads_and(t + 1 < ze ? wait_slot(next_in(s2)) : true);  // plane t+3 for step t+1
        kin = s0;
        kmid = m1;
        return good;
    };
    for (int t = zb; ok && t < ze; t += 3) {
        ok = step(t, cc, ca, cb, mb, mc, ma);
        if (ok && t + 1 < ze) ok = step(t + 1, ca, cb, cc, mc, ma, mb);
        if (ok && t + 2 < ze) ok = step(t + 2, cb, cc, ca, ma, mb, mc);
    }
    if (!ok && threadIdx.x == 0) {
        // let loads still in flight land before the CTA gives up its shared memory
        for (int k = 0; k < kZtbIn; k++)
            if (pending & (1u << k)) mbar_poll(&bar[k], (phase >> k) & 1u, kMaxWaitPolls);
    }
    if (want) {
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// Two sweeps in -> out of a kStar7 functor with neutral +0 on FP32 cells;
// cudaErrorNotSupported when the grid does not suit the kernel.
template <class Fn>
cudaError_t launch_stencil3d_ztb(const float *in, float *out, int depth, int rows, int cols, Fn fn,
                                 unsigned long long *resid, unsigned *err, cudaStream_t st) {
    if (!stencil_tma_ok<float>(in, cols, kZtbPitch, kZtbRows)) return cudaErrorNotSupported;
    CUtensorMap map{};
    cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)depth};
    cuuint64_t strides[2] = {(cuuint64_t)cols * sizeof(float), (cuuint64_t)cols * rows * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)kZtbPitch, (cuuint32_t)kZtbRows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    if (tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(in), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorNotSupported;
    const size_t smem = stencil3d_ztb_smem();
    auto k = stencil3d_ztb_kernel<Fn>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((cols + kT3BX - 1) / kT3BX, (rows + kT3BY - 1) / kT3BY, (depth + kZtbChunk - 1) / kZtbChunk);
    k<<<grid, kT3Threads, smem, st>>>(map, out, depth, rows, cols, fn, resid, err);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
