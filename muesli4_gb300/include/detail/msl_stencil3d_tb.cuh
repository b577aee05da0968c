// Two sweeps per launch of a 7-point 3-D stencil (heat3D) by z-marching:
// temporal blocking without the z halo of a block.
//
// One CTA owns a 64 x 32 (x, y) tile and marches through a chunk of z planes.
// Step t of the march
//   * computes the first sweep ("intermediate") at plane t+1 on the tile plus
//     a one-cell margin into one of two intermediate planes in shared memory:
//     the tile's cells by register strips, the 192 margin cells (the row above
//     and below, the column left and right; a star reads no diagonal, so the
//     corners are not needed) as six whole-warp items;
//   * computes the second sweep at plane t from the intermediate planes t-1,
//     t and t+1, straight to HBM;
// and one barrier ends the step. Input planes (a 72 x 36 window: the tile
// plus two cells on every side, x rounded out to 16 bytes) arrive by TMA in a
// ring of four slots, issued two steps before their first use.
//
// Every thread owns a strip of two adjacent columns by four rows, kept as
// four packed pairs (one per row), and holds its input and intermediate values
// of the three planes a star reads in registers (B, centre and F of both
// sweeps; N and S inside the strip; W of the right column and E of the left).
// The pairs move between registers and shared memory as 64-bit accesses; only
// the strip's outer W and E cells and its two end rows come from shared
// memory cell by cell or pair by pair. The margin lanes keep
// their input values in registers the same way, so no step reads an input
// plane older than t+1 and the slot of plane t takes the load of plane t+4 as
// the step begins. The roles of the register columns rotate with the plane:
// the march is unrolled three times, so no value is copied between steps.
//
// heat3D divides the sum of six neighbours by 6. The sums and the division's
// fast path (div6_core) run on packed FP32 pairs, two cells per instruction;
// a warp vote finds the rare sums outside the fast path's range, and only
// then does the strip divide cell by cell with IEEE division where needed,
// exactly as star7 would compute it.
//
// Requirements (checked by the launcher): FP32 cells, a functor with
// kSum7Div6 (heat3D), neutral value +0 -- outside the grid both the staged
// input (TMA zero fill) and the intermediate sweep (set explicitly) hold 0,
// which is exactly the view's neutral value -- a grid TMA can address and an
// output 16-byte aligned (rows are then 8-byte aligned for the pair stores).
// Results are bit-identical to two launches of the one-sweep kernel: every
// cell of every sweep is computed by the same functor from the same operands;
// only where the operands live differs.
#pragma once

#include "msl_stencil.cuh"

namespace msl {
namespace gpu {

constexpr int kZtbBX = 64, kZtbBY = 32, kZtbRPT = 4, kZtbThreads = 256;
constexpr int kZtbPitch = kZtbBX + 8;                    // 72: window x0-4 .. x0+67
constexpr int kZtbRows = kZtbBY + 4;                     // 36: window y0-2 .. y0+33
constexpr int kZtbPlane = kZtbPitch * kZtbRows;          // floats per input slot (10368 bytes = 81 x 128)
constexpr int kZtbMidPlane = kZtbPitch * (kZtbBY + 2);   // intermediate slot: window rows 1 .. 34
constexpr int kZtbInSlots = 4, kZtbMidSlots = 2;         // plane p in input slot p & 3, intermediate slot p & 1
constexpr int kZtbMarginWarps = 6;                       // 192 margin cells = six warp items

inline size_t stencil3d_ztb_smem() {
    return (size_t)kStHeader + ((size_t)kZtbInSlots * kZtbPlane + (size_t)kZtbMidSlots * kZtbMidPlane) * sizeof(float);
}

// Functors declaring kSum7Div6 compute star7 as sum7 / 6 correctly rounded,
// with sum7 = (((((0 + w) + e) + n) + s) + b) + f (heat3D).
template <class Fn, class = void> struct IsSum7Div6 : std::false_type {};
template <class Fn> struct IsSum7Div6<Fn, std::void_t<decltype(Fn::kSum7Div6)>> : std::bool_constant<Fn::kSum7Div6> {};

// heat3D's sum of six neighbours for a pair, without the order's leading
// 0 + w: ((((w + e) + n) + s) + b) + f. It equals (((((0 + w) + e) + n) + s) +
// b) + f except when every term is -0 (then -0 against +0: the chain from +0
// never reaches -0, and once a nonzero term or a +0 enters, both chains agree
// from there on). Such a sum lies outside the division's fast-path range, and
// div6_pairs' fallback adds +0 before dividing, so the quotient is the same.
MSL_DEV f32x2 sum7x2(f32x2 w, f32x2 e, f32x2 n, f32x2 s, f32x2 b, f32x2 f) {
    f32x2 v = add2(w, e);
    v = add2(v, n);
    v = add2(v, s);
    v = add2(v, b);
    return add2(v, f);
}
// div6_core on both halves: q = x * RN(1/6), r = x - 6q (exact), q + r * RN(1/6).
MSL_DEV f32x2 div6_core2(f32x2 x) {
    const float zh = 0.16666667163372039794921875f;
    const f32x2 z2 = pk2(zh, zh);
    const f32x2 q = mul2(x, z2);
    const f32x2 r = fma2(q, pk2(-6.0f, -6.0f), x);
    return fma2(r, z2, q);
}
// True when all eight halves of the strip's four pairs lie in the division's
// fast-path range 2^-122 <= |x| <= FLT_MAX: one predicate chained through the
// comparisons (NaN compares false).
MSL_DEV bool strip_in_range(const f32x2 (&v)[4]) {
    unsigned r;
    asm("{\n\t.reg .pred p;\n\t.reg .f32 a0, a1, a2, a3, a4, a5, a6, a7;\n\t"
        "mov.b64 {a0, a1}, %1;\n\tmov.b64 {a2, a3}, %2;\n\tmov.b64 {a4, a5}, %3;\n\tmov.b64 {a6, a7}, %4;\n\t"
        "abs.f32 a0, a0;\n\tabs.f32 a1, a1;\n\tabs.f32 a2, a2;\n\tabs.f32 a3, a3;\n\t"
        "abs.f32 a4, a4;\n\tabs.f32 a5, a5;\n\tabs.f32 a6, a6;\n\tabs.f32 a7, a7;\n\t"
        "setp.ge.f32 p, a0, 0f02800000;\n\tsetp.le.and.f32 p, a0, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a1, 0f02800000, p;\n\tsetp.le.and.f32 p, a1, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a2, 0f02800000, p;\n\tsetp.le.and.f32 p, a2, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a3, 0f02800000, p;\n\tsetp.le.and.f32 p, a3, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a4, 0f02800000, p;\n\tsetp.le.and.f32 p, a4, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a5, 0f02800000, p;\n\tsetp.le.and.f32 p, a5, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a6, 0f02800000, p;\n\tsetp.le.and.f32 p, a6, 0f7F7FFFFF, p;\n\t"
        "setp.ge.and.f32 p, a7, 0f02800000, p;\n\tsetp.le.and.f32 p, a7, 0f7F7FFFFF, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "l"(v[0]), "l"(v[1]), "l"(v[2]), "l"(v[3]));
    return r != 0;
}
// IEEE-correct x / 6 for sums outside the fast path's range; out of line so
// that the rare path does not crowd the march's instruction cache. The +0
// turns a -0 sum of sum7x2 into the +0 that the reference's order yields.
static __device__ __noinline__ float div6_cold(float x) { return div6_rn(__fadd_rn(x, 0.0f)); }

// x / 6 for the four pairs of a strip: the fast path for the whole warp when
// every lane's `good` holds (its live cells' sums lie in the fast path's
// range), else div6_rn cell by cell (IEEE division outside the range).
MSL_DEV void div6_pairs(bool good, f32x2 (&x)[4]) {
    if (__all_sync(0xFFFFFFFFu, good)) {
#pragma unroll
        for (int k = 0; k < 4; k++) x[k] = div6_core2(x[k]);
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) x[k] = pk2(div6_cold(lo2(x[k])), div6_cold(hi2(x[k])));
    }
}

// Three CTAs per SM (80 registers, 61 KB each): measured faster than two
// CTAs with the registers the march would take unbounded (114).
constexpr int kZtbMinCtas = 3;
// kResid: the launch folds max |new - old| of the second sweep into *resid
// (one instantiation each, so that registers are allocated for the form that
// runs).
template <class Fn, bool kResid>
__global__ void __launch_bounds__(kZtbThreads, kZtbMinCtas)
    stencil3d_ztb_kernel(const __grid_constant__ CUtensorMap tmap, float *out, int depth, int rows, int cols,
                         int zchunk, Fn fn, unsigned long long *resid, unsigned *err) {
    static_assert(IsSum7Div6<Fn>::value, "the two-sweep kernel takes sum7 / 6 functors");
    static_assert(kZtbRPT == 4 && kZtbBY == 8 * kZtbRPT, "eight warps of 64 x 4 cells");
    constexpr int P = kZtbPitch;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);  // one mbarrier per input slot
    float *in_ring = reinterpret_cast<float *>(smem_raw + kStHeader);
    float *mid_ring = in_ring + kZtbInSlots * kZtbPlane;

    // chunk-major order: the CTAs resident together march neighbouring tiles
    // at the same depth, so the halo lines one fetches are in L2 for the next
    const unsigned tiles_x = (unsigned)(cols + kZtbBX - 1) / kZtbBX;
    const unsigned tiles = tiles_x * ((unsigned)(rows + kZtbBY - 1) / kZtbBY);
    const unsigned tile = blockIdx.x % tiles, chunk = blockIdx.x / tiles;
    const int x0 = (int)(tile % tiles_x) * kZtbBX, y0 = (int)(tile / tiles_x) * kZtbBY;
    const int zb = (int)chunk * zchunk, ze = min(zb + zchunk, depth);
    const int wx0 = x0 - 4, wy0 = y0 - 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the thread that issues and waits for the TMA loads: lane 0 of the last
    // warp, which has no margin item
    const bool leader = threadIdx.x == kZtbThreads - 32;

    // this thread's strip: window columns cx, cx+1 (8-byte aligned), rows cy .. cy+3
    const int cx = 4 + 2 * lane, cy = 2 + warp * kZtbRPT;
    const int gx = wx0 + cx, gy0 = wy0 + cy;
    const int own = cy * P + cx, own_mid = own - P;  // intermediate slots start at window row 1
    const bool x_in = gx < cols;
    // every strip cell lies inside the grid (margin cells are tested one by one)
    const bool full = x0 + kZtbBX <= cols && y0 + kZtbBY <= rows;

    // margin item of warps 0..5: rows 1 and 34 over columns 4..67 (warps
    // 0-3), columns 3 and 68 over rows 2..33 (warps 4-5, half a warp each)
    const bool has_margin = warp < kZtbMarginWarps;
    int mx = cx, my = cy;
    if (warp < 4) {
        mx = 4 + (warp & 1) * 32 + lane;
        my = warp < 2 ? 1 : kZtbBY + 2;
    } else if (has_margin) {
        mx = lane < 16 ? 3 : kZtbBX + 4;
        my = 2 + (warp - 4) * 16 + (lane & 15);
    }
    const int mo = my * P + mx, mo_mid = mo - P;
    const bool m_in = wx0 + mx >= 0 && wx0 + mx < cols && wy0 + my >= 0 && wy0 + my < rows;

    __shared__ int s_fail;  // set by the leader when a plane's wait gives up
    if (threadIdx.x == 0) s_fail = 0;
    uint32_t phase = 0, pending = 0;  // leader: per slot, the parity of its next completion / a load not waited for
    auto slot = [&](int p) { return in_ring + (p & 3) * kZtbPlane; };
    auto issue = [&](int p) {  // leader: TMA load of input plane p (zeros outside the grid)
        const int k = p & 3;
        pending |= 1u << k;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[k], (uint32_t)(kZtbPlane * sizeof(float)));
        tma_load_3d(slot(p), &tmap, &bar[k], wx0, wy0, p);
    };
    // Only the leader waits for a plane (the other warps sleep at the barrier
    // that follows instead of polling); the barrier makes it visible to all.
    auto wait_plane = [&](int p) {
        const int k = p & 3;
        const bool ok = mbar_wait_bounded(&bar[k], (phase >> k) & 1u, err);  // the load has landed either way
        phase ^= 1u << k;
        pending &= ~(1u << k);
        return ok;
    };
    auto drain = [&]() {  // leader, on failure: loads in flight land before the CTA gives up its shared memory
        for (int k = 0; k < kZtbInSlots; k++)
            if (pending & (1u << k)) mbar_poll(&bar[k], (phase >> k) & 1u, kMaxWaitPolls);
    };

    if (leader) {
        for (int k = 0; k < kZtbInSlots; k++) mbar_init(&bar[k], 1);
        fence_barrier_init();
    }
    __syncthreads();
    // Input planes zb-2 .. ze+1 are each loaded once and waited for once:
    // the first four here, plane t+4 at step t, waited for at step t+1.
    bool ok = true;
    if (leader) {
        for (int p = zb - 2; p <= zb + 1; p++) issue(p);
        ok = wait_plane(zb - 2);
        ok = wait_plane(zb - 1) && ok;
        ok = wait_plane(zb) && ok;
    }
    if (!__syncthreads_and(ok)) {
        if (leader) drain();
        return;
    }

    // register columns, pair k = row k of the strip
    auto load_col = [&](f32x2 (&d)[4], const float *plane) {
#pragma unroll
        for (int k = 0; k < 4; k++) d[k] = ld_pair(plane + own + k * P);
    };
    f32x2 ia[4], ib[4], ic[4];  // input columns
    f32x2 ma[4], mb[4], mc[4];  // intermediate columns
    float pa = 0.0f, pb = 0.0f, pc = 0.0f;  // the margin cell's input values
    load_col(ia, slot(zb - 2));
    load_col(ib, slot(zb - 1));
    if (has_margin) {
        pa = slot(zb - 2)[mo];
        pb = slot(zb - 1)[mo];
    }
    __syncthreads();  // plane zb-2's slot is read before step zb-2 reloads it

    double dmax = 0.0;
    auto live_row = [&](auto full_tag, int j) {
        constexpr bool FULL = decltype(full_tag)::value;
        return FULL || (x_in && gy0 + j < rows);
    };
    // One sweep of the strip: W, E and the strip's ends from the plane in
    // shared memory (q: the strip's first cell, rows P apart), B, the centre
    // (N and S inside the strip) and F from the register columns cb, cc, cf:
    // the four pairs' sums, then x / 6.
    auto sweep = [&](auto full_tag, const float *q, const f32x2 (&cb)[4], const f32x2 (&cc)[4],
                     const f32x2 (&cf)[4], f32x2 (&v)[4]) {
        const f32x2 n = ld_pair(q - P), s = ld_pair(q + kZtbRPT * P);
        bool good = true;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const f32x2 w = pk2(q[k * P - 1], lo2(cc[k]));
            const f32x2 e = pk2(hi2(cc[k]), q[k * P + 2]);
            const f32x2 nn = k == 0 ? n : cc[k - 1];
            const f32x2 ss = k == 3 ? s : cc[k + 1];
            v[k] = sum7x2(w, e, nn, ss, cb[k], cf[k]);
            if constexpr (!decltype(full_tag)::value)
                good = good && (!live_row(full_tag, k) || (div6_in_range(lo2(v[k])) && div6_in_range(hi2(v[k]))));
        }
        if constexpr (decltype(full_tag)::value) good = strip_in_range(v);
        div6_pairs(good, v);
    };
    // Step t: intermediate plane t+1 (from input planes t, t+1, t+2), then
    // output plane t (from intermediate planes t-1, t, t+1) when t >= zb.
    // Input roles: xb = plane t, xc = t+1, xf <- t+2; intermediate roles:
    // yb = t-1, yc = t, yf <- t+1; margin: qb = plane t, qf <- t+2.
    auto step = [&](auto full_tag, auto want_tag, int t, f32x2 (&xb)[4], f32x2 (&xc)[4], f32x2 (&xf)[4],
                    f32x2 (&yb)[4], f32x2 (&yc)[4], f32x2 (&yf)[4], float &qb, float &qf) {
        constexpr bool FULL = decltype(full_tag)::value, WANT = decltype(want_tag)::value;
        if (leader && t + 4 <= ze + 1) issue(t + 4);  // into the slot of plane t, last read at step t-1
        const float *pc_ = slot(t + 1), *pf_ = slot(t + 2);
        float *mw = mid_ring + ((t + 1) & 1) * kZtbMidPlane;
        load_col(xf, pf_);
        if (has_margin) qf = pf_[mo];

        // ---- first sweep, plane t+1 ----
        if (t + 1 >= 0 && t + 1 < depth) {
            sweep(full_tag, pc_ + own, xb, xc, xf, yf);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (!FULL && !live_row(full_tag, k)) yf[k] = pk2(0.0f, 0.0f);
                st_pair(mw + own_mid + k * P, yf[k]);
            }
            if (has_margin) {
                const float *r = pc_ + mo;
                const float sum = fn.sum7(r[-1], r[1], r[-P], r[P], qb, qf);
                float v = div6_core(sum);
                if (!__all_sync(0xFFFFFFFFu, !m_in || div6_in_range(sum)) && !div6_in_range(sum)) v = div6_cold(sum);
                mw[mo_mid] = m_in ? v : 0.0f;
            }
        } else {  // outside the grid the intermediate plane is the neutral value
#pragma unroll
            for (int k = 0; k < 4; k++) {
                yf[k] = pk2(0.0f, 0.0f);
                st_pair(mw + own_mid + k * P, yf[k]);
            }
            if (has_margin) mw[mo_mid] = 0.0f;
        }

        // ---- second sweep, plane t ----
        if (t >= zb) {
            f32x2 v[4];
            sweep(full_tag, mid_ring + (t & 1) * kZtbMidPlane + own_mid, yb, yc, yf, v);
            float *o = out + ((size_t)t * rows + gy0) * cols + gx;
#pragma unroll
            for (int k = 0; k < kZtbRPT; k++) {
                if (live_row(full_tag, k)) {
                    if constexpr (WANT) {
                        const double d0 = fabs((double)lo2(v[k]) - (double)lo2(yc[k]));
                        const double d1 = fabs((double)hi2(v[k]) - (double)hi2(yc[k]));
                        if (d0 > dmax || d0 != d0) dmax = d0;
                        if (d1 > dmax || d1 != d1) dmax = d1;
                    }
                    st_pair(o + (size_t)k * cols, v[k]);
                }
            }
        }
        if (leader && t + 3 <= ze + 1 && !wait_plane(t + 3)) s_fail = 1;  // read from step t+1 on
        __syncthreads();
        return s_fail == 0;
    };
    auto march = [&](auto full_tag, auto want_tag) {
        for (int t = zb - 2; ok && t < ze; t += 3) {
            ok = step(full_tag, want_tag, t, ia, ib, ic, ma, mb, mc, pa, pc);
            if (ok && t + 1 < ze) ok = step(full_tag, want_tag, t + 1, ib, ic, ia, mb, mc, ma, pb, pa);
            if (ok && t + 2 < ze) ok = step(full_tag, want_tag, t + 2, ic, ia, ib, mc, ma, mb, pc, pb);
        }
    };
    // one march per case, so that the common one (every strip cell inside)
    // carries no tests it does not need
    if (full) march(std::true_type{}, std::bool_constant<kResid>{});
    else march(std::false_type{}, std::bool_constant<kResid>{});
    if (!ok && leader) drain();
    if constexpr (kResid) {
        dmax = block_max(dmax);
        if (threadIdx.x == 0) atomic_max_nonneg(resid, dmax);
    }
}

// z planes per CTA: the longest chunk (26 planes down to 4) that still gives
// at least two waves of resident CTAs. Longer chunks spend less on the first
// sweep's two extra planes and the march's start; on heat3D 512^3 (128 tiles,
// 456 resident CTAs) 26 planes measured best (10.67 ms per 100 sweeps against
// 10.79 for 24, 10.89 for 20 and 22, 10.97 for 28, 11.1 for 32).
inline int stencil3d_ztb_zchunk(int depth, long long tiles, long long resident) {
    static const int kCand[] = {26, 24, 16, 12, 8, 6, 4};
    for (int z : kCand)
        if (tiles * ((depth + z - 1) / z) >= 2 * resident) return z;
    return 4;
}

// Two sweeps in -> out of a kSum7Div6 functor with neutral +0 on FP32 cells;
// cudaErrorNotSupported when the grid does not suit the kernel. zchunk 0
// picks the chunk length.
template <class Fn>
cudaError_t launch_stencil3d_ztb(const float *in, float *out, int depth, int rows, int cols, Fn fn,
                                 unsigned long long *resid, unsigned *err, cudaStream_t st, int zchunk = 0) {
    if (!stencil_tma_ok<float>(in, cols, kZtbPitch, kZtbRows) || ((uintptr_t)out % 16) != 0)
        return cudaErrorNotSupported;
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
    auto k = resid ? stencil3d_ztb_kernel<Fn, true> : stencil3d_ztb_kernel<Fn, false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    static int per_sm = 0, sms = 0;  // per functor; both forms share launch bounds and shared memory
    if (per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kZtbThreads, smem);
        if (per_sm < 1) per_sm = 1;
    }
    const long long tiles = (long long)((cols + kZtbBX - 1) / kZtbBX) * ((rows + kZtbBY - 1) / kZtbBY);
    const int zc = zchunk > 0 ? zchunk : stencil3d_ztb_zchunk(depth, tiles, (long long)per_sm * sms);
    const long long blocks = tiles * ((depth + zc - 1) / zc);
    if (blocks > 0x7FFFFFFFLL) return cudaErrorNotSupported;
    k<<<(unsigned)blocks, kZtbThreads, smem, st>>>(map, out, depth, rows, cols, zc, fn, resid, err);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
