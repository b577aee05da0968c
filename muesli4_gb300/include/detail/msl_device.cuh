// Device-side building blocks shared by the prebuilt kernels of
// libmsl_gb300.so and by the C++ front end (user functors are instantiated in
// the user's translation unit with the same templates).
//
//  * non-contracting scalar arithmetic (the checkers evaluate a*b+c as two
//    roundings, so the kernels do too),
//  * 16-byte vector loads/stores of any trivially copyable element type,
//  * bfloat16 storage conversions,
//  * inline-PTX wrappers for mbarrier and TMA (cp.async.bulk.tensor), with
//    bounded waits that report a timeout instead of spinning forever.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef MSL_HD
#define MSL_HD __host__ __device__ __forceinline__
#endif
#ifndef MSL_DEV
#define MSL_DEV __device__ __forceinline__
#endif

namespace msl {
namespace gpu {

// ---- device error word -------------------------------------------------------
// Bit flags a kernel sets in a device word the host reads at its next
// synchronisation point (the library keeps one per context).
enum : unsigned {
    kErrBarrierTimeout = 1u,  // an mbarrier/TMA wait gave up
    kErrBadLaunch = 2u,       // a kernel saw launch parameters it cannot handle
};
// Upper bound on mbarrier.try_wait polls (each poll itself blocks for a
// hardware-defined interval); ~seconds in total, far above any legal wait.
constexpr unsigned kMaxWaitPolls = 1u << 22;
// The word after a kernel's error word holds the poll limit of its bounded
// waits: 0 means kMaxWaitPolls (msl_set_wait_limit sets it for the library's
// kernels).
MSL_DEV unsigned wait_poll_limit(const unsigned *err) {
    // set by the host between launches: read through the read-only cache, so
    // the CTAs of a launch do not all queue on one L2 line
    const unsigned v = err ? __ldg(err + 1) : 0u;
    return v ? v : kMaxWaitPolls;
}

MSL_DEV void report_error(unsigned *err, unsigned bits) {
    if (err) atomicOr(err, bits);
}

// ---- non-contracting arithmetic ----------------------------------------------
template <typename T> struct Arith {
    static MSL_HD T add(T a, T b) { return a + b; }
    static MSL_HD T sub(T a, T b) { return a - b; }
    static MSL_HD T mul(T a, T b) { return a * b; }
};
template <> struct Arith<float> {
    static MSL_DEV float add(float a, float b) { return __fadd_rn(a, b); }
    static MSL_DEV float sub(float a, float b) { return __fsub_rn(a, b); }
    static MSL_DEV float mul(float a, float b) { return __fmul_rn(a, b); }
};
template <> struct Arith<double> {
    static MSL_DEV double add(double a, double b) { return __dadd_rn(a, b); }
    static MSL_DEV double sub(double a, double b) { return __dsub_rn(a, b); }
    static MSL_DEV double mul(double a, double b) { return __dmul_rn(a, b); }
};
template <> struct Arith<int32_t> {  // two's-complement wrap-around
    static MSL_HD int32_t add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
    static MSL_HD int32_t sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
    static MSL_HD int32_t mul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
};

// ---- bfloat16 storage ----------------------------------------------------------
struct bf16s {
    uint16_t bits;
};
MSL_HD float bf16_to_f(bf16s h) {
    union { uint32_t u; float f; } c;
    c.u = (uint32_t)h.bits << 16;
    return c.f;
}
MSL_HD bf16s f_to_bf16(float f) {  // round to nearest even, NaN stays quiet
    union { uint32_t u; float f; } c;
    c.f = f;
    uint32_t u = c.u;
    if ((u & 0x7fffffffu) > 0x7f800000u) return bf16s{(uint16_t)((u >> 16) | 0x40u)};
    u += 0x7fffu + ((u >> 16) & 1u);
    return bf16s{(uint16_t)(u >> 16)};
}
// Storage type S -> arithmetic type used by the stencil functors.
template <typename S> struct Compute { using type = S; };
template <> struct Compute<bf16s> { using type = float; };
template <typename S> MSL_HD typename Compute<S>::type widen(S s) { return s; }
template <> MSL_HD float widen<bf16s>(bf16s s) { return bf16_to_f(s); }
template <typename S> MSL_HD S narrow(typename Compute<S>::type v) { return v; }
template <> MSL_HD bf16s narrow<bf16s>(float v) { return f_to_bf16(v); }

// ---- vectors ---------------------------------------------------------------------
template <int BYTES> struct RawWord;
template <> struct RawWord<16> { using type = uint4; };
template <> struct RawWord<8> { using type = uint2; };
template <> struct RawWord<4> { using type = uint32_t; };
template <> struct RawWord<2> { using type = uint16_t; };
template <> struct RawWord<1> { using type = uint8_t; };

template <typename T, int N> struct alignas(sizeof(T) * N <= 16 ? sizeof(T) * N : 16) Vec {
    T v[N];
};

// Load / store N consecutive elements starting at element index i (the address
// must be aligned to sizeof(T)*N when that is a power of two <= 16).
template <typename T, int N> MSL_DEV Vec<T, N> vload(const T *p, size_t i) {
    constexpr int B = (int)sizeof(T) * N;
    if constexpr (B == 16 || B == 8 || B == 4 || B == 2 || B == 1) {
        using W = typename RawWord<B>::type;
        union { W w; Vec<T, N> v; } u;
        u.w = *reinterpret_cast<const W *>(p + i);
        return u.v;
    } else {
        Vec<T, N> r;
#pragma unroll
        for (int k = 0; k < N; k++) r.v[k] = p[i + k];
        return r;
    }
}
template <typename T, int N> MSL_DEV void vstore(T *p, size_t i, const Vec<T, N> &x) {
    constexpr int B = (int)sizeof(T) * N;
    if constexpr (B == 16 || B == 8 || B == 4 || B == 2 || B == 1) {
        using W = typename RawWord<B>::type;
        union { W w; Vec<T, N> v; } u;
        u.v = x;
        *reinterpret_cast<W *>(p + i) = u.w;
    } else {
#pragma unroll
        for (int k = 0; k < N; k++) p[i + k] = x.v[k];
    }
}
// Elements per 16-byte vector for a kernel touching the given element types.
template <typename A> constexpr int vec_width1() {
    return (sizeof(A) <= 16 && 16 % sizeof(A) == 0) ? (int)(16 / sizeof(A)) : 1;
}
template <typename A, typename B> constexpr int vec_width2() {
    return vec_width1<A>() < vec_width1<B>() ? vec_width1<A>() : vec_width1<B>();
}
template <typename A, typename B, typename C> constexpr int vec_width3() {
    return vec_width2<A, B>() < vec_width1<C>() ? vec_width2<A, B>() : vec_width1<C>();
}
template <typename A, typename B, typename C, typename D> constexpr int vec_width4() {
    return vec_width3<A, B, C>() < vec_width1<D>() ? vec_width3<A, B, C>() : vec_width1<D>();
}

// True for +0 (all bits zero): the value TMA and the plain staging loads
// write outside a grid.
template <typename T> MSL_HD bool is_positive_zero(T v) {
    unsigned char b[sizeof(T)];
    memcpy(b, &v, sizeof(T));
    for (size_t i = 0; i < sizeof(T); i++)
        if (b[i]) return false;
    return true;
}

inline bool aligned_to(const void *p, size_t bytes) { return ((uintptr_t)p % bytes) == 0; }

// ---- shared memory / mbarrier / TMA (inline PTX, sm_90+ incl. sm_103a) ----------
MSL_DEV uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

MSL_DEV void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// Make mbarrier initialisation visible to the async (TMA) proxy.
MSL_DEV void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Order this thread's generic-proxy shared-memory accesses before later async-proxy ones.
MSL_DEV void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
MSL_DEV void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
MSL_DEV void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
MSL_DEV bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// At most `limit` polls for phase `parity` of `bar`.
MSL_DEV bool mbar_poll(uint64_t *bar, uint32_t parity, unsigned limit) {
    for (unsigned i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Bounded wait for phase `parity` of a barrier that tracks a copy in flight;
// false (and the error bit set) if the phase did not complete within the
// poll limit. Before returning false it waits again, up to kMaxWaitPolls
// polls, for the copy to land, so that a CTA that gives up does not leave a
// copy writing into shared memory it no longer owns. Not inlined: the
// kernels' hot code stays free of the give-up path (measured 5 % faster on
// the 3-D tile kernel than the original inlined poll loop, and 12 % faster
// than an inlined form with the give-up path).
static __device__ __noinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, unsigned *err) {
    if (mbar_try_wait(bar, parity)) return true;  // the first poll needs no limit
    if (mbar_poll(bar, parity, wait_poll_limit(err) - 1)) return true;
    report_error(err, kErrBarrierTimeout);
    mbar_poll(bar, parity, kMaxWaitPolls);
    return false;
}

// Tiled TMA loads into this CTA's shared memory, completing on `bar`.
// The innermost coordinate times the element size must be a multiple of 16 B.
MSL_DEV void tma_load_2d(void *dst, const void *tmap, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}
MSL_DEV void tma_load_3d(void *dst, const void *tmap, uint64_t *bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}
MSL_DEV void tma_prefetch_desc(const void *tmap) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

// ---- warp helpers ----------------------------------------------------------------
template <typename T> MSL_DEV T shfl_down(T v, int delta, int width = 32) {
    static_assert(sizeof(T) % 4 == 0, "shuffle of 4-byte multiples only");
    union { T t; int w[sizeof(T) / 4]; } u;
    u.t = v;
#pragma unroll
    for (int k = 0; k < (int)(sizeof(T) / 4); k++) u.w[k] = __shfl_down_sync(0xffffffffu, u.w[k], delta, width);
    return u.t;
}

}  // namespace gpu
}  // namespace msl

namespace msl {
namespace gpu {

// Packed FP32 pairs (add/mul/fma.rn.f32x2, sm_100 and later: two independent
// IEEE operations per instruction, each rounded as the scalar one; the low
// half is the first float). The stencil kernels pair two cells of a row.
using f32x2 = unsigned long long;
MSL_DEV f32x2 pk2(float a, float b) {
    f32x2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(a), "f"(b));
    return d;
}
MSL_DEV float lo2(f32x2 v) {
    float a;
    asm("{\n\t.reg .f32 t;\n\tmov.b64 {%0, t}, %1;\n\t}" : "=f"(a) : "l"(v));
    return a;
}
MSL_DEV float hi2(f32x2 v) {
    float b;
    asm("{\n\t.reg .f32 t;\n\tmov.b64 {t, %0}, %1;\n\t}" : "=f"(b) : "l"(v));
    return b;
}
MSL_DEV f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
MSL_DEV f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
MSL_DEV f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
MSL_DEV f32x2 ld_pair(const float *p) { return *reinterpret_cast<const f32x2 *>(p); }  // 8-byte aligned
MSL_DEV void st_pair(float *p, f32x2 v) { *reinterpret_cast<f32x2 *>(p) = v; }

// x / 6 rounded to nearest, via the reciprocal-with-one-correction method for
// a divisor known in advance (P. Markstein, "IA-64 and Elementary Functions",
// 2000; N. Brisebarre, J.-M. Muller, S. K. Raina, "Accelerating correctly
// rounded floating-point division when the divisor is known in advance",
// IEEE Trans. Computers 53(8), 2004): q = RN(x * RN(1/6)), remainder
// r = x - 6q exactly by one FMA, then q' = RN(q + r * RN(1/6)). The result is
// checked against IEEE division for every one of the 2^32 float inputs by the
// GPU test suite. The method needs a normal quotient, so inputs below 2^-122
// in magnitude take IEEE division; infinities and NaNs pass through q.
// Inputs for which the method below is exact: 2^-122 <= |x| <= FLT_MAX.
MSL_DEV bool div6_in_range(float x) {
    const float ax = fabsf(x);
    return ax >= 1.88079096131566e-37f && ax <= 3.40282346638528859812e38f;
}
// The method alone (exact for div6_in_range inputs).
MSL_DEV float div6_core(float x) {
    const float zh = 0.16666667163372039794921875f;  // RN(1/6)
    const float q = __fmul_rn(x, zh);
    const float r = __fmaf_rn(-q, 6.0f, x);
    return __fmaf_rn(r, zh, q);
}
MSL_DEV float div6_rn(float x) {
    // tiny (< 2^-122), infinite and NaN inputs: IEEE division
    if (!div6_in_range(x)) return __fdiv_rn(x, 6.0f);
    return div6_core(x);
}

}  // namespace gpu
}  // namespace msl
