// Fold skeleton: a single-pass reduction with a user functor that needs no
// identity element (each partial is seeded with an element, like the
// reference's foldCPU, src/ds.cpp:924-954).
//
// Reference GPU fold (src/ds.cpp:741-912, foldKernel src/fold_kernels.cu:51-129):
// a full D2H copy of the array, cudaMalloc/cudaFree per call, a shared-memory
// tree with a __syncthreads per level, and a second host-launched stage that
// launches nothing above 2^20 elements. Here: one launch; each thread folds
// 16-byte vectors in a grid-stride loop, warps combine with shuffles, each CTA
// publishes a partial, and the last CTA to finish (atomic ticket) folds the
// partials in CTA order and writes the result. The order of combination is a
// fixed function of n and the grid size, so results are deterministic.
//
// Scratch: `partials`/`have` (one slot per CTA) and a ticket counter that the
// last CTA resets to 0, so the scratch is reusable by the next call on the
// same stream without clearing.
#pragma once

#include "msl_device.cuh"

namespace msl {
namespace gpu {

constexpr int kFoldThreads = 512;
constexpr int kFoldUnroll = 4;  // vectors in flight per thread when a value takes more than 16 bytes a vector
constexpr int kFoldMaxBlocks = 4096;
// Vectors in flight per thread: 8 when a vector of values fits 16 bytes (128 B
// in flight per thread), else 4 (the FP64 residual of FP32 / BF16 inputs).
template <typename R, int V> constexpr int fold_unroll() { return sizeof(R) * V <= 16 ? 8 : kFoldUnroll; }

// Element source over one array.
template <typename T, int V> struct FoldSrcArray {
    using value_type = T;
    const T *p;
    MSL_DEV Vec<T, V> load_vec(size_t vi) const { return vload<T, V>(p, vi * V); }
    MSL_DEV T load(size_t i) const { return p[i]; }
};
// |a[i] - b[i]| evaluated in FP64 (the fused residual of two iterates).
template <typename S> MSL_DEV double as_f64(S s) { return (double)s; }
template <> MSL_DEV double as_f64<bf16s>(bf16s s) { return (double)bf16_to_f(s); }
template <typename T, int V> struct FoldSrcAbsDiff {
    using value_type = double;
    const T *a, *b;
    MSL_DEV Vec<double, V> load_vec(size_t vi) const {
        Vec<T, V> x = vload<T, V>(a, vi * V), y = vload<T, V>(b, vi * V);
        Vec<double, V> r;
#pragma unroll
        for (int k = 0; k < V; k++) r.v[k] = fabs(as_f64(x.v[k]) - as_f64(y.v[k]));
        return r;
    }
    MSL_DEV double load(size_t i) const { return fabs(as_f64(a[i]) - as_f64(b[i])); }
};

// Load bypassing L1 (partials written by other CTAs), word by word.
template <typename T> MSL_DEV T load_cg(const T *p) {
    static_assert(sizeof(T) % 4 == 0, "fold values must be a multiple of 4 bytes");
    union { T t; int w[sizeof(T) / 4]; } u;
#pragma unroll
    for (int k = 0; k < (int)(sizeof(T) / 4); k++) u.w[k] = __ldcg(reinterpret_cast<const int *>(p) + k);
    return u.t;
}

// (value, present) pair: partial folds of an empty range are "absent".
template <typename T, class F> MSL_DEV void fold_in(T &acc, bool &have, T x, bool xh, const F &f) {
    if (xh) {
        acc = have ? f(acc, x) : x;
        have = true;
    }
}

template <typename T, class F> MSL_DEV void warp_fold(T &acc, bool &have, const F &f) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        T o = shfl_down(acc, d);
        bool oh = __shfl_down_sync(0xffffffffu, (int)have, d) != 0;
        fold_in(acc, have, o, oh, f);
    }
}

// CTA-wide fold; the result is valid in thread 0.
template <typename T, class F> MSL_DEV void block_fold(T &acc, bool &have, const F &f) {
    __shared__ T s_val[32];
    __shared__ int s_have[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_fold(acc, have, f);
    if (lane == 0) {
        s_val[warp] = acc;
        s_have[warp] = have;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        have = lane < nw && s_have[lane];
        if (have) acc = s_val[lane];
        warp_fold(acc, have, f);
    }
}

template <int V, int U, class Src, class F>
__global__ void __launch_bounds__(kFoldThreads, 2)
    fold_kernel(Src src, size_t n, F f, typename Src::value_type *partials, int *part_have,
                unsigned *ticket, typename Src::value_type *result, int *result_have) {
    using T = typename Src::value_type;
    const size_t nv = n / V;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    T acc{};
    bool have = false;
    size_t v = tid;
    if (v + (U - 1) * stride < nv) {
        // U independent chains, each seeded with its first element.
        T c[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            Vec<T, V> x = src.load_vec(v + u * stride);
            c[u] = x.v[0];
#pragma unroll
            for (int k = 1; k < V; k++) c[u] = f(c[u], x.v[k]);
        }
        for (v += U * stride; v + (U - 1) * stride < nv; v += U * stride) {
            Vec<T, V> x[U];
#pragma unroll
            for (int u = 0; u < U; u++) x[u] = src.load_vec(v + u * stride);
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int k = 0; k < V; k++) c[u] = f(c[u], x[u].v[k]);
        }
        acc = c[0];
#pragma unroll
        for (int u = 1; u < U; u++) acc = f(acc, c[u]);
        have = true;
    }
    for (; v < nv; v += stride) {
        Vec<T, V> x = src.load_vec(v);
#pragma unroll
        for (int k = 0; k < V; k++) fold_in(acc, have, x.v[k], true, f);
    }
    const size_t i = nv * V + tid;  // ragged tail
    if (i < n) fold_in(acc, have, src.load(i), true, f);

    block_fold(acc, have, f);
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = acc;
        part_have[blockIdx.x] = have;
        __threadfence();
        s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // Last CTA: fold the partials in CTA order (strided over the threads, then
    // the same warp/CTA tree), write the result, reset the ticket.
    acc = T{};
    have = false;
    for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x)
        if (__ldcg(part_have + k)) fold_in(acc, have, load_cg(partials + k), true, f);
    block_fold(acc, have, f);
    if (threadIdx.x == 0) {
        *result = acc;  // may be mapped host memory: fenced system-wide
        *result_have = have;
        *ticket = 0u;
        __threadfence_system();
    }
}

// CTAs of `kernel` (kFoldThreads threads) resident per SM, at least 1.
template <class K> int fold_occupancy(K kernel) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, kFoldThreads, 0) != cudaSuccess || b < 1) b = 1;
    return b;
}

// One wave: as many CTAs as fit on the GPU at once (`per_sm` resident per SM),
// fewer when the input is small. A grid beyond one wave would leave a partial
// last wave (the grid-stride loop gives every CTA the same work).
inline unsigned fold_blocks(size_t units, int sm_count, int per_sm = 2, int unroll = kFoldUnroll) {
    size_t per_block = (size_t)kFoldThreads * unroll;
    size_t b = (units + per_block - 1) / per_block;
    size_t cap = (size_t)(sm_count > 0 ? sm_count : 152) * (size_t)(per_sm > 0 ? per_sm : 1);
    if (cap > (size_t)kFoldMaxBlocks) cap = kFoldMaxBlocks;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

// Scratch layout used by launch_fold (bytes): partial values, partial flags,
// ticket, result value, result flag.
struct FoldScratch {
    void *partials;   // kFoldMaxBlocks * 16 bytes
    int *part_have;   // kFoldMaxBlocks ints
    unsigned *ticket; // 1, zero between calls
    void *result;     // 16 bytes
    int *result_have; // 1
};
constexpr size_t kFoldScratchBytes = (size_t)kFoldMaxBlocks * 16 + (size_t)kFoldMaxBlocks * 4 + 256;
inline FoldScratch carve_fold_scratch(void *base) {
    char *p = (char *)base;
    FoldScratch s;
    s.partials = p;
    s.part_have = (int *)(p + (size_t)kFoldMaxBlocks * 16);
    char *tail = p + (size_t)kFoldMaxBlocks * 20;
    s.ticket = (unsigned *)tail;
    s.result = tail + 64;
    s.result_have = (int *)(tail + 128);
    return s;
}

template <template <typename, int> class SrcT, typename T, class F, typename... P>
cudaError_t launch_fold(size_t n, F f, const FoldScratch &s, cudaStream_t st, int sms, bool vec_ok, P... ptrs) {
    constexpr int V = vec_width1<T>();
    using R = typename SrcT<T, V>::value_type;
    static_assert(sizeof(R) <= 16, "fold value type too large for the scratch slots");
    if (V > 1 && vec_ok) {
        constexpr int U = fold_unroll<R, V>();
        auto k = fold_kernel<V, U, SrcT<T, V>, F>;
        static const int occ = fold_occupancy(k);
        SrcT<T, V> src{ptrs...};
        k<<<fold_blocks(n / V, sms, occ, U), kFoldThreads, 0, st>>>(src, n, f, (R *)s.partials, s.part_have,
                                                                    s.ticket, (R *)s.result, s.result_have);
    } else {
        constexpr int U = fold_unroll<R, 1>();
        auto k = fold_kernel<1, U, SrcT<T, 1>, F>;
        static const int occ = fold_occupancy(k);
        SrcT<T, 1> src{ptrs...};
        k<<<fold_blocks(n, sms, occ, U), kFoldThreads, 0, st>>>(src, n, f, (R *)s.partials, s.part_have, s.ticket,
                                                                (R *)s.result, s.result_have);
    }
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
