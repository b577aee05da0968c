// Element-wise skeleton kernels: map / mapInPlace, zip / zipInPlace, zip of
// three, and their index variants (DA f(i, ..), DM f(row, col, ..),
// DC f(x, y, z, ..)).
//
// Reference behaviour: one thread per element, 32-bit loads, a 1-D grid of
// 1024-thread blocks (mapKernel src/map_kernels.cu:36-43, zipKernel
// src/zip_kernels.cu:37-43, index kernels src/map_kernels.cu:60-101 and
// src/zip_kernels.cu:82-148). Here: a grid-stride loop over 16-byte vectors,
// U vectors in flight per thread, a grid of (a few) CTAs per SM, and the
// coordinates of an index functor advanced incrementally inside a vector
// instead of a div/mod per element. The functor is inlined.
#pragma once

#include "msl_device.cuh"

namespace msl {
namespace gpu {

// ---- coordinate generators for the index skeletons ----------------------------
// at(i) gives the coordinates of flat element i, inc() steps to element i+1.
struct IdxNone {
    struct S {};
    MSL_DEV S at(size_t) const { return {}; }
    MSL_DEV void inc(S &) const {}
};
struct IdxFlat {  // DA: global index = first + local index (src/map_kernels.cu:72-78)
    long long first;
    struct S {
        long long i;
    };
    MSL_DEV S at(size_t i) const { return {first + (long long)i}; }
    MSL_DEV void inc(S &s) const { ++s.i; }
};
struct IdxRowCol {  // DM: (row, col) of a row-major rows x cols matrix
    long long cols;
    struct S {
        int row, col;
    };
    MSL_DEV S at(size_t i) const {
        if (i < 0xffffffffull && cols < 0xffffffffll)
            return {(int)((unsigned)i / (unsigned)cols), (int)((unsigned)i % (unsigned)cols)};
        return {(int)(i / (size_t)cols), (int)(i % (size_t)cols)};
    }
    MSL_DEV void inc(S &s) const {
        if (++s.col == (int)cols) {
            s.col = 0;
            ++s.row;
        }
    }
};
struct IdxXYZ {  // DC: (x=col, y=row, z=depth), index (z*rows + y)*cols + x
    long long cols, rows;
    struct S {
        int x, y, z;
    };
    MSL_DEV S at(size_t i) const {
        size_t layer = (size_t)(cols * rows);
        size_t z = i / layer, rem = i % layer;
        return {(int)(rem % (size_t)cols), (int)(rem / (size_t)cols), (int)z};
    }
    MSL_DEV void inc(S &s) const {
        if (++s.x == (int)cols) {
            s.x = 0;
            if (++s.y == (int)rows) {
                s.y = 0;
                ++s.z;
            }
        }
    }
};

constexpr int kEwThreads = 256;
constexpr int kEwUnroll = 4;

// out[i] = f(coords(i), a[i])
template <int V, int U, class Ix, class F, typename TO, typename TA>
__global__ void __launch_bounds__(kEwThreads) ew_map_kernel(TO *out, const TA *a, size_t n, Ix ix, F f) {
    const size_t nv = n / V;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t v = tid;
    for (; v + (U - 1) * stride < nv; v += U * stride) {
        Vec<TA, V> x[U];
#pragma unroll
        for (int u = 0; u < U; u++) x[u] = vload<TA, V>(a, (v + u * stride) * V);
#pragma unroll
        for (int u = 0; u < U; u++) {
            Vec<TO, V> o;
            auto s = ix.at((v + u * stride) * V);
#pragma unroll
            for (int k = 0; k < V; k++) {
                o.v[k] = f(s, x[u].v[k]);
                ix.inc(s);
            }
            vstore<TO, V>(out, (v + u * stride) * V, o);
        }
    }
    for (; v < nv; v += stride) {
        Vec<TA, V> x = vload<TA, V>(a, v * V);
        Vec<TO, V> o;
        auto s = ix.at(v * V);
#pragma unroll
        for (int k = 0; k < V; k++) {
            o.v[k] = f(s, x.v[k]);
            ix.inc(s);
        }
        vstore<TO, V>(out, v * V, o);
    }
    const size_t i = nv * V + tid;  // ragged tail (< V elements)
    if (i < n) out[i] = f(ix.at(i), a[i]);
}

// out[i] = f(coords(i), a[i], b[i])
template <int V, int U, class Ix, class F, typename TO, typename TA, typename TB>
__global__ void __launch_bounds__(kEwThreads)
    ew_zip_kernel(TO *out, const TA *a, const TB *b, size_t n, Ix ix, F f) {
    const size_t nv = n / V;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t v = tid;
    for (; v + (U - 1) * stride < nv; v += U * stride) {
        Vec<TA, V> x[U];
        Vec<TB, V> y[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            x[u] = vload<TA, V>(a, (v + u * stride) * V);
            y[u] = vload<TB, V>(b, (v + u * stride) * V);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            Vec<TO, V> o;
            auto s = ix.at((v + u * stride) * V);
#pragma unroll
            for (int k = 0; k < V; k++) {
                o.v[k] = f(s, x[u].v[k], y[u].v[k]);
                ix.inc(s);
            }
            vstore<TO, V>(out, (v + u * stride) * V, o);
        }
    }
    for (; v < nv; v += stride) {
        Vec<TA, V> x = vload<TA, V>(a, v * V);
        Vec<TB, V> y = vload<TB, V>(b, v * V);
        Vec<TO, V> o;
        auto s = ix.at(v * V);
#pragma unroll
        for (int k = 0; k < V; k++) {
            o.v[k] = f(s, x.v[k], y.v[k]);
            ix.inc(s);
        }
        vstore<TO, V>(out, v * V, o);
    }
    const size_t i = nv * V + tid;
    if (i < n) out[i] = f(ix.at(i), a[i], b[i]);
}

// out[i] = f(coords(i), a[i], b[i], c[i])
template <int V, int U, class Ix, class F, typename TO, typename TA, typename TB, typename TC>
__global__ void __launch_bounds__(kEwThreads)
    ew_zip3_kernel(TO *out, const TA *a, const TB *b, const TC *c, size_t n, Ix ix, F f) {
    const size_t nv = n / V;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (size_t v = tid; v < nv; v += stride) {
        Vec<TA, V> x = vload<TA, V>(a, v * V);
        Vec<TB, V> y = vload<TB, V>(b, v * V);
        Vec<TC, V> z = vload<TC, V>(c, v * V);
        Vec<TO, V> o;
        auto s = ix.at(v * V);
#pragma unroll
        for (int k = 0; k < V; k++) {
            o.v[k] = f(s, x.v[k], y.v[k], z.v[k]);
            ix.inc(s);
        }
        vstore<TO, V>(out, v * V, o);
    }
    const size_t i = nv * V + tid;
    if (i < n) out[i] = f(ix.at(i), a[i], b[i], c[i]);
}

// ---- host-side launchers ---------------------------------------------------------
inline unsigned ew_blocks(size_t units, int sm_count) {
    size_t per_block = (size_t)kEwThreads * kEwUnroll;
    size_t b = (units + per_block - 1) / per_block;
    size_t cap = (size_t)(sm_count > 0 ? sm_count : 152) * 8;  // 8 x 256 threads = a full SM
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

template <class Ix, class F, typename TO, typename TA>
cudaError_t launch_map(TO *out, const TA *a, size_t n, Ix ix, F f, cudaStream_t st, int sms) {
    constexpr int V = vec_width2<TO, TA>();
    if (V > 1 && aligned_to(out, V * sizeof(TO)) && aligned_to(a, V * sizeof(TA)))
        ew_map_kernel<V, kEwUnroll><<<ew_blocks(n / V, sms), kEwThreads, 0, st>>>(out, a, n, ix, f);
    else
        ew_map_kernel<1, kEwUnroll><<<ew_blocks(n, sms), kEwThreads, 0, st>>>(out, a, n, ix, f);
    return cudaGetLastError();
}

template <class Ix, class F, typename TO, typename TA, typename TB>
cudaError_t launch_zip(TO *out, const TA *a, const TB *b, size_t n, Ix ix, F f, cudaStream_t st, int sms) {
    constexpr int V = vec_width3<TO, TA, TB>();
    if (V > 1 && aligned_to(out, V * sizeof(TO)) && aligned_to(a, V * sizeof(TA)) && aligned_to(b, V * sizeof(TB)))
        ew_zip_kernel<V, kEwUnroll><<<ew_blocks(n / V, sms), kEwThreads, 0, st>>>(out, a, b, n, ix, f);
    else
        ew_zip_kernel<1, kEwUnroll><<<ew_blocks(n, sms), kEwThreads, 0, st>>>(out, a, b, n, ix, f);
    return cudaGetLastError();
}

template <class Ix, class F, typename TO, typename TA, typename TB, typename TC>
cudaError_t launch_zip3(TO *out, const TA *a, const TB *b, const TC *c, size_t n, Ix ix, F f, cudaStream_t st,
                        int sms) {
    constexpr int V = vec_width4<TO, TA, TB, TC>();
    if (V > 1 && aligned_to(out, V * sizeof(TO)) && aligned_to(a, V * sizeof(TA)) &&
        aligned_to(b, V * sizeof(TB)) && aligned_to(c, V * sizeof(TC)))
        ew_zip3_kernel<V, 1><<<ew_blocks(n / V, sms), kEwThreads, 0, st>>>(out, a, b, c, n, ix, f);
    else
        ew_zip3_kernel<1, 1><<<ew_blocks(n, sms), kEwThreads, 0, st>>>(out, a, b, c, n, ix, f);
    return cudaGetLastError();
}

}  // namespace gpu
}  // namespace msl
