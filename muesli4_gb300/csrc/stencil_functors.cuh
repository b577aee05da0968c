// Built-in stencil functors of libmsl_gb300.so (internal header).
//
// Reference functors: examples/heatdiffusion.cpp:55-76 (heat2D, heat3D),
// examples/gameoflife.cpp:22-42 (Life), examples/meanblur2.cpp:46-57 (box).
#pragma once

#include "../include/detail/msl_stencil.cuh"
#include "msl_internal.h"

namespace msl {
namespace builtin {

using namespace msl::gpu;


template <typename T> __device__ __forceinline__ T div_rn(T a, T b);
template <> __device__ __forceinline__ float div_rn<float>(float a, float b) { return __fdiv_rn(a, b); }
template <> __device__ __forceinline__ double div_rn<double>(double a, double b) { return __ddiv_rn(a, b); }

// heat2D: (((0 + W) + E) + N) + S, then / 4 (examples/heatdiffusion.cpp:67-76).
template <typename T, class V> __device__ __forceinline__ T heat5(const V &m, int x, int y) {
    T v = T(0);
    v = Arith<T>::add(v, m(x - 1, y));
    v = Arith<T>::add(v, m(x + 1, y));
    v = Arith<T>::add(v, m(x, y - 1));
    v = Arith<T>::add(v, m(x, y + 1));
    // v / 4 and v * 0.25 are the same real number, each rounded once: the
    // results are identical for every v, and the product is one instruction.
    return Arith<T>::mul(v, T(0.25));
}
template <typename T> struct StHeat5 {
    static constexpr bool kStrip2 = true;
    template <class V> __device__ __forceinline__ T operator()(const V &m, int x, int y) const { return heat5<T>(m, x, y); }
    template <class V> __device__ __forceinline__ void strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) const {
        heat5_strip<false>(m, x, y0, out);
    }
};
// Plain Jacobi: boundary cells keep their value, inside cells take heat2D.
template <typename T> struct StJacobi5 {
    static constexpr bool kStrip2 = true;
    static constexpr bool kStripAnyTile = true;  // strip() reads the window only and handles the edges
    static constexpr bool kPairStrip = std::is_same<T, float>::value;  // packed pairs (jacobi_pair_strip)
    template <class V> __device__ __forceinline__ T operator()(const V &m, int x, int y) const {
        if (x == 0 || y == 0 || x == m.width - 1 || y == m.height - 1) return m(x, y);
        return heat5<T>(m, x, y);
    }
    template <class V> __device__ __forceinline__ void strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) const {
        jacobi_strip_window(m, x, y0, out);
    }
};
// Box over (2R+1)^2 cells, summed dx outer / dy inner as the meanblur loop
// nest (examples/meanblur2.cpp:46-57). strip() computes kSt2RPT vertically
// adjacent outputs reusing each loaded column: for every dx it loads the
// RPT + 2R cells of that column once and adds them to the RPT sums, so each
// output still receives its (dx, dy) terms in the reference's order.
template <typename T, int R, bool MEAN> struct StBoxFixed {
    static constexpr bool kStrip2 = true;  // has a strip() (detected by has_strip2)
    template <class V> __device__ __forceinline__ T finish(T s) const {
        return MEAN ? div_rn<T>(s, T((2 * R + 1) * (2 * R + 1))) : s;
    }
    template <class V> __device__ __forceinline__ T operator()(const V &m, int x, int y) const {
        T s = T(0);
#pragma unroll
        for (int dx = -R; dx <= R; dx++)
#pragma unroll
            for (int dy = -R; dy <= R; dy++) s = Arith<T>::add(s, m(x + dx, y + dy));
        return finish<V>(s);
    }
    template <class V> __device__ __forceinline__ void strip(const V &m, int x, int y0, T (&out)[kSt2RPT]) const {
        T s[kSt2RPT];
#pragma unroll
        for (int j = 0; j < kSt2RPT; j++) s[j] = T(0);
#pragma unroll 1
        for (int dx = -R; dx <= R; dx++) {
            T col[kSt2RPT + 2 * R];
#pragma unroll
            for (int k = 0; k < kSt2RPT + 2 * R; k++) col[k] = m(x + dx, y0 - R + k);
#pragma unroll
            for (int j = 0; j < kSt2RPT; j++)
#pragma unroll
                for (int dy = 0; dy <= 2 * R; dy++) s[j] = Arith<T>::add(s[j], col[j + dy]);
        }
#pragma unroll
        for (int j = 0; j < kSt2RPT; j++) out[j] = finish<V>(s[j]);
    }
};
// Any radius (runtime), one output at a time.
template <typename T> struct StBoxAny {
    int r;
    bool mean;
    template <class V> __device__ __forceinline__ T operator()(const V &m, int x, int y) const {
        T s = T(0);
        for (int dx = -r; dx <= r; dx++)
            for (int dy = -r; dy <= r; dy++) s = Arith<T>::add(s, m(x + dx, y + dy));
        return mean ? div_rn<T>(s, T((2 * r + 1) * (2 * r + 1))) : s;
    }
};
// Conway's rule (examples/gameoflife.cpp:22-42), dead cells outside.
struct StLife {
    static constexpr bool kStrip2 = true;
    __device__ __forceinline__ static int32_t rule(int32_t alive, int32_t sum) {
        int32_t next = 0;
        if (alive == 1 && (sum == 2 || sum == 3)) next = 1;
        if (alive == 0 && sum == 3) next = 1;
        return next;
    }
    template <class V> __device__ __forceinline__ int32_t operator()(const V &m, int x, int y) const {
        int32_t sum = m(x, y - 1) + m(x - 1, y - 1) + m(x + 1, y - 1) + m(x, y + 1) + m(x - 1, y + 1) +
                      m(x + 1, y + 1) + m(x - 1, y) + m(x + 1, y);
        return rule(m(x, y), sum);
    }
    // kSt2RPT cells of one column. int32 addition wraps, so it is associative
    // and commutative: the eight neighbours are summed as three-cell row sums
    // (shared by the cells above and below) plus the left and right cells,
    // which gives the same sum as the reference's order for any inputs.
    template <class V> __device__ __forceinline__ void strip(const V &m, int x, int y0, int32_t (&out)[kSt2RPT]) const {
        uint32_t l[kSt2RPT + 2], c[kSt2RPT + 2], r[kSt2RPT + 2], h[kSt2RPT + 2];
#pragma unroll
        for (int k = 0; k < kSt2RPT + 2; k++) {
            l[k] = (uint32_t)m(x - 1, y0 - 1 + k);
            c[k] = (uint32_t)m(x, y0 - 1 + k);
            r[k] = (uint32_t)m(x + 1, y0 - 1 + k);
            h[k] = l[k] + c[k] + r[k];
        }
#pragma unroll
        for (int j = 0; j < kSt2RPT; j++)
            out[j] = rule((int32_t)c[j + 1], (int32_t)(h[j] + h[j + 2] + l[j + 1] + r[j + 1]));
    }
};
// heat3D: ((((((0 + W) + E) + N) + S) + B) + F) / 6 (examples/heatdiffusion.cpp:55-65).
template <typename T> struct StHeat7 {
    static constexpr bool kStar7 = true;
    // star7 == sum7 / 6 correctly rounded (kernels that split the two take
    // the division's fast path for whole warps at once)
    static constexpr bool kSum7Div6 = std::is_same<T, float>::value;
    __device__ __forceinline__ T sum7(T w, T e, T n, T s, T b, T f) const {
        T v = T(0);
        v = Arith<T>::add(v, w);
        v = Arith<T>::add(v, e);
        v = Arith<T>::add(v, n);
        v = Arith<T>::add(v, s);
        v = Arith<T>::add(v, b);
        v = Arith<T>::add(v, f);
        return v;
    }
    __device__ __forceinline__ T star7(T w, T e, T n, T s, T b, T f) const {
        const T v = sum7(w, e, n, s, b, f);
        if constexpr (std::is_same<T, float>::value) return div6_rn(v);  // == v / 6, correctly rounded
        else return div_rn<T>(v, T(6));
    }
    template <class V> __device__ __forceinline__ T operator()(const V &c, int x, int y, int z) const {
        return star7(c(x - 1, y, z), c(x + 1, y, z), c(x, y - 1, z), c(x, y + 1, z), c(x, y, z - 1), c(x, y, z + 1));
    }
};
// 3-D box, dx outer, dy, dz inner (examples/meanblur2.cpp:46-57).
template <typename T> struct StBox3 {
    int r;
    bool mean;
    template <class V> __device__ __forceinline__ T operator()(const V &c, int x, int y, int z) const {
        T s = T(0);
        for (int dx = -r; dx <= r; dx++)
            for (int dy = -r; dy <= r; dy++)
                for (int dz = -r; dz <= r; dz++) s = Arith<T>::add(s, c(x + dx, y + dy, z + dz));
        return mean ? div_rn<T>(s, T((2 * r + 1) * (2 * r + 1) * (2 * r + 1))) : s;
    }
};

// Launch a fixed-radius box sweep (F32); defined in stencil_box_*.cu.
template <int R>
cudaError_t box_fixed_f32(const float *in, float *out, int rows, int cols, float neutral, bool mean,
                          unsigned long long *resid, bool tma);

}  // namespace builtin
}  // namespace msl

namespace msl {
namespace builtin {
// `depth` fused sweeps (temporal blocking) of a built-in 2-D stencil; defined
// in stencil_tb.cu for Jacobi / heat2D (F32, F64, BF16) and Life (I32).
cudaError_t tb_sweeps_2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int r, int depth,
                         double neutral, unsigned long long *resid, bool tma, int tile_rows);
bool tb_supported_2d(int dtype, int kind);
// `depth` Life generations of an int32 grid whose cells are all 0 or 1, with
// the dead (0) border, on the packed kernel of msl_life.cuh (stencil_tb.cu);
// cudaErrorNotSupported when the grid does not suit it.
constexpr int kLifePackedMaxDepth = 32;  // generations per launch of life_packed_2d
cudaError_t life_packed_2d(const void *in, void *out, int rows, int cols, int depth);
}  // namespace builtin
}  // namespace msl
