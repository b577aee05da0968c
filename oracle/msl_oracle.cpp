// CPU oracle for the skeleton hot path -- TEST INFRASTRUCTURE, not product code.
// See msl_oracle.h. Each function names the reference code whose loop it
// restates (paths inside the Muesli reference project).
#include "msl_oracle.h"

#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <vector>

#include "../include/msl_gb300.h"

namespace {

// ---- bfloat16 storage (round to nearest even; NaN kept quiet) ---------------
struct bf16 {
    uint16_t bits;
};
inline float to_f(bf16 h) {
    uint32_t u = (uint32_t)h.bits << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline bf16 from_f(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return bf16{(uint16_t)((u >> 16) | 0x40)};
    u += 0x7fffu + ((u >> 16) & 1u);
    return bf16{(uint16_t)(u >> 16)};
}

// Scalar arithmetic with int32 wrap-around (the reference relies on the
// two's-complement behaviour of its int functors).
template <typename T> struct Ar {
    static T add(T a, T b) { return a + b; }
    static T sub(T a, T b) { return a - b; }
    static T mul(T a, T b) { return a * b; }
};
template <> struct Ar<int32_t> {
    static int32_t add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
    static int32_t sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
    static int32_t mul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
};
template <typename T> T absval(T x) { return x < 0 ? Ar<T>::sub(0, x) : x; }
template <typename T> T param(const double *p, int k) { return p ? (T)p[k] : T(0); }
template <> int32_t param<int32_t>(const double *p, int k) { return p ? (int32_t)(long long)p[k] : 0; }

// ---- map: DS::map / mapInPlace, src/ds.cpp:614-663 --------------------------
template <typename T>
int map_t(int op, const T *in, T *out, size_t n, const double *p) {
    const T a = param<T>(p, 0), b = param<T>(p, 1);
    switch (op) {
        case MSL_MAP_AFFINE:
#pragma omp parallel for
            for (long long k = 0; k < (long long)n; k++) out[k] = Ar<T>::add(Ar<T>::mul(a, in[k]), b);
            return 0;
        case MSL_MAP_ABS:
#pragma omp parallel for
            for (long long k = 0; k < (long long)n; k++) out[k] = absval(in[k]);
            return 0;
        case MSL_MAP_SQUARE:
#pragma omp parallel for
            for (long long k = 0; k < (long long)n; k++) out[k] = Ar<T>::mul(in[k], in[k]);
            return 0;
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

// ---- zip: DS::zip / zipInPlace, src/ds.cpp:669-727 (GPU argument order) -----
template <typename T> T zip_op(int op, T a, T b) {
    switch (op) {
        case MSL_ZIP_ADD: return Ar<T>::add(a, b);
        case MSL_ZIP_SUB: return Ar<T>::sub(a, b);
        case MSL_ZIP_MUL: return Ar<T>::mul(a, b);
        case MSL_ZIP_MULADD: return Ar<T>::add(Ar<T>::mul(a, b), a);
        case MSL_ZIP_ABSDIFF: return absval(Ar<T>::sub(a, b));
        case MSL_ZIP_MAX: return a > b ? a : b;
        default: return a < b ? a : b;  // MSL_ZIP_MIN
    }
}
template <typename T>
int zip_t(int op, const T *a, const T *b, T *out, size_t n) {
    if (op < MSL_ZIP_ADD || op > MSL_ZIP_MIN) return MSL_ERR_INVALID_ARGUMENT;
#pragma omp parallel for
    for (long long k = 0; k < (long long)n; k++) out[k] = zip_op<T>(op, a[k], b[k]);
    return 0;
}
// DA::zipInPlace3, src/da.cpp:434-459.
template <typename T>
int zip3_t(int op, const T *a, const T *b, const T *c, T *out, size_t n) {
    if (op != MSL_ZIP3_MULADD && op != MSL_ZIP3_SUM) return MSL_ERR_INVALID_ARGUMENT;
#pragma omp parallel for
    for (long long k = 0; k < (long long)n; k++)
        out[k] = op == MSL_ZIP3_MULADD ? Ar<T>::add(Ar<T>::mul(a[k], b[k]), c[k])
                                       : Ar<T>::add(Ar<T>::add(a[k], b[k]), c[k]);
    return 0;
}

// ---- index functors ----------------------------------------------------------
// Coordinates in the reference's argument order: DA f(i, ...) src/da.cpp:249;
// DM f(row, col, ...) src/dm.cpp:393-395; DC f(col, row, depth, ...) via
// mapIndexKernelDC src/map_kernels.cu:88-101.
template <typename T>
T index_op(int op, int nd, const long long *c, const long long *dims, long long flat, T v, T w,
           bool has_w, const double *p) {
    switch (op) {
        case MSL_IDX_LINEAR: {
            T acc = Ar<T>::mul(param<T>(p, 0), (T)c[0]);
            for (int k = 1; k < nd; k++) acc = Ar<T>::add(acc, Ar<T>::mul(param<T>(p, k), (T)c[k]));
            acc = Ar<T>::add(acc, Ar<T>::mul(param<T>(p, nd), v));
            if (has_w) acc = Ar<T>::add(acc, Ar<T>::mul(param<T>(p, nd + 1), w));
            return acc;
        }
        case MSL_IDX_PRODUCT: {
            T acc = (T)c[0];
            for (int k = 1; k < nd; k++) acc = Ar<T>::mul(acc, (T)c[k]);
            acc = Ar<T>::mul(acc, v);
            if (has_w) acc = Ar<T>::mul(acc, w);
            return acc;
        }
        case MSL_IDX_XOR_MASK: {
            int32_t m = (int32_t)(long long)(p ? p[0] : 0);
            return (T)((int32_t)v ^ (int32_t)(flat & m));
        }
        default: {  // MSL_IDX_BORDER
            bool top, edge;
            if (nd == 1) {
                top = c[0] == 0;
                edge = c[0] == dims[0] - 1;
            } else if (nd == 2) {  // (row, col), dims = rows, cols
                top = c[0] == 0;
                edge = c[0] == dims[0] - 1 || c[1] == 0 || c[1] == dims[1] - 1;
            } else {  // (x, y, z), dims = depth, rows, cols
                top = c[1] == 0;
                edge = c[0] == 0 || c[0] == dims[2] - 1 || c[1] == dims[1] - 1 || c[2] == 0 ||
                       c[2] == dims[0] - 1;
            }
            if (top) return param<T>(p, 0);
            if (edge) return param<T>(p, 1);
            return v;
        }
    }
}

template <typename T>
int index_t(int op, const T *a, const T *b, T *out, int nd, const long long *dims, const double *p) {
    if (nd < 1 || nd > 3 || op < MSL_IDX_LINEAR || op > MSL_IDX_BORDER) return MSL_ERR_INVALID_ARGUMENT;
    long long n = 1;
    for (int k = 0; k < nd; k++) n *= dims[k];
#pragma omp parallel for
    for (long long k = 0; k < n; k++) {
        long long c[3];
        if (nd == 1) {
            c[0] = k;
        } else if (nd == 2) {  // src/dm.cpp:393-394
            c[0] = k / dims[1];
            c[1] = k % dims[1];
        } else {  // src/map_kernels.cu:92-96
            long long layer = dims[1] * dims[2];
            c[2] = k / layer;
            long long rem = k % layer;
            c[1] = rem / dims[2];
            c[0] = rem % dims[2];
        }
        out[k] = index_op<T>(op, nd, c, dims, k, a[k], b ? b[k] : T(0), b != nullptr, p);
    }
    return 0;
}

// ---- fold: DS::foldCPU, src/ds.cpp:924-954 -----------------------------------
// A left fold seeded with the first element, run on one thread (the
// reference's omp-parallel version of this loop is a data race).
template <typename T>
int fold_t(int op, const T *in, size_t n, T *res) {
    if (n == 0 || op < MSL_FOLD_SUM || op > MSL_FOLD_MIN) return MSL_ERR_INVALID_ARGUMENT;
    T acc = in[0];
    for (size_t k = 1; k < n; k++) {
        T x = in[k];
        if (op == MSL_FOLD_SUM) acc = Ar<T>::add(acc, x);
        else if (op == MSL_FOLD_MAX) acc = acc > x ? acc : x;
        else acc = acc < x ? acc : x;
    }
    *res = acc;
    return 0;
}

// ---- stencil views -------------------------------------------------------------
// NPLMatrix::operator() on one partition, include/nplmatrix.h:123-139.
template <typename S> struct View2 {
    const S *d;
    int width, height;
    float neutral_f;
    S neutral;
    float operator()(int x, int y) const {
        if (x < 0 || y < 0 || x >= width || y >= height) return neutral_f;
        return (float)d[(long long)y * width + x];
    }
};
template <> struct View2<bf16> {
    const bf16 *d;
    int width, height;
    float neutral_f;
    bf16 neutral;
    float operator()(int x, int y) const {
        if (x < 0 || y < 0 || x >= width || y >= height) return neutral_f;
        return to_f(d[(long long)y * width + x]);
    }
};
struct View2i {
    const int32_t *d;
    int width, height;
    int32_t neutral;
    int32_t operator()(int x, int y) const {
        if (x < 0 || y < 0 || x >= width || y >= height) return neutral;
        return d[(long long)y * width + x];
    }
};
// PLCube::operator() on one partition, include/plcube.h:105-119.
template <typename V> struct View3 {
    const V *d;
    int width, height, depth;
    V neutral;
    V operator()(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= width || y >= height || z >= depth) return neutral;
        return d[((long long)z * height + y) * width + x];
    }
};

// The built-in 2-D functors, evaluated as their reference counterparts are.
template <typename V, typename A>
A stencil2_value(int kind, const V &m, int x, int y, int r) {
    switch (kind) {
        case MSL_ST2_JACOBI5:
            if (x == 0 || y == 0 || x == m.width - 1 || y == m.height - 1) return m(x, y);
            /* fall through */
        case MSL_ST2_HEAT5: {  // examples/heatdiffusion.cpp:67-76
            A v = 0;
            v += m(x - 1, y);
            v += m(x + 1, y);
            v += m(x, y - 1);
            v += m(x, y + 1);
            v /= 4;
            return v;
        }
        case MSL_ST2_BOXMEAN:
        case MSL_ST2_BOXSUM: {  // loop nest of examples/meanblur2.cpp:46-57, in 2-D
            A res = 0;
            for (int mx = x - r; mx <= x + r; mx++)
                for (int my = y - r; my <= y + r; my++) res += m(mx, my);
            if (kind == MSL_ST2_BOXMEAN) res = res / (A)((2 * r + 1) * (2 * r + 1));
            return res;
        }
    }
    return 0;
}
// examples/gameoflife.cpp:22-42 on the NPLMatrix view.
inline int32_t life_value(const View2i &m, int x, int y) {
    int32_t sum = m(x, y - 1) + m(x - 1, y - 1) + m(x + 1, y - 1) + m(x, y + 1) + m(x - 1, y + 1) +
                  m(x + 1, y + 1) + m(x - 1, y) + m(x + 1, y);
    int32_t alive = m(x, y);
    int32_t next = 0;
    if (alive == 1 && (sum == 2 || sum == 3)) next = 1;
    if (alive == 0 && sum == 3) next = 1;
    return next;
}

inline bool kind2_ok(int dtype, int kind) {
    if (dtype == MSL_I32) return kind == MSL_ST2_LIFE;
    if (dtype == MSL_BF16) return kind == MSL_ST2_JACOBI5 || kind == MSL_ST2_HEAT5;
    return kind >= MSL_ST2_JACOBI5 && kind <= MSL_ST2_BOXSUM;
}

// DM::mapStencil<f>, src/dm.cpp:1578-1590, with the functor called as
// f(view, x=col, y=row) (the GPU build's convention, include/detail/map_kernels.cuh:159-168).
int stencil2d_any(int dtype, int kind, const void *in, void *out, int rows, int cols, int r,
                  double neutral) {
    long long n = (long long)rows * cols;
    if (dtype == MSL_I32) {
        View2i m{(const int32_t *)in, cols, rows, (int32_t)(long long)neutral};
        int32_t *o = (int32_t *)out;
#pragma omp parallel for
        for (long long k = 0; k < n; k++) o[k] = life_value(m, (int)(k % cols), (int)(k / cols));
    } else if (dtype == MSL_F32) {
        View2<float> m{(const float *)in, cols, rows, (float)neutral, (float)neutral};
        float *o = (float *)out;
#pragma omp parallel for
        for (long long k = 0; k < n; k++)
            o[k] = stencil2_value<View2<float>, float>(kind, m, (int)(k % cols), (int)(k / cols), r);
    } else if (dtype == MSL_BF16) {  // BF16 storage, FP32 arithmetic
        View2<bf16> m{(const bf16 *)in, cols, rows, (float)neutral, from_f((float)neutral)};
        bf16 *o = (bf16 *)out;
#pragma omp parallel for
        for (long long k = 0; k < n; k++)
            o[k] = from_f(stencil2_value<View2<bf16>, float>(kind, m, (int)(k % cols), (int)(k / cols), r));
    } else {  // MSL_F64
        struct V {
            const double *d;
            int width, height;
            double neutral;
            double operator()(int x, int y) const {
                if (x < 0 || y < 0 || x >= width || y >= height) return neutral;
                return d[(long long)y * width + x];
            }
        } m{(const double *)in, cols, rows, neutral};
        double *o = (double *)out;
#pragma omp parallel for
        for (long long k = 0; k < n; k++)
            o[k] = stencil2_value<V, double>(kind, m, (int)(k % cols), (int)(k / cols), r);
    }
    return 0;
}

template <typename V, typename A>
A stencil3_value(int kind, const V &c, int x, int y, int z, int r) {
    if (kind == MSL_ST3_HEAT7) {  // examples/heatdiffusion.cpp:55-65
        A v = 0;
        v += c(x - 1, y, z);
        v += c(x + 1, y, z);
        v += c(x, y - 1, z);
        v += c(x, y + 1, z);
        v += c(x, y, z - 1);
        v += c(x, y, z + 1);
        v /= 6;
        return v;
    }
    A res = 0;  // examples/meanblur2.cpp:46-57
    for (int mx = x - r; mx <= x + r; mx++)
        for (int my = y - r; my <= y + r; my++)
            for (int mz = z - r; mz <= z + r; mz++) res += c(mx, my, mz);
    if (kind == MSL_ST3_BOXMEAN) res = res / (A)((2 * r + 1) * (2 * r + 1) * (2 * r + 1));
    return res;
}

// DC::mapStencil<f>, src/dc.cpp:578-590.
int stencil3d_any(int dtype, int kind, const void *in, void *out, int depth, int rows, int cols, int r,
                  double neutral) {
    long long layer = (long long)rows * cols, n = layer * depth;
    if (dtype == MSL_F32) {
        View3<float> c{(const float *)in, cols, rows, depth, (float)neutral};
        float *o = (float *)out;
#pragma omp parallel for
        for (long long k = 0; k < n; k++) {
            int z = (int)(k / layer), y = (int)((k % layer) / cols), x = (int)(k % cols);
            o[k] = stencil3_value<View3<float>, float>(kind, c, x, y, z, r);
        }
    } else {
        View3<double> c{(const double *)in, cols, rows, depth, neutral};
        double *o = (double *)out;
#pragma omp parallel for
        for (long long k = 0; k < n; k++) {
            int z = (int)(k / layer), y = (int)((k % layer) / cols), x = (int)(k % cols);
            o[k] = stencil3_value<View3<double>, double>(kind, c, x, y, z, r);
        }
    }
    return 0;
}

size_t dsize(int dtype) {
    switch (dtype) {
        case MSL_F32: case MSL_I32: return 4;
        case MSL_F64: return 8;
        case MSL_BF16: return 2;
    }
    return 0;
}
double as_double(int dtype, const void *p, long long k) {
    switch (dtype) {
        case MSL_F32: return ((const float *)p)[k];
        case MSL_F64: return ((const double *)p)[k];
        case MSL_I32: return ((const int32_t *)p)[k];
        default: return to_f(((const bf16 *)p)[k]);
    }
}


// ---- DM row / column skeletons ------------------------------------------------
template <typename T> T fold_op(int op, T a, T b) {
    switch (op) {
        case MSL_FOLD_SUM: return Ar<T>::add(a, b);
        case MSL_FOLD_MAX: return a > b ? a : b;
        default: return a < b ? a : b;  // MSL_FOLD_MIN
    }
}

// DM::reduceRows on the GPU (src/dm.cpp:1677-1685): foldRowsKernel
// (src/fold_kernels.cu:215-294) with one block of L threads per row,
// L = nextPow2((cols + 1) / 2) below threads_per_block, else threads_per_block.
// Thread t folds row[t], row[t + L], ... ; then sdata[t] = f(sdata[t], sdata[t + h])
// for h = L/2 ... 1.
template <typename T>
void fold_rows_t(int op, const T *in, T *out, long long rows, long long cols, int tpb) {
    long long lanes = tpb;
    if (cols < tpb) {
        lanes = 1;
        while (lanes < (cols + 1) / 2) lanes <<= 1;
    }
    std::vector<T> v((size_t)lanes);
    for (long long r = 0; r < rows; r++) {
        const T *row = in + r * cols;
        for (long long t = 0; t < lanes; t++) {
            T acc = row[t];
            for (long long c = t + lanes; c < cols; c += lanes) acc = fold_op(op, acc, row[c]);
            v[(size_t)t] = acc;
        }
        for (long long h = lanes / 2; h > 0; h /= 2)
            for (long long t = 0; t < h; t++) v[(size_t)t] = fold_op(op, v[(size_t)t], v[(size_t)(t + h)]);
        out[r] = v[0];
    }
}

template <typename T> void fold_cols_t(int op, const T *in, T *out, long long rows, long long cols) {
    for (long long c = 0; c < cols; c++) {
        T acc = in[c];
        for (long long r = 1; r < rows; r++) acc = fold_op(op, acc, in[r * cols + c]);
        out[c] = acc;
    }
}

// DM::rotateRows (src/dm.cpp:1345-1475), one process: the `howmuch` rows that
// wrap around go through a switch buffer, the others shift by `howmuch`.
void rotate_rows_bytes(const unsigned char *in, unsigned char *out, long long rows, long long cols, long long a,
                       size_t es) {
    const bool negative = a < 0;
    const long long howmuch = negative ? -a : a;
    const size_t rb = (size_t)cols * es;
    if (howmuch == rows || a == 0) {
        std::memcpy(out, in, (size_t)rows * rb);
        return;
    }
    std::vector<unsigned char> sw((size_t)howmuch * rb);
    if (negative) std::memcpy(sw.data(), in, sw.size());
    else std::memcpy(sw.data(), in + (size_t)(rows - howmuch) * rb, sw.size());
    for (long long k = 0; k < rows; k++) {
        const unsigned char *src;
        if (negative) src = k >= rows - howmuch ? sw.data() + (size_t)(k - (rows - howmuch)) * rb : in + (size_t)(k + howmuch) * rb;
        else src = k < howmuch ? sw.data() + (size_t)k * rb : in + (size_t)(k - howmuch) * rb;
        std::memcpy(out + (size_t)k * rb, src, rb);
    }
}

// DM::rotateCols (src/dm.cpp:1483-1533).
void rotate_cols_bytes(const unsigned char *in, unsigned char *out, long long rows, long long cols, long long a,
                       size_t es) {
    long long howmuch = a < 0 ? -a : a;
    if (howmuch >= cols) {
        howmuch %= cols;
        a %= cols;
    }
    for (long long i = 0; i < rows; i++)
        for (long long j = 0; j < cols; j++) {
            long long ce = j + a;
            if (ce < 0) ce += cols;
            if (ce >= cols) ce -= cols;
            std::memcpy(out + (size_t)(i * cols + j) * es, in + (size_t)(i * cols + ce) * es, es);
        }
}

}  // namespace

extern "C" {

int oracle_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

int oracle_map(int dtype, int op, const void *in, void *out, size_t n, const double *p) {
    switch (dtype) {
        case MSL_F32: return map_t<float>(op, (const float *)in, (float *)out, n, p);
        case MSL_F64: return map_t<double>(op, (const double *)in, (double *)out, n, p);
        case MSL_I32: return map_t<int32_t>(op, (const int32_t *)in, (int32_t *)out, n, p);
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_zip(int dtype, int op, const void *a, const void *b, void *out, size_t n) {
    switch (dtype) {
        case MSL_F32: return zip_t<float>(op, (const float *)a, (const float *)b, (float *)out, n);
        case MSL_F64: return zip_t<double>(op, (const double *)a, (const double *)b, (double *)out, n);
        case MSL_I32: return zip_t<int32_t>(op, (const int32_t *)a, (const int32_t *)b, (int32_t *)out, n);
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_zip3(int dtype, int op, const void *a, const void *b, const void *c, void *out, size_t n) {
    switch (dtype) {
        case MSL_F32:
            return zip3_t<float>(op, (const float *)a, (const float *)b, (const float *)c, (float *)out, n);
        case MSL_F64:
            return zip3_t<double>(op, (const double *)a, (const double *)b, (const double *)c, (double *)out, n);
        case MSL_I32:
            return zip3_t<int32_t>(op, (const int32_t *)a, (const int32_t *)b, (const int32_t *)c,
                                   (int32_t *)out, n);
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_map_index(int dtype, int op, const void *in, void *out, int nd, const long long *dims,
                     const double *p) {
    if (op == MSL_IDX_XOR_MASK && dtype != MSL_I32) return MSL_ERR_INVALID_ARGUMENT;
    switch (dtype) {
        case MSL_F32: return index_t<float>(op, (const float *)in, nullptr, (float *)out, nd, dims, p);
        case MSL_F64: return index_t<double>(op, (const double *)in, nullptr, (double *)out, nd, dims, p);
        case MSL_I32: return index_t<int32_t>(op, (const int32_t *)in, nullptr, (int32_t *)out, nd, dims, p);
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_zip_index(int dtype, int op, const void *a, const void *b, void *out, int nd,
                     const long long *dims, const double *p) {
    if (op == MSL_IDX_XOR_MASK || op == MSL_IDX_BORDER) return MSL_ERR_INVALID_ARGUMENT;
    switch (dtype) {
        case MSL_F32: return index_t<float>(op, (const float *)a, (const float *)b, (float *)out, nd, dims, p);
        case MSL_F64:
            return index_t<double>(op, (const double *)a, (const double *)b, (double *)out, nd, dims, p);
        case MSL_I32:
            return index_t<int32_t>(op, (const int32_t *)a, (const int32_t *)b, (int32_t *)out, nd, dims, p);
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_fold(int dtype, int op, const void *in, size_t n, void *result) {
    switch (dtype) {
        case MSL_F32: return fold_t<float>(op, (const float *)in, n, (float *)result);
        case MSL_F64: return fold_t<double>(op, (const double *)in, n, (double *)result);
        case MSL_I32: return fold_t<int32_t>(op, (const int32_t *)in, n, (int32_t *)result);
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_fold_absdiff_max(int dtype, const void *a, const void *b, size_t n, double *result) {
    if (n == 0 || dsize(dtype) == 0) return MSL_ERR_INVALID_ARGUMENT;
    double m = 0.0;
    for (size_t k = 0; k < n; k++) {
        double d = std::fabs(as_double(dtype, a, (long long)k) - as_double(dtype, b, (long long)k));
        if (d > m || d != d) m = d;
    }
    *result = m;
    return 0;
}

int oracle_stencil2d(int dtype, int kind, const void *in, void *out, int rows, int cols, int r,
                     double neutral) {
    if (rows <= 0 || cols <= 0 || r < 0 || !kind2_ok(dtype, kind)) return MSL_ERR_INVALID_ARGUMENT;
    return stencil2d_any(dtype, kind, in, out, rows, cols, r, neutral);
}

int oracle_stencil2d_iterate(int dtype, int kind, void *a, void *b, int rows, int cols, int r,
                             double neutral, int iters, double *residual, int *result_in_b) {
    if (rows <= 0 || cols <= 0 || r < 0 || iters < 1 || !kind2_ok(dtype, kind)) return MSL_ERR_INVALID_ARGUMENT;
    void *p = a, *q = b;
    for (int i = 0; i < iters; i++) {
        stencil2d_any(dtype, kind, p, q, rows, cols, r, neutral);
        void *t = p; p = q; q = t;
    }
    if (result_in_b) *result_in_b = (p == b);
    if (residual) oracle_fold_absdiff_max(dtype, p, q, (size_t)rows * cols, residual);
    return 0;
}

// Plain Jacobi (the sweep functor of examples/jacobisolver.cpp:52-62 on the
// heatdiffusion operand order, boundary fixed) by defect correction with
// bfloat16-stored correction d and defect r and an FP32 solution u. The
// reference has no such solver; this restatement checks the GPU's
// MSL_BF16_DC batch step for step: each cycle applies u <- u + d, takes
// r = J(u) - u in FP64 ((((W + E) + N) + S) * 0.25 - u), stops when
// max |r| <= tol or max_iters sweeps are done, else sets d = r and runs
// cycle - 1 sweeps d <- heat5(d) + r (FP32, rounded to bfloat16).
int oracle_jacobi_defect_bf16(float *u, int rows, int cols, double tol, long long max_iters, int cycle,
                              long long *iters, double *residual) {
    if (!u || rows <= 0 || cols <= 0 || cycle < 2 || max_iters < 0) return MSL_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)rows * cols;
    std::vector<bf16> d(n, bf16{0}), d2(n, bf16{0}), r(n, bf16{0});
    auto inside = [&](int x, int y) { return x > 0 && y > 0 && x < cols - 1 && y < rows - 1; };
    long long it = 0;
    double res = 0.0;
    for (;;) {
        for (size_t k = 0; k < n; k++) u[k] = u[k] + to_f(d[k]);
        res = 0.0;
        for (int y = 0; y < rows; y++)
            for (int x = 0; x < cols; x++) {
                const size_t k = (size_t)y * cols + x;
                double dd = 0.0;
                if (inside(x, y)) {
                    double j = (double)u[k - 1] + (double)u[k + 1];
                    j = j + (double)u[k - cols];
                    j = j + (double)u[k + cols];
                    dd = j * 0.25 - (double)u[k];
                    if (std::fabs(dd) > res || dd != dd) res = std::fabs(dd);
                }
                r[k] = from_f((float)dd);
                d[k] = r[k];
            }
        if (!(res > tol) || it >= max_iters) break;
        it += 1;
        for (int s = 1; s < cycle; s++) {
            for (int y = 0; y < rows; y++)
                for (int x = 0; x < cols; x++) {
                    const size_t k = (size_t)y * cols + x;
                    if (!inside(x, y)) {
                        d2[k] = bf16{0};
                        continue;
                    }
                    float v = 0.0f;
                    v = v + to_f(d[k - 1]);
                    v = v + to_f(d[k + 1]);
                    v = v + to_f(d[k - cols]);
                    v = v + to_f(d[k + cols]);
                    v = v * 0.25f;
                    v = v + to_f(r[k]);
                    d2[k] = from_f(v);
                }
            std::swap(d, d2);
        }
        it += cycle - 1;
    }
    if (iters) *iters = it;
    if (residual) *residual = res;
    return 0;
}

int oracle_stencil3d(int dtype, int kind, const void *in, void *out, int depth, int rows, int cols,
                     int r, double neutral) {
    if (depth <= 0 || rows <= 0 || cols <= 0 || r < 0 || (dtype != MSL_F32 && dtype != MSL_F64) ||
        kind < MSL_ST3_HEAT7 || kind > MSL_ST3_BOXMEAN)
        return MSL_ERR_INVALID_ARGUMENT;
    return stencil3d_any(dtype, kind, in, out, depth, rows, cols, r, neutral);
}

int oracle_stencil3d_iterate(int dtype, int kind, void *a, void *b, int depth, int rows, int cols,
                             int r, double neutral, int iters, double *residual, int *result_in_b) {
    if (iters < 1) return MSL_ERR_INVALID_ARGUMENT;
    void *p = a, *q = b;
    for (int i = 0; i < iters; i++) {
        int rc = oracle_stencil3d(dtype, kind, p, q, depth, rows, cols, r, neutral);
        if (rc) return rc;
        void *t = p; p = q; q = t;
    }
    if (result_in_b) *result_in_b = (p == b);
    if (residual) oracle_fold_absdiff_max(dtype, p, q, (size_t)depth * rows * cols, residual);
    return 0;
}

int oracle_fold_rows(int dtype, int op, const void *in, long long rows, long long cols, int tpb, void *out) {
    if (rows <= 0 || cols <= 0 || tpb < 1 || tpb > 1024 || (tpb & (tpb - 1))) return MSL_ERR_INVALID_ARGUMENT;
    switch (dtype) {
        case MSL_F32: fold_rows_t<float>(op, (const float *)in, (float *)out, rows, cols, tpb); return 0;
        case MSL_F64: fold_rows_t<double>(op, (const double *)in, (double *)out, rows, cols, tpb); return 0;
        case MSL_I32: fold_rows_t<int32_t>(op, (const int32_t *)in, (int32_t *)out, rows, cols, tpb); return 0;
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_fold_cols(int dtype, int op, const void *in, long long rows, long long cols, void *out) {
    if (rows <= 0 || cols <= 0) return MSL_ERR_INVALID_ARGUMENT;
    switch (dtype) {
        case MSL_F32: fold_cols_t<float>(op, (const float *)in, (float *)out, rows, cols); return 0;
        case MSL_F64: fold_cols_t<double>(op, (const double *)in, (double *)out, rows, cols); return 0;
        case MSL_I32: fold_cols_t<int32_t>(op, (const int32_t *)in, (int32_t *)out, rows, cols); return 0;
    }
    return MSL_ERR_INVALID_ARGUMENT;
}

int oracle_zip_rows(int dtype, int op, const void *m, const void *v, void *out, long long rows, long long cols) {
    if (rows <= 0 || cols <= 0) return MSL_ERR_INVALID_ARGUMENT;
    for (long long r = 0; r < rows; r++)
        for (long long c = 0; c < cols; c++) {
            const long long k = r * cols + c;
            switch (dtype) {
                case MSL_F32: ((float *)out)[k] = zip_op<float>(op, ((const float *)m)[k], ((const float *)v)[r]); break;
                case MSL_F64: ((double *)out)[k] = zip_op<double>(op, ((const double *)m)[k], ((const double *)v)[r]); break;
                case MSL_I32: ((int32_t *)out)[k] = zip_op<int32_t>(op, ((const int32_t *)m)[k], ((const int32_t *)v)[r]); break;
                default: return MSL_ERR_INVALID_ARGUMENT;
            }
        }
    return 0;
}

int oracle_rotate_rows(int dtype, const void *in, void *out, long long rows, long long cols, long long a) {
    const size_t es = dsize(dtype);
    if (rows <= 0 || cols <= 0 || es == 0) return MSL_ERR_INVALID_ARGUMENT;
    if ((a < 0 ? -a : a) > rows) return MSL_ERR_NOT_IMPLEMENTED;  // RotateRowManyNotImplementedException
    rotate_rows_bytes((const unsigned char *)in, (unsigned char *)out, rows, cols, a, es);
    return 0;
}

int oracle_rotate_cols(int dtype, const void *in, void *out, long long rows, long long cols, long long a) {
    const size_t es = dsize(dtype);
    if (rows <= 0 || cols <= 0 || es == 0) return MSL_ERR_INVALID_ARGUMENT;
    rotate_cols_bytes((const unsigned char *)in, (unsigned char *)out, rows, cols, a, es);
    return 0;
}

// DM::setColumn on one process (src/dm.cpp:1874-1877).
int oracle_set_column(int dtype, void *dm, const void *da, long long rows, long long cols, long long col) {
    const size_t es = dsize(dtype);
    if (rows <= 0 || cols <= 0 || es == 0) return MSL_ERR_INVALID_ARGUMENT;
    if (col < 0 || col >= cols) return MSL_ERR_INVALID_ARGUMENT;
    for (long long i = 0; i < rows; i++)
        std::memcpy((unsigned char *)dm + (size_t)(i * cols + col) * es, (const unsigned char *)da + (size_t)i * es, es);
    return 0;
}

// The result dumps of examples/heatdiffusion.cpp:99-114 (2-D) and :156-170
// (3-D), generalised from size^2 / size^3 to rows x cols / depth x rows x cols:
// an std::ofstream in append mode, `out << value << ";"`, "\n" per line.
int oracle_dump_text(const char *path, int dtype, const void *grid, int depth, int rows, int cols) {
    if (!path || depth < 1 || rows < 1 || cols < 1 || dsize(dtype) == 0) return MSL_ERR_INVALID_ARGUMENT;
    std::ofstream out(path, std::ios::app | std::ios::binary);
    if (!out) return MSL_ERR_INVALID_ARGUMENT;
    auto put = [&](long long index) {
        switch (dtype) {
            case MSL_F32: out << ((const float *)grid)[index]; break;
            case MSL_F64: out << ((const double *)grid)[index]; break;
            case MSL_I32: out << ((const int32_t *)grid)[index]; break;
            default: out << to_f(((const bf16 *)grid)[index]); break;
        }
        out << ";";
    };
    if (depth == 1) {
        for (int x = 0; x < rows; x++) {
            for (int y = 0; y < cols; y++) put(y + (long long)cols * x);
            out << "\n";
        }
    } else {
        for (int x = 0; x < cols; x++)
            for (int y = 0; y < rows; y++) {
                for (int z = 0; z < depth; z++) put(x + (long long)cols * y + (long long)cols * rows * z);
                out << "\n";
            }
    }
    return out.good() ? 0 : MSL_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
