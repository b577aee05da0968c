// Driver that runs the Muesli reference's own OpenMP skeletons on raw input
// files and writes raw output files. Test infrastructure only: it is compiled
// from the reference headers by oracle/Makefile into oracle/_ref/ and used to
// generate and re-check the golden fixtures under tests/golden/.
//
// Usage: ref_harness <op> <ints...> -- <input files...> -- <output file>
//
// Adapters for the reference's known CPU-build quirks (each one keeps the
// reference's own loop and view code and only fixes how the harness calls it):
//  * DM::mapStencil passes (row, col) as (x, y) on the CPU (src/dm.cpp:1585-1589);
//    every DM stencil below is wrapped in swapxy<> so the functor sees x=col, y=row.
//  * DS::map / DS::zip read the nCPUPartition shadow copy (src/ds.cpp:652,714);
//    inputs are loaded with setLocalPartition(), which refreshes it.
//  * DS::zip(b, c, f) computes f(c[i], b[i]) on the CPU (src/ds.cpp:720); the
//    harness passes (b, a) so the result is f(a[i], b[i]), the GPU build's order.
//  * DS::foldCPU is a racy omp-parallel left fold (src/ds.cpp:930-935); the
//    harness runs folds with one OpenMP thread.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "muesli.h"
#include "da.h"
#include "dm.h"
#include "dc.h"

using namespace msl;

namespace {

template <typename T>
std::vector<T> load(const char *path, size_t n) {
    std::vector<T> v(n);
    FILE *f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "ref_harness: cannot read %zu elements from %s\n", n, path);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <typename T>
void store(const char *path, const T *p, size_t n) {
    FILE *f = std::fopen(path, "wb");
    if (!f || std::fwrite(p, sizeof(T), n, f) != n) {
        std::fprintf(stderr, "ref_harness: cannot write %s\n", path);
        std::exit(2);
    }
    std::fclose(f);
}

// ---- element-wise functors of the benchmark workloads -----------------------
struct Affine : public Functor<float, float> {  // x -> 2.5f*x + 1.0f
    MSL_USERFUNC float operator()(float x) const override { return 2.5f * x + 1.0f; }
};
struct MulAdd : public Functor2<float, float, float> {  // (a, b) -> a*b + a
    MSL_USERFUNC float operator()(float a, float b) const override { return a * b + a; }
};
struct SumF : public Functor2<float, float, float> {
    MSL_USERFUNC float operator()(float a, float b) const override { return a + b; }
};
struct SumI : public Functor2<int, int, int> {
    MSL_USERFUNC int operator()(int a, int b) const override {
        return (int)((unsigned)a + (unsigned)b);
    }
};
struct MaxF : public Functor2<float, float, float> {
    MSL_USERFUNC float operator()(float x, float y) const override { return x > y ? x : y; }
};
struct AbsDiff : public Functor2<float, float, float> {
    MSL_USERFUNC float operator()(float x, float y) const override {
        float d = x - y;
        if (d < 0) d *= (-1);
        return d;
    }
};
// reducetwoColumns functor: (x, y, s) -> s + x*y  (two roundings)
struct DotNext : public Functor3<float, float, float, float> {
    MSL_USERFUNC float operator()(float x, float y, float s) const override { return s + x * y; }
};
struct XorIndex : public Functor2<int, int, int> {  // (i, x) -> x ^ (i & 1023)
    MSL_USERFUNC int operator()(int i, int x) const override { return x ^ (i & 1023); }
};
// Non-commutative index functors pin the argument order of the index skeletons.
struct DaIdx : public Functor2<int, int, int> {  // (i, x) -> 3*i - x
    MSL_USERFUNC int operator()(int i, int x) const override { return 3 * i - x; }
};
struct DaZipIdx : public Functor3<int, int, int, int> {  // (i, a, b) -> i + 2a - 3b
    MSL_USERFUNC int operator()(int i, int a, int b) const override { return i + 2 * a - 3 * b; }
};
struct DmIdx : public Functor3<int, int, int, int> {  // (row, col, x) -> 1000*row + 7*col - x
    MSL_USERFUNC int operator()(int r, int c, int x) const override { return 1000 * r + 7 * c - x; }
};
struct DmZipIdx : public Functor4<int, int, int, int, int> {  // (row, col, a, b)
    MSL_USERFUNC int operator()(int r, int c, int a, int b) const override {
        return 1000 * r + 7 * c + 2 * a - 3 * b;
    }
};
struct DcIdx : public Functor4<int, int, int, int, int> {  // (x, y, z, v)
    MSL_USERFUNC int operator()(int x, int y, int z, int v) const override {
        return 100000 * z + 1000 * y + 7 * x - v;
    }
};
struct DcZipIdx : public Functor5<int, int, int, int, int, int> {  // (x, y, z, a, b)
    MSL_USERFUNC int operator()(int x, int y, int z, int a, int b) const override {
        return 100000 * z + 1000 * y + 7 * x + 2 * a - 3 * b;
    }
};

// ---- stencil functors --------------------------------------------------------
// 2-D Jacobi of the plain-Jacobi workload: fixed border cells, 4-neighbour
// average inside, accumulated in the order of heat2D (examples/heatdiffusion.cpp:67-76).
MSL_USERFUNC float jacobi5(const NPLMatrix<float> &m, int x, int y) {
    if (x == 0 || y == 0 || x == m.width - 1 || y == m.height - 1) return m(x, y);
    float v = 0;
    v += m(x - 1, y);
    v += m(x + 1, y);
    v += m(x, y - 1);
    v += m(x, y + 1);
    v /= 4;
    return v;
}
// heat2D as in examples/heatdiffusion.cpp:67-76 (every cell updated).
MSL_USERFUNC float heat2d(const NPLMatrix<float> &m, int x, int y) {
    float v = 0;
    v += m(x - 1, y);
    v += m(x + 1, y);
    v += m(x, y - 1);
    v += m(x, y + 1);
    v /= 4;
    return v;
}
// 2-D box mean: the meanblur loop nest (examples/meanblur2.cpp:46-57) in 2-D,
// x outer and y inner, divided by the box size.
template <int R>
MSL_USERFUNC float boxmean(const NPLMatrix<float> &m, int x, int y) {
    float res = 0;
    for (int mx = x - R; mx <= x + R; mx++)
        for (int my = y - R; my <= y + R; my++) res += m(mx, my);
    return res / (float)((2 * R + 1) * (2 * R + 1));
}
// Game of Life rule of examples/gameoflife.cpp:22-42 on the NPLMatrix view.
MSL_USERFUNC int life8(const NPLMatrix<int> &m, int x, int y) {
    int sum = m(x, y - 1) + m(x - 1, y - 1) + m(x + 1, y - 1) + m(x, y + 1) + m(x - 1, y + 1) +
              m(x + 1, y + 1) + m(x - 1, y) + m(x + 1, y);
    int alive = m(x, y);
    int next = 0;
    if (alive == 1 && (sum == 2 || sum == 3)) next = 1;
    if (alive == 0 && sum == 3) next = 1;
    return next;
}
// heat3D, examples/heatdiffusion.cpp:55-65.
MSL_USERFUNC float heat3d(const PLCube<float> &c, int x, int y, int z) {
    float v = 0;
    v += c(x - 1, y, z);
    v += c(x + 1, y, z);
    v += c(x, y - 1, z);
    v += c(x, y + 1, z);
    v += c(x, y, z - 1);
    v += c(x, y, z + 1);
    v /= 6;
    return v;
}
// meanblur update<radius>, examples/meanblur2.cpp:46-57 (3-D box sum).
template <int R>
MSL_USERFUNC float boxsum3d(const PLCube<float> &c, int x, int y, int z) {
    float res = 0;
    for (int mx = x - R; mx <= x + R; mx++)
        for (int my = y - R; my <= y + R; my++)
            for (int mz = z - R; mz <= z + R; mz++) res += c(mx, my, mz);
    return res;
}

// The CPU DM::mapStencil calls f(matrix, row, col); swap back to (x=col, y=row).
template <typename T, NPLMMapStencilFunctor<T> g>
MSL_USERFUNC T swapxy(const NPLMatrix<T> &m, int a, int b) { return g(m, b, a); }

template <typename T, NPLMMapStencilFunctor<T> g>
void dm_stencil(int rows, int cols, int r, T neutral, int iters, const char *in, const char *out) {
    std::vector<T> h = load<T>(in, (size_t)rows * cols);
    DM<T> a(rows, cols, T(0), true), b(rows, cols, T(0), true);
    a.setLocalPartition(h.data());
    DM<T> *p = &a, *q = &b;
    for (int i = 0; i < iters; i++) {
        p->template mapStencil<swapxy<T, g>>(*q, (size_t)r, neutral, false);
        std::swap(p, q);
    }
    store(out, p->getLocalPartition(), (size_t)rows * cols);
}

template <DCMapStencilFunctor<float> g>
void dc_stencil(int depth, int rows, int cols, int r, float neutral, int iters, const char *in,
                const char *out) {
    size_t n = (size_t)depth * rows * cols;
    std::vector<float> h = load<float>(in, n);
    DC<float> a(rows, cols, depth, 0.0f, false), b(rows, cols, depth, 0.0f, false);
    a.setLocalPartition(h.data());
    DC<float> *p = &a, *q = &b;
    for (int i = 0; i < iters; i++) {
        p->template mapStencil<g>(*q, (size_t)r, neutral);
        std::swap(p, q);
    }
    store(out, p->getLocalPartition(), n);
}

int usage() {
    std::fprintf(stderr, "usage: ref_harness <op> <ints...> -- <inputs...> -- <output>\n");
    return 2;
}

}  // namespace

// DM x DA broadcast zips and the DA-with-matrix-rows skeletons (src/dm.cpp:1757-1853,
// src/dm.cpp:505-535, src/da.cpp:256-324); non-commutative integer functors.
struct BcMA {  // (r, c, a, b[r][c], u[r])
    MSL_USERFUNC int operator()(int r, int c, int a, int b, int u) const { return 1000 * r + 7 * c + 2 * a - 3 * b + 5 * u; }
};
struct BcA {  // (r, c, a, u[r])
    MSL_USERFUNC int operator()(int r, int c, int a, int u) const { return 1000 * r + 7 * c - a + 11 * u; }
};
struct BcAAA {  // (r, c, a, u[r], v[r], w[r])
    MSL_USERFUNC int operator()(int r, int c, int a, int u, int v, int w) const {
        return 1000 * r + 7 * c + a - 2 * u + 3 * v - 5 * w;
    }
};
// crossZipIndexInPlace: a[r][c] <- b[c][r] + a[r][c]. The CPU build calls
// f(r, c, a[r][c], b_partition) and stores the result (src/dm.cpp:528-532).
struct BcCross {
    int n;
    MSL_USERFUNC int operator()(int r, int c, int a, int *b) const { return b[c * n + r] + a; }
};
struct BcRowSum {  // this[i] <- i + sum(row i) - this[i]
    int cols;
    MSL_USERFUNC int operator()(int i, int *row, int x) const {
        int s = 0;
        for (int k = 0; k < cols; k++) s += row[k];
        return i + s - x;
    }
};
struct BcRowPick {  // this[i] <- row[i % cols] * b[i] + this[i] + i
    int cols;
    MSL_USERFUNC int operator()(int i, int *row, int b, int x) const { return row[i % cols] * b + x + i; }
};

int main(int argc, char **argv) {
    if (argc < 2) return usage();
    std::string op = argv[1];
    std::vector<long> iv;
    std::vector<const char *> ins;
    const char *out = nullptr;
    int k = 2;
    for (; k < argc && std::strcmp(argv[k], "--") != 0; k++) iv.push_back(std::atol(argv[k]));
    for (k++; k < argc && std::strcmp(argv[k], "--") != 0; k++) ins.push_back(argv[k]);
    if (k + 1 < argc) out = argv[k + 1];
    if (!out) return usage();

    int fake_argc = 1;
    char *fake_argv[] = {argv[0], nullptr};
    msl::initSkeletons(fake_argc, fake_argv);
    auto I = [&](size_t i) { return i < iv.size() ? iv[i] : 0L; };

    if (op == "da_map_affine") {  // n
        int n = (int)I(0);
        std::vector<float> x = load<float>(ins.at(0), n);
        DA<float> a(n, 0.0f), o(n, 0.0f);
        a.setLocalPartition(x.data());
        Affine f;
        o.map(f, a);
        store(out, o.getLocalPartition(), n);
    } else if (op == "da_map_inplace_affine") {
        int n = (int)I(0);
        std::vector<float> x = load<float>(ins.at(0), n);
        DA<float> a(n, 0.0f);
        a.setLocalPartition(x.data());
        Affine f;
        a.mapInPlace(f);
        store(out, a.getLocalPartition(), n);
    } else if (op == "da_zip_muladd") {  // out = a*b + a
        int n = (int)I(0);
        std::vector<float> x = load<float>(ins.at(0), n), y = load<float>(ins.at(1), n);
        DA<float> a(n, 0.0f), b(n, 0.0f), o(n, 0.0f);
        a.setLocalPartition(x.data());
        b.setLocalPartition(y.data());
        MulAdd f;
        o.zip(b, a, f);  // CPU build computes f(second, first)
        store(out, o.getLocalPartition(), n);
    } else if (op == "da_zip_inplace_muladd") {  // a <- a*b + a
        int n = (int)I(0);
        std::vector<float> x = load<float>(ins.at(0), n), y = load<float>(ins.at(1), n);
        DA<float> a(n, 0.0f), b(n, 0.0f);
        a.setLocalPartition(x.data());
        b.setLocalPartition(y.data());
        MulAdd f;
        a.zipInPlace(b, f);
        store(out, a.getLocalPartition(), n);
    } else if (op == "da_fold_sum_f32" || op == "da_fold_max_f32") {
        omp_set_num_threads(1);
        int n = (int)I(0);
        std::vector<float> x = load<float>(ins.at(0), n);
        DA<float> a(n, 0.0f);
        a.setLocalPartition(x.data());
        float r;
        if (op == "da_fold_sum_f32") { SumF f; r = a.fold(f, true); }
        else { MaxF f; r = a.fold(f, true); }
        store(out, &r, 1);
    } else if (op == "da_fold_sum_i32") {
        omp_set_num_threads(1);
        int n = (int)I(0);
        std::vector<int> x = load<int>(ins.at(0), n);
        DA<int> a(n, 0);
        a.setLocalPartition(x.data());
        SumI f;
        int r = a.fold(f, true);
        store(out, &r, 1);
    } else if (op == "da_mapindex_xor") {
        int n = (int)I(0);
        std::vector<int> x = load<int>(ins.at(0), n);
        DA<int> a(n, 0), o(n, 0);
        a.setLocalPartition(x.data());
        XorIndex f;
        o.mapIndex(f, a);
        store(out, o.getLocalPartition(), n);
    } else if (op == "da_mapindex_inplace") {  // (i, x) -> 3i - x
        int n = (int)I(0);
        std::vector<int> x = load<int>(ins.at(0), n);
        DA<int> a(n, 0);
        a.setLocalPartition(x.data());
        DaIdx f;
        a.mapIndexInPlace(f);
        store(out, a.getLocalPartition(), n);
    } else if (op == "da_zipindex") {  // out = f(i, a, b); CPU passes (i, c, b)
        int n = (int)I(0);
        std::vector<int> x = load<int>(ins.at(0), n), y = load<int>(ins.at(1), n);
        DA<int> a(n, 0), b(n, 0), o(n, 0);
        a.setLocalPartition(x.data());
        b.setLocalPartition(y.data());
        DaZipIdx f;
        o.zipIndex(b, a, f);
        store(out, o.getLocalPartition(), n);
    } else if (op == "da_zipindex_inplace") {  // a <- f(i, a, b)
        int n = (int)I(0);
        std::vector<int> x = load<int>(ins.at(0), n), y = load<int>(ins.at(1), n);
        DA<int> a(n, 0), b(n, 0);
        a.setLocalPartition(x.data());
        b.setLocalPartition(y.data());
        DaZipIdx f;
        a.zipIndexInPlace(b, f);
        store(out, a.getLocalPartition(), n);
    } else if (op == "dm_mapindex" || op == "dm_mapindex_inplace") {  // rows cols
        int rows = (int)I(0), cols = (int)I(1);
        size_t n = (size_t)rows * cols;
        std::vector<int> x = load<int>(ins.at(0), n);
        DM<int> a(rows, cols, 0, true), o(rows, cols, 0, true);
        a.setLocalPartition(x.data());
        DmIdx f;
        if (op == "dm_mapindex") { o.mapIndex(f, a); store(out, o.getLocalPartition(), n); }
        else { a.mapIndexInPlace(f); store(out, a.getLocalPartition(), n); }
    } else if (op == "dm_zipindex" || op == "dm_zipindex_inplace") {
        int rows = (int)I(0), cols = (int)I(1);
        size_t n = (size_t)rows * cols;
        std::vector<int> x = load<int>(ins.at(0), n), y = load<int>(ins.at(1), n);
        DM<int> a(rows, cols, 0, true), b(rows, cols, 0, true), o(rows, cols, 0, true);
        a.setLocalPartition(x.data());
        b.setLocalPartition(y.data());
        DmZipIdx f;
        if (op == "dm_zipindex") { o.zipIndex(b, a, f); store(out, o.getLocalPartition(), n); }
        else { a.zipIndexInPlace(b, f); store(out, a.getLocalPartition(), n); }
    } else if (op == "dc_mapindex" || op == "dc_mapindex_inplace") {  // depth rows cols
        int depth = (int)I(0), rows = (int)I(1), cols = (int)I(2);
        size_t n = (size_t)depth * rows * cols;
        std::vector<int> x = load<int>(ins.at(0), n);
        DC<int> a(rows, cols, depth, 0, false), o(rows, cols, depth, 0, false);
        a.setLocalPartition(x.data());
        DcIdx f;
        if (op == "dc_mapindex") { o.mapIndex(f, a); store(out, o.getLocalPartition(), n); }
        else { a.mapIndexInPlace(f); store(out, a.getLocalPartition(), n); }
    } else if (op == "dc_zipindex" || op == "dc_zipindex_inplace") {
        int depth = (int)I(0), rows = (int)I(1), cols = (int)I(2);
        size_t n = (size_t)depth * rows * cols;
        std::vector<int> x = load<int>(ins.at(0), n), y = load<int>(ins.at(1), n);
        DC<int> a(rows, cols, depth, 0, false), b(rows, cols, depth, 0, false), o(rows, cols, depth, 0, false);
        a.setLocalPartition(x.data());
        b.setLocalPartition(y.data());
        DcZipIdx f;
        if (op == "dc_zipindex") { o.zipIndex(b, a, f); store(out, o.getLocalPartition(), n); }
        else { a.zipIndexInPlace(b, f); store(out, a.getLocalPartition(), n); }
    } else if (op == "dm_jacobi5") {  // rows cols iters
        dm_stencil<float, jacobi5>((int)I(0), (int)I(1), 1, 0.0f, (int)I(2), ins.at(0), out);
    } else if (op == "dm_heat2d") {  // rows cols iters neutral*1000
        dm_stencil<float, heat2d>((int)I(0), (int)I(1), 1, (float)I(3) / 1000.0f, (int)I(2), ins.at(0), out);
    } else if (op == "dm_life8") {  // rows cols iters
        dm_stencil<int, life8>((int)I(0), (int)I(1), 1, 0, (int)I(2), ins.at(0), out);
    } else if (op == "dm_boxmean") {  // rows cols r iters
        int rows = (int)I(0), cols = (int)I(1), r = (int)I(2), it = (int)I(3);
        switch (r) {
            case 1: dm_stencil<float, boxmean<1>>(rows, cols, 1, 0.0f, it, ins.at(0), out); break;
            case 2: dm_stencil<float, boxmean<2>>(rows, cols, 2, 0.0f, it, ins.at(0), out); break;
            case 3: dm_stencil<float, boxmean<3>>(rows, cols, 3, 0.0f, it, ins.at(0), out); break;
            case 4: dm_stencil<float, boxmean<4>>(rows, cols, 4, 0.0f, it, ins.at(0), out); break;
            case 6: dm_stencil<float, boxmean<6>>(rows, cols, 6, 0.0f, it, ins.at(0), out); break;
            case 8: dm_stencil<float, boxmean<8>>(rows, cols, 8, 0.0f, it, ins.at(0), out); break;
            case 10: dm_stencil<float, boxmean<10>>(rows, cols, 10, 0.0f, it, ins.at(0), out); break;
            default: std::fprintf(stderr, "unsupported radius %d\n", r); return 2;
        }
    } else if (op == "dc_heat3d") {  // depth rows cols iters
        dc_stencil<heat3d>((int)I(0), (int)I(1), (int)I(2), 1, 0.0f, (int)I(3), ins.at(0), out);
    } else if (op == "dc_boxsum") {  // depth rows cols r iters
        int d = (int)I(0), rows = (int)I(1), cols = (int)I(2), r = (int)I(3), it = (int)I(4);
        switch (r) {
            case 1: dc_stencil<boxsum3d<1>>(d, rows, cols, 1, 0.0f, it, ins.at(0), out); break;
            case 2: dc_stencil<boxsum3d<2>>(d, rows, cols, 2, 0.0f, it, ins.at(0), out); break;
            default: std::fprintf(stderr, "unsupported radius %d\n", r); return 2;
        }
    } else if (op == "dm_jacobi_residual") {  // rows cols iters: sweeps, then zip(|a-b|), fold(max)
        omp_set_num_threads(1);
        int rows = (int)I(0), cols = (int)I(1), it = (int)I(2);
        size_t n = (size_t)rows * cols;
        std::vector<float> h = load<float>(ins.at(0), n);
        DM<float> a(rows, cols, 0.0f, true), b(rows, cols, 0.0f, true), d(rows, cols, 0.0f, true);
        a.setLocalPartition(h.data());
        DM<float> *p = &a, *q = &b;
        for (int i = 0; i < it; i++) {
            p->mapStencil<swapxy<float, jacobi5>>(*q, 1, 0.0f, false);
            std::swap(p, q);
        }
        // p holds sweep `it`, q sweep `it-1`; refresh the shadow copies first.
        p->setLocalPartition(p->getLocalPartition());
        q->setLocalPartition(q->getLocalPartition());
        AbsDiff ad;
        MaxF mx;
        d.zip(*q, *p, ad);  // f(p, q) = |new - old|
        float res = d.fold(mx, true);
        std::vector<float> o(n + 1);
        std::memcpy(o.data(), p->getLocalPartition(), n * sizeof(float));
        o[n] = res;
        store(out, o.data(), n + 1);
    } else if (op == "dm_reduce_rows_sum_i32" || op == "dm_reduce_rows_max_f32") {  // rows cols
        omp_set_num_threads(1);  // the CPU build folds each row with a racy omp loop
        int rows = (int)I(0), cols = (int)I(1);
        size_t n = (size_t)rows * cols;
        if (op == "dm_reduce_rows_sum_i32") {
            std::vector<int> x = load<int>(ins.at(0), n);
            DM<int> a(rows, cols, 0, true);
            DA<int> c(rows, 0);
            a.setLocalPartition(x.data());
            SumI f;
            a.reduceRows(c, f);
            store(out, c.getLocalPartition(), rows);
        } else {
            std::vector<float> x = load<float>(ins.at(0), n);
            DM<float> a(rows, cols, 0.0f, true);
            DA<float> c(rows, 0.0f);
            a.setLocalPartition(x.data());
            MaxF f;
            a.reduceRows(c, f);
            store(out, c.getLocalPartition(), rows);
        }
    } else if (op == "dm_reduce_two_columns") {  // rows cols
        int rows = (int)I(0), cols = (int)I(1);
        size_t n = (size_t)rows * cols;
        std::vector<float> x = load<float>(ins.at(0), n);
        DM<float> a(rows, cols, 0.0f, true);
        DA<float> c(rows, 0.0f);
        a.setLocalPartition(x.data());
        DotNext f;
        a.reducetwoColumns(c, f);
        store(out, c.getLocalPartition(), rows);
    } else if (op == "dm_rotate_rows" || op == "dm_rotate_cols") {  // rows cols a
        int rows = (int)I(0), cols = (int)I(1), a = (int)I(2);
        size_t n = (size_t)rows * cols;
        std::vector<int> x = load<int>(ins.at(0), n);
        DM<int> m(rows, cols, 0, true);
        m.setLocalPartition(x.data());
        if (op == "dm_rotate_rows") m.rotateRows(a);
        else m.rotateCols(a);
        store(out, m.getLocalPartition(), n);
    } else if (op == "dm_set_column") {  // rows cols col
        int rows = (int)I(0), cols = (int)I(1), col = (int)I(2);
        size_t n = (size_t)rows * cols;
        std::vector<float> x = load<float>(ins.at(0), n), v = load<float>(ins.at(1), rows);
        DM<float> m(rows, cols, 0.0f, true);
        DA<float> d(rows, 0.0f);
        m.setLocalPartition(x.data());
        d.setLocalPartition(v.data());
        m.setColumn(d, col);
        store(out, m.getLocalPartition(), n);
    } else if (op == "dm_zipindex_ma" || op == "dm_zipindex_a" || op == "dm_zipindex_aaa" ||
               op == "dm_crosszip") {  // rows cols; inputs a, b (rows x cols), u, v, w (rows)
        int rows = (int)I(0), cols = (int)I(1);
        size_t n = (size_t)rows * cols;
        std::vector<int> a = load<int>(ins.at(0), n), b = load<int>(ins.at(1), n);
        std::vector<int> u = load<int>(ins.at(2), rows), v = load<int>(ins.at(3), rows), w = load<int>(ins.at(4), rows);
        DM<int> ma(rows, cols, 0, true), mb(rows, cols, 0, true);
        DA<int> du(rows, 0), dv(rows, 0), dw(rows, 0);
        ma.setLocalPartition(a.data());
        mb.setLocalPartition(b.data());
        du.setLocalPartition(u.data());
        dv.setLocalPartition(v.data());
        dw.setLocalPartition(w.data());
        if (op == "dm_zipindex_ma") { BcMA f; ma.zipIndexInPlaceMA(mb, du, f); }
        else if (op == "dm_zipindex_a") { BcA f; ma.zipIndexInPlaceA(du, f); }
        else if (op == "dm_zipindex_aaa") { BcAAA f; ma.zipIndexInPlaceAAA(du, dv, dw, f); }
        else { BcCross f{cols}; ma.crossZipIndexInPlace(mb, f); }
        store(out, ma.getLocalPartition(), n);
    } else if (op == "da_mapindex_dmrows" || op == "da_zipindex_dmrows") {  // rows cols; inputs m, u, v
        int rows = (int)I(0), cols = (int)I(1);
        size_t n = (size_t)rows * cols;
        std::vector<int> a = load<int>(ins.at(0), n), u = load<int>(ins.at(1), rows), v = load<int>(ins.at(2), rows);
        DM<int> ma(rows, cols, 0, true);
        DA<int> du(rows, 0), dv(rows, 0);
        ma.setLocalPartition(a.data());
        du.setLocalPartition(u.data());
        dv.setLocalPartition(v.data());
        if (op == "da_mapindex_dmrows") { BcRowSum f{cols}; du.mapIndexInPlaceDMRows(ma, f); }
        else { BcRowPick f{cols}; du.zipIndexInPlaceDMRows(dv, ma, f); }
        store(out, du.getLocalPartition(), rows);
    } else {
        std::fprintf(stderr, "ref_harness: unknown op %s\n", op.c_str());
        return 2;
    }
    msl::terminateSkeletons();
    return 0;
}
