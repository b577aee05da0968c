// Checks of the drop-in C++ front end (muesli.h, da.h, dm.h, dc.h) with
// user functors written the way reference programs write them: classes
// deriving from Functor..Functor5 with MSL_USERFUNC operators, MSL_USERFUNC
// lambdas, and stencil functions passed as template arguments.
//
// Built into a shared library by tests/test_gpu_frontend.py; each extern "C"
// entry point either runs a known-answer check (returns the number of
// failures) or runs a skeleton on host arrays so the test can compare the
// result with the CPU oracle.
#include <cstdio>
#include <cstring>

#include "da.h"
#include "dc.h"
#include "dm.h"
#include "muesli.h"

using namespace msl;

namespace {

int failures = 0;
template <typename T> void expect_all(const char *what, DS<T> &a, T v) {
    T *p = a.gather();
    for (int i = 0; i < a.getSize(); i++)
        if (p[i] != v) {
            std::printf("KAT %s: element %d is %g, expected %g\n", what, i, (double)p[i], (double)v);
            failures++;
            return;
        }
}
template <typename T, class G> void expect_each(const char *what, DS<T> &a, G g) {
    T *p = a.gather();
    for (int i = 0; i < a.getSize(); i++)
        if (p[i] != g(i)) {
            std::printf("KAT %s: element %d is %g, expected %g\n", what, i, (double)p[i], (double)g(i));
            failures++;
            return;
        }
}

// ---- functors in the reference's style ---------------------------------------------
class Mult : public Functor<int, int> {
   public:
    explicit Mult(int factor) : y(factor) {}
    MSL_USERFUNC int operator()(int x) const override { return x * y; }

   private:
    int y;
};
class Sum : public Functor2<int, int, int> {
   public:
    MSL_USERFUNC int operator()(int x, int y) const override { return x + y; }
};
class Sum3 : public Functor3<int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int i, int j, int x) const override { return i + j + x; }
};
class Sum4 : public Functor4<int, int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int i, int j, int x, int y) const override { return i + j + x + y; }
};
class Sum5 : public Functor5<int, int, int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int i, int j, int k, int x, int y) const override { return i + j + k + x + y; }
};
class Product3 : public Functor3<int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int i, int a, int b) const override { return i * a * b; }
};
// Non-commutative index functors (pin the argument order).
class DmIdx : public Functor3<int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int r, int c, int x) const override { return 1000 * r + 7 * c - x; }
};
class DcIdx : public Functor4<int, int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int x, int y, int z, int v) const override { return 100000 * z + 1000 * y + 7 * x - v; }
};
class DmZipIdx : public Functor4<int, int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int r, int c, int a, int b) const override { return 1000 * r + 7 * c + 2 * a - 3 * b; }
};
class DcZipIdx : public Functor5<int, int, int, int, int, int> {
   public:
    MSL_USERFUNC int operator()(int x, int y, int z, int a, int b) const override {
        return 100000 * z + 1000 * y + 7 * x + 2 * a - 3 * b;
    }
};
class AbsDiff : public Functor2<float, float, float> {
   public:
    MSL_USERFUNC float operator()(float x, float y) const override {
        float d = x - y;
        if (d < 0) d *= (-1);
        return d;
    }
};
class MaxF : public Functor2<float, float, float> {
   public:
    MSL_USERFUNC float operator()(float x, float y) const override { return x > y ? x : y; }
};

// Row / column skeletons and the DM x DA zips (functors of the ACO examples' shape).
class DotNext : public Functor3<float, float, float, float> {  // reducetwoColumns: s + x*y
   public:
    MSL_USERFUNC float operator()(float x, float y, float s) const override { return s + x * y; }
};
class ZipMA : public Functor5<int, int, int, int, int, int> {  // (r, c, a, b[r][c], v[r])
   public:
    MSL_USERFUNC int operator()(int r, int c, int a, int b, int v) const override {
        return 1000 * r + 7 * c + 2 * a - 3 * b + 5 * v;
    }
};
class ZipA : public Functor4<int, int, int, int, int> {  // (r, c, a, v[r])
   public:
    MSL_USERFUNC int operator()(int r, int c, int a, int v) const override { return 1000 * r + 7 * c - a + 11 * v; }
};
class ZipAAA : public Functor6<int, int, int, int, int, int, int> {  // (r, c, a, u[r], v[r], w[r])
   public:
    MSL_USERFUNC int operator()(int r, int c, int a, int u, int v, int w) const override {
        return 1000 * r + 7 * c + a - 2 * u + 3 * v - 5 * w;
    }
};
// crossZipIndexInPlace: a[r][c] = b[c][r] + a[r][c] on a square matrix (the
// functor indexes both matrices through their device pointers).
struct CrossT {
    int n;
    MSL_USERFUNC void operator()(int r, int c, int *a, int *b) const { a[r * n + c] = b[c * n + r] + a[r * n + c]; }
};
// mapIndexInPlaceDMRows: this[i] = i + sum of row i - this[i]
struct RowSum {
    int cols;
    MSL_USERFUNC int operator()(int i, int *row, int x) const {
        int s = 0;
        for (int k = 0; k < cols; k++) s += row[k];
        return i + s - x;
    }
};
// zipIndexInPlaceDMRows: this[i] = row[i % cols] * b[i] + this[i] + i
struct RowPick {
    int cols;
    MSL_USERFUNC int operator()(int i, int *row, int b, int x) const { return row[i % cols] * b + x + i; }
};

// ---- stencil functions -----------------------------------------------------------
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
template <int R> MSL_USERFUNC float boxsum3d(const PLCube<float> &c, int x, int y, int z) {
    float res = 0;
    for (int mx = x - R; mx <= x + R; mx++)
        for (int my = y - R; my <= y + R; my++)
            for (int mz = z - R; mz <= z + R; mz++) res += c(mx, my, mz);
    return res;
}
MSL_USERFUNC float add27(const PLCube<float> &c, int x, int y, int z) { return boxsum3d<1>(c, x, y, z); }
// Game of Life through the legacy PLMatrix interface (mapStencilMM).
class GoL : public DMMapStencilFunctor<int, int> {
   public:
    MSL_USERFUNC int operator()(int row, int col, PLMatrix<int> *in, int ncol, int nrow) const {
        int sum = in->get(row - 1, col) + in->get(row - 1, col - 1) + in->get(row - 1, col + 1) + in->get(row + 1, col) +
                  in->get(row + 1, col - 1) + in->get(row + 1, col + 1) + in->get(row, col - 1) + in->get(row, col + 1);
        int alive = in->get(row, col);
        int next = 0;
        if (alive == 1 && (sum == 2 || sum == 3)) next = 1;
        if (alive == 0 && sum == 3) next = 1;
        return next;
    }
};

// mapStencilMM with a neutral-value functor, written like the reference's
// Jacobi solver (examples/jacobisolver.cpp:15-63): the neutral functor takes
// (row, col) of a cell outside the matrix; neither functor is symmetric, so
// the argument order and the halo cells' coordinates are pinned.
class EdgeValues : public Functor2<int, int, float> {
   public:
    EdgeValues(int rows, int cols) : rows_(rows), cols_(cols) {}
    MSL_USERFUNC float operator()(int row, int col) const override {
        if (row >= 0 && row < rows_ && col >= 0 && col < cols_) return -1.0f;  // never read
        return 3.0f * row - 7.0f * col + 0.25f;
    }

   private:
    int rows_, cols_;
};
class WeightedCross : public DMNVFMapStencilFunctor<float, float, EdgeValues> {
   public:
    WeightedCross() : DMNVFMapStencilFunctor() {}
    MSL_USERFUNC float operator()(int row, int col, PLMatrix<float> *in, int ncol, int nrow) const {
        const int r = stencil_size;
        float sum = 0;
        sum += in->get(row - r, col);
        sum += 2 * in->get(row + r, col);
        sum += 4 * in->get(row, col - r);
        sum += 8 * in->get(row, col + r);
        return sum / (4 * r);
    }
};

}  // namespace

extern "C" {

int fe_init(void) {
    static char name[] = "frontend_checks";
    static char *argv[] = {name, nullptr};
    initSkeletons(1, argv);
    return 0;
}

int fe_terminate(void) {
    terminateSkeletons();
    return 0;
}

// Known answers of the reference's da_test: Fill 2, Initfill 3, Map 9,
// mapInPlace 6, mapIndex j+6, mapIndexInPlace j+3, Fold 3*dim, Zip 30,
// zipInPlace 30, zipIndex j+12, zipIndexInPlace j*6.
int fe_da_kat(int dim) {
    failures = 0;
    DA<int> a(dim);
    a.fill(2);
    expect_all("Fill", a, 2);
    DA<int> b(dim, 3);
    expect_all("Initfill", b, 3);
    Mult mult(3);
    Sum sum;
    DA<int> map_dest(dim, 3);
    b.map(mult, map_dest);
    expect_all("Map", b, 9);
    b.fill(2);
    b.mapInPlace(mult);
    expect_all("mapInPlace", b, 6);
    b.fill(6);
    a.mapIndex(sum, b);
    expect_each("mapIndex", a, [](int j) { return j + 6; });
    b.fill(3);
    b.mapIndexInPlace(sum);
    expect_each("mapIndexInPlace", b, [](int j) { return j + 3; });
    b.fill(3);
    int folded = b.fold(sum, true);
    if (folded != 3 * dim) {
        std::printf("KAT Fold: %d, expected %d\n", folded, 3 * dim);
        failures++;
    }
    DA<int> c(dim, 3);
    c.fill(20);
    b.fill(10);
    a.zip(b, c, sum);
    expect_all("Zip", a, 30);
    b.fill(20);
    c.fill(10);
    b.zipInPlace(c, sum);
    expect_all("zipInPlace", b, 30);
    a.fill(7);
    c.fill(5);
    Sum3 sum3;
    b.zipIndex(c, a, sum3);
    expect_each("zipIndex", b, [](int j) { return j + 7 + 5; });
    b.fill(3);
    c.fill(2);
    Product3 pr;
    b.zipIndexInPlace(c, pr);
    expect_each("zipIndexInPlace", b, [](int j) { return j * 3 * 2; });
    // a lambda functor, as in the reference's da_test (examples/da_test.cpp:97)
    auto product = [] MSL_USERFUNC(int i, int j) { return i * j; };
    a.fill(4);
    c.fill(5);
    a.zipInPlace(c, product);
    expect_all("zipInPlace(lambda)", a, 20);
    // host-side element access and copies
    const int k = dim - 1;
    a.set(k, 99);
    if (a.get(k) != 99) failures++;
    DA<int> copy(a);
    if (copy.get(k) != 99 || (k > 0 && copy.get(0) != 20)) failures++;
    return failures;
}

// Known answers of the reference's dm_test: Map 9, mapIndex row+col+6,
// mapIndexInPlace row+col+x, Fold 2*elements, Zip 30, zipIndex row+col+a+b.
int fe_dm_kat(int rows, int cols) {
    failures = 0;
    DM<int> a(rows, cols, 3, true), b(rows, cols, 6, true), c(rows, cols, 0, true);
    Mult mult(3);
    a.mapInPlace(mult);
    expect_all("DM Map", a, 9);
    Sum3 sum3;
    c.mapIndex(sum3, b);
    expect_each("DM mapIndex", c, [cols](int k) { return k / cols + k % cols + 6; });
    b.mapIndexInPlace(sum3);
    expect_each("DM mapIndexInPlace", b, [cols](int k) { return k / cols + k % cols + 6; });
    DM<int> two(rows, cols, 2, true);
    Sum sum;
    if (two.fold(sum, true) != 2 * rows * cols) failures++;
    DM<int> ten(rows, cols, 10, true), twenty(rows, cols, 20, true);
    c.zip(ten, twenty, sum);
    expect_all("DM Zip", c, 30);
    Sum4 sum4;
    c.zipIndex(ten, twenty, sum4);
    expect_each("DM zipIndex", c, [cols](int k) { return k / cols + k % cols + 30; });
    if (a.get2D(rows - 1, cols - 1) != 9) failures++;
    a.set2D(0, 1, 5);
    if (a.get(1) != 5) failures++;
    return failures;
}

// dc_test: mapIndex depth+row+col+x, zipIndex, fold; and the stencil test of
// examples/dc_map_stencil_test.cpp (27-point sum of ones: 27 inside, 18 on a
// face, 12 on an edge, 8 in a corner).
int fe_dc_kat(int rows, int cols, int depth) {
    failures = 0;
    DC<int> a(rows, cols, depth, 6), c(rows, cols, depth, 0);
    Sum4 sum4;
    c.mapIndex(sum4, a);
    expect_each("DC mapIndex", c, [rows, cols](int k) {
        int x = k % cols, y = (k / cols) % rows, z = k / (rows * cols);
        return x + y + z + 6;
    });
    Sum5 sum5;
    c.zipIndex(a, a, sum5);
    expect_each("DC zipIndex", c, [rows, cols](int k) {
        int x = k % cols, y = (k / cols) % rows, z = k / (rows * cols);
        return x + y + z + 12;
    });
    Sum sum;
    if (a.fold(sum, true) != 6 * rows * cols * depth) failures++;
    DC<float> ones(rows, cols, depth, 1.0f), out(rows, cols, depth, 0.0f);
    ones.mapStencil<add27>(out, 1, 0.0f);
    float *p = out.gather();
    for (int z = 0; z < depth; z++)
        for (int y = 0; y < rows; y++)
            for (int x = 0; x < cols; x++) {
                int inside = (x > 0 && x < cols - 1) + (y > 0 && y < rows - 1) + (z > 0 && z < depth - 1);
                float want = inside == 3 ? 27.f : inside == 2 ? 18.f : inside == 1 ? 12.f : 8.f;
                if (cols == 1 || rows == 1 || depth == 1) continue;
                if (p[(z * rows + y) * cols + x] != want) {
                    failures++;
                    return failures;
                }
            }
    if (out.get(0, 0, 0) != 8.f) failures++;
    return failures;
}

// Plain Jacobi through DM::mapStencil, then the residual the reference way:
// zip(|new - old|) and fold(max). out receives the last sweep.
int fe_jacobi(const float *grid, int rows, int cols, int iters, float *out, float *residual) {
    DM<float> a(rows, cols, 0.0f, true), b(rows, cols, 0.0f, true), d(rows, cols, 0.0f, true);
    a.setLocalPartition(const_cast<float *>(grid));
    DM<float> *p = &a, *q = &b;
    for (int i = 0; i < iters; i++) {
        p->mapStencil<jacobi5>(*q, 1, 0.0f, false);
        std::swap(p, q);
    }
    AbsDiff ad;
    MaxF mx;
    d.zip(*p, *q, ad);
    *residual = d.fold(mx, true);
    std::memcpy(out, p->gather(), sizeof(float) * rows * cols);
    return 0;
}

int fe_heat3d(const float *cube, int depth, int rows, int cols, int iters, float *out) {
    DC<float> a(rows, cols, depth, 0.0f), b(rows, cols, depth, 0.0f);
    a.setLocalPartition(const_cast<float *>(cube));
    DC<float> *p = &a, *q = &b;
    for (int i = 0; i < iters; i++) {
        p->mapStencil<heat3d>(*q, 1, 0.0f);
        std::swap(p, q);
    }
    std::memcpy(out, p->gather(), sizeof(float) * depth * rows * cols);
    return 0;
}

int fe_boxsum3d_r2(const float *cube, int depth, int rows, int cols, float *out) {
    DC<float> a(rows, cols, depth, 0.0f), b(rows, cols, depth, 0.0f);
    a.setLocalPartition(const_cast<float *>(cube));
    a.mapStencil<boxsum3d<2>>(b, 2, 0.0f);
    std::memcpy(out, b.gather(), sizeof(float) * depth * rows * cols);
    return 0;
}

int fe_life_mm(const int *board, int rows, int cols, int iters, int *out) {
    DM<int> a(rows, cols, 0, true), b(rows, cols, 0, true);
    a.setLocalPartition(const_cast<int *>(board));
    GoL gol;
    gol.setStencilSize(1);
    for (int i = 0; i < iters; i++) {
        if (i % 2 == 0) a.mapStencilMM(b, gol, 0);
        else b.mapStencilMM(a, gol, 0);
    }
    std::memcpy(out, (iters % 2 ? b : a).gather(), sizeof(int) * rows * cols);
    return 0;
}

int fe_stencil_mm_nvf(const float *grid, int rows, int cols, int radius, int iters, float *out) {
    DM<float> a(rows, cols, 0.0f, true), b(rows, cols, 0.0f, true);
    a.setLocalPartition(const_cast<float *>(grid));
    EdgeValues edges(rows, cols);
    WeightedCross f;
    f.setStencilSize(radius);
    for (int i = 0; i < iters; i++) {
        if (i % 2 == 0) a.mapStencilMM(b, f, edges);
        else b.mapStencilMM(a, f, edges);
    }
    std::memcpy(out, (iters % 2 ? b : a).gather(), sizeof(float) * rows * cols);
    return 0;
}

// The float part of the map/zip/fold microbench with MSL_USERFUNC lambdas
// (built with -fmad=false: each * and + rounds separately, as in the oracle).
int fe_mapzipfold(const float *x, const float *y, int n, float *mapped, float *zipped, float *folded) {
    DA<float> a(n, 0.0f), b(n, 0.0f), m(n, 0.0f), z(n, 0.0f);
    a.setLocalPartition(const_cast<float *>(x));
    b.setLocalPartition(const_cast<float *>(y));
    auto affine = [] MSL_USERFUNC(float v) { return 2.5f * v + 1.0f; };
    auto muladd = [] MSL_USERFUNC(float p, float q) { return p * q + p; };
    auto plus = [] MSL_USERFUNC(float p, float q) { return p + q; };
    m.map(affine, a);
    z.zip(m, b, muladd);
    *folded = z.fold(plus, true);
    std::memcpy(mapped, m.gather(), sizeof(float) * n);
    std::memcpy(zipped, z.gather(), sizeof(float) * n);
    return 0;
}

int fe_dm_index(const int *in, const int *in2, int rows, int cols, int *mapped, int *zipped) {
    DM<int> a(rows, cols, 0, true), b(rows, cols, 0, true), o(rows, cols, 0, true);
    a.setLocalPartition(const_cast<int *>(in));
    b.setLocalPartition(const_cast<int *>(in2));
    DmIdx f;
    o.mapIndex(f, a);
    std::memcpy(mapped, o.gather(), sizeof(int) * rows * cols);
    DmZipIdx g;
    a.zipIndexInPlace(b, g);
    std::memcpy(zipped, a.gather(), sizeof(int) * rows * cols);
    return 0;
}

int fe_dc_index(const int *in, const int *in2, int depth, int rows, int cols, int *mapped, int *zipped) {
    DC<int> a(rows, cols, depth, 0), b(rows, cols, depth, 0), o(rows, cols, depth, 0);
    a.setLocalPartition(const_cast<int *>(in));
    b.setLocalPartition(const_cast<int *>(in2));
    DcIdx f;
    o.mapIndex(f, a);
    std::memcpy(mapped, o.gather(), sizeof(int) * depth * rows * cols);
    DcZipIdx g;
    a.zipIndexInPlace(b, g);
    std::memcpy(zipped, a.gather(), sizeof(int) * depth * rows * cols);
    return 0;
}

// DM::reduceRows with a Functor2 class (int) or a lambda (float) and a given
// threads-per-block setting.
int fe_reduce_rows_i32(const int *in, int rows, int cols, int tpb, int *out) {
    DM<int> a(rows, cols, 0, true);
    DA<int> c(rows, 0);
    a.setLocalPartition(const_cast<int *>(in));
    const int keep = Muesli::threads_per_block;
    setThreadsPerBlock(tpb);
    Sum f;
    a.reduceRows(c, f);
    setThreadsPerBlock(keep);
    std::memcpy(out, c.gather(), sizeof(int) * rows);
    return 0;
}
int fe_reduce_rows_f32(const float *in, int rows, int cols, int tpb, int op, float *out) {
    DM<float> a(rows, cols, 0.0f, true);
    DA<float> c(rows, 0.0f);
    a.setLocalPartition(const_cast<float *>(in));
    const int keep = Muesli::threads_per_block;
    setThreadsPerBlock(tpb);
    if (op == 0) {
        auto plus = [] MSL_USERFUNC(float x, float y) { return x + y; };
        a.reduceRows(c, plus);
    } else {
        MaxF mx;
        a.reduceRows(c, mx);
    }
    setThreadsPerBlock(keep);
    std::memcpy(out, c.gather(), sizeof(float) * rows);
    return 0;
}
int fe_reduce_two_columns(const float *in, int rows, int cols, float *out) {
    DM<float> a(rows, cols, 0.0f, true);
    DA<float> c(rows, 0.0f);
    a.setLocalPartition(const_cast<float *>(in));
    DotNext f;
    a.reducetwoColumns(c, f);
    std::memcpy(out, c.gather(), sizeof(float) * rows);
    return 0;
}
// which: 0 rotateRows, 1 rotateCols; the matrix is rotated in place.
int fe_rotate(const int *in, int rows, int cols, int a, int which, int *out) {
    DM<int> m(rows, cols, 0, true);
    m.setLocalPartition(const_cast<int *>(in));
    if (which == 0) m.rotateRows(a);
    else m.rotateCols(a);
    std::memcpy(out, m.gather(), sizeof(int) * rows * cols);
    return 0;
}
int fe_set_column(const float *in, const float *v, int rows, int cols, int col, float *out) {
    DM<float> m(rows, cols, 0.0f, true);
    DA<float> d(rows, 0.0f);
    m.setLocalPartition(const_cast<float *>(in));
    d.setLocalPartition(const_cast<float *>(v));
    m.setColumn(d, col);
    m.broadcastPartition(0);
    std::memcpy(out, m.gather(), sizeof(float) * rows * cols);
    return 0;
}
// kind: 0 zipIndexInPlaceMA(b, u), 1 zipIndexInPlaceA(u), 2 zipIndexInPlaceAAA(u, v, w),
// 3 crossZipIndexInPlace(b) (square), 4 DA::mapIndexInPlaceDMRows (on u, rows = a),
// 5 DA::zipIndexInPlaceDMRows (on u, b-vector = v, rows = a).
int fe_dm_da(int kind, const int *a, const int *b, const int *u, const int *v, const int *w, int rows, int cols,
             int *out) {
    DM<int> ma(rows, cols, 0, true), mb(rows, cols, 0, true);
    DA<int> du(rows, 0), dv(rows, 0), dw(rows, 0);
    ma.setLocalPartition(const_cast<int *>(a));
    mb.setLocalPartition(const_cast<int *>(b));
    du.setLocalPartition(const_cast<int *>(u));
    dv.setLocalPartition(const_cast<int *>(v));
    dw.setLocalPartition(const_cast<int *>(w));
    if (kind == 0) { ZipMA f; ma.zipIndexInPlaceMA(mb, du, f); }
    else if (kind == 1) { ZipA f; ma.zipIndexInPlaceA(du, f); }
    else if (kind == 2) { ZipAAA f; ma.zipIndexInPlaceAAA(du, dv, dw, f); }
    else if (kind == 3) { CrossT f{cols}; ma.crossZipIndexInPlace(mb, f); }
    if (kind <= 3) {
        std::memcpy(out, ma.gather(), sizeof(int) * rows * cols);
        return 0;
    }
    if (kind == 4) { RowSum f{cols}; du.mapIndexInPlaceDMRows(ma, f); }
    else { RowPick f{cols}; du.zipIndexInPlaceDMRows(dv, ma, f); }
    std::memcpy(out, du.gather(), sizeof(int) * rows);
    return 0;
}

}  // extern "C"
