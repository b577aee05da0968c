// dm.h -- DM<T>, the row-major matrix (drop-in for the reference's
// include/dm.h:71-667 and src/dm.cpp). Index functors are called
// f(row, col, ...); stencil functors f(view, x=col, y=row).
#pragma once

#include "da.h"
#include "detail/msl_matrix.cuh"
#include "detail/msl_stencil.cuh"
#include "ds.h"

namespace msl {

namespace detail {
template <typename T, NPLMMapStencilFunctor<T> f> struct NplCall {
    __device__ __forceinline__ T operator()(const NPLMatrix<T> &m, int x, int y) const { return f(m, x, y); }
};
// mapStencilMM functors: f(row, col, PLMatrix<T>* input, ncol, nrow).
template <typename T, class F> struct PlmCall {
    F f;
    __device__ __forceinline__ T operator()(const NPLMatrix<T> &m, int x, int y) const {
        PLMatrix<T> pl(m);
        if constexpr (std::is_class<F>::value) return f.F::operator()(y, x, &pl, m.width, m.height);
        else return f(y, x, &pl, m.width, m.height);
    }
};
// mapStencilMM with a neutral-value functor: the view reads cells outside the
// matrix from the halo ring the functor filled.
template <typename T, class F> struct PlmNvfCall {
    F f;
    const T *halo;
    int r;
    __device__ __forceinline__ T operator()(const NPLMatrix<T> &m, int x, int y) const {
        PLMatrix<T> pl(m, halo, r);
        if constexpr (std::is_class<F>::value) return f.F::operator()(y, x, &pl, m.width, m.height);
        else return f(y, x, &pl, m.width, m.height);
    }
};
// halo[k] = nvf(row, col) for every cell (row, col) of the ring.
template <typename T, class NVF> __global__ void halo_ring_kernel(T *halo, HaloRing ring, NVF nvf) {
    const long long n = ring.size(), stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        int row, col;
        ring.cell(k, row, col);
        halo[k] = invoke(nvf, row, col);
    }
}
// Device buffer of a container's halo ring, kept between calls. A copy of the
// container starts without one; a move takes it along.
struct HaloBuffer {
    void *p = nullptr;
    size_t bytes = 0;
    HaloBuffer() = default;
    HaloBuffer(const HaloBuffer &) {}
    HaloBuffer &operator=(const HaloBuffer &) { return *this; }
    HaloBuffer(HaloBuffer &&o) noexcept : p(o.p), bytes(o.bytes) {
        o.p = nullptr;
        o.bytes = 0;
    }
    HaloBuffer &operator=(HaloBuffer &&o) noexcept {
        std::swap(p, o.p);
        std::swap(bytes, o.bytes);
        return *this;
    }
    ~HaloBuffer() {
        if (p) msl_free(p);
    }
    void *reserve(size_t need) {
        if (need <= bytes) return p;
        if (p) msl_free(p);
        p = nullptr;
        bytes = 0;
        if (!check_status(msl_alloc(&p, need), "halo ring allocation")) return nullptr;
        bytes = need;
        return p;
    }
};

// DM x DA broadcast zips (src/zip_kernels.cu:45-71): a[r][c] = f(r, c, a[r][c], ...).
template <typename T, typename T2, typename T3, class F> struct ZipMAOp {  // ..., b[r][c], v[r]
    T *a;
    const T2 *b;
    const T3 *v;
    long long cols;
    F f;
    struct Row { long long base; T3 x; int r; };
    __device__ __forceinline__ Row row(long long r) const { return Row{r * cols, v[r], (int)r}; }
    __device__ __forceinline__ void operator()(const Row &w, long long, long long c) const {
        const long long k = w.base + c;
        a[k] = invoke(f, w.r, (int)c, a[k], b[k], w.x);
    }
};
template <typename T, typename T3, class F> struct ZipAOp {  // ..., v[r]
    T *a;
    const T3 *v;
    long long cols;
    F f;
    struct Row { long long base; T3 x; int r; };
    __device__ __forceinline__ Row row(long long r) const { return Row{r * cols, v[r], (int)r}; }
    __device__ __forceinline__ void operator()(const Row &w, long long, long long c) const {
        const long long k = w.base + c;
        a[k] = invoke(f, w.r, (int)c, a[k], w.x);
    }
};
template <typename T, typename T2, typename T3, typename T4, class F> struct ZipAAAOp {  // ..., u[r], v[r], w[r]
    T *a;
    const T2 *u;
    const T3 *v;
    const T4 *w;
    long long cols;
    F f;
    struct Row { long long base; T2 x; T3 y; T4 z; int r; };
    __device__ __forceinline__ Row row(long long r) const { return Row{r * cols, u[r], v[r], w[r], (int)r}; }
    __device__ __forceinline__ void operator()(const Row &q, long long, long long c) const {
        const long long k = q.base + c;
        a[k] = invoke(f, q.r, (int)c, a[k], q.x, q.y, q.z);
    }
};
// crossZipIndexInPlace on the GPU (src/zip_kernels.cu:158-163): f(r, c, a, b)
// with both containers' device pointers; the functor writes through them.
template <typename T, typename T2, class F> struct CrossZipOp {
    T *a;
    T2 *b;
    long long cols;
    F f;
    __device__ __forceinline__ int row(long long r) const { return (int)r; }
    __device__ __forceinline__ void operator()(int r, long long, long long c) const { invoke(f, r, (int)c, a, b); }
};
// reducetwoColumns (src/dm.cpp:1729-1752): per row, s = 0, then
// s = f(row[j], row[(j + 1) % cols], s) for j = 0 ... cols-1.
template <typename T, typename R, class F>
__global__ void reduce_two_columns_kernel(const T *in, R *out, long long rows, long long cols, F f) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += stride) {
        const T *row = in + r * cols;
        R s = R(0);
        for (long long j = 0; j < cols; j++) s = invoke(f, row[j], row[j + 1 == cols ? 0 : j + 1], s);
        out[r] = s;
    }
}
}  // namespace detail

template <typename T> class DM : public DS<T> {
   public:
    DM() = default;
    DM(int row, int col) : DS<T>(row * col), nrow(row), ncol(col) {}
    DM(int row, int col, const T &v) : DS<T>(row * col, v), nrow(row), ncol(col) {}
    DM(int row, int col, const T &v, bool rowComplete) : DS<T>(row * col, v), nrow(row), ncol(col) { (void)rowComplete; }

    int getnCol() const { return ncol; }
    int getnRow() const { return nrow; }
    T get2D(int row, int col) { return this->get(row * ncol + col); }
    void set2D(int row, int col, T value) { this->set(row * ncol + col, value); }

    // this[r][c] = f(r, c, this[r][c])  (src/dm.cpp:372-401)
    template <typename MapIndexFunctor> void mapIndexInPlace(MapIndexFunctor &f) {
        this->ensure_device();
        detail::launched(gpu::launch_map(this->d_, (const T *)this->d_, (size_t)this->n, gpu::IdxRowCol{ncol},
                                         detail::IndexCall2<MapIndexFunctor>{f}, stream(), sm_count()),
                         "mapIndexInPlace");
        this->device_written();
    }
    // this[r][c] = f(r, c, b[r][c])  (src/dm.cpp:405-429)
    template <typename MapIndexFunctor> void mapIndex(MapIndexFunctor &f, DM<T> &b) {
        if (b.getSize() != this->n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        detail::launched(gpu::launch_map(this->d_, (const T *)b.getDeviceData(), (size_t)this->n, gpu::IdxRowCol{ncol},
                                         detail::IndexCall2<MapIndexFunctor>{f}, stream(), sm_count()),
                         "mapIndex");
        this->device_written();
    }
    // this[r][c] = f(r, c, this[r][c], b[r][c])  (src/dm.cpp:435-464)
    template <typename T2, typename ZipIndexFunctor> void zipIndexInPlace(DM<T2> &b, ZipIndexFunctor &f) {
        if (b.getSize() != this->n) return throws(detail::NotSameSizeException());
        this->ensure_device();
        b.ensure_device();
        detail::launched(gpu::launch_zip(this->d_, (const T *)this->d_, (const T2 *)b.getDeviceData(), (size_t)this->n,
                                         gpu::IdxRowCol{ncol}, detail::IndexCall2<ZipIndexFunctor>{f}, stream(),
                                         sm_count()),
                         "zipIndexInPlace");
        this->device_written();
    }
    // this[r][c] = f(r, c, b[r][c], c2[r][c])  (src/dm.cpp:468-501, GPU argument order)
    template <typename T2, typename ZipIndexFunctor> void zipIndex(DM<T2> &b, DM<T2> &c, ZipIndexFunctor &f) {
        if (b.getSize() != this->n || c.getSize() != this->n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        c.ensure_device();
        detail::launched(gpu::launch_zip(this->d_, (const T2 *)b.getDeviceData(), (const T2 *)c.getDeviceData(),
                                         (size_t)this->n, gpu::IdxRowCol{ncol}, detail::IndexCall2<ZipIndexFunctor>{f},
                                         stream(), sm_count()),
                         "zipIndex");
        this->device_written();
    }
    // this[r][c] = f(r, c, this[r][c], b[r][c], c2[r][c])
    template <typename T2, typename T3, typename ZipIndexFunctor>
    void zipIndexInPlace3(DM<T2> &b, DM<T3> &c, ZipIndexFunctor &f) {
        this->ensure_device();
        b.ensure_device();
        c.ensure_device();
        detail::launched(gpu::launch_zip3(this->d_, (const T *)this->d_, (const T2 *)b.getDeviceData(),
                                          (const T3 *)c.getDeviceData(), (size_t)this->n, gpu::IdxRowCol{ncol},
                                          detail::IndexCall2<ZipIndexFunctor>{f}, stream(), sm_count()),
                         "zipIndexInPlace3");
        this->device_written();
    }

    // result[y][x] = f(view of this, x, y), view = neutral outside the matrix
    // (src/dm.cpp:1535-1591). shared_mem is a hint the tile kernel does not need.
    template <NPLMMapStencilFunctor<T> f>
    void mapStencil(DM<T> &result, size_t stencilSize, T neutralValue, bool shared_mem = false) {
        (void)shared_mem;
        if (result.getSize() != this->n || &result == this) return throws(detail::IllegalArgumentException());
        this->ensure_device();
        detail::launched(gpu::launch_stencil2d<T>((const T *)this->d_, result.getDeviceData(), nrow, ncol,
                                                  (int)stencilSize, neutralValue, detail::NplCall<T, f>{}, nullptr,
                                                  detail::front_scratch().err, stream()),
                         "mapStencil");
        result.device_written();
    }
    // Legacy PLMatrix stencil (src/dm.cpp:615-1331), on the same tile kernel:
    // result[r][c] = f(r, c, PLMatrix*, ncol, nrow), neutral outside.
    template <typename T2, typename MapStencilFunctor>
    void mapStencilMM(DM<T2> &result, MapStencilFunctor &f, T neutral_value) {
        if (result.getSize() != this->n || (void *)&result == (void *)this)
            return throws(detail::IllegalArgumentException());
        this->ensure_device();
        int r = f.getStencilSize();
        detail::launched(gpu::launch_stencil2d<T>((const T *)this->d_, (T *)result.getDeviceData(), nrow, ncol, r,
                                                  neutral_value, detail::PlmCall<T, MapStencilFunctor>{f}, nullptr,
                                                  detail::front_scratch().err, stream()),
                         "mapStencilMM");
        result.device_written();
    }
    // The same with a neutral-value functor (src/dm.cpp:615-919; the
    // examples' jacobi solver, examples/jacobisolver.cpp:127-136): a read of a
    // cell (row, col) outside the matrix returns nvf(row, col). The functor
    // is evaluated on the device once per call for the ring of cells within
    // the stencil size of the matrix (kept in a buffer of this container
    // between calls); reads farther out return T{}.
    template <typename T2, typename MapStencilFunctor, typename NeutralValueFunctor,
              typename std::enable_if<std::is_class<NeutralValueFunctor>::value, int>::type = 0>
    void mapStencilMM(DM<T2> &result, MapStencilFunctor &f, NeutralValueFunctor &nvf) {
        if (result.getSize() != this->n || (void *)&result == (void *)this)
            return throws(detail::IllegalArgumentException());
        const int r = f.getStencilSize();
        if (r < 0) return throws(detail::IllegalArgumentException());
        this->ensure_device();
        const HaloRing ring{nrow, ncol, r};
        T *halo = nullptr;
        if (ring.size() > 0) {
            halo = (T *)halo_.reserve((size_t)ring.size() * sizeof(T));
            if (!halo) return;
            const int threads = 256;
            long long blocks = (ring.size() + threads - 1) / threads;
            if (blocks > 4LL * sm_count()) blocks = 4LL * sm_count();
            detail::halo_ring_kernel<<<(unsigned)blocks, threads, 0, stream()>>>(halo, ring, nvf);
            detail::launched(cudaGetLastError(), "mapStencilMM neutral values");
        }
        detail::launched(gpu::launch_stencil2d<T>((const T *)this->d_, (T *)result.getDeviceData(), nrow, ncol, r,
                                                  T{}, detail::PlmNvfCall<T, MapStencilFunctor>{f, halo, r}, nullptr,
                                                  detail::front_scratch().err, stream()),
                         "mapStencilMM");
        result.device_written();
    }

    // ---- row / column skeletons ----
    // c[r] = fold of row r with f, in the GPU build's row-fold order
    // (src/dm.cpp:1677-1685, kernel src/fold_kernels.cu:215-294): lanes per row
    // from Muesli::threads_per_block, element-seeded.
    template <typename ReduceFunctor> void reduceRows(DA<T> &c, ReduceFunctor &f) {
        static_assert(sizeof(T) % 4 == 0, "reduceRows shuffles 4-byte words");
        if (c.getSize() != nrow) return throws(detail::SizeMismatchException());
        const int tpb = Muesli::threads_per_block;
        if (tpb < 1 || tpb > 1024 || (tpb & (tpb - 1))) return throws(detail::IllegalArgumentException());
        this->ensure_device();
        detail::launched(gpu::launch_fold_rows((const T *)this->d_, c.getDeviceData(), nrow, ncol, tpb,
                                               detail::FoldCall<ReduceFunctor, T>{f}, stream(), sm_count()),
                         "reduceRows");
        c.device_written();
    }
    // c[r] = f(row[ncol-1], row[0], ... f(row[1], row[2], f(row[0], row[1], 0)))
    // (src/dm.cpp:1729-1752), one device thread per row.
    template <typename T2, typename ReduceFunctor> void reducetwoColumns(DA<T2> &c, ReduceFunctor &f) {
        if (c.getSize() != nrow) return throws(detail::SizeMismatchException());
        if (!nrow || !ncol) return;
        this->ensure_device();
        detail::reduce_two_columns_kernel<<<gpu::rows_blocks(nrow, 256, sm_count()), 256, 0, stream()>>>(
            (const T *)this->d_, c.getDeviceData(), (long long)nrow, (long long)ncol, f);
        detail::launched(cudaGetLastError(), "reducetwoColumns");
        c.device_written();
    }

    // this[r][c] = f(r, c, this[r][c], b[r][c], v[r])  (src/dm.cpp:1757-1787)
    template <typename T2, typename T3, typename ZipIndexFunctor>
    void zipIndexInPlaceMA(DM<T2> &b, DA<T3> &v, ZipIndexFunctor &f) {
        if (b.getSize() != this->n || v.getSize() < nrow) return throws(detail::NotSameSizeException());
        this->ensure_device();
        b.ensure_device();
        v.ensure_device();
        detail::ZipMAOp<T, T2, T3, ZipIndexFunctor> op{this->d_, b.getDeviceData(), v.getDeviceData(), ncol, f};
        detail::launched(gpu::launch_row_cells(nrow, ncol, op, stream(), sm_count()), "zipIndexInPlaceMA");
        this->device_written();
    }
    // this[r][c] = f(r, c, this[r][c], v[r])  (src/dm.cpp:1790-1812)
    template <typename T3, typename ZipIndexFunctor> void zipIndexInPlaceA(DA<T3> &v, ZipIndexFunctor &f) {
        if (v.getSize() < nrow) return throws(detail::NotSameSizeException());
        this->ensure_device();
        v.ensure_device();
        detail::ZipAOp<T, T3, ZipIndexFunctor> op{this->d_, v.getDeviceData(), ncol, f};
        detail::launched(gpu::launch_row_cells(nrow, ncol, op, stream(), sm_count()), "zipIndexInPlaceA");
        this->device_written();
    }
    // this[r][c] = f(r, c, this[r][c], u[r], v[r], w[r])  (src/dm.cpp:1815-1853)
    template <typename T2, typename T3, typename T4, typename ZipIndexFunctor>
    void zipIndexInPlaceAAA(DA<T2> &u, DA<T3> &v, DA<T4> &w, ZipIndexFunctor &f) {
        if (u.getSize() < nrow || v.getSize() < nrow || w.getSize() < nrow)
            return throws(detail::NotSameSizeException());
        this->ensure_device();
        u.ensure_device();
        v.ensure_device();
        w.ensure_device();
        detail::ZipAAAOp<T, T2, T3, T4, ZipIndexFunctor> op{this->d_, u.getDeviceData(), v.getDeviceData(),
                                                             w.getDeviceData(), ncol, f};
        detail::launched(gpu::launch_row_cells(nrow, ncol, op, stream(), sm_count()), "zipIndexInPlaceAAA");
        this->device_written();
    }
    // f(r, c, this_data, b_data) for every cell (src/dm.cpp:505-536, GPU build):
    // the functor reads and writes both matrices through the device pointers.
    template <typename T2, typename ZipIndexFunctor> void crossZipIndexInPlace(DM<T2> &b, ZipIndexFunctor &f) {
        this->ensure_device();
        b.ensure_device();
        detail::CrossZipOp<T, T2, ZipIndexFunctor> op{this->d_, b.getDeviceData(), ncol, f};
        detail::launched(gpu::launch_row_cells(nrow, ncol, op, stream(), sm_count()), "crossZipIndexInPlace");
        this->device_written();
        b.device_written();
    }

    // Row k becomes row (k - a) mod nrow (src/dm.cpp:1345-1475); |a| > nrow is
    // the reference's RotateRowManyNotImplementedException (matrix unchanged).
    void rotateRows(int a) {
        const long long howmuch = a < 0 ? -(long long)a : a;
        if (a == 0 || howmuch == nrow || !this->n) return;
        if (howmuch > nrow) return throws(detail::RotateRowManyNotImplementedException());
        permute(a, true);
    }
    // Column j becomes column (j + a) mod ncol (src/dm.cpp:1483-1533).
    void rotateCols(int a) {
        if (!this->n || a % ncol == 0) return;
        permute(a, false);
    }
    // this[r][col] = da[r]  (src/dm.cpp:1856-1879)
    void setColumn(DA<T> &da, int col) {
        if (col < 0 || col >= ncol) return throws(detail::IndexOutOfBoundsException());
        if (da.getSize() != nrow) return throws(detail::SizeMismatchException());
        this->ensure_device();
        da.ensure_device();
        gpu::set_column_kernel<<<gpu::rows_blocks(nrow, 256, sm_count()), 256, 0, stream()>>>(
            this->d_, (const T *)da.getDeviceData(), (long long)nrow, (long long)ncol, (long long)col);
        detail::launched(cudaGetLastError(), "setColumn");
        this->device_written();
    }
    // One process holds every partition: broadcasting partition 0 leaves the
    // data as it is; any other index is an IllegalPartitionException
    // (src/dm.cpp:301-310).
    void broadcastPartition(int partitionIndex) {
        if (partitionIndex != 0) throws(detail::IllegalPartitionException());
    }

    void show(const std::string &descr = std::string(), int limited = 0) {
        this->ensure_host();
        std::ostringstream s;
        if (!descr.empty()) s << descr << std::endl;
        int rows = limited > 0 ? std::min(limited, nrow) : nrow;
        for (int r = 0; r < rows; r++) {
            s << "[";
            for (int c = 0; c < ncol; c++) s << this->localPartition[(size_t)r * ncol + c] << (c + 1 < ncol ? " " : "");
            s << "]" << std::endl;
        }
        if (isRootProcess()) std::cout << s.str();
    }

   private:
    int nrow = 0, ncol = 0;
    detail::HaloBuffer halo_;

    // Rotation into a fresh device buffer, which then replaces the partition.
    void permute(int a, bool rows) {
        this->ensure_device();
        T *tmp = nullptr;
        if (!check_status(msl_alloc((void **)&tmp, this->bytes()), "rotate buffer")) return;
        cudaError_t e;
        if (rows) {
            long long s = a % nrow;
            if (s < 0) s += nrow;
            e = gpu::launch_row_cells(nrow, ncol, gpu::RotateRowsOp<T>{this->d_, tmp, nrow, ncol, s}, stream(), sm_count());
        } else {
            long long s = a % ncol;
            if (s < 0) s += ncol;
            e = gpu::launch_row_cells(nrow, ncol, gpu::RotateColsOp<T>{this->d_, tmp, ncol, s}, stream(), sm_count());
        }
        detail::launched(e, rows ? "rotateRows" : "rotateCols");
        msl_free(this->d_);  // waits for the rotation to finish
        this->d_ = tmp;
        this->device_written();
    }
};

}  // namespace msl
