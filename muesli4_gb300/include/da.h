// da.h -- DA<T>, the one-dimensional container (drop-in for the reference's
// include/da.h:69-284 and src/da.cpp).
#pragma once

#include "detail/msl_matrix.cuh"
#include "ds.h"

namespace msl {

template <typename T> class DM;

namespace detail {
// this[i] = f(i, &rows[i][0], this[i])  (src/map_kernels.cu:80-86)
template <typename T, typename T2, class F> struct MapDMRowsOp {
    T *a;
    T2 *rows;
    long long cols;
    F f;
    __device__ __forceinline__ void operator()(long long i) const { a[i] = invoke(f, (int)i, rows + i * cols, a[i]); }
};
// this[i] = f(i, &rows[i][0], b[i], this[i])  (src/zip_kernels.cu:73-78)
template <typename T, typename T1, typename T2, class F> struct ZipDMRowsOp {
    T *a;
    const T1 *b;
    T2 *rows;
    long long cols;
    F f;
    __device__ __forceinline__ void operator()(long long i) const {
        a[i] = invoke(f, (int)i, rows + i * cols, b[i], a[i]);
    }
};
}  // namespace detail

template <typename T> class DA : public DS<T> {
   public:
    DA() = default;
    explicit DA(int size) : DS<T>(size) {}
    DA(int size, const T &v) : DS<T>(size, v) {}

    // this[i] = f(i, this[i])  (src/da.cpp:232-255)
    template <typename MapIndexFunctor> void mapIndexInPlace(MapIndexFunctor &f) {
        this->ensure_device();
        detail::launched(gpu::launch_map(this->d_, (const T *)this->d_, (size_t)this->n, gpu::IdxFlat{0},
                                         detail::IndexCall1<MapIndexFunctor>{f}, stream(), sm_count()),
                         "mapIndexInPlace");
        this->device_written();
    }
    // this[i] = f(i, b[i])  (src/da.cpp:328-355)
    template <typename MapIndexFunctor> void mapIndex(MapIndexFunctor &f, DA<T> &b) {
        if (b.getSize() != this->n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        detail::launched(gpu::launch_map(this->d_, (const T *)b.getDeviceData(), (size_t)this->n, gpu::IdxFlat{0},
                                         detail::IndexCall1<MapIndexFunctor>{f}, stream(), sm_count()),
                         "mapIndex");
        this->device_written();
    }
    // this[i] = f(i, this[i], b[i])  (src/da.cpp:375-399)
    template <typename T2, typename ZipIndexFunctor> void zipIndexInPlace(DA<T2> &b, ZipIndexFunctor &f) {
        if (b.getSize() != this->n) return throws(detail::NotSameSizeException());
        this->ensure_device();
        b.ensure_device();
        detail::launched(gpu::launch_zip(this->d_, (const T *)this->d_, (const T2 *)b.getDeviceData(), (size_t)this->n,
                                         gpu::IdxFlat{0}, detail::IndexCall1<ZipIndexFunctor>{f}, stream(), sm_count()),
                         "zipIndexInPlace");
        this->device_written();
    }
    // this[i] = f(i, b[i], c[i])  (src/da.cpp:403-430, GPU argument order)
    template <typename T2, typename ZipIndexFunctor> void zipIndex(DA<T2> &b, DA<T2> &c, ZipIndexFunctor &f) {
        if (b.getSize() != this->n || c.getSize() != this->n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        c.ensure_device();
        detail::launched(gpu::launch_zip(this->d_, (const T2 *)b.getDeviceData(), (const T2 *)c.getDeviceData(),
                                         (size_t)this->n, gpu::IdxFlat{0}, detail::IndexCall1<ZipIndexFunctor>{f},
                                         stream(), sm_count()),
                         "zipIndex");
        this->device_written();
    }
    // this[i] = f(i, row i of `rows` (device pointer), this[i])  (src/da.cpp:256-287)
    template <typename MapIndexFunctor, typename T2> void mapIndexInPlaceDMRows(DM<T2> &rows, MapIndexFunctor &f) {
        if (rows.getnRow() < this->n) return throws(detail::SizeMismatchException());
        this->ensure_device();
        rows.ensure_device();
        detail::MapDMRowsOp<T, T2, MapIndexFunctor> op{this->d_, rows.getDeviceData(), rows.getnCol(), f};
        detail::launched(gpu::launch_for_each_index(this->n, op, stream(), sm_count()), "mapIndexInPlaceDMRows");
        this->device_written();
    }
    // this[i] = f(i, row i of `rows`, b[i], this[i])  (src/da.cpp:290-324)
    template <typename ZipIndexFunctor, typename T1, typename T2>
    void zipIndexInPlaceDMRows(DA<T1> &b, DM<T2> &rows, ZipIndexFunctor &f) {
        if (rows.getnRow() < this->n || b.getSize() != this->n) return throws(detail::SizeMismatchException());
        this->ensure_device();
        b.ensure_device();
        rows.ensure_device();
        detail::ZipDMRowsOp<T, T1, T2, ZipIndexFunctor> op{this->d_, b.getDeviceData(), rows.getDeviceData(),
                                                           rows.getnCol(), f};
        detail::launched(gpu::launch_for_each_index(this->n, op, stream(), sm_count()), "zipIndexInPlaceDMRows");
        this->device_written();
    }
    // One process holds every partition (src/da.cpp:166-175).
    void broadcastPartition(int partitionIndex) {
        if (partitionIndex != 0) throws(detail::IllegalPartitionException());
    }
    void show(const std::string &descr = std::string(), int limited = 0) { DS<T>::show(descr, limited); }
};

}  // namespace msl
