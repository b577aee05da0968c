// dc.h -- DC<T>, the cube (drop-in for the reference's include/dc.h and
// src/dc.cpp). Layout (z * rows + y) * cols + x; index and stencil functors
// are called f(x=col, y=row, z=depth, ...).
#pragma once

#include "detail/msl_stencil.cuh"
#include "ds.h"

namespace msl {

namespace detail {
template <typename T, DCMapStencilFunctor<T> f> struct PlcCall {
    __device__ __forceinline__ T operator()(const PLCube<T> &c, int x, int y, int z) const { return f(c, x, y, z); }
};
}  // namespace detail

template <typename T> class DC : public DS<T> {
   public:
    DC() = default;
    DC(int row, int col, int depth) : DS<T>(row * col * depth), nrow(row), ncol(col), ndepth(depth) {}
    DC(int row, int col, int depth, const T &v) : DS<T>(row * col * depth, v), nrow(row), ncol(col), ndepth(depth) {}
    DC(int row, int col, int depth, const T &v, bool rowComplete)
        : DS<T>(row * col * depth, v), nrow(row), ncol(col), ndepth(depth) {
        (void)rowComplete;
    }

    int getCols() const { return ncol; }
    int getRows() const { return nrow; }
    int getDepth() const { return ndepth; }
    // src/dc.cpp:602-608: element (col, row, depth)
    T get(int col, int row, int depth) { return DS<T>::get(index(col, row, depth)); }
    void set(int col, int row, int depth, T value) { DS<T>::set(index(col, row, depth), value); }
    using DS<T>::get;
    using DS<T>::set;

    // this = f(x, y, z, this)  (src/dc.cpp:387-414)
    template <typename MapIndexFunctor> void mapIndexInPlace(MapIndexFunctor &f) {
        this->ensure_device();
        detail::launched(gpu::launch_map(this->d_, (const T *)this->d_, (size_t)this->n, gpu::IdxXYZ{ncol, nrow},
                                         detail::IndexCall3<MapIndexFunctor>{f}, stream(), sm_count()),
                         "mapIndexInPlace");
        this->device_written();
    }
    // this = f(x, y, z, b)  (src/dc.cpp:418-448)
    template <typename MapIndexFunctor> void mapIndex(MapIndexFunctor &f, DC<T> &b) {
        if (b.getSize() != this->n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        detail::launched(gpu::launch_map(this->d_, (const T *)b.getDeviceData(), (size_t)this->n,
                                         gpu::IdxXYZ{ncol, nrow}, detail::IndexCall3<MapIndexFunctor>{f}, stream(),
                                         sm_count()),
                         "mapIndex");
        this->device_written();
    }
    // this = f(x, y, z, this, b)  (src/dc.cpp:456-485)
    template <typename T2, typename ZipIndexFunctor> void zipIndexInPlace(DC<T2> &b, ZipIndexFunctor &f) {
        if (b.getSize() != this->n) return throws(detail::NotSameSizeException());
        this->ensure_device();
        b.ensure_device();
        detail::launched(gpu::launch_zip(this->d_, (const T *)this->d_, (const T2 *)b.getDeviceData(), (size_t)this->n,
                                         gpu::IdxXYZ{ncol, nrow}, detail::IndexCall3<ZipIndexFunctor>{f}, stream(),
                                         sm_count()),
                         "zipIndexInPlace");
        this->device_written();
    }
    // this = f(x, y, z, b, c)  (src/dc.cpp:519-550, GPU argument order)
    template <typename T2, typename ZipIndexFunctor> void zipIndex(DC<T2> &b, DC<T2> &c, ZipIndexFunctor &f) {
        if (b.getSize() != this->n || c.getSize() != this->n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        c.ensure_device();
        detail::launched(gpu::launch_zip(this->d_, (const T2 *)b.getDeviceData(), (const T2 *)c.getDeviceData(),
                                         (size_t)this->n, gpu::IdxXYZ{ncol, nrow}, detail::IndexCall3<ZipIndexFunctor>{f},
                                         stream(), sm_count()),
                         "zipIndex");
        this->device_written();
    }

    // result = f(view of this, x, y, z), view = neutral outside the cube (src/dc.cpp:559-592).
    template <DCMapStencilFunctor<T> f> void mapStencil(DC<T> &result, size_t stencilSize, T neutralValue) {
        if (result.getSize() != this->n || &result == this) return throws(detail::IllegalArgumentException());
        this->ensure_device();
        detail::launched(gpu::launch_stencil3d<T>((const T *)this->d_, result.getDeviceData(), ndepth, nrow, ncol,
                                                  (int)stencilSize, neutralValue, detail::PlcCall<T, f>{}, nullptr,
                                                  detail::front_scratch().err, stream(), sm_count()),
                         "mapStencil");
        result.device_written();
    }

   private:
    int nrow = 0, ncol = 0, ndepth = 0;
    int index(int col, int row, int depth) const { return (depth * nrow + row) * ncol + col; }
};

}  // namespace msl
