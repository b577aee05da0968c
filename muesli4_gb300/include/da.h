// da.h -- DA<T>, the one-dimensional container (drop-in for the reference's
// include/da.h:69-284 and src/da.cpp).
#pragma once

#include "ds.h"

namespace msl {

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
    void show(const std::string &descr = std::string(), int limited = 0) { DS<T>::show(descr, limited); }
};

}  // namespace msl
