// dm.h -- DM<T>, the row-major matrix (drop-in for the reference's
// include/dm.h:71-667 and src/dm.cpp). Index functors are called
// f(row, col, ...); stencil functors f(view, x=col, y=row).
#pragma once

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
};

}  // namespace msl
