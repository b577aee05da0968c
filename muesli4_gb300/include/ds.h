// ds.h -- DS<T>, the base of the distributed containers (drop-in for the
// reference's include/ds.h:69-642 and src/ds.cpp).
//
// GB300 design: one device-resident partition per container (msl_alloc), a
// pinned host mirror allocated on first host access, and a two-flag
// coherence state (device copy valid / host copy valid). Skeletons run on
// the device and only invalidate the host copy; host reads (gather, get,
// getLocalPartition, show) download on demand and synchronise; host writes
// (set, setLocal, fill(T*), setLocalPartition) go to the mirror and are
// uploaded before the next skeleton. Skeleton calls are asynchronous on the
// library stream, where the reference synchronises after every call
// (src/muesli.cpp:213-223).
//
// User functors are inlined into the kernels of detail/msl_elementwise.cuh and
// detail/msl_fold.cuh, instantiated in the caller's translation unit.
#pragma once

#include <algorithm>
#include <cstring>
#include <iomanip>
#include <sstream>
#include <type_traits>
#include <utility>

#include "detail/msl_elementwise.cuh"
#include "detail/msl_fold.cuh"
#include "functors.h"
#include "muesli.h"

namespace msl {
namespace detail {

// Calls the functor's own operator() with a qualified name, so the call is
// resolved statically even when the functor class declares it virtual (the
// object's virtual-table pointer is a host address and is never used).
template <class F, class... A>
__device__ __forceinline__ auto invoke(const F &f, A &&...a) -> decltype(f(static_cast<A &&>(a)...)) {
    if constexpr (std::is_class<F>::value) return f.F::operator()(static_cast<A &&>(a)...);
    else return f(static_cast<A &&>(a)...);
}

// Adapters from the reference's functor signatures to the kernels' (coords, values...) convention.
template <class F> struct MapCall {
    F f;
    template <class S, class X> __device__ __forceinline__ auto operator()(S, X x) const { return invoke(f, x); }
    template <class S, class X, class Y> __device__ __forceinline__ auto operator()(S, X x, Y y) const {
        return invoke(f, x, y);
    }
    template <class S, class X, class Y, class Z> __device__ __forceinline__ auto operator()(S, X x, Y y, Z z) const {
        return invoke(f, x, y, z);
    }
};
template <class F> struct IndexCall1 {  // DA: f(i, ...)
    F f;
    template <class... X> __device__ __forceinline__ auto operator()(gpu::IdxFlat::S s, X... x) const {
        return invoke(f, (int)s.i, x...);
    }
};
template <class F> struct IndexCall2 {  // DM: f(row, col, ...)
    F f;
    template <class... X> __device__ __forceinline__ auto operator()(gpu::IdxRowCol::S s, X... x) const {
        return invoke(f, s.row, s.col, x...);
    }
};
template <class F> struct IndexCall3 {  // DC: f(x=col, y=row, z=depth, ...)
    F f;
    template <class... X> __device__ __forceinline__ auto operator()(gpu::IdxXYZ::S s, X... x) const {
        return invoke(f, s.x, s.y, s.z, x...);
    }
};
template <class F, typename T> struct FoldCall {
    F f;
    __device__ __forceinline__ T operator()(T a, T b) const { return invoke(f, a, b); }
};

template <typename T> __global__ void fill_value_kernel(T *p, size_t n, T v) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

// Device scratch of the front end: fold partials and ticket, device error
// word. Allocated once on first use, released by terminateSkeletons().
struct FrontScratch {
    void *base = nullptr;
    gpu::FoldScratch fold{};
    unsigned *err = nullptr;
};
inline FrontScratch &front_scratch() {
    static FrontScratch s;
    if (!s.base) {
        const size_t bytes = gpu::kFoldScratchBytes + 256;
        if (!check_status(msl_alloc(&s.base, bytes), "scratch allocation")) return s;
        cudaMemsetAsync(s.base, 0, bytes, stream());
        s.fold = gpu::carve_fold_scratch(s.base);
        s.err = (unsigned *)((char *)s.base + gpu::kFoldScratchBytes);
        at_terminate().push_back([] {
            msl_free(front_scratch().base);
            front_scratch() = FrontScratch{};
        });
    }
    return s;
}

inline void launched(cudaError_t e, const char *what) {
    if (e != cudaSuccess) check_status(MSL_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
    if (Muesli::debug) syncStreams();
}

}  // namespace detail

template <typename T> class DS {
   public:
    // Host mirror of the partition (valid after updateHost()/gather(); the
    // reference's public localPartition, include/ds.h:604).
    T *localPartition = nullptr;

    DS() = default;
    explicit DS(int size) : n(size) { allocate(); }
    DS(int size, const T &v) : n(size) {
        allocate();
        fill(v);
    }
    DS(const DS &o) : n(o.n) {
        allocate();
        copy_from(o);
    }
    DS &operator=(const DS &o) {
        if (this != &o) {
            if (n != o.n) {
                release();
                n = o.n;
                allocate();
            }
            copy_from(o);
        }
        return *this;
    }
    DS(DS &&o) noexcept { steal(o); }
    DS &operator=(DS &&o) noexcept {
        if (this != &o) {
            release();
            steal(o);
        }
        return *this;
    }
    virtual ~DS() { release(); }

    // ---- sizes (src/ds.cpp:189-211 collapse to one partition) ----
    int getSize() const { return (int)n; }
    int getLocalSize() const { return (int)n; }
    int getFirstIndex() const { return 0; }
    bool isLocal(int index) const { return index >= 0 && index < n; }
    long getnCPU() { return 0; }
    T *getDeviceData() const { return d_; }

    // ---- fill / transfers ----
    // DS::fill(const T&) (src/ds.cpp:290-305): a device fill kernel.
    void fill(const T &v) {
        if (!n) return;
        detail::fill_value_kernel<T><<<gpu::ew_blocks(n, sm_count()), 256, 0, stream()>>>(d_, (size_t)n, v);
        detail::launched(cudaGetLastError(), "fill");
        device_written();
    }
    // DS::fill(T*) (src/ds.cpp:307-321): copy n values from host memory.
    void fill(T *const values) { setLocalPartition(values); }
    void setLocalPartition(T *elements) {
        if (!n) return;
        ensure_mirror();
        if (elements != localPartition) std::memcpy(localPartition, elements, bytes());
        host_written();
        updateDevice();
    }
    T *getLocalPartition() {
        ensure_host();
        return localPartition;
    }
    // DS::updateDevice (src/ds.cpp:442-462): push the host mirror if it is newer.
    void updateDevice(bool force = false) {
        if (!n || !localPartition) return;
        if (force || !dev_valid_) {
            check_status(msl_upload(d_, localPartition, bytes()), "updateDevice");
            dev_valid_ = true;
        }
    }
    // DS::updateHost (src/ds.cpp:465-484).
    void updateHost() { ensure_host(); }
    void setCpuMemoryInSync(bool b) { host_valid_ = b; }

    // ---- gather (src/ds.cpp:539-591) ----
    // Returns the internal host buffer (borrowed, as in the reference).
    T *gather() {
        ensure_host();
        return localPartition;
    }
    // Copies the values into b; a null b receives the internal buffer (borrowed).
    void gather(T *&b) {
        ensure_host();
        if (!b) b = localPartition;
        else if (b != localPartition) std::memcpy(b, localPartition, bytes());
    }
    // Device-to-device copy into another container of the same size.
    void gather(DS<T> &da) {
        if (da.n != n) return throws(detail::SizeMismatchException());
        ensure_device();
        check_status(msl_copy(da.d_, d_, bytes()), "gather");
        da.device_written();
    }

    // ---- element access ----
    T get(int index) {
        ensure_host();
        return localPartition[index];
    }
    void set(int globalIndex, const T &v) {
        ensure_host();
        localPartition[globalIndex] = v;
        host_written();
    }
    T getLocal(int localIndex) { return get(localIndex); }
    void setLocal(int localIndex, const T &v) { set(localIndex, v); }

    // ---- map (src/ds.cpp:614-663) ----
    template <typename MapFunctor> void mapInPlace(MapFunctor &f) {
        ensure_device();
        detail::launched(gpu::launch_map(d_, (const T *)d_, (size_t)n, gpu::IdxNone{}, detail::MapCall<MapFunctor>{f},
                                         stream(), sm_count()),
                         "mapInPlace");
        device_written();
    }
    // this[i] = f(b[i])
    template <typename F> void map(F &f, DS<T> &b) {
        if (b.n != n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        detail::launched(
            gpu::launch_map(d_, (const T *)b.d_, (size_t)n, gpu::IdxNone{}, detail::MapCall<F>{f}, stream(), sm_count()),
            "map");
        device_written();
    }

    // ---- zip (src/ds.cpp:669-727), the GPU build's argument order ----
    // this[i] = f(this[i], b[i])
    template <typename T2, typename ZipFunctor> void zipInPlace(DS<T2> &b, ZipFunctor &f) {
        if (b.getSize() != n) return throws(detail::NotSameSizeException());
        ensure_device();
        b.ensure_device();
        detail::launched(gpu::launch_zip(d_, (const T *)d_, (const T2 *)b.getDeviceData(), (size_t)n, gpu::IdxNone{},
                                         detail::MapCall<ZipFunctor>{f}, stream(), sm_count()),
                         "zipInPlace");
        device_written();
    }
    // this[i] = f(b[i], c[i])
    template <typename T2, typename ZipFunctor> void zip(DS<T2> &b, DS<T2> &c, ZipFunctor &f) {
        if (b.getSize() != n || c.getSize() != n) return throws(detail::NotSameSizeException());
        b.ensure_device();
        c.ensure_device();
        detail::launched(gpu::launch_zip(d_, (const T2 *)b.getDeviceData(), (const T2 *)c.getDeviceData(), (size_t)n,
                                         gpu::IdxNone{}, detail::MapCall<ZipFunctor>{f}, stream(), sm_count()),
                         "zip");
        device_written();
    }
    // this[i] = f(this[i], b[i], c[i])
    template <typename T2, typename T3, typename ZipFunctor> void zipInPlace3(DS<T2> &b, DS<T3> &c, ZipFunctor &f) {
        ensure_device();
        b.ensure_device();
        c.ensure_device();
        detail::launched(gpu::launch_zip3(d_, (const T *)d_, (const T2 *)b.getDeviceData(), (const T3 *)c.getDeviceData(),
                                          (size_t)n, gpu::IdxNone{}, detail::MapCall<ZipFunctor>{f}, stream(), sm_count()),
                         "zipInPlace3");
        device_written();
    }

    // ---- fold (src/ds.cpp:741-954) ----
    // Single-pass device fold seeded with elements; f must be associative and
    // commutative. final_fold_on_cpu is accepted for compatibility: the last
    // combination step always runs on the device.
    template <typename FoldFunctor> T fold(FoldFunctor &f, bool final_fold_on_cpu = false) {
        (void)final_fold_on_cpu;
        static_assert(sizeof(T) % 4 == 0 && sizeof(T) <= 16, "fold supports element types of 4..16 bytes (multiple of 4)");
        if (!n) {
            throws(detail::IllegalArgumentException());
            return T{};
        }
        ensure_device();
        auto &s = detail::front_scratch();
        constexpr int V = gpu::vec_width1<T>();
        detail::launched(gpu::launch_fold<gpu::FoldSrcArray, T>((size_t)n, detail::FoldCall<FoldFunctor, T>{f}, s.fold,
                                                                 stream(), sm_count(), gpu::aligned_to(d_, V * sizeof(T)),
                                                                 (const T *)d_),
                         "fold");
        T result{};
        cudaMemcpyAsync(&result, s.fold.result, sizeof(T), cudaMemcpyDeviceToHost, stream());
        check_status(msl_sync(), "fold");
        return result;
    }
    template <typename FoldFunctor> T foldCPU(FoldFunctor &f) { return fold(f, true); }

    // ---- printing ----
    void show(const std::string &descr = std::string(), int limited = 0) {
        ensure_host();
        std::ostringstream s;
        if (!descr.empty()) s << descr << std::endl;
        s << "[";
        long lim = limited > 0 ? std::min<long>(limited, n) : n;
        for (long i = 0; i < lim; i++) s << localPartition[i] << (i + 1 < lim ? " " : "");
        s << "]" << std::endl;
        if (isRootProcess()) std::cout << s.str();
    }
    void showLocal(const std::string &descr) { show(descr); }

    // ---- coherence (public so containers of other element types can use them) ----
    void ensure_device() {
        if (!dev_valid_ && localPartition) {
            check_status(msl_upload(d_, localPartition, bytes()), "updateDevice");
            dev_valid_ = true;
        }
    }
    void ensure_host() {
        if (!n) return;
        ensure_mirror();
        if (!host_valid_) {
            check_status(msl_download(localPartition, d_, bytes()), "updateHost");
            host_valid_ = true;
        }
    }
    void device_written() {
        dev_valid_ = true;
        host_valid_ = false;
    }
    void host_written() {
        host_valid_ = true;
        dev_valid_ = false;
    }

   protected:
    long n = 0;
    T *d_ = nullptr;
    bool dev_valid_ = true, host_valid_ = false;

    size_t bytes() const { return (size_t)n * sizeof(T); }
    void allocate() {
        if (Muesli::proc_entrance == UNDEFINED) throws(detail::MissingInitializationException());
        if (n > 0) check_status(msl_alloc((void **)&d_, bytes()), "DS allocation");
        dev_valid_ = true;
        host_valid_ = false;
    }
    void ensure_mirror() {
        if (!localPartition && n) {
            if (cudaMallocHost((void **)&localPartition, bytes()) != cudaSuccess) {
                localPartition = nullptr;
                check_status(MSL_ERR_OUT_OF_MEMORY, "host mirror allocation");
            }
        }
    }
    void copy_from(const DS &o) {
        if (!n) return;
        const_cast<DS &>(o).ensure_device();
        check_status(msl_copy(d_, o.d_, bytes()), "copy");
        device_written();
    }
    void release() {
        if (d_) msl_free(d_);
        if (localPartition) {
            cudaStreamSynchronize(stream());
            cudaFreeHost(localPartition);
        }
        d_ = nullptr;
        localPartition = nullptr;
    }
    void steal(DS &o) {
        n = o.n;
        d_ = o.d_;
        localPartition = o.localPartition;
        dev_valid_ = o.dev_valid_;
        host_valid_ = o.host_valid_;
        o.n = 0;
        o.d_ = nullptr;
        o.localPartition = nullptr;
    }
};

}  // namespace msl
