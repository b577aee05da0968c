// Runtime and partition storage of libmsl_gb300.so: context, stream, errors,
// device buffers, host<->device transfers, the device copy kernel and fill.
//
// Reference counterparts: msl::initSkeletons / terminateSkeletons /
// syncStreams (src/muesli.cpp:63-223); DS<T> storage and transfers
// (src/ds.cpp:215-239, 290-305, 442-591); copyKernel (src/copy_kernel.cu:33-43).
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "../include/detail/msl_elementwise.cuh"
#include "msl_internal.h"

namespace msl {
namespace rt {

namespace {
thread_local std::string g_last_error;
}

Context &ctx() {
    static Context c;
    return c;
}

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    int code = (e == cudaErrorMemoryAllocation) ? MSL_ERR_OUT_OF_MEMORY : MSL_ERR_CUDA;
    return fail(code, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

int require_init() {
    if (!ctx().initialised) return fail(MSL_ERR_NOT_INITIALIZED, "msl_init has not been called");
    return MSL_OK;
}

int check_device_errors(const char *what) {
    Context &c = ctx();
    MSL_TRY_CUDA(cudaMemcpyAsync(c.host_result, c.err_word, sizeof(unsigned), cudaMemcpyDeviceToHost, c.stream),
                 what);
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), what);
    unsigned bits = *(volatile unsigned *)c.host_result;
    if (bits) {
        MSL_TRY_CUDA(cudaMemsetAsync(c.err_word, 0, sizeof(unsigned), c.stream), what);
        MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), what);
        if (bits & gpu::kErrBarrierTimeout)
            return fail(MSL_ERR_TIMEOUT, "%s: a kernel gave up waiting on a TMA/mbarrier phase", what);
        return fail(MSL_ERR_CUDA, "%s: device error bits 0x%x", what, bits);
    }
    return MSL_OK;
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case MSL_F32: case MSL_I32: return 4;
        case MSL_F64: return 8;
        case MSL_BF16: return 2;
    }
    return 0;
}

}  // namespace rt
}  // namespace msl

namespace {
// Allocations still allowed before injected failures start (-1: no injection).
std::atomic<long long> g_alloc_allowance{-1};

// One CTA waits on an mbarrier through the library's bounded poll; with
// `arrive` thread 0 completes the phase first, without it nothing ever does.
__global__ void wait_selftest_kernel(unsigned *err, unsigned polls, bool arrive) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        msl::gpu::mbar_init(&bar, 1);
        msl::gpu::fence_barrier_init();
    }
    __syncthreads();
    if (arrive && threadIdx.x == 0) msl::gpu::mbar_arrive(&bar);
    if (!msl::gpu::mbar_poll(&bar, 0, polls)) msl::gpu::report_error(err, msl::gpu::kErrBarrierTimeout);
}
}  // namespace

bool msl::rt::alloc_fault() {
    long long a = g_alloc_allowance.load();
    while (a > 0 && !g_alloc_allowance.compare_exchange_weak(a, a - 1)) {
    }
    return a == 0;
}

using namespace msl;
using msl::rt::ctx;

namespace {

constexpr size_t kScratchBytes = gpu::kFoldScratchBytes + 256;

template <typename T> __global__ void fill_kernel(T *p, size_t n, T v) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

struct CopyOp {
    template <class S, typename T> __device__ __forceinline__ T operator()(S, T x) const { return x; }
};

template <typename T> int fill_t(void *dst, size_t n, T v) {
    auto &c = ctx();
    if (n == 0) return MSL_OK;
    // 16-byte stores when possible: fill a vector-typed view.
    constexpr int V = 16 / sizeof(T);
    if (((uintptr_t)dst % 16) == 0 && V > 1) {
        gpu::Vec<T, V> vv;
        for (int k = 0; k < V; k++) vv.v[k] = v;
        size_t nv = n / V;
        if (nv) {
            fill_kernel<gpu::Vec<T, V>><<<gpu::ew_blocks(nv, c.sm_count), gpu::kEwThreads, 0, c.stream>>>(
                (gpu::Vec<T, V> *)dst, nv, vv);
            rt::count_launch();
        }
        size_t rest = n - nv * V;
        if (rest) {
            fill_kernel<T><<<1, 32, 0, c.stream>>>((T *)dst + nv * V, rest, v);
            rt::count_launch();
        }
    } else {
        fill_kernel<T><<<gpu::ew_blocks(n, c.sm_count), gpu::kEwThreads, 0, c.stream>>>((T *)dst, n, v);
        rt::count_launch();
    }
    MSL_TRY_CUDA(cudaGetLastError(), "msl_fill");
    return MSL_OK;
}

}  // namespace

extern "C" {

int msl_init(int device) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (c.initialised) {
        if (c.device == device) return MSL_OK;
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_init: already bound to device %d", c.device);
    }
    int count = 0;
    MSL_TRY_CUDA(cudaGetDeviceCount(&count), "msl_init: cudaGetDeviceCount");
    if (device < 0 || device >= count)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_init: device %d out of range (%d devices)", device, count);
    MSL_TRY_CUDA(cudaSetDevice(device), "msl_init: cudaSetDevice");
    cudaDeviceProp prop;
    MSL_TRY_CUDA(cudaGetDeviceProperties(&prop, device), "msl_init: cudaGetDeviceProperties");
    if (prop.major < 9)
        return rt::fail(MSL_ERR_UNSUPPORTED_DEVICE, "msl_init: device %d is sm_%d%d; TMA kernels need sm_90 or newer",
                        device, prop.major, prop.minor);
    c.sm_count = prop.multiProcessorCount;
    MSL_TRY_CUDA(cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking), "msl_init: stream");
    c.stream = c.own_stream;
    MSL_TRY_CUDA(cudaMalloc(&c.scratch, kScratchBytes), "msl_init: scratch");
    MSL_TRY_CUDA(cudaMemset(c.scratch, 0, kScratchBytes), "msl_init: scratch clear");
    c.fold = gpu::carve_fold_scratch(c.scratch);
    c.err_word = (unsigned *)((char *)c.scratch + gpu::kFoldScratchBytes);
    c.resid = (unsigned long long *)((char *)c.scratch + gpu::kFoldScratchBytes + 64);
    MSL_TRY_CUDA(cudaMallocHost(&c.host_result, 256), "msl_init: pinned result slot");
    MSL_TRY_CUDA(cudaHostAlloc(&c.host_fold, 256, cudaHostAllocMapped), "msl_init: mapped fold slot");
    MSL_TRY_CUDA(cudaHostGetDevicePointer(&c.host_fold_dev, c.host_fold, 0), "msl_init: mapped fold slot");
    c.device = device;
    c.launches = 0;
    c.initialised = true;
    return MSL_OK;
}

int msl_terminate(void) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (!c.initialised) return MSL_OK;
    cudaStreamSynchronize(c.stream);
    cudaFree(c.scratch);
    cudaFreeHost(c.host_result);
    cudaFreeHost(c.host_fold);
    cudaStreamDestroy(c.own_stream);
    c.scratch = nullptr;
    c.host_result = nullptr;
    c.host_fold = c.host_fold_dev = nullptr;
    c.own_stream = c.stream = nullptr;
    c.initialised = false;
    c.device = -1;
    return MSL_OK;
}

int msl_sync(void) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_sync");
    return rt::check_device_errors("msl_sync");
}

const char *msl_last_error_string(void) {
    return msl::rt::g_last_error.c_str();
}

int msl_get_stream(void **stream) {
    auto &c = ctx();
    if (int e = rt::require_init()) return e;
    if (!stream) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_get_stream: NULL");
    *stream = (void *)c.stream;
    return MSL_OK;
}

int msl_set_stream(void *stream) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    c.stream = stream ? (cudaStream_t)stream : c.own_stream;
    return MSL_OK;
}

int msl_device_info(int *sm_count, size_t *free_bytes, size_t *total_bytes) {
    auto &c = ctx();
    if (int e = rt::require_init()) return e;
    size_t f = 0, t = 0;
    MSL_TRY_CUDA(cudaMemGetInfo(&f, &t), "msl_device_info");
    if (sm_count) *sm_count = c.sm_count;
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return MSL_OK;
}

int msl_set_wait_limit(unsigned polls) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    MSL_TRY_CUDA(cudaMemcpyAsync(c.err_word + 1, &polls, sizeof polls, cudaMemcpyHostToDevice, c.stream),
                 "msl_set_wait_limit");
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_set_wait_limit");
    return MSL_OK;
}

int msl_wait_selftest(unsigned polls, int arrive) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (polls == 0) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_wait_selftest: polls must be >= 1");
    wait_selftest_kernel<<<1, 64, 0, c.stream>>>(c.err_word, polls, arrive != 0);
    MSL_TRY_CUDA(cudaGetLastError(), "msl_wait_selftest");
    rt::count_launch();
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_wait_selftest");
    return rt::check_device_errors("msl_wait_selftest");
}

int msl_debug_fail_allocs(long long after) {
    g_alloc_allowance.store(after < 0 ? -1 : after);
    return MSL_OK;
}

int msl_launch_count(unsigned long long *count) {
    if (!count) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_launch_count: NULL");
    *count = ctx().launches.load();
    return MSL_OK;
}

int msl_alloc(void **dptr, size_t bytes) {
    if (!dptr) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_alloc: NULL result pointer");
    *dptr = nullptr;
    if (bytes && rt::alloc_fault())
        return rt::fail(MSL_ERR_OUT_OF_MEMORY, "msl_alloc: %zu bytes: allocation failure injected", bytes);
    if (int e = rt::require_init()) return e;
    if (bytes == 0) return MSL_OK;
    MSL_TRY_CUDA(cudaMalloc(dptr, bytes), "msl_alloc");
    return MSL_OK;
}

int msl_free(void *dptr) {
    if (int e = rt::require_init()) return e;
    if (!dptr) return MSL_OK;
    MSL_TRY_CUDA(cudaStreamSynchronize(ctx().stream), "msl_free: sync");
    MSL_TRY_CUDA(cudaFree(dptr), "msl_free");
    return MSL_OK;
}

int msl_upload(void *dst, const void *src, size_t bytes) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (bytes == 0) return MSL_OK;
    if (!dst || !src) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_upload: NULL pointer");
    MSL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c.stream), "msl_upload");
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_upload: sync");
    return MSL_OK;
}

int msl_download(void *dst, const void *src, size_t bytes) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (bytes == 0) return MSL_OK;
    if (!dst || !src) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_download: NULL pointer");
    MSL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c.stream), "msl_download");
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_download: sync");
    return MSL_OK;
}

// Stream-ordered transfers: enqueued on `stream` (a cudaStream_t; NULL = the
// library stream) without waiting, so copies of one buffer can overlap
// kernels working on another. The caller orders them against its other work
// (events) and keeps the host buffer alive and unchanged until the copy is
// done; with pinned host memory the copy engines run them asynchronously.
int msl_upload_async(void *dst, const void *src, size_t bytes, void *stream) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (bytes == 0) return MSL_OK;
    if (!dst || !src) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_upload_async: NULL pointer");
    MSL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream ? (cudaStream_t)stream : c.stream),
                 "msl_upload_async");
    return MSL_OK;
}

int msl_download_async(void *dst, const void *src, size_t bytes, void *stream) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (bytes == 0) return MSL_OK;
    if (!dst || !src) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_download_async: NULL pointer");
    MSL_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream ? (cudaStream_t)stream : c.stream),
                 "msl_download_async");
    return MSL_OK;
}

int msl_copy(void *dst, const void *src, size_t bytes) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (bytes == 0) return MSL_OK;
    if (!dst || !src) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_copy: NULL pointer");
    cudaError_t e;
    if (((uintptr_t)dst | (uintptr_t)src | bytes) % 16 == 0)
        e = gpu::launch_map((uint4 *)dst, (const uint4 *)src, bytes / 16, gpu::IdxNone{}, CopyOp{}, c.stream,
                            c.sm_count);
    else
        e = gpu::launch_map((uint8_t *)dst, (const uint8_t *)src, bytes, gpu::IdxNone{}, CopyOp{}, c.stream,
                            c.sm_count);
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_copy");
    rt::count_launch();
    return MSL_OK;
}

int msl_fill(int dtype, void *dst, size_t n, double value) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (n && !dst) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fill: NULL pointer");
    switch (dtype) {
        case MSL_F32: return fill_t<float>(dst, n, (float)value);
        case MSL_F64: return fill_t<double>(dst, n, value);
        case MSL_I32: return fill_t<int32_t>(dst, n, (int32_t)(long long)value);
        case MSL_BF16: return fill_t<gpu::bf16s>(dst, n, gpu::f_to_bf16((float)value));
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fill: unknown dtype %d", dtype);
}

}  // extern "C"
