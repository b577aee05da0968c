// msl_fold_noalloc: the fold skeleton for callers that must not allocate.
//
// Some callers cannot call cudaMalloc: real-time loops that must never hit the
// implicit device synchronisation cudaMalloc/cudaFree can cause, and plugins
// running inside a host whose device memory is entirely owned by that host's
// own allocator. msl_fold needs msl_init, which
// allocates the fold scratch; this variant needs nothing but the caller's
// input, the caller's one-element device result and a stream.
//
// Its scratch -- one partial value and one flag per CTA, and the CTAs' ticket
// counter -- lives in the static device array g_fold_noalloc_scratch below,
// which every GPU that loads the library holds until the process exits. All
// calls share it: two calls that overlap on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.
#include <mutex>

#include "../include/detail/msl_fold.cuh"
#include "msl_internal.h"

using namespace msl;
using namespace msl::gpu;

namespace {

// Capacity: 2048 CTA partials of up to 16 bytes, their flags and the ticket.
constexpr int kNoAllocSlots = 2048;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocSlots * 16 + (size_t)kNoAllocSlots * 4 + 256;
// Each thread folds at most this many elements (the rounding bound of a float
// sum grows with the longest serial chain), so a call covers at most
// kNoAllocSlots * kFoldThreads * kMaxPerThread = 2^30 elements.
constexpr size_t kMaxPerThread = 1024;
constexpr size_t kNoAllocMaxElems = (size_t)kNoAllocSlots * kFoldThreads * kMaxPerThread;

static __device__ __align__(256) unsigned char g_fold_noalloc_scratch[kNoAllocBytes];

// The device address of the static array is looked up on every call, with the
// caller's device and context current: a module loaded into another context
// (a plugin host's own context, or the primary context rebuilt after
// cudaDeviceReset) has its own copy of the array at another address, so an
// address cached from an earlier call could point at memory this context does
// not own. The lookup allocates nothing. The SM count is a property of the
// device and is cached per device ordinal.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
int g_sm_count[kMaxDevices];

int setup_call(int dev, void **base, int *sms) {
    if (dev < 0 || dev >= kMaxDevices) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_noalloc: device %d", dev);
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_fold_noalloc_scratch);
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_fold_noalloc: cudaGetSymbolAddress");
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_sm_count[dev]) {
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return rt::cuda_fail(e, "msl_fold_noalloc: SM count");
        g_sm_count[dev] = n;
    }
    *base = p;
    *sms = g_sm_count[dev];
    return MSL_OK;
}

template <typename T, int OP> struct NoAllocOp {
    __device__ __forceinline__ T operator()(T a, T b) const {
        if constexpr (OP == MSL_FOLD_SUM) return Arith<T>::add(a, b);
        else if constexpr (OP == MSL_FOLD_MAX) return a > b ? a : b;
        else return a < b ? a : b;
    }
};

template <typename T, int OP> cudaError_t launch(const void *in, size_t n, void *result, char *base, int sms,
                                                 cudaStream_t st) {
    constexpr int V = vec_width1<T>();
    const bool vec = aligned_to(in, V * sizeof(T));
    const size_t units = vec ? n / V : n;
    // The usual one-wave grid, raised when needed so that no thread folds
    // more than kMaxPerThread elements; never more CTAs than partial slots.
    constexpr int UV = fold_unroll<T, V>(), U1 = fold_unroll<T, 1>();
    size_t blocks = fold_blocks(units, sms, 2, vec ? UV : U1);
    const size_t need = (n + (size_t)kFoldThreads * kMaxPerThread - 1) / ((size_t)kFoldThreads * kMaxPerThread);
    if (blocks < need) blocks = need;
    if (blocks > (size_t)kNoAllocSlots) blocks = kNoAllocSlots;
    T *partials = reinterpret_cast<T *>(base);
    int *have = reinterpret_cast<int *>(base + (size_t)kNoAllocSlots * 16);
    char *tail = base + (size_t)kNoAllocSlots * 20;
    unsigned *ticket = reinterpret_cast<unsigned *>(tail);
    int *result_have = reinterpret_cast<int *>(tail + 128);
    // The ticket must start at zero (a previous call leaves it at zero, but a
    // call interrupted by an error would not).
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (vec) {
        FoldSrcArray<T, V> src{(const T *)in};
        fold_kernel<V, UV><<<(unsigned)blocks, kFoldThreads, 0, st>>>(src, n, NoAllocOp<T, OP>{}, partials, have,
                                                                     ticket, (T *)result, result_have);
    } else {
        FoldSrcArray<T, 1> src{(const T *)in};
        fold_kernel<1, U1><<<(unsigned)blocks, kFoldThreads, 0, st>>>(src, n, NoAllocOp<T, OP>{}, partials, have,
                                                                     ticket, (T *)result, result_have);
    }
    return cudaGetLastError();
}

template <typename T> cudaError_t dispatch(int op, const void *in, size_t n, void *result, char *base, int sms,
                                           cudaStream_t st) {
    switch (op) {
        case MSL_FOLD_SUM: return launch<T, MSL_FOLD_SUM>(in, n, result, base, sms, st);
        case MSL_FOLD_MAX: return launch<T, MSL_FOLD_MAX>(in, n, result, base, sms, st);
        default: return launch<T, MSL_FOLD_MIN>(in, n, result, base, sms, st);
    }
}

}  // namespace

extern "C" {

int msl_fold_noalloc(int dtype, int op, const void *in, size_t n, void *result_device, void *stream) {
    if (n == 0) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_noalloc: empty input has no fold");
    if (n > kNoAllocMaxElems)
        return rt::fail(MSL_ERR_SIZE_MISMATCH,
                        "msl_fold_noalloc: %zu elements exceed the %zu-element capacity of its static scratch "
                        "(%d partial slots x %d threads x %zu elements per thread)",
                        n, kNoAllocMaxElems, kNoAllocSlots, kFoldThreads, kMaxPerThread);
    if (!in || !result_device) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_noalloc: NULL pointer");
    if (op < MSL_FOLD_SUM || op > MSL_FOLD_MIN) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_noalloc: op %d", op);
    if (dtype != MSL_F32 && dtype != MSL_F64 && dtype != MSL_I32)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_fold_noalloc: dtype %d", dtype);
    int dev = 0;
    MSL_TRY_CUDA(cudaGetDevice(&dev), "msl_fold_noalloc: cudaGetDevice");
    void *base = nullptr;
    int sms = 0;
    if (int e = setup_call(dev, &base, &sms)) return e;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    switch (dtype) {
        case MSL_F32: e = dispatch<float>(op, in, n, result_device, (char *)base, sms, st); break;
        case MSL_F64: e = dispatch<double>(op, in, n, result_device, (char *)base, sms, st); break;
        default: e = dispatch<int32_t>(op, in, n, result_device, (char *)base, sms, st); break;
    }
    if (e != cudaSuccess) return rt::cuda_fail(e, "msl_fold_noalloc");
    rt::count_launch();
    return MSL_OK;
}

}  // extern "C"
