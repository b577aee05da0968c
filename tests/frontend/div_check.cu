// Exhaustive check of msl::gpu::div6_rn against IEEE division (__fdiv_rn) over
// all 2^32 float bit patterns. NaN results compare equal to NaN results.
#include <cstdint>

#include "detail/msl_device.cuh"

__global__ void div6_check_kernel(unsigned long long *mismatches, unsigned *first_bad) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < (1ull << 32); i += stride) {
        const float x = __uint_as_float((unsigned)i);
        const float a = msl::gpu::div6_rn(x), b = __fdiv_rn(x, 6.0f);
        const bool same = (__float_as_uint(a) == __float_as_uint(b)) || (a != a && b != b);
        if (!same) {
            local++;
            atomicMin(first_bad, (unsigned)i);
        }
    }
    if (local) atomicAdd(mismatches, local);
}

extern "C" int div6_exhaustive(unsigned long long *mismatches_out, unsigned *first_bad_out) {
    unsigned long long *m;
    unsigned *f;
    if (cudaMalloc(&m, sizeof(*m)) != cudaSuccess || cudaMalloc(&f, sizeof(*f)) != cudaSuccess) return 1;
    cudaMemset(m, 0, sizeof(*m));
    cudaMemset(f, 0xff, sizeof(*f));
    div6_check_kernel<<<152 * 8, 256>>>(m, f);
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(mismatches_out, m, sizeof(*m), cudaMemcpyDeviceToHost);
    cudaMemcpy(first_bad_out, f, sizeof(*f), cudaMemcpyDeviceToHost);
    cudaFree(m);
    cudaFree(f);
    return 0;
}
