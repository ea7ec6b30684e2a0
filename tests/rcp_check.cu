// Exhaustive check of rcp_bounded against the IEEE division, compiled by
// tests/test_gpu_rcp.py with the encoder's flags (-prec-div=true, -ftz=false).
// Usage: rcp_check LO_BITS HI_BITS -> prints "<mismatches> <first bad bits>"
// over every float bit pattern in [LO_BITS, HI_BITS] and its negation.
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

#include "bc1_device.cuh"

using namespace icbc_gpu;

__global__ void k_check(uint32_t lo, uint32_t n, unsigned long long *bad, unsigned int *first) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (uint32_t sign = 0; sign < 2; sign++) {
            const uint32_t u = (lo + i) | (sign << 31);
            const float d = __uint_as_float(u);
            const float a = rcp_bounded(d), b = 1.0f / d;
            if (__float_as_uint(a) != __float_as_uint(b)) {
                atomicAdd(bad, 1ull);
                atomicMin(first, u);
            }
        }
    }
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    const uint32_t lo = (uint32_t)strtoul(argv[1], nullptr, 0), hi = (uint32_t)strtoul(argv[2], nullptr, 0);
    if (hi < lo || hi >= 0x80000000u) return 2;
    unsigned long long *bad;
    unsigned int *first;
    if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess || cudaMalloc(&first, sizeof(*first)) != cudaSuccess) return 3;
    cudaMemset(bad, 0, sizeof(*bad));
    cudaMemset(first, 0xff, sizeof(*first));
    k_check<<<152 * 8, 256>>>(lo, hi - lo + 1, bad, first);
    unsigned long long hb = 0;
    unsigned int hf = 0;
    if (cudaMemcpy(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    if (cudaMemcpy(&hf, first, sizeof(hf), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    printf("%llu 0x%08x\n", hb, hf);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 3;
}
