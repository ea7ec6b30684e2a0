// Exhaustive and sampled checks of rcp_bounded and div_bounded against the
// IEEE division, compiled by tests/test_gpu_rcp.py with the encoder's flags
// (-prec-div=true, -ftz=false).
//   rcp_check rcp LO_BITS HI_BITS   every float bit pattern in [LO_BITS, HI_BITS] and its negation
//   rcp_check div LO_BITS HI_BITS   every b in [LO_BITS, HI_BITS] with 16 dividends a: 0, seven
//                                   floats spread over the bit patterns of [2^-24, 64], eight
//                                   uniform in [0, 64)
// Prints "<mismatches> <first bad bits>".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>

#include "bc1_device.cuh"

using namespace icbc_gpu;

__device__ __forceinline__ uint32_t mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__global__ void k_rcp(uint32_t lo, uint32_t n, unsigned long long *bad, unsigned int *first) {
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

__global__ void k_div(uint32_t lo, uint32_t n, unsigned long long *bad, unsigned int *first) {
    const uint32_t top = 0x42800000u;  // 64.0f
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float b = __uint_as_float(lo + i);
        for (uint32_t k = 0; k < 16; k++) {
            const uint32_t r = mix((lo + i) * 16u + k);
            const uint32_t low = 0x33800000u;  // 2^-24
            const float a = k == 7  ? 0.0f
                            : k < 7 ? __uint_as_float(low + r % (top - low + 1))
                                    : (float)(r >> 8) * (64.0f / 16777216.0f);
            const float q = div_bounded(a, b), e = a / b;
            if (__float_as_uint(q) != __float_as_uint(e)) {
                atomicAdd(bad, 1ull);
                atomicMin(first, lo + i);
            }
        }
    }
}

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    const bool div = strcmp(argv[1], "div") == 0;
    const uint32_t lo = (uint32_t)strtoul(argv[2], nullptr, 0), hi = (uint32_t)strtoul(argv[3], nullptr, 0);
    if (hi < lo || hi >= 0x80000000u) return 2;
    unsigned long long *bad;
    unsigned int *first;
    if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess || cudaMalloc(&first, sizeof(*first)) != cudaSuccess) return 3;
    cudaMemset(bad, 0, sizeof(*bad));
    cudaMemset(first, 0xff, sizeof(*first));
    if (div) k_div<<<152 * 8, 256>>>(lo, hi - lo + 1, bad, first);
    else k_rcp<<<152 * 8, 256>>>(lo, hi - lo + 1, bad, first);
    unsigned long long hb = 0;
    unsigned int hf = 0;
    if (cudaMemcpy(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    if (cudaMemcpy(&hf, first, sizeof(hf), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    printf("%llu 0x%08x\n", hb, hf);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 3;
}
