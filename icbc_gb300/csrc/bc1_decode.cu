// bc1_decode.cu -- decode_bc1 / evaluate_bc1_error and the reference's
// decode_bc3 / evaluate_bc3_error over many blocks.
#include <cuda_runtime.h>

#include "bc1_kernels.h"

namespace icbc_gpu {

// decode_bc1 (icbc.h:2915-2927), one thread per block.
__global__ void k_decode(const uint2 *blocks, uint4 *rgba, int64_t n, int decoder) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint2 v = blocks[b];
    const Pal32 p = palette32(v.x & 0xffff, v.x >> 16, decoder);
    const bool four = (v.x & 0xffff) > (v.x >> 16);
    uint32_t pk[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t a = (i == 3 && !four) ? 0u : 255u;
        pk[i] = (uint32_t)p.r[i] | ((uint32_t)p.g[i] << 8) | ((uint32_t)p.b[i] << 16) | (a << 24);
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
        uint32_t q[4];
#pragma unroll
        for (int x = 0; x < 4; x++) q[x] = pk[(v.y >> (2 * (4 * r + x))) & 3];
        rgba[4 * b + r] = make_uint4(q[0], q[1], q[2], q[3]);
    }
}

// evaluate_bc1_error (icbc.h:3030-3046): integer squared error per texel,
// accumulated as float in texel order.
__global__ void k_evaluate(const uint4 *rgba, const uint2 *blocks, float *errors, int64_t n, int decoder) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint2 v = blocks[b];
    const Pal32 p = palette32(v.x & 0xffff, v.x >> 16, decoder);
    float error = 0.0f;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const uint4 q = rgba[4 * b + r];
        const uint32_t px[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int x = 0; x < 4; x++) {
            const int i = (v.y >> (2 * (4 * r + x))) & 3;
            const int dr = p.r[i] - (int)(px[x] & 255), dg = p.g[i] - (int)((px[x] >> 8) & 255),
                      db = p.b[i] - (int)((px[x] >> 16) & 255);
            error += (float)(dr * dr + dg * dg + db * db);
        }
    }
    errors[b] = error;
}

// decode_bc3 (icbc.h:2929-2947): a 16-byte block is the BC4 alpha half
// (alpha0, alpha1, 6 index bytes) and a BC1 block.  The colour palette is
// always the 4-colour form; the reference's alpha index is always 0, so every
// texel takes alpha0.  One thread per block.
__global__ void k_decode_bc3(const uint4 *blocks, uint4 *rgba, int64_t n, int decoder) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint4 v = blocks[b];
    const Pal32 p = palette32_form(v.z & 0xffff, v.z >> 16, decoder, true);
    const uint32_t a = (v.x & 255u) << 24;
    uint32_t pk[4];
#pragma unroll
    for (int i = 0; i < 4; i++) pk[i] = (uint32_t)p.r[i] | ((uint32_t)p.g[i] << 8) | ((uint32_t)p.b[i] << 16) | a;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        uint32_t q[4];
#pragma unroll
        for (int x = 0; x < 4; x++) q[x] = pk[(v.w >> (2 * (4 * r + x))) & 3];
        rgba[4 * b + r] = make_uint4(q[0], q[1], q[2], q[3]);
    }
}

// evaluate_bc3_error (icbc.h:3048-3071): per texel in order, the integer
// colour error (scaled by alpha / 255.0f when alpha_blend), then the squared
// difference of alpha0 and the texel's alpha, accumulated as float.
__global__ void k_evaluate_bc3(const uint4 *rgba, const uint4 *blocks, float *errors, int64_t n, int alpha_blend,
                               int decoder) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint4 v = blocks[b];
    const Pal32 p = palette32_form(v.z & 0xffff, v.z >> 16, decoder, true);
    const int alpha0 = (int)(v.x & 255u);
    float error = 0.0f;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const uint4 q = rgba[4 * b + r];
        const uint32_t px[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int x = 0; x < 4; x++) {
            const int i = (v.w >> (2 * (4 * r + x))) & 3;
            const int dr = p.r[i] - (int)(px[x] & 255), dg = p.g[i] - (int)((px[x] >> 8) & 255),
                      db = p.b[i] - (int)((px[x] >> 16) & 255), ta = (int)(px[x] >> 24);
            const float scale = alpha_blend ? __fdiv_rn((float)ta * 1.0f, 255.0f) : 1.0f;
            error += scale * (float)(dr * dr + dg * dg + db * db);
            error += (float)((alpha0 - ta) * (alpha0 - ta));
        }
    }
    errors[b] = error;
}

cudaError_t launch_decode_bc3(const void *blocks, void *rgba, int64_t n, int decoder, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    k_decode_bc3<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(
        reinterpret_cast<const uint4 *>(blocks), reinterpret_cast<uint4 *>(rgba), n, decoder);
    return cudaGetLastError();
}

cudaError_t launch_evaluate_bc3(const void *rgba, const void *blocks, float *errors, int64_t n, int alpha_blend,
                                int decoder, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    k_evaluate_bc3<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(
        reinterpret_cast<const uint4 *>(rgba), reinterpret_cast<const uint4 *>(blocks), errors, n, alpha_blend,
        decoder);
    return cudaGetLastError();
}

cudaError_t launch_decode(const void *blocks, void *rgba, int64_t n, int decoder, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    k_decode<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(
        reinterpret_cast<const uint2 *>(blocks), reinterpret_cast<uint4 *>(rgba), n, decoder);
    return cudaGetLastError();
}

cudaError_t launch_evaluate(const void *rgba, const void *blocks, float *errors, int64_t n, int decoder,
                            cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    k_evaluate<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(
        reinterpret_cast<const uint4 *>(rgba), reinterpret_cast<const uint2 *>(blocks), errors, n, decoder);
    return cudaGetLastError();
}

}  // namespace icbc_gpu
