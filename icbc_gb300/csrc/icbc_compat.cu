// icbc_compat.cu -- icbc's C++ entry points (icbc.h:10-52) on the GPU.
//
// Each call stages one block in per-thread device buffers, runs the block
// kernels through the C ABI on a per-thread stream and copies the result
// back.  Semantics follow the reference: compress_bc1 uses the decoder set by
// init and leaves the output untouched for a level outside 0..9 (returning
// FLT_MAX, the error the reference's empty option set yields); any other
// failure is reported as a NaN error, since these signatures carry no status.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstring>

#include "../../include/icbc_compat.hpp"
#include "../../include/icbc_gpu.h"

namespace {

struct ThreadState {
    cudaStream_t stream = nullptr;
    float *d_colors = nullptr;   // 64 floats
    float *d_weights = nullptr;  // 16 floats
    uint8_t *d_block = nullptr;  // 16 bytes (a BC1 or BC3 block)
    float *d_error = nullptr;
    uint8_t *d_rgba = nullptr;   // 64 bytes
    bool ok = false;

    bool ready() {
        if (ok) return true;
        if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (cudaMalloc(&d_colors, 64 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&d_weights, 16 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&d_block, 16) != cudaSuccess) return false;
        if (cudaMalloc(&d_error, 16) != cudaSuccess) return false;
        if (cudaMalloc(&d_rgba, 64) != cudaSuccess) return false;
        ok = true;
        return true;
    }
    ~ThreadState() {
        if (stream) cudaStreamDestroy(stream);
        cudaFree(d_colors);
        cudaFree(d_weights);
        cudaFree(d_block);
        cudaFree(d_error);
        cudaFree(d_rgba);
    }
};

thread_local ThreadState t_state;

}  // namespace

namespace icbc {

void init(Decoder decoder) { icbc_gpu_init((int)decoder); }

float compress_bc1(Quality level, const float *input_colors, const float *input_weights, const float color_weights[3],
                   bool three_color_mode, bool three_color_black, void *output) {
    if ((int)level < 0 || (int)level > 9) return FLT_MAX;
    ThreadState &T = t_state;
    if (!T.ready()) return NAN;
    cudaError_t e = cudaMemcpyAsync(T.d_colors, input_colors, 64 * sizeof(float), cudaMemcpyHostToDevice, T.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(T.d_weights, input_weights, 16 * sizeof(float), cudaMemcpyHostToDevice, T.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T.d_block, output, 8, cudaMemcpyHostToDevice, T.stream);
    if (e != cudaSuccess) return NAN;
    if (icbc_gpu_compress_bc1_blocks((int)level, T.d_colors, T.d_weights, color_weights, three_color_mode,
                                     three_color_black, ICBC_GPU_DECODER_DEFAULT, T.d_block, T.d_error, 1,
                                     T.stream) != ICBC_GPU_OK)
        return NAN;
    float error = NAN;
    e = cudaMemcpyAsync(output, T.d_block, 8, cudaMemcpyDeviceToHost, T.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&error, T.d_error, sizeof(float), cudaMemcpyDeviceToHost, T.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(T.stream);
    return e == cudaSuccess ? error : NAN;
}

void decode_bc1(const void *block, unsigned char rgba_block[16 * 4], Decoder decoder) {
    ThreadState &T = t_state;
    if (!T.ready()) return;
    if (cudaMemcpyAsync(T.d_block, block, 8, cudaMemcpyHostToDevice, T.stream) != cudaSuccess) return;
    if (icbc_gpu_decode_bc1(T.d_block, T.d_rgba, 1, (int)decoder, T.stream) != ICBC_GPU_OK) return;
    if (cudaMemcpyAsync(rgba_block, T.d_rgba, 64, cudaMemcpyDeviceToHost, T.stream) != cudaSuccess) return;
    cudaStreamSynchronize(T.stream);
}

float evaluate_bc1_error(const unsigned char rgba_block[16 * 4], const void *block, Decoder decoder) {
    ThreadState &T = t_state;
    if (!T.ready()) return NAN;
    cudaError_t e = cudaMemcpyAsync(T.d_block, block, 8, cudaMemcpyHostToDevice, T.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T.d_rgba, rgba_block, 64, cudaMemcpyHostToDevice, T.stream);
    if (e != cudaSuccess) return NAN;
    if (icbc_gpu_evaluate_bc1_error(T.d_rgba, T.d_block, T.d_error, 1, (int)decoder, T.stream) != ICBC_GPU_OK)
        return NAN;
    float error = NAN;
    e = cudaMemcpyAsync(&error, T.d_error, sizeof(float), cudaMemcpyDeviceToHost, T.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(T.stream);
    return e == cudaSuccess ? error : NAN;
}

void decode_bc3(const void *block, unsigned char rgba_block[16 * 4], Decoder decoder) {
    ThreadState &T = t_state;
    if (!T.ready()) return;
    if (cudaMemcpyAsync(T.d_block, block, 16, cudaMemcpyHostToDevice, T.stream) != cudaSuccess) return;
    if (icbc_gpu_decode_bc3(T.d_block, T.d_rgba, 1, (int)decoder, T.stream) != ICBC_GPU_OK) return;
    if (cudaMemcpyAsync(rgba_block, T.d_rgba, 64, cudaMemcpyDeviceToHost, T.stream) != cudaSuccess) return;
    cudaStreamSynchronize(T.stream);
}

float evaluate_bc3_error(const unsigned char rgba_block[16 * 4], const void *block, bool alpha_blend,
                         Decoder decoder) {
    ThreadState &T = t_state;
    if (!T.ready()) return NAN;
    cudaError_t e = cudaMemcpyAsync(T.d_block, block, 16, cudaMemcpyHostToDevice, T.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T.d_rgba, rgba_block, 64, cudaMemcpyHostToDevice, T.stream);
    if (e != cudaSuccess) return NAN;
    if (icbc_gpu_evaluate_bc3_error(T.d_rgba, T.d_block, T.d_error, 1, alpha_blend, (int)decoder, T.stream) !=
        ICBC_GPU_OK)
        return NAN;
    float error = NAN;
    e = cudaMemcpyAsync(&error, T.d_error, sizeof(float), cudaMemcpyDeviceToHost, T.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(T.stream);
    return e == cudaSuccess ? error : NAN;
}

// The reference has no BC3 encoder: compress_bc3 returns 0 and leaves the
// output untouched (icbc.h:3850-3853).
float compress_bc3(Quality, const float *, const float *, const float *, bool, void *) { return 0.0f; }

}  // namespace icbc
