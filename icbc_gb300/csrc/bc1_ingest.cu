// bc1_ingest.cu -- the input side of the encoder on the device: 8-bit images
// of 1..4 channels expanded to RGBA8, and mip chains whose levels are encoded
// in one batch.
//
// The reference's test driver loads images with stbi_load(..., 4)
// (icbc_test.cpp:345), which expands grey to (g, g, g, 255), grey + alpha to
// (g, g, g, a) and RGB to (r, g, b, 255); k_expand_rgba8 does the same on the
// device so raw decoded pixels can be uploaded as they are.  The reference
// encodes one image; callers such as texture pipelines encode a mip chain,
// built here with a 2x2 box filter: level k + 1 has size
// max(1, w >> 1) x max(1, h >> 1), each channel (a + b + c + d + 2) >> 2 over
// source texels (2x, 2y) .. (2x + 1, 2y + 1), coordinates clamped to the
// source (a 1-texel-wide level repeats its column).  Both kernels move bytes:
// HBM-bound, one thread per output texel, coalesced 4-byte accesses.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/icbc_gpu.h"
#include "bc1_kernels.h"

namespace icbc_gpu {

__global__ void k_expand_rgba8(const uint8_t *src, int channels, int width, int64_t total, int64_t src_pitch,
                               uint8_t *dst, int64_t dst_pitch) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t y = i / width, x = i - y * width;
        const uint8_t *s = src + y * src_pitch + x * channels;
        uchar4 o;
        if (channels == 1) o = make_uchar4(s[0], s[0], s[0], 255);
        else if (channels == 2) o = make_uchar4(s[0], s[0], s[0], s[1]);
        else if (channels == 3) o = make_uchar4(s[0], s[1], s[2], 255);
        else o = make_uchar4(s[0], s[1], s[2], s[3]);
        *reinterpret_cast<uchar4 *>(dst + y * dst_pitch + 4 * x) = o;
    }
}

__global__ void k_mip_down(const uint8_t *src, int sw, int sh, int64_t sp, uint8_t *dst, int dw, int64_t total,
                           int64_t dp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t y = i / dw, x = i - y * dw;
        const int64_t x0 = 2 * x < sw ? 2 * x : sw - 1, x1 = 2 * x + 1 < sw ? 2 * x + 1 : sw - 1;
        const int64_t y0 = 2 * y < sh ? 2 * y : sh - 1, y1 = 2 * y + 1 < sh ? 2 * y + 1 : sh - 1;
        const uchar4 a = *reinterpret_cast<const uchar4 *>(src + y0 * sp + 4 * x0);
        const uchar4 b = *reinterpret_cast<const uchar4 *>(src + y0 * sp + 4 * x1);
        const uchar4 c = *reinterpret_cast<const uchar4 *>(src + y1 * sp + 4 * x0);
        const uchar4 d = *reinterpret_cast<const uchar4 *>(src + y1 * sp + 4 * x1);
        uchar4 o;
        o.x = (uint8_t)((a.x + b.x + c.x + d.x + 2) >> 2);
        o.y = (uint8_t)((a.y + b.y + c.y + d.y + 2) >> 2);
        o.z = (uint8_t)((a.z + b.z + c.z + d.z + 2) >> 2);
        o.w = (uint8_t)((a.w + b.w + c.w + d.w + 2) >> 2);
        *reinterpret_cast<uchar4 *>(dst + y * dp + 4 * x) = o;
    }
}

namespace {

int grid_of(int64_t total) {
    const int64_t g = (total + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)current_sm_count() * 32));
}

// Sizes of levels 0..levels-1 and the prefix of their block counts.
void layout(int32_t w, int32_t h, int32_t levels, std::vector<int32_t> &ws, std::vector<int32_t> &hs,
            std::vector<int64_t> &offsets) {
    ws.clear();
    hs.clear();
    offsets.assign(1, 0);
    for (int k = 0; k < levels; k++) {
        ws.push_back(w);
        hs.push_back(h);
        offsets.push_back(offsets.back() + (int64_t)((w + 3) / 4) * ((h + 3) / 4));
        w = std::max(1, w >> 1);
        h = std::max(1, h >> 1);
    }
}

}  // namespace
}  // namespace icbc_gpu

using namespace icbc_gpu;

extern "C" {

int icbc_gpu_expand_rgba8(const uint8_t *d_src, int32_t channels, int32_t width, int32_t height, int64_t src_pitch,
                          uint8_t *d_rgba, int64_t rgba_pitch, void *stream) {
    if (!d_src || !d_rgba || channels < 1 || channels > 4 || width < 1 || height < 1 ||
        src_pitch < (int64_t)width * channels || rgba_pitch < 4 * (int64_t)width)
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(d_rgba) & 3) || (rgba_pitch & 3)) return ICBC_GPU_ERR_MISALIGNED;
    const int64_t total = (int64_t)width * height;
    k_expand_rgba8<<<grid_of(total), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        d_src, channels, width, total, src_pitch, d_rgba, rgba_pitch);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ICBC_GPU_OK : ICBC_GPU_ERR_CUDA;
}

int icbc_gpu_mip_levels(int32_t width, int32_t height) {
    if (width < 1 || height < 1) return 0;
    int n = 1;
    while (width > 1 || height > 1) {
        width = std::max(1, width >> 1);
        height = std::max(1, height >> 1);
        n++;
    }
    return n;
}

int icbc_gpu_mip_layout(int32_t width, int32_t height, int32_t levels, int32_t *widths, int32_t *heights,
                        int64_t *block_offsets) {
    if (width < 1 || height < 1 || levels < 1 || levels > icbc_gpu_mip_levels(width, height))
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::vector<int32_t> ws, hs;
    std::vector<int64_t> off;
    layout(width, height, levels, ws, hs, off);
    for (int k = 0; k < levels; k++) {
        if (widths) widths[k] = ws[k];
        if (heights) heights[k] = hs[k];
    }
    if (block_offsets)
        for (int k = 0; k <= levels; k++) block_offsets[k] = off[k];
    return ICBC_GPU_OK;
}

int icbc_gpu_build_mips(const uint8_t *d_rgba, int32_t width, int32_t height, int64_t pitch, int32_t levels,
                        uint8_t *d_chain, void *stream) {
    if (!d_rgba || width < 1 || height < 1 || pitch < 4 * (int64_t)width || levels < 1 ||
        levels > icbc_gpu_mip_levels(width, height) || (levels > 1 && !d_chain))
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(d_rgba) & 3) || (pitch & 3) || (reinterpret_cast<uintptr_t>(d_chain) & 3))
        return ICBC_GPU_ERR_MISALIGNED;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint8_t *src = d_rgba;
    int sw = width, sh = height;
    int64_t sp = pitch;
    uint8_t *dst = d_chain;
    for (int k = 1; k < levels; k++) {
        const int dw = std::max(1, sw >> 1), dh = std::max(1, sh >> 1);
        const int64_t total = (int64_t)dw * dh;
        k_mip_down<<<grid_of(total), 256, 0, s>>>(src, sw, sh, sp, dst, dw, total, 4 * (int64_t)dw);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return ICBC_GPU_ERR_CUDA;
        src = dst;
        sw = dw;
        sh = dh;
        sp = 4 * (int64_t)dw;
        dst += 4 * total;
    }
    return ICBC_GPU_OK;
}

int icbc_gpu_compress_bc1_mips(const icbc_gpu_image *image, int32_t levels, void *stream) {
    if (!image || !image->out || levels < 1 || image->width < 1 || image->height < 1 ||
        levels > icbc_gpu_mip_levels(image->width, image->height) || image->weight_mode == ICBC_GPU_WEIGHTS_PLANE)
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::vector<int32_t> ws, hs;
    std::vector<int64_t> off;
    layout(image->width, image->height, levels, ws, hs, off);
    int64_t chain_bytes = 0;
    for (int k = 1; k < levels; k++) chain_bytes += 4 * (int64_t)ws[k] * hs[k];
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    void *chain = nullptr;
    if (chain_bytes) {
        const cudaError_t e = scratch_alloc(&chain, (size_t)chain_bytes, s);
        if (e != cudaSuccess) return ICBC_GPU_ERR_OUT_OF_MEMORY;
    }
    int st = icbc_gpu_build_mips(image->rgba, image->width, image->height, image->pitch, levels,
                                 static_cast<uint8_t *>(chain), stream);
    if (st == ICBC_GPU_OK) {
        std::vector<icbc_gpu_image> ims((size_t)levels, *image);
        const uint8_t *lv = static_cast<const uint8_t *>(chain);
        for (int k = 0; k < levels; k++) {
            icbc_gpu_image &m = ims[k];
            if (k > 0) {
                m.rgba = lv;
                m.width = ws[k];
                m.height = hs[k];
                m.pitch = 4 * (int64_t)ws[k];
                lv += 4 * (int64_t)ws[k] * hs[k];
            }
            m.out = static_cast<uint8_t *>(image->out) + 8 * off[k];
            m.errors = image->errors ? image->errors + off[k] : nullptr;
        }
        st = icbc_gpu_compress_bc1_images(ims.data(), levels, stream);
    }
    if (chain) {
        scratch_free(chain, s);
        if (cudaStreamSynchronize(s) != cudaSuccess && st == ICBC_GPU_OK) st = ICBC_GPU_ERR_CUDA;
    }
    return st;
}

}  // extern "C"
