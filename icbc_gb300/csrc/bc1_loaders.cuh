// bc1_loaders.cuh -- texel loaders and per-CTA staging shared by the kernels.
#pragma once

#include "bc1_kernels.h"

namespace icbc_gpu {

// ------------------------------------------------------------- loaders --

// Cooperative coalesced load of up to 32 consecutive float blocks into the
// warp's texel rows; weights default to 1.0f.
__device__ __forceinline__ void load_float_blocks(const BlocksSrc &s, int64_t base, int nb, float *in, int lane) {
    const float4 *src = reinterpret_cast<const float4 *>(s.colors) + base * 16;
    for (int j = lane; j < nb * 16; j += 32) {
        const float4 v = __ldg(src + j);
        float *r = in + (j >> 4) * kInStride + 4 * (j & 15);
        r[0] = v.x;
        r[1] = v.y;
        r[2] = v.z;
    }
    if (s.weights) {
        const float4 *ws = reinterpret_cast<const float4 *>(s.weights) + base * 4;
        for (int j = lane; j < nb * 4; j += 32) {
            const float4 v = __ldg(ws + j);
            float *r = in + (j >> 2) * kInStride + 16 * (j & 3);
            r[3] = v.x;
            r[7] = v.y;
            r[11] = v.z;
            r[15] = v.w;
        }
    } else if (lane < nb) {
        float *r = in + lane * kInStride;
#pragma unroll
        for (int t = 0; t < 16; t++) r[4 * t + 3] = 1.0f;
    }
}

// The 16 RGBA8 texels of block b of an image: four 16-byte row loads when
// the block is whole and rows are 16-byte aligned, else clamped texel loads
// (edge replication).
__device__ __forceinline__ void fetch_image_block(const ImageDesc &d, int64_t b, uint32_t px[16]) {
    const int bx = (int)(b % d.bw), by = (int)(b / d.bw);
    const int x0 = bx * 4, y0 = by * 4;
    if (d.vec16 && x0 + 4 <= d.width && y0 + 4 <= d.height) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const uint4 q = __ldg(reinterpret_cast<const uint4 *>(d.rgba + (int64_t)(y0 + r) * d.pitch) + bx);
            px[4 * r + 0] = q.x;
            px[4 * r + 1] = q.y;
            px[4 * r + 2] = q.z;
            px[4 * r + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int t = 0; t < 16; t++) {
            const int x = min(x0 + (t & 3), d.width - 1), y = min(y0 + (t >> 2), d.height - 1);
            px[t] = __ldg(reinterpret_cast<const uint32_t *>(d.rgba + (int64_t)y * d.pitch) + x);
        }
    }
}

// One block of an RGBA8 image into this lane's float row.  u8 -> float is
// the exact table of i / 255.0f.
__device__ __forceinline__ void load_image_block(const ImageDesc &d, int64_t b, float *row, const float *lut) {
    const int bx = (int)(b % d.bw), by = (int)(b / d.bw);
    const int x0 = bx * 4, y0 = by * 4;
    uint32_t px[16];
    fetch_image_block(d, b, px);
#pragma unroll
    for (int t = 0; t < 16; t++) {
        row[4 * t + 0] = lut[px[t] & 255];
        row[4 * t + 1] = lut[(px[t] >> 8) & 255];
        row[4 * t + 2] = lut[(px[t] >> 16) & 255];
        float w = 1.0f;
        if (d.weight_mode == 1) {
            w = lut[px[t] >> 24];
        } else if (d.weight_mode == 2) {
            const int x = min(x0 + (t & 3), d.width - 1), y = min(y0 + (t >> 2), d.height - 1);
            w = __ldg(d.weight_plane + (int64_t)y * d.weight_pitch + x);
        }
        row[4 * t + 3] = w;
    }
}

// One block of an RGBA8 image into this lane's byte row (the words as they are).
__device__ __forceinline__ void load_image_block_bytes(const ImageDesc &d, int64_t b, uint32_t *row) {
    uint32_t px[16];
    fetch_image_block(d, b, px);
#pragma unroll
    for (int t = 0; t < 16; t++) row[t] = px[t];
}

__device__ __forceinline__ void stage_tables(SharedTables &T, const GlobalTables *G) {
    const uint4 *src = reinterpret_cast<const uint4 *>(&G->s);
    uint4 *dst = reinterpret_cast<uint4 *>(&T);
    for (int i = threadIdx.x; i < (int)(sizeof(SharedTables) / 16); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
}

template <int L>
__device__ __forceinline__ WarpCtx warp_ctx(unsigned char *smem, const SharedTables &T, const GlobalTables *G, int decoder) {
    const int warp = threadIdx.x >> 5;
    float *base = reinterpret_cast<float *>(smem + sizeof(SharedTables)) +
                  warp * (Level<L>::cluster ? kWarpFloatsHigh : kWarpFloatsLow);
    WarpCtx w;
    w.T = &T;
    w.D = &G->dec[decoder];
    w.in = base;
    w.sat = base + 32 * kInStride;
    w.slots = reinterpret_cast<unsigned long long *>(base + 32 * kInStride + 32 * kSatStride);
    w.info = reinterpret_cast<int *>(base + 32 * kInStride + 32 * kSatStride + 64);
    w.lane = threadIdx.x & 31;
    return w;
}

// The warp's context with byte texel rows (levels 2..9): w.in holds 32 rows
// of kInWordsByte words.
__device__ __forceinline__ WarpCtx warp_ctx_byte_rows(unsigned char *smem, const SharedTables &T, const GlobalTables *G,
                                                      int decoder) {
    const int warp = threadIdx.x >> 5;
    float *base = reinterpret_cast<float *>(smem + sizeof(SharedTables)) + warp * kWarpFloatsByte;
    WarpCtx w;
    w.T = &T;
    w.D = &G->dec[decoder];
    w.in = base;
    w.sat = base + 32 * kInWordsByte;
    w.slots = reinterpret_cast<unsigned long long *>(base + 32 * kInWordsByte + 32 * kSatStride);
    w.info = reinterpret_cast<int *>(base + 32 * kInWordsByte + 32 * kSatStride + 64);
    w.lane = threadIdx.x & 31;
    return w;
}

__device__ __forceinline__ ByteRow byte_row(const WarpCtx &w, int alpha) {
    return ByteRow{reinterpret_cast<const uint32_t *>(w.in) + w.lane * kInWordsByte, w.T->lut255, alpha};
}

}  // namespace icbc_gpu
