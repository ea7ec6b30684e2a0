// bc1_simd.cu -- encoders that reproduce the reference's SIMD builds.
//
// icbc.h compiled with ICBC_SIMD = SSE2 .. AVX512 gives different blocks from
// its scalar build for a few blocks per thousand: only the cluster-fit loops
// differ (vector width and lane tie-break, fused vmadd/vmsub, vround01
// rounding; icbc.h:2089-2344, :2362-2742).  This kernel runs the level
// encoders with those loops (encode_warp_ex<L, false, true>), one launch per
// call, refinement inline at level 9.  It is a parity mode: the plain kernels
// stay the fast path for the scalar profile.  -fmad=false as everywhere; the
// fused operations are explicit __fmaf_rn calls.
#include <cuda_runtime.h>

#include "bc1_loaders.cuh"

namespace icbc_gpu {

__global__ void __launch_bounds__(kWarpsPerCta * 32) k_encode_simd(const GlobalTables *G, ImageDesc d, BlocksSrc s,
                                                                    EncodeParams p, uint2 *out, float *errors,
                                                                    int64_t n, int level, int image) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const WarpCtx w = warp_ctx<9>(smem, T, G, p.decoder);
    const int64_t groups = (n + 31) / 32;
    for (int64_t g = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); g < groups;
         g += (int64_t)gridDim.x * kWarpsPerCta) {
        const int64_t base = g * 32;
        const int nb = (int)(n - base < 32 ? n - base : 32);
        const bool active = w.lane < nb;
        const int64_t b = base + w.lane;
        __syncwarp();
        if (image) {
            if (active) load_image_block(d, b, w.in + w.lane * kInStride, T.lut255);
        } else {
            load_float_blocks(s, base, nb, w.in, w.lane);
        }
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (level >= 4 && active) {
            const uint2 prev = out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool unused;
        float e = 0.0f;
        switch (level) {
            case 2: e = encode_warp_ex<2, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            case 3: e = encode_warp_ex<3, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            case 4: e = encode_warp_ex<4, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            case 5: e = encode_warp_ex<5, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            case 6: e = encode_warp_ex<6, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            case 7: e = encode_warp_ex<7, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            case 8: e = encode_warp_ex<8, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
            default: e = encode_warp_ex<9, false, true>(w, float_row(w), p, active, c0, c1, idx, unused); break;
        }
        if (active) {
            out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (errors) errors[b] = e;
        }
    }
}

cudaError_t launch_simd(const GlobalTables *G, const ImageDesc *image, const BlocksSrc *blocks, const EncodeParams &p,
                        uint2 *out, float *errors, int64_t n, int level, cudaStream_t stream) {
    const size_t smem = smem_bytes(true);
    cudaError_t e = cudaFuncSetAttribute(k_encode_simd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t groups = (n + 31) / 32;
    const int64_t ctas = (groups + kWarpsPerCta - 1) / kWarpsPerCta;
    const int grid = (int)(ctas < 1 ? 1 : ctas < 0x7fffffff ? ctas : 0x7fffffff);
    const ImageDesc dd = image ? *image : ImageDesc{};
    const BlocksSrc ss = blocks ? *blocks : BlocksSrc{nullptr, nullptr};
    k_encode_simd<<<grid, kWarpsPerCta * 32, smem, stream>>>(G, dd, ss, p, out, errors, n, level, image ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace icbc_gpu
