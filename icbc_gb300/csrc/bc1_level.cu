// bc1_level.cu -- encoder kernels of one quality level.
//
// Compiled once per level with -DICBC_LEVEL=<0..9> so the ten
// specialisations build in parallel.  -fmad=false keeps every multiply and
// add separately rounded, as the reference's scalar build does.
#include <cuda_runtime.h>

#include "bc1_batch_task.cuh"

#ifndef ICBC_LEVEL
#error "compile with -DICBC_LEVEL=<0..9>"
#endif

namespace icbc_gpu {

// ------------------------------------------------------------- kernels --

// With DEFER (level 9 only) refinement is left to k_refine: the kernel
// records each block's starting error and whether refinement applies.
template <int L, bool DEFER>
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_encode_blocks(const GlobalTables *G, BlocksSrc s, EncodeParams p,
                                                                     uint2 *out, float *errors, int64_t n,
                                                                     RefineSlot *st) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const WarpCtx w = warp_ctx<L>(smem, T, G, p.decoder);
    const int64_t groups = (n + 31) / 32;
    for (int64_t g = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); g < groups;
         g += (int64_t)gridDim.x * kWarpsPerCta) {
        const int64_t base = g * 32;
        const int nb = (int)(n - base < 32 ? n - base : 32);
        __syncwarp();
        load_float_blocks(s, base, nb, w.in, w.lane);
        __syncwarp();
        const bool active = w.lane < nb;
        const int64_t b = base + w.lane;
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (L >= 4 && active) {
            const uint2 prev = out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool pending;
        const float e = encode_warp_ex<L, DEFER>(w, float_row(w), p, active, c0, c1, idx, pending);
        if (active) {
            out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (errors) errors[b] = e;
            if (DEFER) st[b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

template <int L, bool DEFER>
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_encode_image(const GlobalTables *G, ImageDesc d, EncodeParams p,
                                                                    RefineSlot *st) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const WarpCtx w = warp_ctx<L>(smem, T, G, p.decoder);
    const int64_t groups = (d.nblocks + 31) / 32;
    for (int64_t g = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); g < groups;
         g += (int64_t)gridDim.x * kWarpsPerCta) {
        const int64_t b = g * 32 + w.lane;
        const bool active = b < d.nblocks;
        __syncwarp();
        if (active) load_image_block(d, b, w.in + w.lane * kInStride, T.lut255);
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (L >= 4 && active) {
            const uint2 prev = d.out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool pending;
        const float e = encode_warp_ex<L, DEFER>(w, float_row(w), p, active, c0, c1, idx, pending);
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (DEFER) st[b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

// k_encode_image with byte texel rows, for RGBA8 images with uniform or alpha
// weights at levels 2..9: 11 KB of shared memory per warp and at most 128
// registers per thread, so four CTAs (16 warps) fit on an SM instead of three.
template <int L, bool DEFER>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 4) k_encode_image_bytes(const GlobalTables *G, ImageDesc d,
                                                                             EncodeParams p, RefineSlot *st) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const WarpCtx w = warp_ctx_byte_rows(smem, T, G, p.decoder);
    const ByteRow row = byte_row(w, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA);
    const int64_t groups = (d.nblocks + 31) / 32;
    for (int64_t g = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); g < groups;
         g += (int64_t)gridDim.x * kWarpsPerCta) {
        const int64_t b = g * 32 + w.lane;
        const bool active = b < d.nblocks;
        __syncwarp();
        if (active) load_image_block_bytes(d, b, reinterpret_cast<uint32_t *>(w.in) + w.lane * kInWordsByte);
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (L >= 4 && active) {
            const uint2 prev = d.out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool pending;
        const float e = encode_warp_ex<L, DEFER>(w, row, p, active, c0, c1, idx, pending);
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (DEFER) st[b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

// Levels 2..9 in two passes (RGBA8 images, byte rows).  Many blocks reduce
// to 0 or 1 colours (on the quality-sweep image 99% at level 2, 86% at level
// 4, 61% at level 5, 21-29% at levels 6-9), and a warp with one other block
// among them runs that block's whole cluster fit with some lanes idle (with
// one lane busy at the low levels).  Pass 1 finishes the blocks of 0 or 1
// colours and lists the rest; pass 2 runs the full encoder over the list, 32
// listed blocks per warp.  Each block's computation is the single-pass one
// (pass 2 reduces again).  Levels 2-4 take half the time, levels 5-8 2-25%
// less.
// Pass 1 needs only to tell blocks of 0 or 1 reduced colours from the rest,
// so it follows reduce_colors (icbc.h:1683-1728) only while one colour has
// been kept: the texels and the running colour stay in registers (a ByteRow
// over a register array, every index known at compile time), and a block
// is listed as soon as a second colour appears.  For the blocks it finishes
// the arithmetic is reduce_colors' (every texel merged into the first
// colour).  Shared memory holds only the i / 255 table; six CTAs per SM
// (80 registers) beat both four (126 registers) and eight (more spills).
template <int L>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 6) k_image_trivial(const GlobalTables *G, ImageDesc d, EncodeParams p,
                                                                     uint32_t *list, unsigned int *listed,
                                                                     RefineSlot *st) {
    __shared__ float lut[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = G->s.lut255[i];
    __syncthreads();
    const DecoderTables *D = &G->dec[p.decoder];
    const int lane = threadIdx.x & 31;
    const int alpha = d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA;
    const int64_t groups = (d.nblocks + 31) / 32;
    for (int64_t g = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); g < groups;
         g += (int64_t)gridDim.x * kWarpsPerCta) {
        const int64_t b = g * 32 + lane;
        const bool active = b < d.nblocks;
        bool other = false;
        if (active) {
            uint32_t px[16];
            fetch_image_block(d, b, px);
            const ByteRow row{px, lut, alpha};
            V3 c;
            int count;
            other = !reduce_to_one(row, Level<L>::threshold, c, count);
            if (!other) {
                uint32_t c0, c1, idx;
                const float e = trivial_block<16>(D, lut, row, p, c, count, c0, c1, idx);
                d.out[b] = make_uint2(c0 | (c1 << 16), idx);
                if (d.errors) d.errors[b] = e;
                if (st) st[b] = RefineSlot{e, 0u};  // level 9: nothing to refine
            }
        }
        const unsigned m = __ballot_sync(kFull, other);
        if (m) {
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(listed, (unsigned)__popc(m));
            base = __shfl_sync(kFull, base, 0);
            if (other) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)b;
        }
    }
}

template <int L, bool DEFER>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 4) k_image_listed(const GlobalTables *G, ImageDesc d,
                                                                       EncodeParams p, const uint32_t *list,
                                                                       const unsigned int *listed, RefineSlot *st) {
    const int64_t n = *listed;
    const int64_t groups = (n + 31) / 32;
    if ((int64_t)blockIdx.x * kWarpsPerCta >= groups) return;  // the whole CTA has no work
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const WarpCtx w = warp_ctx_byte_rows(smem, T, G, p.decoder);
    const ByteRow row = byte_row(w, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA);
    for (int64_t g = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); g < groups;
         g += (int64_t)gridDim.x * kWarpsPerCta) {
        const int64_t k = g * 32 + w.lane;
        const bool active = k < n;
        const int64_t b = active ? (int64_t)list[k] : 0;
        __syncwarp();
        if (active) load_image_block_bytes(d, b, reinterpret_cast<uint32_t *>(w.in) + w.lane * kInWordsByte);
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (L >= 4 && active) {
            const uint2 prev = d.out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool pending;
        const float e = encode_warp_ex<L, DEFER>(w, row, p, active, c0, c1, idx, pending);
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (DEFER) st[b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

// The batched form's kernel for this level's tasks of a byte-row batch:
// run_batch with the level fixed, so the kernel holds one level's code as the
// plain kernels do (the all-levels kernel stalls about twice as often on
// instruction fetch for the same blocks).
template <int LV>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 4)
    k_batch_level(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks, int task0, int ntasks,
                  int *counter, const int64_t *refine_base, RefineSlot *slots, BatchLists lists) {
    extern __shared__ __align__(16) unsigned char smem[];
    run_batch<true, LV>(G, smem, images, tasks, nullptr, 0, task0, ntasks, counter, refine_base, slots, lists);
}

constexpr int L = ICBC_LEVEL;
constexpr bool kCompact = Level<L>::cluster;

// CTAs for n blocks, from the level's launch shape: every warp takes
// groups_per_warp groups of 32 blocks; a persistent grid is exactly the
// resident CTAs (from the occupancy API), each warp striding over the image,
// otherwise there are enough CTAs for the work and the hardware balances
// them (better when block costs vary, as they do from level 2 on).
template <class K>
static int grid_for(K kernel, int64_t n, int sms, size_t smem, int &resident) {
    const LaunchShape shape = launch_shape(L);
    const int64_t groups = (n + 31) / 32;
    const int64_t per_cta = (int64_t)kWarpsPerCta * shape.groups_per_warp;
    int64_t ctas = (groups + per_cta - 1) / per_cta;
    if (shape.persistent) {
        if (!resident) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarpsPerCta * 32, smem) !=
                    cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
            resident = per_sm;
        }
        const int64_t cap = (int64_t)sms * resident;
        const int64_t all = (groups + kWarpsPerCta - 1) / kWarpsPerCta;
        ctas = all < cap ? all : cap;
    }
    return (int)(ctas < 1 ? 1 : ctas < 0x7fffffff ? ctas : 0x7fffffff);
}

#define ICBC_CAT2(a, b) a##b
#define ICBC_CAT(a, b) ICBC_CAT2(a, b)

// Level 9 encodes in two launches: the encoder without refinement, then
// k_refine, handing over through a RefineSlot per block in stream-ordered
// scratch.  Other levels are one launch.
constexpr bool kDefer = Level<L>::refine;

// The level-9 hand-over lives in stream-ordered scratch, or in the caller's
// `ext_st` (n slots) and `ext_counter` when given (graph captures, where
// nothing is allocated).
template <class Kernel, class Launch>
static cudaError_t run(Kernel kernel, size_t smem, int &resident, int64_t n, int sms, cudaStream_t stream,
                       Launch launch, const GlobalTables *G, const ImageDesc *image, const BlocksSrc *blocks,
                       const EncodeParams &p, uint2 *out, float *errors, RefineSlot *ext_st = nullptr,
                       unsigned long long *ext_counter = nullptr) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = grid_for(kernel, n, sms, smem, resident);
    if (!kDefer) {
        launch(grid, smem, nullptr);
        return cudaGetLastError();
    }
    void *scratch = nullptr;
    RefineSlot *st = ext_st;
    unsigned long long *counter = ext_counter;
    if (!st) {
        const size_t slots = ((size_t)n * sizeof(RefineSlot) + 15) / 16 * 16;
        e = scratch_alloc(&scratch, slots + 16, stream);
        if (e != cudaSuccess) return e;
        st = reinterpret_cast<RefineSlot *>(scratch);
        counter = reinterpret_cast<unsigned long long *>(static_cast<char *>(scratch) + slots);
    }
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (e == cudaSuccess) {
        launch(grid, smem, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_refine(G, image, blocks, p, out, errors, st, n, counter, stream, sms);
    if (!scratch) return e;
    const cudaError_t f = scratch_free(scratch, stream);
    return e != cudaSuccess ? e : f;
}

// Resident CTAs per SM of each kernel (persistent launch shapes), found once.
static int g_resident_blocks = 0, g_resident_image = 0, g_resident_bytes = 0;

// Byte rows apply to the cluster-fit levels and to RGBA8 weights (uniform or
// alpha); weight planes need float rows.
static bool use_byte_rows(const ImageDesc &d) { return Level<L>::cluster && d.weight_mode != ICBC_GPU_WEIGHTS_PLANE; }

static int g_resident_trivial = 0, g_resident_listed = 0;

// The two passes of kCompact levels, with the list (and at level 9 the
// refinement hand-over, unless the caller gives one) in stream-ordered
// scratch; level 9 then runs its refinement pass over every block.
static cudaError_t launch_image_compacted(const GlobalTables *G, const ImageDesc &d, const EncodeParams &p,
                                          cudaStream_t stream, int sms, RefineSlot *ext_st,
                                          unsigned long long *ext_counter) {
    const size_t smem = smem_bytes_byte_rows();
    cudaError_t e =
        cudaFuncSetAttribute(k_image_listed<L, kDefer>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && !g_resident_listed) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_image_listed<L, kDefer>, kWarpsPerCta * 32, smem);
        g_resident_listed = per_sm > 0 ? per_sm : 1;
    }
    if (e != cudaSuccess) return e;
    const size_t list_bytes = ((size_t)d.nblocks * 4 + 15) / 16 * 16;
    const size_t slot_bytes = (kDefer && !ext_st) ? ((size_t)d.nblocks * sizeof(RefineSlot) + 15) / 16 * 16 + 16 : 0;
    void *scratch = nullptr;
    e = scratch_alloc(&scratch, list_bytes + 16 + slot_bytes, stream);
    if (e != cudaSuccess) return e;
    char *base = static_cast<char *>(scratch);
    uint32_t *list = reinterpret_cast<uint32_t *>(base);
    unsigned int *listed = reinterpret_cast<unsigned int *>(base + list_bytes);
    RefineSlot *st = ext_st;
    unsigned long long *counter = ext_counter;
    if (kDefer && !ext_st) {
        st = reinterpret_cast<RefineSlot *>(base + list_bytes + 16);
        counter = reinterpret_cast<unsigned long long *>(base + list_bytes + 16 + slot_bytes - 16);
    }
    e = cudaMemsetAsync(listed, 0, sizeof(unsigned int), stream);
    if (e == cudaSuccess && kDefer) e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (e == cudaSuccess) {
        const int grid = grid_for(k_image_trivial<L>, d.nblocks, sms, 0, g_resident_trivial);
        k_image_trivial<L><<<grid, kWarpsPerCta * 32, 0, stream>>>(G, d, p, list, listed, kDefer ? st : nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        // Persistent over the list, whose length only the device knows.
        const int64_t most = ((int64_t)d.nblocks + 32 * kWarpsPerCta - 1) / (32 * kWarpsPerCta);
        const int64_t cap = (int64_t)sms * g_resident_listed;
        const int grid = (int)(most < cap ? most : cap);
        k_image_listed<L, kDefer><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, d, p, list, listed, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && kDefer) e = launch_refine(G, &d, nullptr, p, d.out, d.errors, st, d.nblocks, counter, stream, sms);
    const cudaError_t f = scratch_free(scratch, stream);
    return e != cudaSuccess ? e : f;
}

static cudaError_t launch_image(const GlobalTables *G, const ImageDesc &d, const EncodeParams &p, cudaStream_t stream,
                                int sms, RefineSlot *ext_st, unsigned long long *ext_counter) {
    if constexpr (kCompact) {
        if (use_byte_rows(d) && d.nblocks < (int64_t(1) << 32))
            return launch_image_compacted(G, d, p, stream, sms, ext_st, ext_counter);
    }
    if constexpr (Level<L>::cluster) {
        if (use_byte_rows(d))
            return run(k_encode_image_bytes<L, kDefer>, smem_bytes_byte_rows(), g_resident_bytes, d.nblocks, sms,
                       stream,
                       [&](int grid, size_t smem, RefineSlot *slots) {
                           k_encode_image_bytes<L, kDefer><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, d, p, slots);
                       },
                       G, &d, nullptr, p, d.out, d.errors, ext_st, ext_counter);
    }
    return run(k_encode_image<L, kDefer>, smem_bytes(Level<L>::cluster), g_resident_image, d.nblocks, sms, stream,
               [&](int grid, size_t smem, RefineSlot *slots) {
                   k_encode_image<L, kDefer><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, d, p, slots);
               },
               G, &d, nullptr, p, d.out, d.errors, ext_st, ext_counter);
}

cudaError_t ICBC_CAT(launch_blocks_l, ICBC_LEVEL)(const GlobalTables *G, const BlocksSrc &s, const EncodeParams &p,
                                                  void *out, float *errors, int64_t n, cudaStream_t stream, int sms) {
    uint2 *o = reinterpret_cast<uint2 *>(out);
    return run(k_encode_blocks<L, kDefer>, smem_bytes(Level<L>::cluster), g_resident_blocks, n, sms, stream,
               [&](int grid, size_t smem, RefineSlot *st) {
                   k_encode_blocks<L, kDefer><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, s, p, o, errors, n, st);
               },
               G, nullptr, &s, p, o, errors);
}

cudaError_t ICBC_CAT(launch_batch_level_l, ICBC_LEVEL)(const GlobalTables *G, const ImageDesc *images,
                                                        const BatchTask *tasks, int task0, int ntasks, int *counter,
                                                        cudaStream_t stream, int grid, const int64_t *refine_base,
                                                        RefineSlot *slots, BatchLists lists) {
    const size_t smem = smem_bytes_byte_rows();
    cudaError_t e = cudaFuncSetAttribute(k_batch_level<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_batch_level<L><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, images, tasks, task0, ntasks, counter, refine_base,
                                                               slots, lists);
    return cudaGetLastError();
}

cudaError_t ICBC_CAT(launch_image_l, ICBC_LEVEL)(const GlobalTables *G, const ImageDesc &d, const EncodeParams &p,
                                                 cudaStream_t stream, int sms) {
    return launch_image(G, d, p, stream, sms, nullptr, nullptr);
}

// As launch_image_l<L>, with level 9's hand-over in the caller's memory
// (d.nblocks slots and a counter; unused at the other levels).
cudaError_t ICBC_CAT(launch_image_ext_l, ICBC_LEVEL)(const GlobalTables *G, const ImageDesc &d, const EncodeParams &p,
                                                     cudaStream_t stream, int sms, RefineSlot *st,
                                                     unsigned long long *counter) {
    return launch_image(G, d, p, stream, sms, st, counter);
}

}  // namespace icbc_gpu
