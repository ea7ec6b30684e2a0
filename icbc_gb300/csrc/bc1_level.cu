// bc1_level.cu -- encoder kernels of one quality level.
//
// Compiled once per level with -DICBC_LEVEL=<0..9> so the ten
// specialisations build in parallel.  -fmad=false keeps every multiply and
// add separately rounded, as the reference's scalar build does.
#include <cuda_runtime.h>

#include <algorithm>

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
// k_image_listed with the CTA as the unit: NW warps take 32 * NW listed
// blocks at a time and move through the encoder's stages together -- colour
// reduction and summed-area tables one block per lane, then the cluster
// searches over all the CTA's blocks at once (flat_search_group), then the
// output blocks.  All warps of an SM run the same stage's code at the same
// time, and a search balances over 32 * NW blocks instead of 32.  Same
// arithmetic and the same winner per block as k_image_listed.  Shared memory:
// the tables, then the CTA's byte rows, SAT rows and the sentinel's SAT row,
// argmin slots, info words with the sentinel's (padded to 16 bytes) and NW
// scan sums (group_smem_bytes).
template <int NW>
__host__ __device__ constexpr size_t group_smem_bytes() {
    return sizeof(SharedTables) + (size_t)NW * 32 * (kInWordsByte * 4 + kSatStride * 4 + 8 + 4) + NW * 4 +
           kSatStride * 4 + 16;
}

// The batched CTA-wide kernel's layout: the group layout (16-byte aligned
// size), NW 16-byte round keys and the round's first task.
template <int NW>
__host__ __device__ constexpr size_t batch_smem_bytes() {
    return group_smem_bytes<NW>() + NW * 16 + 16;
}
static_assert(group_smem_bytes<8>() % 16 == 0 && group_smem_bytes<16>() % 16 == 0, "round keys need 16-byte alignment");

// The warp's and the CTA's contexts in the group layout, and the scan sums.
template <int NW>
__device__ __forceinline__ void group_ctx(unsigned char *smem, const SharedTables &T, const DecoderTables *D,
                                          WarpCtx &w, WarpCtx &g, int *&sums) {
    uint32_t *in = reinterpret_cast<uint32_t *>(smem + sizeof(SharedTables));
    float *sat = reinterpret_cast<float *>(in + NW * 32 * kInWordsByte);
    unsigned long long *slots = reinterpret_cast<unsigned long long *>(sat + (NW * 32 + 1) * kSatStride);
    int *info = reinterpret_cast<int *>(slots + NW * 32);
    sums = info + NW * 32 + 4;
    // The group search's sentinel block (flat_search_group), read only after
    // the search's first barrier.
    const float nan = __int_as_float(0x7fffffff);
    if (threadIdx.x < 17) st4(sat + NW * 32 * kSatStride + 4 * threadIdx.x, make_float4(nan, nan, nan, nan));
    if (threadIdx.x == 0) info[NW * 32] = 16 << kInfoShift;
    const int warp = threadIdx.x >> 5;
    g.T = &T;
    g.D = D;
    g.in = reinterpret_cast<float *>(in);
    g.sat = sat;
    g.slots = slots;
    g.info = info;
    g.lane = threadIdx.x;
    w = g;
    w.in = reinterpret_cast<float *>(in + warp * 32 * kInWordsByte);
    w.sat = sat + warp * 32 * kSatStride;
    w.slots = slots + warp * 32;
    w.info = info + warp * 32;
    w.lane = threadIdx.x & 31;
}

template <int L, bool DEFER, int NW>
__global__ void __launch_bounds__(NW * 32, 512 / (NW * 32))
    k_image_listed_cta(const GlobalTables *G, ImageDesc d, EncodeParams p, const uint32_t *list,
                       const unsigned int *listed, RefineSlot *st) {
    const int64_t n = *listed;
    const int64_t groups = (n + 32 * NW - 1) / (32 * NW);
    if ((int64_t)blockIdx.x >= groups) return;  // the whole CTA has no work
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    WarpCtx w, g;
    int *sums;
    group_ctx<NW>(smem, T, &G->dec[p.decoder], w, g, sums);
    uint32_t *in = reinterpret_cast<uint32_t *>(g.in);
    const ByteRow row = byte_row(w, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA);
    for (int64_t grp = blockIdx.x; grp < groups; grp += gridDim.x) {
        const int64_t k = grp * (32 * NW) + threadIdx.x;
        const bool active = k < n;
        const int64_t b = active ? (int64_t)list[k] : 0;
        __syncwarp();
        if (active) load_image_block_bytes(d, b, in + threadIdx.x * kInWordsByte);
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (L >= 4 && active) {
            const uint2 prev = d.out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool pending;
        const float e = encode_warp_ex<L, DEFER, false, NW>(w, row, p, active, c0, c1, idx, pending, &g, sums);
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (DEFER) st[b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

// k_batch_level with the CTA as the unit: the CTA takes NW tasks at a time
// (one per warp; past the end of the queue a warp has no blocks, but its
// threads still walk the round's combinations) and moves through the
// encoder's stages together, the cluster searches over all its blocks at
// once -- when every task of the round has the same decoder and colour
// weights (every walker must use the same fit weights); otherwise each warp
// searches its own blocks that round.  Levels 2-9 of a byte-row batch; at
// level 9 every image refines in k_refine's batch mode (the planner gives
// each level-9 image of the shared kernel a slot range).
template <int LV, int NW>
__global__ void __launch_bounds__(NW * 32, 512 / (NW * 32))
    k_batch_level_cta(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks, int task0, int ntasks,
                      int *counter, const int64_t *refine_base, RefineSlot *slots, BatchLists lists) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    WarpCtx w, g;
    int *sums;
    group_ctx<NW>(smem, T, &G->dec[0], w, g, sums);
    // Round state past the group layout: each warp's (decoder, colour
    // weights), then the CTA's first task (batch_smem_bytes).
    uint4 *warp_key = reinterpret_cast<uint4 *>(smem + group_smem_bytes<NW>());
    int *round_task = reinterpret_cast<int *>(warp_key + NW);
    uint32_t *in = reinterpret_cast<uint32_t *>(g.in);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (;;) {
        if (threadIdx.x == 0) *round_task = atomicAdd(counter, NW);
        __syncthreads();
        const int t = *round_task + warp;
        if (t - warp >= ntasks) break;
        const bool has_task = t < ntasks;
        const BatchTask task = has_task ? tasks[task0 + t] : BatchTask{0u, 0u};
        const ImageDesc &d = images[task.image];
        const int64_t lb = lists.list ? lists.list_base[task.image] : -1;
        int64_t b = (int64_t)task.first_block + lane;
        bool active = has_task && b < d.nblocks;
        if (has_task && lb >= 0) {
            const int64_t n = lists.listed[task.image];
            active = b < n;  // tasks past the list's end: finished by the first pass
            b = active ? (int64_t)lists.list[lb + b] : 0;
        }
        if (lane == 0)
            warp_key[warp] = has_task ? make_uint4((uint32_t)d.decoder, __float_as_uint(d.cw[0]),
                                                   __float_as_uint(d.cw[1]), __float_as_uint(d.cw[2]))
                                      : make_uint4(0xffffffffu, 0u, 0u, 0u);
        __syncthreads();
        // One search over the CTA when every warp with a task has the same key.
        bool group = true;
        uint4 first = make_uint4(0xffffffffu, 0u, 0u, 0u);
#pragma unroll
        for (int k = 0; k < NW; k++) {
            const uint4 v = warp_key[k];
            if (v.x == 0xffffffffu) continue;
            if (first.x == 0xffffffffu) first = v;
            group &= v.x == first.x && v.y == first.y && v.z == first.z && v.w == first.w;
        }
        // Every thread walks the group's combinations with its own fit
        // weights, so a warp without a task takes the round's (decoder,
        // colour weights); warp 0 always has a task.
        EncodeParams p;
        p.decoder = has_task ? d.decoder : (int)first.x;
        p.three_color_mode = d.three_color_mode;
        p.three_color_black = d.three_color_black;
        p.cw = has_task ? v3(d.cw[0], d.cw[1], d.cw[2])
                        : v3(__uint_as_float(first.y), __uint_as_float(first.z), __uint_as_float(first.w));
        w.D = &G->dec[p.decoder];
        const ByteRow row = byte_row(w, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA);
        __syncwarp();
        if (active) load_image_block_bytes(d, b, in + threadIdx.x * kInWordsByte);
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (LV >= 4 && active) {
            const uint2 prev = d.out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        bool pending = false;
        const float e = encode_warp_ex<LV, LV == 9, false, NW>(w, row, p, active, c0, c1, idx, pending, &g, sums,
                                                                group);
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (LV == 9) slots[refine_base[task.image] + b] = RefineSlot{e, pending ? 1u : 0u};
        }
        __syncthreads();  // round_task and warp_key are rewritten next round
    }
}

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

static int g_resident_trivial = 0, g_resident_listed = 0, g_resident_listed8 = 0, g_resident_listed16 = 0;
static int g_resident_batch8 = 0, g_resident_batch16 = 0;

// The listed pass's CTA size at this level: the launch shape's, else the
// level's default -- 16-warp CTAs from level 4 on, 4 at levels 2-3, whose
// short lists gain nothing from CTA-wide searches.
static int listed_cta_warps() {
    const int c = launch_shape(L).cta_warps;
    if (c == 4 || c == 8 || c == 16) return c;
    return L >= 4 ? 16 : 4;
}

// The CTA size for an image of `nblocks` blocks: a CTA-wide pass takes
// 32 * cta_warps listed blocks per CTA, so an image with fewer blocks than
// two such rounds over every SM would run on a fraction of the SMs; it takes
// 4-warp CTAs instead.
static int listed_cta_warps(int64_t nblocks, int sms) {
    const int c = listed_cta_warps();
    return c > 4 && nblocks >= (int64_t)sms * 32 * c * 2 ? c : 4;
}

// The batched form's per-level kernel's CTA size: the launch shape's, else 4
// (on a mixed batch of small images CTA-wide searches do not pay: a round's
// tasks often differ in decoder or colour weights).
static int batch_cta_warps() {
    const int c = launch_shape(L).batch_cta_warps;
    return c == 8 || c == 16 ? c : 4;
}

// Shared-memory limit of a listed-pass kernel and, once, its resident CTAs per SM.
template <class K>
static cudaError_t listed_attributes(K kernel, int warps, size_t smem, int *resident) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && !*resident) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, warps * 32, smem);
        *resident = per_sm > 0 ? per_sm : 1;
    }
    return e;
}

// The two passes of kCompact levels, with the list (and at level 9 the
// refinement hand-over, unless the caller gives one) in stream-ordered
// scratch; level 9 then runs its refinement pass over every block.
static cudaError_t launch_image_compacted(const GlobalTables *G, const ImageDesc &d, const EncodeParams &p,
                                          cudaStream_t stream, int sms, RefineSlot *ext_st,
                                          unsigned long long *ext_counter) {
    const int cta_warps = listed_cta_warps(d.nblocks, sms);
    const size_t smem = cta_warps == 16 ? group_smem_bytes<16>()
                        : cta_warps == 8 ? group_smem_bytes<8>()
                                         : smem_bytes_byte_rows();
    cudaError_t e = cudaSuccess;
    int *resident = cta_warps == 16 ? &g_resident_listed16 : cta_warps == 8 ? &g_resident_listed8 : &g_resident_listed;
    if (cta_warps == 16) e = listed_attributes(k_image_listed_cta<L, kDefer, 16>, 16, smem, resident);
    else if (cta_warps == 8) e = listed_attributes(k_image_listed_cta<L, kDefer, 8>, 8, smem, resident);
    else e = listed_attributes(k_image_listed<L, kDefer>, kWarpsPerCta, smem, resident);
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
        const int per_cta = 32 * (cta_warps == 4 ? kWarpsPerCta : cta_warps);
        const int64_t most = ((int64_t)d.nblocks + per_cta - 1) / per_cta;
        const int64_t cap = (int64_t)sms * *resident;
        const int grid = (int)(most < cap ? most : cap);
        if (cta_warps == 16)
            k_image_listed_cta<L, kDefer, 16><<<grid, 16 * 32, smem, stream>>>(G, d, p, list, listed, st);
        else if (cta_warps == 8)
            k_image_listed_cta<L, kDefer, 8><<<grid, 8 * 32, smem, stream>>>(G, d, p, list, listed, st);
        else
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
    // `grid` counts 4-warp CTAs; a CTA-wide kernel gets as many warps in all.
    const int cta_warps = Level<L>::cluster && (L < 9 || refine_base) ? batch_cta_warps() : 4;
    if (cta_warps != 4) {
        const size_t smem = cta_warps == 16 ? batch_smem_bytes<16>() : batch_smem_bytes<8>();
        int *resident = cta_warps == 16 ? &g_resident_batch16 : &g_resident_batch8;
        cudaError_t e = cta_warps == 16 ? listed_attributes(k_batch_level_cta<L, 16>, 16, smem, resident)
                                        : listed_attributes(k_batch_level_cta<L, 8>, 8, smem, resident);
        if (e != cudaSuccess) return e;
        const int want = (grid * kWarpsPerCta + cta_warps - 1) / cta_warps;
        const int ctas = std::max(1, std::min(want, current_sm_count() * *resident));
        if (cta_warps == 16)
            k_batch_level_cta<L, 16><<<ctas, 16 * 32, smem, stream>>>(G, images, tasks, task0, ntasks, counter,
                                                                       refine_base, slots, lists);
        else
            k_batch_level_cta<L, 8><<<ctas, 8 * 32, smem, stream>>>(G, images, tasks, task0, ntasks, counter,
                                                                     refine_base, slots, lists);
        return cudaGetLastError();
    }
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
