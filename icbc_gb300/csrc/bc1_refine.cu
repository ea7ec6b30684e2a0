// bc1_refine.cu -- endpoint refinement of level 9 as its own pass.
//
// refine_endpoints (icbc.h:3574-3651) runs 33 to 256 sequential steps per
// block, different for every block.  Run inside the encoder, each lane
// refines its own block and the warp waits for its slowest lane.  Here the
// encoder leaves, per block, the error refinement starts from and whether it
// applies (RefineSlot); this kernel then refines with a queue per lane: a
// lane that finishes a block takes the next pending one (warp-aggregated
// atomics on one counter), so lanes stay busy until the queue is empty.
// Every step is the reference's step; only the scheduling differs.
#include <cuda_runtime.h>

#include <mutex>

#include "bc1_loaders.cuh"

namespace icbc_gpu {

// One float block (the compress_bc1 layout) into a lane's texel row.
__device__ __forceinline__ void load_float_block_lane(const BlocksSrc &s, int64_t b, float *row) {
    const float4 *c = reinterpret_cast<const float4 *>(s.colors) + b * 16;
#pragma unroll 4
    for (int t = 0; t < 16; t++) {
        const float4 v = __ldg(c + t);
        row[4 * t + 0] = v.x;
        row[4 * t + 1] = v.y;
        row[4 * t + 2] = v.z;
    }
    if (s.weights) {
        const float4 *w4 = reinterpret_cast<const float4 *>(s.weights) + b * 4;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float4 v = __ldg(w4 + j);
            row[16 * j + 3] = v.x;
            row[16 * j + 7] = v.y;
            row[16 * j + 11] = v.z;
            row[16 * j + 15] = v.w;
        }
    } else {
#pragma unroll
        for (int t = 0; t < 16; t++) row[4 * t + 3] = 1.0f;
    }
}

constexpr size_t kRefineLutBytes = 256 * sizeof(float);
// Texel rows of 68 floats (16-byte aligned, 17 float4): a texel's colour and
// weight are one 16-byte load, and the 16-byte accesses of any 8 lanes to
// the same texel of their rows fall in 8 different bank groups.
constexpr int kRefineStride = 68;
constexpr size_t kRefineRowBytes = kWarpsPerCta * sizeof(float) * 32 * kRefineStride;
// Then each warp's candidate palettes, 4 entries x 32 lanes of float4
// (block_error_pal): 44 KB per CTA, five CTAs per SM.
constexpr size_t kRefineSmem = kRefineLutBytes + kRefineRowBytes + kWarpsPerCta * 4 * 32 * sizeof(float4);

constexpr int kRefillBatch = 16;  // 4: 3% slower, 8: 0.4%, 12: as 16 (hard mixture, level 9)

__device__ __forceinline__ V3 shfl3(V3 v, int src) {
    return v3(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src));
}

// Bit t of x (t < 16) to bit 2t.
__device__ __forceinline__ uint32_t spread_bits(uint32_t x) {
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    return (x | (x << 1)) & 0x55555555u;
}

// MODE 0: float blocks (s), 1: one image (d), 2: the deferred level-9 blocks
// of a batch (images + map), each lane with its own image's decoder and
// parameters.
template <int MODE>
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_refine(const GlobalTables *G, ImageDesc d, BlocksSrc s,
                                                              EncodeParams p, uint2 *out, float *errors,
                                                              const RefineSlot *st, int64_t n,
                                                              unsigned long long *counter, const ImageDesc *images,
                                                              RefineMap map) {
    // Shared memory: the u8 table (all refinement needs of the staged
    // tables), each warp's 32 float texel rows, then its candidate palettes.
    extern __shared__ __align__(16) unsigned char smem[];
    float *lut = reinterpret_cast<float *>(smem);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = G->s.lut255[i];
    __syncthreads();
    WarpCtx w{};
    w.D = &G->dec[p.decoder];
    w.in = reinterpret_cast<float *>(smem + kRefineLutBytes) + (threadIdx.x >> 5) * 32 * kRefineStride;
    w.lane = threadIdx.x & 31;
    const int lane = w.lane;
    float *row = w.in + lane * kRefineStride;
    float4 *pal = reinterpret_cast<float4 *>(smem + kRefineLutBytes + kRefineRowBytes) + (threadIdx.x >> 5) * 128 + lane;
    EncodeParams lp = p;
    RefineLane r;
    uint2 *o = nullptr;
    float *er = nullptr;
    bool have = false, exhausted = false;
    // The last accepted candidate's palette times the colour weights, the
    // source of the index update the warp computes for this lane.
    V3 q0 = v3(0.0f, 0.0f, 0.0f), q1 = q0, q2 = q0, q3 = q0;
    for (;;) {
        // Lanes without a block take the next ones; blocks that need no
        // refinement are skipped (their error and bytes are final already).
        // Refills run in batches: a lane that finished waits until
        // kRefillBatch lanes (or all) need a block, so the divergent refill
        // code runs for many lanes at once instead of one at a time.
        unsigned need = __ballot_sync(kFull, !have && !exhausted);
        if (__popc(need) < kRefillBatch && __any_sync(kFull, have)) need = 0;
        while (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (!have && !exhausted) {
                const int64_t mine = (int64_t)base + __popc(need & ((1u << lane) - 1u));
                if (mine >= n) {
                    exhausted = true;
                } else {
                    const RefineSlot sl = st[mine];
                    if (sl.pending) {
                        if (MODE == 2) {
                            int lo = 0, hi = map.n;
                            while (hi - lo > 1) {
                                const int mid = (lo + hi) >> 1;
                                if (map.map_start[mid] <= mine) lo = mid;
                                else hi = mid;
                            }
                            const ImageDesc &di = images[map.map_image[lo]];
                            const int64_t b = mine - map.map_start[lo];
                            lp.decoder = di.decoder;
                            lp.three_color_mode = di.three_color_mode;
                            lp.three_color_black = di.three_color_black;
                            lp.cw = v3(di.cw[0], di.cw[1], di.cw[2]);
                            w.D = &G->dec[di.decoder];
                            load_image_block(di, b, row, lut);
                            o = di.out + b;
                            er = di.errors ? di.errors + b : nullptr;
                        } else {
                            if (MODE == 1) load_image_block(d, mine, row, lut);
                            else load_float_block_lane(s, mine, row);
                            o = out + mine;
                            er = errors ? errors + mine : nullptr;
                        }
                        const uint2 cur = *o;
                        refine_begin(w, lut, FloatRow4{row}, lp, sl.error, cur.x & 0xffff, cur.x >> 16, cur.y, r);
                        have = true;
                    }
                }
            }
            need = __ballot_sync(kFull, !have && !exhausted);
        }
        if (!__any_sync(kFull, have)) break;
        bool accepted = false, stop = false;
        if (have) {
            PalF pr;
            accepted = refine_try(w, lut, FloatRow4{row}, lp, r, pr, stop, pal);
            if (accepted) {
                q0 = pr.c[0] * lp.cw;
                q1 = pr.c[1] * lp.cw;
                q2 = pr.c[2] * lp.cw;
                q3 = pr.c[3] * lp.cw;
            }
        }
        // An accepted step's lane needs indices_generic of its new palette
        // before its next step.  Each texel's index depends on that texel
        // alone, so the warp computes them for two such lanes at a time: the
        // half-warp of lane l takes texel l & 15 of one block, and two ballots
        // pack the 2-bit indices in texel order.
        unsigned m = __ballot_sync(kFull, accepted);
        while (m) {
            const int l0 = __ffs(m) - 1;
            m &= m - 1;
            const int l1 = m ? __ffs(m) - 1 : l0;
            m &= m - 1;
            const int src = lane < 16 ? l0 : l1;
            const V3 p0 = shfl3(q0, src), p1 = shfl3(q1, src), p2 = shfl3(q2, src), p3 = shfl3(q3, src);
            const V3 cw = shfl3(lp.cw, src);
            const uint32_t x =
                index_generic(FloatRow4{w.in + src * kRefineStride}.color(lane & 15), cw, p0, p1, p2, p3);
            const unsigned lo = __ballot_sync(kFull, x & 1u), hi = __ballot_sync(kFull, x >> 1);
            if (lane == l0) r.base_idx = spread_bits(lo & 0xffffu) | (spread_bits(hi & 0xffffu) << 1);
            else if (lane == l1) r.base_idx = spread_bits(lo >> 16) | (spread_bits(hi >> 16) << 1);
        }
        if (have && stop) {
            *o = make_uint2(r.c0 | (r.c1 << 16), r.idx);
            if (er) *er = r.best;
            have = false;
        }
    }
}

namespace {

std::mutex g_pool_mutex;
cudaMemPool_t g_pool[64] = {};

}  // namespace

// The library-owned pool of the current device, created on first use.
static cudaError_t device_pool(cudaMemPool_t *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pool[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        e = cudaMemPoolCreate(&g_pool[dev], &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = 1ull << 30;
        cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

// Creates the pool of the current device if it does not exist yet.  Pool
// creation is not allowed while a stream captures, so code that captures
// launches which take scratch calls this first.
cudaError_t scratch_prepare() {
    cudaMemPool_t pool;
    return device_pool(&pool);
}

// Stream-ordered scratch from a library-owned pool of the current device
// (freed memory stays cached in the pool for the next call).
cudaError_t scratch_alloc(void **ptr, size_t bytes, cudaStream_t stream) {
    cudaMemPool_t pool;
    const cudaError_t e = device_pool(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(ptr, bytes, pool, stream);
}

cudaError_t scratch_free(void *ptr, cudaStream_t stream) { return cudaFreeAsync(ptr, stream); }

template <int MODE>
static cudaError_t refine_grid(int64_t n, int sms, size_t smem, int *grid) {
    static int resident = 0;
    cudaError_t e = cudaFuncSetAttribute(k_refine<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (!resident) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_refine<MODE>, kWarpsPerCta * 32, smem);
        if (e != cudaSuccess) return e;
        resident = per_sm > 0 ? per_sm : 1;
    }
    const int64_t want = (n + kWarpsPerCta * 32 - 1) / (kWarpsPerCta * 32);
    const int64_t cap = (int64_t)sms * resident;
    *grid = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    return cudaSuccess;
}

cudaError_t launch_refine(const GlobalTables *G, const ImageDesc *image, const BlocksSrc *blocks,
                          const EncodeParams &p, uint2 *out, float *errors, const RefineSlot *st, int64_t n,
                          unsigned long long *counter, cudaStream_t stream, int sms) {
    const size_t smem = kRefineSmem;
    const ImageDesc dd = image ? *image : ImageDesc{};
    const BlocksSrc ss = blocks ? *blocks : BlocksSrc{nullptr, nullptr};
    const RefineMap none{nullptr, nullptr, 0};
    int grid = 0;
    cudaError_t e = image ? refine_grid<1>(n, sms, smem, &grid) : refine_grid<0>(n, sms, smem, &grid);
    if (e != cudaSuccess) return e;
    if (image)
        k_refine<1><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, dd, ss, p, out, errors, st, n, counter, nullptr, none);
    else
        k_refine<0><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, dd, ss, p, out, errors, st, n, counter, nullptr, none);
    return cudaGetLastError();
}

cudaError_t launch_refine_batch(const GlobalTables *G, const ImageDesc *images, RefineMap map,
                                const RefineSlot *slots, int64_t total, unsigned long long *counter,
                                cudaStream_t stream, int sms) {
    const size_t smem = kRefineSmem;
    int grid = 0;
    cudaError_t e = refine_grid<2>(total, sms, smem, &grid);
    if (e != cudaSuccess) return e;
    EncodeParams p{};
    k_refine<2><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, ImageDesc{}, BlocksSrc{nullptr, nullptr}, p, nullptr,
                                                           nullptr, slots, total, counter, images, map);
    return cudaGetLastError();
}

}  // namespace icbc_gpu
