// bc1_batch.cu -- persistent batched encoder over mixed images, levels and
// decoders.  -fmad=false as for every encoder translation unit.  Compiled
// twice: -DICBC_BATCH_BYTES=1 keeps texels as bytes (batches without weight
// planes: four CTAs per SM, as the plain image kernels), =0 as floats.
#include <cuda_runtime.h>

#include "bc1_loaders.cuh"

#ifndef ICBC_BATCH_BYTES
#error "compile with -DICBC_BATCH_BYTES=<0|1>"
#endif

namespace icbc_gpu {

constexpr bool kBytes = ICBC_BATCH_BYTES != 0;

// Encodes the warp's task at level L on its texel rows.
template <int L, bool DEFER>
__device__ __forceinline__ float encode_task(const WarpCtx &w, const ImageDesc &d, const EncodeParams &p, bool active,
                                             uint32_t &c0, uint32_t &c1, uint32_t &idx, bool &pending) {
    if (kBytes) return encode_warp_ex<L, DEFER>(w, byte_row(w, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA), p, active,
                                                c0, c1, idx, pending);
    return encode_warp_ex<L, DEFER>(w, float_row(w), p, active, c0, c1, idx, pending);
}

// Task t of a batch: an entry of the explicit list, or -- without one --
// found from per-image offsets: task t belongs to the last image whose first
// task (`task_start[i]`, n_images + 1 entries) is <= t.
__device__ __forceinline__ BatchTask batch_task(const BatchTask *tasks, const uint32_t *task_start, int n_images,
                                                int t) {
    if (tasks) return tasks[t];
    int lo = 0, hi = n_images;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((int)task_start[mid] <= t) lo = mid;
        else hi = mid;
    }
    BatchTask task;
    task.image = (uint32_t)lo;
    task.first_block = (uint32_t)(t - (int)task_start[lo]) * 32u;
    return task;
}

// Persistent batched encoder: every warp takes the next task (32 blocks of
// one image) from an atomic counter until the queue is empty.  Tasks are
// ordered most expensive level first by the planner (batch_task: an explicit
// list, or per-image offsets).  With `refine_base`, the
// level-9 images leave refinement to k_refine's batch mode (bc1_refine.cu),
// which runs after this kernel in the same stream: the same split as the
// plain level-9 launches, so lanes do not wait for each other's refinement.
// With `lists.list` (second pass of a two-pass batch), the tasks of an image
// with list_base >= 0 cover the image's list instead of its blocks: task
// blocks first_block .. first_block + 31 are list entries, and tasks past
// the list's end have nothing to do.
template <bool BYTES>
__global__ void __launch_bounds__(kWarpsPerCta * 32, BYTES ? 4 : 1)
    k_encode_batch(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks, const uint32_t *task_start,
                   int n_images, int ntasks, int *counter, const int64_t *refine_base, RefineSlot *slots,
                   BatchLists lists) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(counter, 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= ntasks) break;
        const BatchTask task = batch_task(tasks, task_start, n_images, t);
        const ImageDesc &d = images[task.image];
        const int level = d.level;
        const int64_t lb = lists.list ? lists.list_base[task.image] : -1;
        int64_t b = (int64_t)task.first_block + lane;
        bool active = b < d.nblocks;
        if (lb >= 0) {
            const int64_t n = lists.listed[task.image];
            if ((int64_t)task.first_block >= n) continue;  // the whole task was finished by the first pass
            active = b < n;
            b = active ? (int64_t)lists.list[lb + b] : 0;
        }
        EncodeParams p;
        p.decoder = d.decoder;
        p.three_color_mode = d.three_color_mode;
        p.three_color_black = d.three_color_black;
        p.cw = v3(d.cw[0], d.cw[1], d.cw[2]);
        const WarpCtx w = BYTES ? warp_ctx_byte_rows(smem, T, G, p.decoder) : warp_ctx<9>(smem, T, G, p.decoder);
        __syncwarp();
        if (active) {
            if (BYTES) load_image_block_bytes(d, b, reinterpret_cast<uint32_t *>(w.in) + lane * kInWordsByte);
            else load_image_block(d, b, w.in + lane * kInStride, T.lut255);
        }
        __syncwarp();
        uint32_t c0 = 0, c1 = 0, idx = 0;
        if (level >= 4 && active) {
            const uint2 prev = d.out[b];
            c0 = prev.x & 0xffff;
            c1 = prev.x >> 16;
            idx = prev.y;
        }
        // Level 9 with a refinement slot range: encode now, refine in
        // k_refine's batch mode (warp-uniform: one image per task).
        const int64_t base = (level == 9 && refine_base) ? refine_base[task.image] : -1;
        bool pending = false;
        float e = 0.0f;
        switch (level) {
            case 0: e = encode_task<0, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 1: e = encode_task<1, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 2: e = encode_task<2, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 3: e = encode_task<3, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 4: e = encode_task<4, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 5: e = encode_task<5, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 6: e = encode_task<6, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 7: e = encode_task<7, false>(w, d, p, active, c0, c1, idx, pending); break;
            case 8: e = encode_task<8, false>(w, d, p, active, c0, c1, idx, pending); break;
            default:
                if (base >= 0) e = encode_task<9, true>(w, d, p, active, c0, c1, idx, pending);
                else e = encode_task<9, false>(w, d, p, active, c0, c1, idx, pending);
                break;
        }
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (base >= 0) slots[base + b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

#if ICBC_BATCH_BYTES
// First pass of a two-pass batch: every warp takes tasks of the listed
// images (list_base >= 0, levels 2..9) in a grid stride and follows
// reduce_colors (icbc.h:1683-1728) in registers for its 32 blocks, as
// k_image_trivial does for one image: a block of 0 or 1 reduced colours is
// finished here (icbc.h:3752-3764; at level 9 with an empty refinement slot),
// any other goes to its image's list with one atomic per warp.  Only the u8
// table is in shared memory, so six CTAs fit on an SM.
__global__ void __launch_bounds__(kWarpsPerCta * 32, 6)
    k_batch_trivial(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks, const uint32_t *task_start,
                    int n_images, int ntasks, BatchLists lists, const int64_t *refine_base, RefineSlot *slots) {
    __shared__ float lut[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = G->s.lut255[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5); t < ntasks; t += gridDim.x * kWarpsPerCta) {
        const BatchTask task = batch_task(tasks, task_start, n_images, t);
        const int64_t lb = lists.list_base[task.image];
        if (lb < 0) continue;
        const ImageDesc &d = images[task.image];
        const int64_t b = (int64_t)task.first_block + lane;
        const bool active = b < d.nblocks;
        const int64_t sb = (d.level == 9 && refine_base) ? refine_base[task.image] : -1;
        bool other = false;
        if (active) {
            uint32_t px[16];
            fetch_image_block(d, b, px);
            const ByteRow row{px, lut, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA};
            V3 c;
            int count;
            other = !reduce_to_one(row, level_threshold(d.level), c, count);
            if (!other) {
                EncodeParams p;
                p.decoder = d.decoder;
                p.three_color_mode = d.three_color_mode;
                p.three_color_black = d.three_color_black;
                p.cw = v3(d.cw[0], d.cw[1], d.cw[2]);
                uint32_t c0, c1, idx;
                const float e = trivial_block<16>(&G->dec[d.decoder], lut, row, p, c, count, c0, c1, idx);
                d.out[b] = make_uint2(c0 | (c1 << 16), idx);
                if (d.errors) d.errors[b] = e;
                if (sb >= 0) slots[sb + b] = RefineSlot{e, 0u};  // level 9: nothing to refine
            }
        }
        const unsigned m = __ballot_sync(kFull, other);
        if (m) {
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(lists.listed + task.image, (unsigned)__popc(m));
            base = __shfl_sync(kFull, base, 0);
            if (other) lists.list[lb + base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)b;
        }
    }
}

cudaError_t launch_batch_trivial(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                 const uint32_t *task_start, int n_images, int ntasks, BatchLists lists,
                                 const int64_t *refine_base, RefineSlot *slots, cudaStream_t stream, int sms) {
    if (ntasks <= 0) return cudaSuccess;
    static int resident = 0;
    if (!resident &&
        (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_batch_trivial, kWarpsPerCta * 32, 0) !=
             cudaSuccess ||
         resident < 1))
        resident = 1;
    const int64_t need = ((int64_t)ntasks + kWarpsPerCta - 1) / kWarpsPerCta;
    const int64_t cap = (int64_t)sms * resident;
    const int grid = (int)(need < cap ? need : cap);
    k_batch_trivial<<<grid, kWarpsPerCta * 32, 0, stream>>>(G, images, tasks, task_start, n_images, ntasks, lists,
                                                            refine_base, slots);
    return cudaGetLastError();
}
#endif

#define ICBC_BATCH_CAT2(a, b) a##b
#define ICBC_BATCH_CAT(a, b) ICBC_BATCH_CAT2(a, b)
#if ICBC_BATCH_BYTES
#define ICBC_BATCH_FN(name) ICBC_BATCH_CAT(name, _bytes)
#else
#define ICBC_BATCH_FN(name) ICBC_BATCH_CAT(name, _float)
#endif

static size_t batch_smem() { return kBytes ? smem_bytes_byte_rows() : smem_bytes(true); }

cudaError_t ICBC_BATCH_FN(launch_encode_batch)(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                               const uint32_t *task_start, int n_images, int ntasks, int *counter,
                                               cudaStream_t stream, int grid, const int64_t *refine_base,
                                               RefineSlot *slots, BatchLists lists) {
    const size_t smem = batch_smem();
    cudaError_t e = cudaFuncSetAttribute(k_encode_batch<kBytes>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_encode_batch<kBytes><<<grid, kWarpsPerCta * 32, smem, stream>>>(G, images, tasks, task_start, n_images, ntasks,
                                                                       counter, refine_base, slots, lists);
    return cudaGetLastError();
}

int ICBC_BATCH_FN(batch_ctas_per_sm)() {
    int n = 0;
    const size_t smem = batch_smem();
    cudaFuncSetAttribute(k_encode_batch<kBytes>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_encode_batch<kBytes>, kWarpsPerCta * 32, smem) !=
        cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

}  // namespace icbc_gpu
