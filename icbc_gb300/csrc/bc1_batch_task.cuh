// bc1_batch_task.cuh -- one task of the batched form (32 blocks of one image)
// and the persistent loop over a task queue, shared by the all-levels batch
// kernels (bc1_batch.cu) and the per-level ones (bc1_level.cu).
#pragma once

#include "bc1_loaders.cuh"

namespace icbc_gpu {

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

// Encodes the warp's task at level L on its texel rows (bytes or floats).
template <bool BYTES, int L, bool DEFER>
__device__ __forceinline__ float encode_task(const WarpCtx &w, const ImageDesc &d, const EncodeParams &p, bool active,
                                             uint32_t &c0, uint32_t &c1, uint32_t &idx, bool &pending) {
    if constexpr (BYTES)
        return encode_warp_ex<L, DEFER>(w, byte_row(w, d.weight_mode == ICBC_GPU_WEIGHTS_ALPHA), p, active, c0, c1,
                                        idx, pending);
    else
        return encode_warp_ex<L, DEFER>(w, float_row(w), p, active, c0, c1, idx, pending);
}

// Level-L encode of a task, L = -1: the image's level at run time.
template <bool BYTES, int L>
__device__ __forceinline__ float encode_task_at(int level, bool defer, const WarpCtx &w, const ImageDesc &d,
                                                const EncodeParams &p, bool active, uint32_t &c0, uint32_t &c1,
                                                uint32_t &idx, bool &pending) {
    if constexpr (L == 9) {
        return defer ? encode_task<BYTES, 9, true>(w, d, p, active, c0, c1, idx, pending)
                     : encode_task<BYTES, 9, false>(w, d, p, active, c0, c1, idx, pending);
    } else if constexpr (L >= 0) {
        return encode_task<BYTES, L, false>(w, d, p, active, c0, c1, idx, pending);
    } else {
        switch (level) {
            case 0: return encode_task<BYTES, 0, false>(w, d, p, active, c0, c1, idx, pending);
            case 1: return encode_task<BYTES, 1, false>(w, d, p, active, c0, c1, idx, pending);
            case 2: return encode_task<BYTES, 2, false>(w, d, p, active, c0, c1, idx, pending);
            case 3: return encode_task<BYTES, 3, false>(w, d, p, active, c0, c1, idx, pending);
            case 4: return encode_task<BYTES, 4, false>(w, d, p, active, c0, c1, idx, pending);
            case 5: return encode_task<BYTES, 5, false>(w, d, p, active, c0, c1, idx, pending);
            case 6: return encode_task<BYTES, 6, false>(w, d, p, active, c0, c1, idx, pending);
            case 7: return encode_task<BYTES, 7, false>(w, d, p, active, c0, c1, idx, pending);
            case 8: return encode_task<BYTES, 8, false>(w, d, p, active, c0, c1, idx, pending);
            default:
                return defer ? encode_task<BYTES, 9, true>(w, d, p, active, c0, c1, idx, pending)
                             : encode_task<BYTES, 9, false>(w, d, p, active, c0, c1, idx, pending);
        }
    }
}

// The persistent loop of a batched kernel: every warp takes the next task of
// tasks task0 .. task0 + ntasks - 1 from an atomic counter until the queue
// is empty (L >= 0: every image of those tasks has level L).  With
// `refine_base`, the level-9 images leave refinement to k_refine's batch
// mode (bc1_refine.cu), which runs after the batch: the same split as the
// plain level-9 launches, so lanes do not wait for each other's refinement.
// With `lists.list` (second pass of a two-pass batch), the tasks of an image
// with list_base >= 0 cover the image's list instead of its blocks: task
// blocks first_block .. first_block + 31 are list entries, and tasks past
// the list's end have nothing to do.
template <bool BYTES, int L>
__device__ __forceinline__ void run_batch(const GlobalTables *G, unsigned char *smem, const ImageDesc *images,
                                          const BatchTask *tasks, const uint32_t *task_start, int n_images, int task0,
                                          int ntasks, int *counter, const int64_t *refine_base, RefineSlot *slots,
                                          BatchLists lists) {
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(counter, 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= ntasks) break;
        const BatchTask task = batch_task(tasks, task_start, n_images, task0 + t);
        const ImageDesc &d = images[task.image];
        const int level = L >= 0 ? L : d.level;
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
        const float e = encode_task_at<BYTES, L>(level, base >= 0, w, d, p, active, c0, c1, idx, pending);
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (base >= 0) slots[base + b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

}  // namespace icbc_gpu
