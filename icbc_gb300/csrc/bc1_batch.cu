// bc1_batch.cu -- persistent batched encoder over mixed images, levels and
// decoders.  -fmad=false as for every encoder translation unit.
#include <cuda_runtime.h>

#include "bc1_loaders.cuh"

namespace icbc_gpu {

// Persistent batched encoder: every warp takes the next task (32 blocks of
// one image) from an atomic counter until the queue is empty.  Tasks are
// ordered most expensive level first by the planner.  A task is either an
// entry of an explicit list (`tasks`), or -- when `tasks` is NULL -- found from
// per-image offsets: task t belongs to the last image whose first task
// (`task_start[i]`, n_images + 1 entries) is <= t.  With `refine_base`, the
// level-9 images leave refinement to k_refine's batch mode (bc1_refine.cu),
// which runs after this kernel in the same stream: the same split as the
// plain level-9 launches, so lanes do not wait for each other's refinement.
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_encode_batch(const GlobalTables *G, const ImageDesc *images,
                                                                     const BatchTask *tasks, const uint32_t *task_start,
                                                                     int n_images, int ntasks, int *counter,
                                                                     const int64_t *refine_base, RefineSlot *slots) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, G);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(counter, 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= ntasks) break;
        BatchTask task;
        if (tasks) {
            task = tasks[t];
        } else {
            int lo = 0, hi = n_images;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if ((int)task_start[mid] <= t) lo = mid;
                else hi = mid;
            }
            task.image = (uint32_t)lo;
            task.first_block = (uint32_t)(t - (int)task_start[lo]) * 32u;
        }
        const ImageDesc &d = images[task.image];
        const int level = d.level;
        const int64_t b = (int64_t)task.first_block + lane;
        const bool active = b < d.nblocks;
        EncodeParams p;
        p.decoder = d.decoder;
        p.three_color_mode = d.three_color_mode;
        p.three_color_black = d.three_color_black;
        p.cw = v3(d.cw[0], d.cw[1], d.cw[2]);
        const WarpCtx w = warp_ctx<9>(smem, T, G, p.decoder);
        __syncwarp();
        if (active) load_image_block(d, b, w.in + lane * kInStride, T.lut255);
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
            case 0: e = encode_warp<0>(w, p, active, c0, c1, idx); break;
            case 1: e = encode_warp<1>(w, p, active, c0, c1, idx); break;
            case 2: e = encode_warp<2>(w, p, active, c0, c1, idx); break;
            case 3: e = encode_warp<3>(w, p, active, c0, c1, idx); break;
            case 4: e = encode_warp<4>(w, p, active, c0, c1, idx); break;
            case 5: e = encode_warp<5>(w, p, active, c0, c1, idx); break;
            case 6: e = encode_warp<6>(w, p, active, c0, c1, idx); break;
            case 7: e = encode_warp<7>(w, p, active, c0, c1, idx); break;
            case 8: e = encode_warp<8>(w, p, active, c0, c1, idx); break;
            default:
                if (base >= 0) e = encode_warp_ex<9, true>(w, float_row(w), p, active, c0, c1, idx, pending);
                else e = encode_warp<9>(w, p, active, c0, c1, idx);
                break;
        }
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
            if (base >= 0) slots[base + b] = RefineSlot{e, pending ? 1u : 0u};
        }
    }
}

cudaError_t launch_encode_batch(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                const uint32_t *task_start, int n_images, int ntasks, int *counter,
                                cudaStream_t stream, int grid, const int64_t *refine_base, RefineSlot *slots) {
    const size_t smem = smem_bytes(true);
    cudaError_t e = cudaFuncSetAttribute(k_encode_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_encode_batch<<<grid, kWarpsPerCta * 32, smem, stream>>>(G, images, tasks, task_start, n_images, ntasks, counter,
                                                               refine_base, slots);
    return cudaGetLastError();
}

int batch_ctas_per_sm() {
    int n = 0;
    const size_t smem = smem_bytes(true);
    cudaFuncSetAttribute(k_encode_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_encode_batch, kWarpsPerCta * 32, smem) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

}  // namespace icbc_gpu
