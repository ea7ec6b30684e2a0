// bc1_batch.cu -- persistent batched encoder over mixed images, levels and
// decoders.  -fmad=false as for every encoder translation unit.  Compiled
// twice: -DICBC_BATCH_BYTES=1 keeps texels as bytes (batches without weight
// planes: four CTAs per SM, as the plain image kernels), =0 as floats.
#include <cuda_runtime.h>

#include "bc1_batch_task.cuh"

#ifndef ICBC_BATCH_BYTES
#error "compile with -DICBC_BATCH_BYTES=<0|1>"
#endif

namespace icbc_gpu {

constexpr bool kBytes = ICBC_BATCH_BYTES != 0;

// Persistent batched encoder over mixed levels and decoders: every warp
// takes the next task (32 blocks of one image) from an atomic counter until
// the queue is empty (run_batch); tasks are ordered most expensive level
// first by the planner.
template <bool BYTES>
__global__ void __launch_bounds__(kWarpsPerCta * 32, BYTES ? 4 : 1)
    k_encode_batch(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks, const uint32_t *task_start,
                   int n_images, int ntasks, int *counter, const int64_t *refine_base, RefineSlot *slots,
                   BatchLists lists) {
    extern __shared__ __align__(16) unsigned char smem[];
    run_batch<BYTES, -1>(G, smem, images, tasks, task_start, n_images, 0, ntasks, counter, refine_base, slots, lists);
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

// CTAs of k_batch_trivial per SM; the query also loads the kernel's code
// (modules load on first use), so a caller can take that cost up front.
static int batch_trivial_resident() {
    static int resident = 0;
    if (!resident &&
        (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_batch_trivial, kWarpsPerCta * 32, 0) !=
             cudaSuccess ||
         resident < 1))
        resident = 1;
    return resident;
}

void prepare_batch_trivial() { batch_trivial_resident(); }

cudaError_t launch_batch_trivial(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                 const uint32_t *task_start, int n_images, int ntasks, BatchLists lists,
                                 const int64_t *refine_base, RefineSlot *slots, cudaStream_t stream, int sms) {
    if (ntasks <= 0) return cudaSuccess;
    const int resident = batch_trivial_resident();
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
