// bc1_noalloc.cu -- batched BC1 encode that allocates no memory.
//
// Some callers cannot allocate device memory: an engine or texture streamer
// that reserves the whole device budget up front and hands out every byte
// itself, code that runs inside such an allocator's callbacks, or a
// latency-critical path that cannot afford cudaMalloc/cudaFree (both may
// synchronise the device).  The regular batched form (icbc_gpu_batch_create)
// allocates a work queue per batch, so it is closed to them.
//
// icbc_gpu_compress_bc1_images_noalloc gives them the same encode with no
// allocation at all: its work queue -- the image descriptors, the first task
// of every image and the queue counter -- lives in g_noalloc_scratch, one
// file-scope __device__ array sized for ICBC_GPU_NOALLOC_MAX_IMAGES images,
// and its tables in g_noalloc_tables.  Both are part of the loaded module, so
// every GPU that loads this library holds them (about 38 KB) until the process
// exits.  The caller passes device inputs and outputs as for the other forms.
//
// A call plans its queue on the host in one static staging record (guarded by
// a mutex, so no stack or heap is used for it) and hands it to the GPU as the
// by-value parameter of a small staging kernel, which writes it into the
// array and clears the counter; the encode kernel follows in stream order.
// Nothing on the GPU refers to host memory of the call once it has returned.
//
// All calls share the one array and it keeps the last call's contents: each
// call rewrites the descriptors and offsets it uses and clears the counter.
// Calls whose GPU work overlaps (different streams without ordering, or two
// host threads) race on the array and give wrong results; order them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/icbc_gpu.h"
#include "bc1_loaders.cuh"

namespace icbc_gpu {

int resolve_image_desc(const icbc_gpu_image &image, ImageDesc &desc);

namespace {

struct NoAllocQueue {
    ImageDesc images[ICBC_GPU_NOALLOC_MAX_IMAGES];
    uint32_t task_start[ICBC_GPU_NOALLOC_MAX_IMAGES + 1];  // first task of image i; [n] = total
    int counter;                                            // next task to hand out
};

// The scratch of every call.  In host code this name is only a stand-in for
// the symbol, never a device address: the address comes from
// cudaGetSymbolAddress at set-up.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocQueue)];
static __device__ __align__(16) GlobalTables g_noalloc_tables;

// One call's queue as planned on the host: passed by value as a kernel
// parameter (within the 32,764-byte parameter limit), so the launch itself
// carries it to the device.
struct NoAllocPlan {
    ImageDesc images[ICBC_GPU_NOALLOC_MAX_IMAGES];
    uint32_t task_start[ICBC_GPU_NOALLOC_MAX_IMAGES + 1];
    int n_images;
};
static_assert(sizeof(NoAllocPlan) <= 32000, "the plan must fit in a kernel parameter");

// Writes the plan's first n_images descriptors and n_images + 1 offsets into
// the scratch array and clears the queue counter (device code names the array
// directly).
__global__ void k_noalloc_stage(const __grid_constant__ NoAllocPlan plan) {
    NoAllocQueue *q = reinterpret_cast<NoAllocQueue *>(g_noalloc_scratch);
    const int n = plan.n_images;
    for (int i = threadIdx.x; i < n; i += blockDim.x) q->images[i] = plan.images[i];
    for (int i = threadIdx.x; i <= n; i += blockDim.x) q->task_start[i] = plan.task_start[i];
    if (threadIdx.x == 0) q->counter = 0;
}

// Same work loop as k_encode_batch, with tasks found from per-image offsets
// instead of an allocated task list: task t belongs to the last image whose
// first task is <= t.
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_encode_batch_noalloc(NoAllocQueue *q, int n_images,
                                                                             int total_tasks) {
    extern __shared__ __align__(16) unsigned char smem[];
    SharedTables &T = *reinterpret_cast<SharedTables *>(smem);
    stage_tables(T, &g_noalloc_tables);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&q->counter, 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total_tasks) break;
        int lo = 0, hi = n_images;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if ((int)q->task_start[mid] <= t) lo = mid;
            else hi = mid;
        }
        const ImageDesc &d = q->images[lo];
        const int level = d.level;
        const int64_t b = (int64_t)(t - (int)q->task_start[lo]) * 32 + lane;
        const bool active = b < d.nblocks;
        EncodeParams p;
        p.decoder = d.decoder;
        p.three_color_mode = d.three_color_mode;
        p.three_color_black = d.three_color_black;
        p.cw = v3(d.cw[0], d.cw[1], d.cw[2]);
        const WarpCtx w = warp_ctx<9>(smem, T, &g_noalloc_tables, p.decoder);
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
            default: e = encode_warp<9>(w, p, active, c0, c1, idx); break;
        }
        if (active) {
            d.out[b] = make_uint2(c0 | (c1 << 16), idx);
            if (d.errors) d.errors[b] = e;
        }
    }
}

// Status of a failed CUDA call, without touching the library's error text
// (which lives in a heap-allocated string); cudaGetLastError still has it.
int cuda_status(cudaError_t e) {
    return e == cudaErrorMemoryAllocation ? ICBC_GPU_ERR_OUT_OF_MEMORY : ICBC_GPU_ERR_CUDA;
}

struct DeviceState {
    NoAllocQueue *queue = nullptr;  // device address of g_noalloc_scratch on this device
    int grid = 0;
};

std::mutex g_setup_mutex;
DeviceState g_state[64];

// Once per device, with that device current: the scratch address, the
// tables, the kernel's shared-memory limit and its persistent grid size.
int setup_current_device(DeviceState *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e);
    if (dev < 0 || dev >= 64) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceState &S = g_state[dev];
    if (!S.queue) {
        NoAllocQueue *ptr = nullptr;
        e = cudaGetSymbolAddress(reinterpret_cast<void **>(&ptr), g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e);
        e = cudaMemcpyToSymbol(g_noalloc_tables, &host_tables(), sizeof(GlobalTables), 0, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_status(e);
        const int smem = (int)smem_bytes(true);
        e = cudaFuncSetAttribute(k_encode_batch_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return cuda_status(e);
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_encode_batch_noalloc, kWarpsPerCta * 32, smem);
        if (e != cudaSuccess) return cuda_status(e);
        S.grid = current_sm_count() * (per_sm > 0 ? per_sm : 1);
        S.queue = ptr;
    }
    *out = S;
    return ICBC_GPU_OK;
}

}  // namespace
}  // namespace icbc_gpu

using namespace icbc_gpu;

namespace {
// The host staging record of every call (about 27 KB), outside any stack.
std::mutex g_plan_mutex;
icbc_gpu::NoAllocPlan g_plan;
}  // namespace

extern "C" int icbc_gpu_compress_bc1_images_noalloc(const icbc_gpu_image *images, int n_images, void *stream) {
    if (n_images < 0 || (n_images > 0 && !images)) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_images > ICBC_GPU_NOALLOC_MAX_IMAGES) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_images == 0) return ICBC_GPU_OK;
    DeviceState S;
    int st = setup_current_device(&S);
    if (st) return st;
    std::lock_guard<std::mutex> lock(g_plan_mutex);
    // Descriptors most expensive level first (larger images first inside a
    // level), as the allocated batch orders them, then each image's first task.
    ImageDesc *descs = g_plan.images;
    for (int i = 0; i < n_images; i++) {
        st = resolve_image_desc(images[i], descs[i]);
        if (st) return st;
    }
    for (int i = 1; i < n_images; i++) {
        const ImageDesc key = descs[i];
        int j = i - 1;
        while (j >= 0 && (level_cost(descs[j].level) < level_cost(key.level) ||
                          (level_cost(descs[j].level) == level_cost(key.level) && descs[j].nblocks < key.nblocks))) {
            descs[j + 1] = descs[j];
            j--;
        }
        descs[j + 1] = key;
    }
    int64_t total = 0;
    for (int i = 0; i < n_images; i++) {
        g_plan.task_start[i] = (uint32_t)total;
        total += (descs[i].nblocks + 31) / 32;
        if (total > 0x7fffffff) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    }
    g_plan.task_start[n_images] = (uint32_t)total;
    g_plan.n_images = n_images;

    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // The launch copies the plan; g_plan may be rewritten once it returns.
    k_noalloc_stage<<<1, 256, 0, s>>>(g_plan);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    k_encode_batch_noalloc<<<S.grid, kWarpsPerCta * 32, smem_bytes(true), s>>>(S.queue, n_images, (int)total);
    e = cudaGetLastError();
    return e == cudaSuccess ? ICBC_GPU_OK : cuda_status(e);
}
