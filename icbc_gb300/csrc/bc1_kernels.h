// bc1_kernels.h -- launcher interface between the host API and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/icbc_gpu.h"
#include "bc1_encode.cuh"

namespace icbc_gpu {

// Float-block source (the compress_bc1 layout): colors n x 16 x RGBA floats,
// weights n x 16 floats or NULL.  Both 16-byte aligned.
struct BlocksSrc {
    const float *colors;
    const float *weights;
};

// An RGBA8 image resolved for the kernels.
struct ImageDesc {
    const uint8_t *rgba;
    int64_t pitch;
    const float *weight_plane;
    int64_t weight_pitch;
    uint2 *out;
    float *errors;
    int64_t nblocks;
    int width, height, bw;
    int weight_mode;
    int vec16;  // rgba and pitch are 16-byte aligned: whole rows of a block load as one uint4
    int level, decoder, three_color_mode, three_color_black;
    float cw[3];
};

// A warp's unit of batched work: 32 consecutive blocks of one image.
struct BatchTask {
    uint32_t image;
    uint32_t first_block;
};

using BlocksLauncher = cudaError_t (*)(const GlobalTables *, const BlocksSrc &, const EncodeParams &, void *, float *,
                                       int64_t, cudaStream_t, int);
using ImageLauncher = cudaError_t (*)(const GlobalTables *, const ImageDesc &, const EncodeParams &, cudaStream_t, int);
using ImageLauncherExt = cudaError_t (*)(const GlobalTables *, const ImageDesc &, const EncodeParams &, cudaStream_t,
                                         int, RefineSlot *, unsigned long long *);

#define ICBC_DECLARE_LEVEL(L)                                                                                    \
    cudaError_t launch_blocks_l##L(const GlobalTables *, const BlocksSrc &, const EncodeParams &, void *, float *, \
                                   int64_t, cudaStream_t, int);                                                  \
    cudaError_t launch_image_l##L(const GlobalTables *, const ImageDesc &, const EncodeParams &, cudaStream_t, int); \
    cudaError_t launch_image_ext_l##L(const GlobalTables *, const ImageDesc &, const EncodeParams &, cudaStream_t, int, \
                                      RefineSlot *, unsigned long long *);
ICBC_DECLARE_LEVEL(0)
ICBC_DECLARE_LEVEL(1)
ICBC_DECLARE_LEVEL(2)
ICBC_DECLARE_LEVEL(3)
ICBC_DECLARE_LEVEL(4)
ICBC_DECLARE_LEVEL(5)
ICBC_DECLARE_LEVEL(6)
ICBC_DECLARE_LEVEL(7)
ICBC_DECLARE_LEVEL(8)
ICBC_DECLARE_LEVEL(9)
#undef ICBC_DECLARE_LEVEL

// With refine_base (one entry per image; -1: refine inline) a level-9 image's
// refinement is deferred: block b's RefineSlot goes to slots[refine_base[i] + b]
// and launch_refine_batch finishes it.  NULL refine_base: all inline.
// The blocks the first pass of a two-pass batch left to the second: image
// i's are list[list_base[i] .. list_base[i] + listed[i]) (list_base[i] < 0:
// the image is not in two passes and its tasks cover its blocks in order).
struct BatchLists {
    uint32_t *list;
    unsigned int *listed;
    const int64_t *list_base;
};

// The batched form's kernel for the tasks task0 .. task0 + ntasks - 1 of a
// byte-row batch, all of one level (each level's own code, compiled with
// that level's plain kernels); otherwise as launch_encode_batch.
using BatchLevelLauncher = cudaError_t (*)(const GlobalTables *, const ImageDesc *, const BatchTask *, int, int, int *,
                                           cudaStream_t, int, const int64_t *, RefineSlot *, BatchLists);
#define ICBC_DECLARE_BATCH_LEVEL(L)                                                                                \
    cudaError_t launch_batch_level_l##L(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,     \
                                        int task0, int ntasks, int *counter, cudaStream_t stream, int grid,        \
                                        const int64_t *refine_base, RefineSlot *slots, BatchLists lists);
ICBC_DECLARE_BATCH_LEVEL(0)
ICBC_DECLARE_BATCH_LEVEL(1)
ICBC_DECLARE_BATCH_LEVEL(2)
ICBC_DECLARE_BATCH_LEVEL(3)
ICBC_DECLARE_BATCH_LEVEL(4)
ICBC_DECLARE_BATCH_LEVEL(5)
ICBC_DECLARE_BATCH_LEVEL(6)
ICBC_DECLARE_BATCH_LEVEL(7)
ICBC_DECLARE_BATCH_LEVEL(8)
ICBC_DECLARE_BATCH_LEVEL(9)
#undef ICBC_DECLARE_BATCH_LEVEL

// byte_rows: the kernel with byte texel rows (no image of the batch has a
// weight plane), four CTAs per SM; else float rows.  With lists.list, the
// tasks of listed images take their blocks from the lists.
cudaError_t launch_encode_batch_float(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                      const uint32_t *task_start, int n_images, int ntasks, int *counter,
                                      cudaStream_t stream, int grid, const int64_t *refine_base, RefineSlot *slots,
                                      BatchLists lists);
cudaError_t launch_encode_batch_bytes(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                      const uint32_t *task_start, int n_images, int ntasks, int *counter,
                                      cudaStream_t stream, int grid, const int64_t *refine_base, RefineSlot *slots,
                                      BatchLists lists);
int batch_ctas_per_sm_float();
int batch_ctas_per_sm_bytes();
inline cudaError_t launch_encode_batch(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                       const uint32_t *task_start, int n_images, int ntasks, int *counter,
                                       cudaStream_t stream, int grid, const int64_t *refine_base = nullptr,
                                       RefineSlot *slots = nullptr, bool byte_rows = false,
                                       BatchLists lists = BatchLists{nullptr, nullptr, nullptr}) {
    return byte_rows ? launch_encode_batch_bytes(G, images, tasks, task_start, n_images, ntasks, counter, stream, grid,
                                                 refine_base, slots, lists)
                     : launch_encode_batch_float(G, images, tasks, task_start, n_images, ntasks, counter, stream, grid,
                                                 refine_base, slots, lists);
}
// First pass of a two-pass batch (byte rows): finishes the blocks of 0 or 1
// reduced colours of the images with list_base >= 0 (level-9 ones with an
// empty refinement slot) and lists the rest.  A grid stride over the first
// ntasks tasks (`tasks`, or per-image offsets as for launch_encode_batch).
cudaError_t launch_batch_trivial(const GlobalTables *G, const ImageDesc *images, const BatchTask *tasks,
                                 const uint32_t *task_start, int n_images, int ntasks, BatchLists lists,
                                 const int64_t *refine_base, RefineSlot *slots, cudaStream_t stream, int sms);
// Loads launch_batch_trivial's kernel (which otherwise loads on its first launch).
void prepare_batch_trivial();
inline int batch_ctas_per_sm(bool byte_rows = false) {
    return byte_rows ? batch_ctas_per_sm_bytes() : batch_ctas_per_sm_float();
}
cudaError_t launch_decode(const void *blocks, void *rgba, int64_t n, int decoder, cudaStream_t stream);
cudaError_t launch_evaluate(const void *rgba, const void *blocks, float *errors, int64_t n, int decoder,
                            cudaStream_t stream);
cudaError_t launch_decode_bc3(const void *blocks, void *rgba, int64_t n, int decoder, cudaStream_t stream);
cudaError_t launch_evaluate_bc3(const void *rgba, const void *blocks, float *errors, int64_t n, int alpha_blend,
                                int decoder, cudaStream_t stream);

// Level-9 refinement pass (bc1_refine.cu) and its stream-ordered scratch.
cudaError_t scratch_alloc(void **ptr, size_t bytes, cudaStream_t stream);
cudaError_t scratch_prepare();
cudaError_t scratch_free(void *ptr, cudaStream_t stream);
cudaError_t launch_refine(const GlobalTables *G, const ImageDesc *image, const BlocksSrc *blocks,
                          const EncodeParams &p, uint2 *out, float *errors, const RefineSlot *st, int64_t n,
                          unsigned long long *counter, cudaStream_t stream, int sms);

// The deferred level-9 blocks of a batch: refinement index r belongs to image
// map_image[k] for the k with map_start[k] <= r < map_start[k + 1] (n + 1
// entries), block r - map_start[k]; slots[r] is its hand-over.
struct RefineMap {
    const int64_t *map_start;
    const uint32_t *map_image;
    int n;
};
cudaError_t launch_refine_batch(const GlobalTables *G, const ImageDesc *images, RefineMap map,
                                const RefineSlot *slots, int64_t total, unsigned long long *counter,
                                cudaStream_t stream, int sms);

// The SIMD-profile encoder (bc1_simd.cu), levels 2..9: an image (`image`)
// or float blocks (`blocks`), p.simd_* set.
cudaError_t launch_simd(const GlobalTables *G, const ImageDesc *image, const BlocksSrc *blocks, const EncodeParams &p,
                        uint2 *out, float *errors, int64_t n, int level, cudaStream_t stream);

// Launch shape of the plain kernels of a level (autotuned or default).
struct LaunchShape {
    int groups_per_warp;
    bool persistent;
    int cta_warps;        // the listed pass's CTA size (0: the level's default)
    int batch_cta_warps;  // the batched form's per-level kernel's (0: 4)
};
LaunchShape launch_shape(int level);

// Host-side services of icbc_gpu_api.cu used by other translation units.
const GlobalTables &host_tables();
int ensure_tables_on_device(const GlobalTables **out);
int resolve_image_desc_checked(const icbc_gpu_image &image, ImageDesc &desc);
int level_cost(int level);
int current_sm_count();

}  // namespace icbc_gpu
