/*
 * icbc_gpu.h -- C ABI of the GB300 (sm_103a) BC1 encoder.
 *
 * Drop-in for the compress path of icbc (icbc.h v1.05): the same encoder,
 * bit-exact with the reference's scalar build, run as CUDA kernels over many
 * blocks at once.  Plain C types only: pointers, sizes, ints and floats.
 * Every entry point returns an icbc_gpu_status; nothing throws across the ABI.
 *
 * Pointers documented as "device" are CUDA device (or managed) memory owned by
 * the caller; "host" pointers are ordinary host memory.  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  Calls that
 * take a stream are asynchronous unless stated otherwise.
 *
 * Block layout (icbc.h:234-258): 8 bytes, little-endian
 *   u16 col0 (RGB565, r<<11 | g<<5 | b), u16 col1, u32 indices (texel i in bits 2i..2i+1).
 * Texel order inside a block is row-major: texel i = (x = i % 4, y = i / 4).
 */
#ifndef ICBC_GPU_H
#define ICBC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum icbc_gpu_status {
    ICBC_GPU_OK = 0,
    ICBC_GPU_ERR_INVALID_ARGUMENT = 1, /* bad level, decoder, size, flag or NULL pointer */
    ICBC_GPU_ERR_NOT_INITIALIZED = 2,  /* icbc_gpu_init has not run */
    ICBC_GPU_ERR_CUDA = 3,             /* a CUDA runtime call failed; see icbc_gpu_last_error */
    ICBC_GPU_ERR_OUT_OF_MEMORY = 4,    /* a device or pinned allocation failed */
    ICBC_GPU_ERR_MISALIGNED = 5,       /* a pointer or pitch breaks the documented alignment */
    ICBC_GPU_ERR_BUDGET = 6,           /* serving: request larger than the HBM budget */
    ICBC_GPU_ERR_NOT_READY = 7,        /* serving: result not finished yet */
    ICBC_GPU_ERR_CANCELLED = 8,        /* serving: request cancelled or server stopped */
    ICBC_GPU_ERR_NOT_FOUND = 9         /* serving: unknown request id */
};

/* Hardware decoders (values of icbc::Decoder, icbc.h:12-17). */
enum icbc_gpu_decoder {
    ICBC_GPU_DECODER_DEFAULT = -1,     /* the decoder chosen by icbc_gpu_init */
    ICBC_GPU_DECODER_D3D10 = 0,
    ICBC_GPU_DECODER_NVIDIA = 1,
    ICBC_GPU_DECODER_AMD = 2,
    ICBC_GPU_DECODER_INTEL = 3
};

/* Quality levels are icbc::Quality (icbc.h:21-36): 0..9, Fast = 1,
 * Default = 8, Max = 9. */
#define ICBC_GPU_QUALITY_FAST 1
#define ICBC_GPU_QUALITY_DEFAULT 8
#define ICBC_GPU_QUALITY_MAX 9

/* Where the per-texel input_weights of an RGBA8 image come from. */
enum icbc_gpu_weight_mode {
    ICBC_GPU_WEIGHTS_UNIFORM = 0,      /* 1.0f for every texel (icbc_test.cpp:405) */
    ICBC_GPU_WEIGHTS_ALPHA = 1,        /* alpha / 255.0f */
    ICBC_GPU_WEIGHTS_PLANE = 2         /* a float plane of width x height */
};

/* Uploads the init-time tables for all four decoders and selects `decoder`
 * as the default.  Replaces icbc::init (icbc.h:19, :3813-3818).  Safe to call
 * again (only the default decoder changes); serialised by an internal lock.
 * Must not race with encodes that use ICBC_GPU_DECODER_DEFAULT. */
int icbc_gpu_init(int decoder);

/* The default decoder, or -1 before icbc_gpu_init. */
int icbc_gpu_get_decoder(void);

/* Short text for a status code; the last CUDA error text of this thread. */
const char *icbc_gpu_status_string(int status);
const char *icbc_gpu_last_error(void);

/* Encodes n_blocks independent blocks.  Replaces n calls of
 * icbc::compress_bc1 (icbc.h:48, :3846-3848), each with the same arguments:
 *   d_colors  device, n_blocks x 16 texels x RGBA float (alpha ignored),
 *             16-byte aligned;
 *   d_weights device, n_blocks x 16 floats, 16-byte aligned, or NULL for 1.0f;
 *   color_weights host, 3 floats (the reference's color_weights[3]);
 *   d_out     device, n_blocks x 8 bytes, 8-byte aligned.  At levels 4..9 a
 *             block whose search finds no finite error keeps the bytes that
 *             were there, as the reference leaves its output untouched;
 *   d_errors  device, n_blocks floats or NULL: the value icbc::compress_bc1
 *             returns for each block (its weighted error).
 * decoder is ICBC_GPU_DECODER_DEFAULT or 0..3; level is 0..9. */
int icbc_gpu_compress_bc1_blocks(int level, const float *d_colors, const float *d_weights,
                                 const float color_weights[3], int three_color_mode,
                                 int three_color_black, int decoder, void *d_out, float *d_errors,
                                 int64_t n_blocks, void *stream);

/* One RGBA8 image and how to encode it. */
typedef struct icbc_gpu_image {
    const uint8_t *rgba;        /* device, RGBA8 rows */
    int32_t width, height;      /* >= 1 */
    int64_t pitch;              /* bytes between rows, >= 4 * width */
    int32_t weight_mode;        /* icbc_gpu_weight_mode */
    const float *weight_plane;  /* device, used with ICBC_GPU_WEIGHTS_PLANE */
    int64_t weight_pitch;       /* floats between weight-plane rows */
    int32_t level;              /* 0..9 */
    int32_t decoder;            /* ICBC_GPU_DECODER_DEFAULT or 0..3 */
    int32_t three_color_mode;
    int32_t three_color_black;
    float color_weights[3];
    void *out;                  /* device, ceil(w/4) * ceil(h/4) * 8 bytes, 8-byte aligned */
    float *errors;              /* device, one float per block, or NULL */
} icbc_gpu_image;

/* Encodes one image (plain form: one kernel launch).  Blocks are written in
 * row-major block order; partial blocks at the right and bottom edges
 * replicate the last column / row.  Texels convert as u8 / 255.0f with alpha
 * 1.0f, as icbc_test.cpp:398-406 does before calling compress_bc1. */
int icbc_gpu_compress_bc1_image(const icbc_gpu_image *image, void *stream);

/* ------------------------------------------------------------------------
 * SIMD profiles.  The reference gives slightly different blocks depending on
 * the SIMD backend it was compiled with (ICBC_SIMD, icbc.h:59-117): the
 * cluster-fit loops (icbc.h:2089-2344, :2362-2742) run over vectors of 4, 8
 * or 16 combinations whose lanes keep their own minimum, fuse vmadd/vmsub on
 * AVX2 and AVX-512 (icbc.h:734-752, :970-976), round vround01 half to even
 * from SSE4.1 on and on NEON (icbc.h:518-524, :764-766, :988-990,
 * :1159-1162), and on NEON keep a NaN through vsaturate (vmaxq_f32 /
 * vminq_f32, icbc.h:1155-1157).  These entry points reproduce the output of
 * such a build compiled without FP contraction (-ffp-contract=off; for NEON
 * that makes vmlaq_f32 / vmlsq_f32 a multiply then an add, icbc.h:1142-1153),
 * for callers whose stored assets came from one.  Profile
 * ICBC_GPU_SIMD_SCALAR (and levels 0-1, which have no cluster fit) is the
 * plain path.  Same arguments and results otherwise as
 * icbc_gpu_compress_bc1_blocks / icbc_gpu_compress_bc1_image, which they
 * replace for that build (icbc.h:48, :3846).  Values are ICBC_SIMD's.
 * ---------------------------------------------------------------------- */
enum {
    ICBC_GPU_SIMD_NEON = -1,  /* 4 lanes, half to even, vsaturate keeps NaN (ICBC_NEON) */
    ICBC_GPU_SIMD_SCALAR = 0, /* ICBC_SIMD=0 (the plain path) */
    ICBC_GPU_SIMD_SSE2 = 1,   /* 4 lanes, vround01 = int(x + 0.5f) */
    ICBC_GPU_SIMD_SSE41 = 2,  /* 4 lanes, half to even */
    ICBC_GPU_SIMD_AVX = 3,    /* 8 lanes, half to even */
    ICBC_GPU_SIMD_AVX2 = 4,   /* 8 lanes, half to even, fused vmadd/vmsub */
    ICBC_GPU_SIMD_AVX512 = 5  /* 16 lanes, half to even, fused vmadd/vmsub */
};
int icbc_gpu_compress_bc1_blocks_simd(int simd_profile, int level, const float *d_colors, const float *d_weights,
                                      const float color_weights[3], int three_color_mode, int three_color_black,
                                      int decoder, void *d_out, float *d_errors, int64_t n_blocks, void *stream);
int icbc_gpu_compress_bc1_image_simd(int simd_profile, const icbc_gpu_image *image, void *stream);

/* Batched form: many images of any size, level and decoder in one persistent
 * launch that drains a device work queue of (image, block range) tiles,
 * largest cost first.  A batch is planned once and can be launched many
 * times (the launch is a captured CUDA graph).  The image descriptors are
 * copied at create time; the pixel and output buffers they point to must stay
 * valid while the batch is launched. */
typedef struct icbc_gpu_batch icbc_gpu_batch;
int icbc_gpu_batch_create(const icbc_gpu_image *images, int n_images, icbc_gpu_batch **batch);
int icbc_gpu_batch_launch(icbc_gpu_batch *batch, void *stream);
int icbc_gpu_batch_destroy(icbc_gpu_batch *batch);
/* Convenience: create, launch on `stream`, synchronise, destroy. */
int icbc_gpu_compress_bc1_images(const icbc_gpu_image *images, int n_images, void *stream);

/* Plain form over many images: one kernel launch per image, in order, on
 * `stream` (what a caller looping over icbc_gpu_compress_bc1_image gets,
 * without per-call host overhead).  The reference for the batched form's
 * speed-up; same output. */
int icbc_gpu_compress_bc1_images_each(const icbc_gpu_image *images, int n_images, void *stream);

/* Largest batch icbc_gpu_compress_bc1_images_noalloc accepts. */
#define ICBC_GPU_NOALLOC_MAX_IMAGES 256

/* Batched encode that allocates nothing.  No counterpart in the reference:
 * icbc encodes one block per call on the CPU and owns no device memory.
 *
 * For callers that may not allocate device memory -- an engine or texture
 * streamer that reserves the whole device budget itself, code running inside
 * such an allocator, or a latency-critical path that cannot pay for
 * cudaMalloc/cudaFree, which can synchronise the device.  Encodes up to
 * ICBC_GPU_NOALLOC_MAX_IMAGES images of any size, level and decoder, with the
 * same output as icbc_gpu_compress_bc1_images, and calls no cudaMalloc,
 * cudaFree or other allocating routine: its work queue (image descriptors,
 * task offsets, queue counter) lives in one fixed array inside this library's
 * device code, about 38 KB with its tables, which every GPU that loads the
 * library holds until the process exits.  Inputs and outputs are the
 * caller's device buffers, as for icbc_gpu_compress_bc1_image.
 *   - More than ICBC_GPU_NOALLOC_MAX_IMAGES images: ICBC_GPU_ERR_INVALID_ARGUMENT,
 *     returned before any device work.
 *   - The first call on a device sets that device up (looks up the array's
 *     address, uploads the tables) synchronously, with the device current;
 *     make that first call before any stream capture.  icbc_gpu_init is not
 *     needed unless an image uses ICBC_GPU_DECODER_DEFAULT.
 *   - Asynchronous on `stream`; `images` may be reused once the call returns.
 *     The queue is planned in a static host record (about 27 KB, not on the
 *     caller's stack) and reaches the device as a kernel parameter, so no
 *     host memory of the call is read after it returns; host threads take
 *     turns on that record.
 *   - Every call shares the one array and each call clears its queue counter.
 *     Calls whose GPU work overlaps (unordered streams, concurrent host
 *     threads) race on the array and corrupt each other: order them. */
int icbc_gpu_compress_bc1_images_noalloc(const icbc_gpu_image *images, int n_images, void *stream);

/* Decodes n blocks to RGBA8 texels (64 bytes per block).  Replaces
 * icbc::decode_bc1 (icbc.h:38, :2915-2927). */
int icbc_gpu_decode_bc1(const void *d_blocks, uint8_t *d_rgba, int64_t n_blocks, int decoder,
                        void *stream);

/* Unweighted squared RGB error of n blocks against their RGBA8 texels
 * (64 bytes per block).  Replaces icbc::evaluate_bc1_error (icbc.h:43,
 * :3030-3046). */
int icbc_gpu_evaluate_bc1_error(const uint8_t *d_rgba, const void *d_blocks, float *d_errors,
                                int64_t n_blocks, int decoder, void *stream);

/* BC3 as the reference implements it (its BC3 encoder is not written:
 * icbc::compress_bc3 returns 0 without touching the block, icbc.h:3850-3853).
 * A 16-byte block is a BC4 alpha half (alpha0, alpha1, 6 index bytes) then a
 * BC1 block.  Decoding uses the colour block's 4-colour palette whatever the
 * endpoint order, and the reference's alpha index is always 0, so every texel
 * gets alpha0.  Replace icbc::decode_bc3 (icbc.h:39, :2929-2947) and
 * icbc::evaluate_bc3_error (icbc.h:44, :3048-3071): per texel, the squared
 * colour error (times alpha / 255 when alpha_blend) plus the squared alpha0
 * difference.  Blocks 16-byte aligned. */
int icbc_gpu_decode_bc3(const void *d_blocks, uint8_t *d_rgba, int64_t n_blocks, int decoder, void *stream);
int icbc_gpu_evaluate_bc3_error(const uint8_t *d_rgba, const void *d_blocks, float *d_errors, int64_t n_blocks,
                                int alpha_blend, int decoder, void *stream);

/* End-to-end call with HOST buffers: copies the image in, encodes, copies the
 * blocks (and errors if non-NULL) out, and returns when they are on the host.
 * rgba is host memory (pitch bytes per row), weight_plane host floats
 * (width per row) or NULL.  Synchronous. */
int icbc_gpu_compress_bc1_image_host(const uint8_t *rgba, int32_t width, int32_t height, int64_t pitch,
                                     int32_t weight_mode, const float *weight_plane, int32_t level,
                                     int32_t decoder, int32_t three_color_mode, int32_t three_color_black,
                                     const float color_weights[3], void *out, float *errors);

/* ------------------------------------------------------------------------
 * Serving form (no counterpart in the reference, which encodes on the
 * caller's thread): a request loop that batches encode requests of any size
 * and level as they arrive.  Texels and blocks are staged in one device arena
 * of hbm_budget_bytes allocated at create (per request: its texels at rows
 * of 16-byte multiples, 8 bytes per block, 4 per block for errors if asked,
 * and 4 per block of working space at levels 2-9, each rounded up to 256
 * bytes); a request is admitted (FIFO) once
 * its bytes fit in the arena, so requests that arrive while others run join
 * the next batched launch as memory frees up, and up to max_inflight batches
 * run on the GPU at once.  Results equal the single-image encode bit for bit.
 * ---------------------------------------------------------------------- */
typedef struct icbc_gpu_server icbc_gpu_server;

typedef struct icbc_gpu_server_config {
    int64_t hbm_budget_bytes;   /* device arena for staged texels and blocks (> 0) */
    int32_t max_inflight;       /* batched launches on the GPU at once (1..8) */
    int32_t max_batch_images;   /* images per batched launch (1..4096) */
} icbc_gpu_server_config;

/* One encode request.  Host buffers stay owned by the caller and must stay
 * valid until the request completes or is cancelled. */
typedef struct icbc_gpu_request {
    const uint8_t *rgba;        /* host RGBA8 rows */
    int32_t width, height;
    int64_t pitch;              /* bytes between rows */
    int32_t weight_mode;        /* ICBC_GPU_WEIGHTS_UNIFORM or _ALPHA */
    int32_t level, decoder, three_color_mode, three_color_black;
    float color_weights[3];
    void *out;                  /* host, ceil(w/4) * ceil(h/4) * 8 bytes, written on completion */
    float *errors;              /* host, one float per block, or NULL */
} icbc_gpu_request;

typedef struct icbc_gpu_server_stats {
    int64_t submitted, completed, rejected, cancelled, failed;
    int64_t pending, in_flight, batches;
    int64_t arena_bytes, arena_used, arena_peak;
    double pixels_completed;
    double latency_mean_ms, latency_p50_ms, latency_p99_ms, latency_max_ms;  /* submit -> blocks on host */
} icbc_gpu_server_stats;

/* Creates the server on the current device: allocates the arena and pinned
 * staging, starts the scheduler thread (admission, launches) and the
 * delivery thread (finished blocks into the callers' buffers). */
int icbc_gpu_server_create(const icbc_gpu_server_config *config, icbc_gpu_server **server);
/* Queues a request; returns its id.  The texels are copied to pinned staging
 * on the calling thread when there is room (else at launch, from `rgba`).
 * ICBC_GPU_ERR_BUDGET if it can never fit in the arena,
 * ICBC_GPU_ERR_INVALID_ARGUMENT for a malformed request.  Thread-safe. */
int icbc_gpu_server_submit(icbc_gpu_server *server, const icbc_gpu_request *request, uint64_t *id);
/* ICBC_GPU_OK when done, ICBC_GPU_ERR_NOT_READY while queued or running,
 * ICBC_GPU_ERR_CANCELLED, ICBC_GPU_ERR_NOT_FOUND, or the failure status. */
int icbc_gpu_server_poll(icbc_gpu_server *server, uint64_t id);
/* As poll, blocking up to timeout_ms (< 0: no limit). */
int icbc_gpu_server_wait(icbc_gpu_server *server, uint64_t id, int32_t timeout_ms);
/* Cancels a request that has not been admitted yet (ICBC_GPU_ERR_NOT_READY if
 * it is already on the GPU). */
int icbc_gpu_server_cancel(icbc_gpu_server *server, uint64_t id);
int icbc_gpu_server_get_stats(icbc_gpu_server *server, icbc_gpu_server_stats *stats);
/* Stops the scheduler; pending requests are cancelled, running ones finish.
 * Must not run concurrently with other calls on the same server. */
int icbc_gpu_server_destroy(icbc_gpu_server *server);

/* ------------------------------------------------------------------------
 * Containers for encoded images (icbc_test.cpp:155-279).  `blocks` are
 * ceil(w/4) * ceil(h/4) BC1 blocks in row-major block order, in host or
 * device memory (device blocks are copied out first, after the caller has
 * synchronised the stream that wrote them).  Headers hold the image's own
 * width and height; the data size is 8 bytes per block.
 * ---------------------------------------------------------------------- */
/* DDS with a DXT1 FourCC and one mip level (icbc_test.cpp:155-211). */
int icbc_gpu_write_dds(const char *path, int32_t width, int32_t height, const void *blocks);
/* DDS of a whole mip chain: `levels` levels (as icbc_gpu_mip_layout lays
 * them out, level 0 first, blocks contiguous), mip count and mipmap caps set. */
int icbc_gpu_write_dds_mips(const char *path, int32_t width, int32_t height, int32_t levels, const void *blocks);
/* KTX 1.1, GL_COMPRESSED_RGB_S3TC_DXT1_EXT (icbc_test.cpp:233-279). */
int icbc_gpu_write_ktx(const char *path, int32_t width, int32_t height, const void *blocks);
/* Golden-file check (icbc_test.cpp:213-231): 1 when the DDS file's block
 * data equals `blocks`, 0 when it differs, a negative status on error
 * (-ICBC_GPU_ERR_NOT_FOUND: file missing or short). */
int icbc_gpu_compare_dds(const char *path, int32_t width, int32_t height, const void *blocks);

/* ------------------------------------------------------------------------
 * Input side.  The reference's driver decodes files with
 * stbi_load(..., 4) (icbc_test.cpp:345): 1..4-channel 8-bit pixels expanded
 * to RGBA8.  icbc_gpu_expand_rgba8 does that expansion on the device (grey ->
 * (g, g, g, 255), grey + alpha -> (g, g, g, a), RGB -> (r, g, b, 255), RGBA as
 * is), so decoded pixels are uploaded as they are.  (The driver also drops
 * partial edge blocks, icbc_test.cpp:353-358; pass width & ~3 and
 * height & ~3 to get that.)
 *
 * Mip chains (no counterpart in the reference, which encodes one level; the
 * role of its callers' texture pipelines): level k + 1 is
 * max(1, w >> 1) x max(1, h >> 1), each channel (a + b + c + d + 2) >> 2 over
 * the 2x2 source texels (2x, 2y) .. (2x + 1, 2y + 1), coordinates clamped to
 * the source.  Levels down to 1 x 1: icbc_gpu_mip_levels(w, h).
 * ---------------------------------------------------------------------- */
int icbc_gpu_expand_rgba8(const uint8_t *d_src, int32_t channels, int32_t width, int32_t height, int64_t src_pitch,
                          uint8_t *d_rgba, int64_t rgba_pitch, void *stream);
int icbc_gpu_mip_levels(int32_t width, int32_t height);
/* Sizes of levels 0..levels-1 and the first block of each in a chain's block
 * array (levels + 1 offsets; the last is the total).  Any output may be NULL. */
int icbc_gpu_mip_layout(int32_t width, int32_t height, int32_t levels, int32_t *widths, int32_t *heights,
                        int64_t *block_offsets);
/* Levels 1..levels-1 of d_rgba into d_chain, each tightly packed (pitch
 * 4 * width), one after another.  Device pointers, 4-byte aligned. */
int icbc_gpu_build_mips(const uint8_t *d_rgba, int32_t width, int32_t height, int64_t pitch, int32_t levels,
                        uint8_t *d_chain, void *stream);
/* Builds the chain of `image` and encodes its `levels` levels in one batch
 * with the image's level, decoder, flags, colour weights and weight mode
 * (uniform or alpha).  image->out (and image->errors, if set) receive every
 * level's blocks at icbc_gpu_mip_layout's offsets.  Synchronous. */
int icbc_gpu_compress_bc1_mips(const icbc_gpu_image *image, int32_t levels, void *stream);

/* Launch shape of the kernels of one quality level, chosen by an autotuner
 * (icbc_gb300.autotune, icbc_gb300.autotune_batch) or set by hand.
 * groups_per_warp: groups of 32 blocks each warp takes (1..64); persistent:
 * 1 = exactly the resident CTAs, striding over the image, 0 = enough CTAs for
 * the work, balanced by the hardware.  cta_warps (levels 2-9, RGBA8 images
 * with uniform or alpha weights: the pass that encodes the blocks of two or
 * more colours) and batch_cta_warps (the same for the batched form's kernel
 * of that level, read when a batch is created): 4 = CTAs of 4 warps,
 * each warp searching its own 32 blocks' cluster combinations; 8 or 16 =
 * CTAs of that many warps moving through the encoder's stages together, the
 * combinations of all the CTA's blocks searched by all its threads (an image
 * too small for two rounds of such CTAs on every SM takes 4); 0 = the
 * level's default.  Defaults: 1 / persistent at levels 0-1, 2 / not
 * persistent at levels 2-9, cta_warps 16 from level 4 on (else 4),
 * batch_cta_warps 4.  Not for use while launches run or batches are
 * created. */
typedef struct icbc_gpu_launch_config {
    int32_t groups_per_warp;
    int32_t persistent;
    int32_t cta_warps;
    int32_t batch_cta_warps;  /* 0 = 4 */
} icbc_gpu_launch_config;
int icbc_gpu_set_launch_config(int level, const icbc_gpu_launch_config *config);
int icbc_gpu_get_launch_config(int level, icbc_gpu_launch_config *config);

/* Number of SMs of the current device (for sizing host-side work). */
int icbc_gpu_sm_count(void);

/* Diagnostics, host only (no CUDA call): copies the init-time tables the
 * library builds -- the single-colour match tables of a decoder
 * (s_match5/s_match6, icbc.h:3374-3375, as [256][2] {max, min}), its cluster
 * weights {w1_3, w2_3, w1_9, w4_9, w2_9} (icbc.h:1961-1962) and the cluster
 * enumerations packed c0 | c1 << 8 | c2 << 16 with their prefix totals
 * (icbc.h:1947-1950).  Any output pointer may be NULL. */
int icbc_gpu_debug_tables(int decoder, uint8_t match5[512], uint8_t match6[512], float weights[5],
                          uint32_t four[968], int32_t four_total[16], uint32_t three[152],
                          int32_t three_total[16]);

#ifdef __cplusplus
}
#endif

#endif /* ICBC_GPU_H */
