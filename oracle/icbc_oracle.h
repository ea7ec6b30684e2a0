/*
 * icbc_oracle.h -- CPU restatement of icbc's BC1 compress path (scalar profile).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU encoder is compared
 * against and the CPU baseline that bench.py times; no product code path may
 * link, load or call it.  Parity of this restatement with the reference is
 * pinned two ways: against the reference's own icbc.h compiled unmodified in
 * its scalar profile (oracle/build_ref.sh -> oracle/_ref/, where the reference
 * sources are present) and against the committed golden vectors in
 * tests/golden/ that the same compiled reference produced.
 *
 * Semantics follow icbc.h v1.05 compiled with ICBC_SIMD=0 and FP contraction
 * off: every float operation is an IEEE binary32 operation in the order the
 * reference writes it.  Build with -ffp-contract=off (no FMA fusion).
 */
#ifndef ICBC_ORACLE_H
#define ICBC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Decoder and quality enums keep the reference's values (icbc.h:12-36). */
enum { ORACLE_D3D10 = 0, ORACLE_NVIDIA = 1, ORACLE_AMD = 2, ORACLE_INTEL = 3 };

/* Every `decoder` argument below may carry a SIMD profile of the reference
 * in bits 8..10: (profile << ORACLE_PROFILE_SHIFT) | decoder.  Profile 0 is
 * the scalar build (ICBC_SIMD=0); 1..5 reproduce the cluster-fit loops of the
 * ICBC_SSE2, ICBC_SSE41, ICBC_AVX1, ICBC_AVX2 and ICBC_AVX512 builds (vector
 * width, lane tie-break, fused vmadd/vmsub, vround01 rounding), and 6 those of
 * the ICBC_NEON build (ICBC_SIMD=-1: four lanes, half-even rounding, NaN kept
 * by vsaturate), each compiled without FP contraction.  Nothing else in the
 * encoder depends on ICBC_SIMD. */
#define ORACLE_PROFILE_SHIFT 8
/* With a 4-lane profile (SSE2, SSE4.1, NEON), this bit of `decoder` runs the
 * cluster loops as 4-lane vector code: the same results, a vectorised CPU
 * encoder to time.  Ignored with the other profiles. */
#define ORACLE_VECTOR_LOOPS (1 << 11)
enum { ORACLE_SCALAR = 0, ORACLE_SSE2 = 1, ORACLE_SSE41 = 2, ORACLE_AVX1 = 3, ORACLE_AVX2 = 4, ORACLE_AVX512 = 5,
       ORACLE_NEON = 6 };

/* Per-block work counters used to derive the algorithmic FP32 operation
 * count of a workload (units of the reference's scalar inner loops). */
typedef struct {
    int64_t blocks;          /* blocks encoded */
    int64_t zero_blocks;     /* count == 0 path (icbc.h:3752) */
    int64_t single_blocks;   /* count == 1 path (icbc.h:3761) */
    int64_t reduce_pairs;    /* equal() tests in reduce_colors (icbc.h:1703) */
    int64_t reduce_merges;   /* merges in reduce_colors (icbc.h:1705) */
    int64_t sat_builds;      /* compute_sat calls (icbc.h:1857) */
    int64_t sat_points;      /* sum of counts over compute_sat calls */
    int64_t cf4_combos;      /* cluster_fit_four iterations (icbc.h:2362) */
    int64_t cf3_combos;      /* cluster_fit_three iterations (icbc.h:2089) */
    int64_t out4_blocks;     /* output_block4 calls (icbc.h:3257) */
    int64_t out3_blocks;     /* output_block3 calls (icbc.h:3238) */
    int64_t box_fits;        /* fit_colors_bbox+inset+select_diagonal (icbc.h:3769-3773) */
    int64_t box_points;      /* sum of counts over box fits */
    int64_t lsq_fits;        /* optimize_end_points4 calls (icbc.h:3278) */
    int64_t refine_steps;    /* refine_endpoints iterations (icbc.h:3614) */
} oracle_stats;

/* Builds every decoder's tables; idempotent and thread-safe
 * (the reference's init, icbc.h:3813-3818, for all four decoders at once). */
void oracle_init(void);

/* One block: icbc::compress_bc1 (icbc.h:3846-3848 -> :3734-3808) with the
 * decoder that icbc::init(decoder) would have selected.  colors = 16 x RGBA
 * float, weights = 16 floats, out = 8 bytes.  Returns the weighted error. */
float oracle_compress_bc1(int decoder, int level, const float *colors,
                          const float *weights, const float color_weights[3],
                          int three_color_mode, int three_color_black,
                          void *out, oracle_stats *stats);

/* n blocks over nthreads host threads, chunks of 32 blocks taken from an
 * atomic counter as icbc_test.cpp:397 / ic_pfor.h:669-681 do.
 * colors: n*64 floats, weights: n*16 floats (NULL = all 1.0f),
 * errors: n floats or NULL.  Returns the thread count used. */
int oracle_compress_blocks(int decoder, int level, const float *colors,
                           const float *weights, const float color_weights[3],
                           int three_color_mode, int three_color_black,
                           void *out, float *errors, int64_t n, int nthreads,
                           oracle_stats *stats);

/* Weight sources for RGBA8 images. */
enum { ORACLE_W_UNIFORM = 0, ORACLE_W_ALPHA = 1, ORACLE_W_PLANE = 2 };

/* RGBA8 image -> BC1 blocks, blocks in row-major block order.  Partial edge
 * blocks replicate the last row/column.  Texels convert as u8 / 255.0f
 * (icbc_test.cpp:401-405); weights are 1.0f, alpha / 255.0f or a float plane
 * (w*h floats, row pitch w).  Returns the thread count used. */
int oracle_encode_image(const uint8_t *rgba, int w, int h, int64_t pitch_bytes,
                        int weight_mode, const float *weight_plane,
                        int decoder, int level, const float color_weights[3],
                        int three_color_mode, int three_color_black,
                        void *out, float *errors, int nthreads,
                        oracle_stats *stats);

/* Gathers the 16 texels of block (bx, by) with edge replication. */
void oracle_fetch_block(const uint8_t *rgba, int w, int h, int64_t pitch_bytes,
                        int bx, int by, uint8_t texels[64]);

/* icbc::decode_bc1 (icbc.h:2915-2927) and icbc::evaluate_bc1_error
 * (icbc.h:3030-3046). */
void oracle_decode_bc1(const void *block, uint8_t rgba[64], int decoder);
float oracle_evaluate_bc1_error(const uint8_t rgba[64], const void *block, int decoder);

/* icbc::decode_bc3 (icbc.h:39, :2929-2947) and icbc::evaluate_bc3_error
 * (icbc.h:44, :3048-3071) as the reference implements them: 16-byte blocks,
 * 4-colour palette, alpha0 for every texel. */
void oracle_decode_bc3(const void *block, uint8_t rgba[64], int decoder);
float oracle_evaluate_bc3_error(const uint8_t rgba[64], const void *block, int alpha_blend, int decoder);

/* FP64 decode-and-compare of a whole image: sum of squared RGB differences
 * over every texel of every (edge-replicated) block.  Returns the sum; mse
 * per texel = sum / (16 * blocks). */
double oracle_image_sse(const uint8_t *rgba, int w, int h, int64_t pitch_bytes,
                        const void *blocks, int decoder);

/* Table accessors for cross-checking the GPU library's init tables. */
void oracle_tables(int decoder, uint8_t match5[512], uint8_t match6[512], float weights5[5]);
int oracle_cluster_tables(uint32_t four[968], int four_total[16], uint32_t three[152], int three_total[16]);

#ifdef __cplusplus
}
#endif

#endif
