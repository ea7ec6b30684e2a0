/*
 * icbc_oracle.c -- CPU restatement of icbc's BC1 compress path (scalar profile).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU encoder and the CPU
 * baseline timed by bench.py.  Nothing in the product links or calls this.
 *
 * Each function names the icbc.h (v1.05) lines it restates.  The arithmetic is
 * the reference's ICBC_SIMD=0 profile: binary32 operations in source order, no
 * FMA contraction (compile with -ffp-contract=off), IEEE division, and the
 * reference's template min/max/clamp semantics (icbc.h:207-217), which differ
 * from fminf/fmaxf on NaN.
 */
#include "icbc_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } v3;
typedef struct { int r, g, b, a; } c32;             /* Color32 as channels */
typedef struct { uint16_t col0, col1; uint32_t indices; } blk;

/* ---------------------------------------------------------------- helpers */

/* Template max/min/clamp (icbc.h:207-217): max(a,b) = (b < a) ? a : b. */
static inline float tmax(float a, float b) { return (b < a) ? a : b; }
static inline float tmin(float a, float b) { return (a < b) ? a : b; }
static inline float tclamp(float x, float a, float b) { return tmin(tmax(x, a), b); }
static inline float saturate(float x) { return tclamp(x, 0.0f, 1.0f); }          /* :332 */
static inline float vsaturate(float a) { return tmin(tmax(a, 0.0f), 1.0f); }     /* :416 */
static inline float vround01(float a) { return (float)(int)(a + 0.5f); }          /* :417 */

static inline v3 v3_make(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 v3_add(v3 a, v3 b) { return v3_make(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v3_sub(v3 a, v3 b) { return v3_make(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v3_mul(v3 a, v3 b) { return v3_make(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 v3_scale(v3 v, float s) { return v3_make(v.x * s, v.y * s, v.z * s); }
static inline v3 v3_div(v3 v, float s) { return v3_make(v.x / s, v.y / s, v.z / s); }
static inline float v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }   /* :316 */
static inline v3 v3_saturate(v3 v) { return v3_make(saturate(v.x), saturate(v.y), saturate(v.z)); }
static inline v3 v3_max(v3 a, v3 b) { return v3_make(tmax(a.x, b.x), tmax(a.y, b.y), tmax(a.z, b.z)); }
static inline v3 v3_min(v3 a, v3 b) { return v3_make(tmin(a.x, b.x), tmin(a.y, b.y), tmin(a.z, b.z)); }

/* equal(a, b, eps) = fabsf(a - b) < eps (icbc.h:360-368). */
static inline int feq(float a, float b, float eps) { return fabsf(a - b) < eps; }
static inline int v3_eq(v3 a, v3 b, float eps) { return feq(a.x, b.x, eps) && feq(a.y, b.y, eps) && feq(a.z, b.z, eps); }

static inline v3 load_xyz(const float *colors, int i) {
    return v3_make(colors[4 * i + 0], colors[4 * i + 1], colors[4 * i + 2]);
}

/* ------------------------------------------------------ colour conversion */

/* Rounding thresholds between adjacent 5/6-bit expanded values
 * (icbc.h:1560-1570; data of the BC1 format, kept identical). */
static const float k_mid5[32] = {
    0.015686f, 0.047059f, 0.078431f, 0.111765f, 0.145098f, 0.176471f, 0.207843f, 0.241176f,
    0.274510f, 0.305882f, 0.337255f, 0.370588f, 0.403922f, 0.435294f, 0.466667f, 0.5f,
    0.533333f, 0.564706f, 0.596078f, 0.629412f, 0.662745f, 0.694118f, 0.725490f, 0.758824f,
    0.792157f, 0.823529f, 0.854902f, 0.888235f, 0.921569f, 0.952941f, 0.984314f, FLT_MAX};
static const float k_mid6[64] = {
    0.007843f, 0.023529f, 0.039216f, 0.054902f, 0.070588f, 0.086275f, 0.101961f, 0.117647f,
    0.133333f, 0.149020f, 0.164706f, 0.180392f, 0.196078f, 0.211765f, 0.227451f, 0.245098f,
    0.262745f, 0.278431f, 0.294118f, 0.309804f, 0.325490f, 0.341176f, 0.356863f, 0.372549f,
    0.388235f, 0.403922f, 0.419608f, 0.435294f, 0.450980f, 0.466667f, 0.482353f, 0.500000f,
    0.517647f, 0.533333f, 0.549020f, 0.564706f, 0.580392f, 0.596078f, 0.611765f, 0.627451f,
    0.643137f, 0.658824f, 0.674510f, 0.690196f, 0.705882f, 0.721569f, 0.737255f, 0.754902f,
    0.772549f, 0.788235f, 0.803922f, 0.819608f, 0.835294f, 0.850980f, 0.866667f, 0.882353f,
    0.898039f, 0.913725f, 0.929412f, 0.945098f, 0.960784f, 0.976471f, 0.992157f, FLT_MAX};

/* SIMD profiles of the reference (ICBC_SIMD, icbc.h:59-66): the vector
 * width of the cluster-fit loops, whether vmadd/vmsub are fused (AVX2 and
 * AVX-512: icbc.h:734-752, :970-980), whether vround01 rounds half to even
 * (SSE4.1 and later, NEON: icbc.h:518-524, :764-766, :988-990, :1159-1162)
 * instead of int(x + 0.5f) (scalar, SSE2: icbc.h:417, :522), and whether
 * vsaturate keeps a NaN (NEON: vmaxq_f32 / vminq_f32 return NaN for a NaN
 * operand, icbc.h:1155-1157; the x86 max/min and the scalar template return
 * the other operand, so NaN saturates to 0).  Index 0 is the scalar profile;
 * 1..5 are ICBC_SSE2, ICBC_SSE41, ICBC_AVX1, ICBC_AVX2, ICBC_AVX512; 6 is
 * ICBC_NEON (ICBC_SIMD=-1) built without FP contraction, where vmlaq_f32 /
 * vmlsq_f32 are a multiply then an add (icbc.h:1142-1153). */
/* vx: run the cluster loops of a 4-lane profile as 4-lane vector code
 * (cluster_fit_four_v4 / cluster_fit_three_v4), set per call from
 * ORACLE_VECTOR_LOOPS. */
typedef struct { int vec, fma, rne, nan, gather, vx; } prof_t;

/* How a profile's cluster loops fetch SAT entry c for a lane (c >= 0).
 * GATHER_FULL: the entry itself, FLT_MAX past the colour count (the scalar
 * lane loads of SSE2 and AVX1, icbc.h:2652-2682; AVX-512's masked loads,
 * icbc.h:2387-2417; SSE4.1's byte shuffles, icbc.h:2473-2522, whose
 * out-of-table case no padding lane reaches).  GATHER_TBL: NEON's table
 * lookups over the first 8, 12 or 16 entries by count (vqtbl2q / vqtbl3q /
 * vqtbl4q, icbc.h:2586-2650 and :2224-2270), which read zero past the table,
 * so the padding lanes of a 12-colour block read zero for entry 12.
 * GATHER_PERM8: AVX2's permutevar8x32 over the first 8 entries when
 * count <= 8 (icbc.h:2428-2445, :2128-2145, vpermuteif at :867-870), which
 * takes the index modulo 8, so the padding lanes of an 8-colour block read
 * entry c - 8. */
enum { GATHER_FULL = 0, GATHER_TBL = 1, GATHER_PERM8 = 2 };
static const prof_t k_prof[7] = {{1, 0, 0, 0, GATHER_FULL, 0},  {4, 0, 0, 0, GATHER_FULL, 0},
                                 {4, 0, 1, 0, GATHER_FULL, 0},  {8, 0, 1, 0, GATHER_FULL, 0},
                                 {8, 1, 1, 0, GATHER_PERM8, 0}, {16, 1, 1, 0, GATHER_FULL, 0},
                                 {4, 0, 1, 1, GATHER_TBL, 0}};

/* The SAT entry a lane of the profile reads for entry c of a count-colour
 * SAT, -1 for a lane that reads zero. */
static inline int p_gather(const prof_t *p, int count, int c) {
    if (c < 0) return c;
    if (p->gather == GATHER_TBL) return c < (count <= 8 ? 8 : count <= 12 ? 12 : 16) ? c : -1;
    if (p->gather == GATHER_PERM8 && count <= 8) return c & 7;
    return c;
}

static inline float p_madd(const prof_t *p, float a, float b, float c) { return p->fma ? fmaf(a, b, c) : a * b + c; }
static inline float p_msub(const prof_t *p, float a, float b, float c) { return p->fma ? fmaf(a, b, -c) : a * b - c; }
/* vm2sub(a, b, c, d) = vmsub(a, b, c * d) (icbc.h:415, :754-756, :978-980). */
static inline float p_m2sub(const prof_t *p, float a, float b, float c, float d) { return p_msub(p, a, b, c * d); }
static inline float p_round01(const prof_t *p, float a) { return p->rne ? nearbyintf(a) : (float)(int)(a + 0.5f); }
static inline float p_saturate(const prof_t *p, float a) { return (p->nan && a != a) ? a : vsaturate(a); }
static inline v3 p_round_ept(const prof_t *p, v3 v) {
    v3 r;
    r.x = p_round01(p, p_saturate(p, v.x) * 31.0f) * (1.0f / 31.0f);
    r.y = p_round01(p, p_saturate(p, v.y) * 63.0f) * (1.0f / 63.0f);
    r.z = p_round01(p, p_saturate(p, v.z) * 31.0f) * (1.0f / 31.0f);
    return r;
}

/* vround5 / vround6 / vround_ept without ICBC_PERFECT_ROUND (icbc.h:1588-1622). */
static inline float vround5(float x) { return vround01(x * 31.0f) * (1.0f / 31.0f); }
static inline float vround6(float x) { return vround01(x * 63.0f) * (1.0f / 63.0f); }
static inline v3 vround_ept(v3 v) {
    return v3_make(vround5(vsaturate(v.x)), vround6(vsaturate(v.y)), vround5(vsaturate(v.z)));
}

/* vector3_to_color16: truncate, then round up past the expanded midpoint (icbc.h:1624-1639). */
static uint16_t vector3_to_color16(v3 v) {
    unsigned r = (unsigned)tclamp(v.x * 31.0f, 0.0f, 31.0f);
    unsigned g = (unsigned)tclamp(v.y * 63.0f, 0.0f, 63.0f);
    unsigned b = (unsigned)tclamp(v.z * 31.0f, 0.0f, 31.0f);
    r += (v.x > k_mid5[r]);
    g += (v.y > k_mid6[g]);
    b += (v.z > k_mid5[b]);
    return (uint16_t)((r << 11) | (g << 5) | b);
}

/* 565 -> 888 bit replication (icbc.h:1641-1654), per channel. */
static c32 expand565(uint16_t c) {
    int r5 = (c >> 11) & 31, g6 = (c >> 5) & 63, b5 = c & 31;
    c32 o = {(r5 << 3) | (r5 >> 2), (g6 << 2) | (g6 >> 4), (b5 << 3) | (b5 >> 2), 255};
    return o;
}

/* color_to_vector3 (icbc.h:1656-1658). */
static inline v3 c32_to_v3(c32 c) { return v3_make(c.r / 255.0f, c.g / 255.0f, c.b / 255.0f); }

/* vector3_to_color32 (icbc.h:1660-1667). */
static c32 vector3_to_color32(v3 v) {
    c32 c;
    c.r = (uint8_t)(saturate(v.x) * 255 + 0.5f);
    c.g = (uint8_t)(saturate(v.y) * 255 + 0.5f);
    c.b = (uint8_t)(saturate(v.z) * 255 + 0.5f);
    c.a = 255;
    return c;
}

/* ------------------------------------------------------------- palettes */

/* Palette of a block for each hardware decoder (icbc.h:2751-2881): the
 * 4-colour form when `four`, else the 3-colour form with palette[3] = 0. */
static void eval_palette32_form(uint16_t u0, uint16_t u1, c32 p[4], int decoder, int four) {
    p[0] = expand565(u0);
    p[1] = expand565(u1);
    const int r0 = (u0 >> 11) & 31, b0 = u0 & 31, r1 = (u1 >> 11) & 31, b1 = u1 & 31;
    const c32 zero = {0, 0, 0, 0};
    if (decoder == ORACLE_D3D10) {                               /* :2752-2779 */
        if (four) {
            p[2].r = (2 * p[0].r + p[1].r) / 3; p[2].g = (2 * p[0].g + p[1].g) / 3;
            p[2].b = (2 * p[0].b + p[1].b) / 3; p[2].a = 255;
            p[3].r = (2 * p[1].r + p[0].r) / 3; p[3].g = (2 * p[1].g + p[0].g) / 3;
            p[3].b = (2 * p[1].b + p[0].b) / 3; p[3].a = 255;
        } else {
            p[2].r = (p[0].r + p[1].r) / 2; p[2].g = (p[0].g + p[1].g) / 2;
            p[2].b = (p[0].b + p[1].b) / 2; p[2].a = 255;
            p[3] = zero;
        }
    } else if (decoder == ORACLE_NVIDIA) {                       /* :2782-2812 */
        int gdiff = p[1].g - p[0].g;
        if (four) {
            p[2].r = (((2 * r0 + r1) * 22) / 8) & 255;
            p[2].g = ((256 * p[0].g + gdiff / 4 + 128 + gdiff * 80) / 256) & 255;
            p[2].b = (((2 * b0 + b1) * 22) / 8) & 255;
            p[2].a = 255;
            p[3].r = (((2 * r1 + r0) * 22) / 8) & 255;
            p[3].g = ((256 * p[1].g - gdiff / 4 + 128 - gdiff * 80) / 256) & 255;
            p[3].b = (((2 * b1 + b0) * 22) / 8) & 255;
            p[3].a = 255;
        } else {
            p[2].r = (((r0 + r1) * 33) / 8) & 255;
            p[2].g = ((256 * p[0].g + gdiff / 4 + 128 + gdiff * 128) / 256) & 255;
            p[2].b = (((b0 + b1) * 33) / 8) & 255;
            p[2].a = 255;
            p[3] = zero;
        }
    } else if (decoder == ORACLE_AMD) {                          /* :2815-2843 */
        if (four) {
            p[2].r = (43 * p[0].r + 21 * p[1].r + 32) >> 6; p[2].g = (43 * p[0].g + 21 * p[1].g + 32) >> 6;
            p[2].b = (43 * p[0].b + 21 * p[1].b + 32) >> 6; p[2].a = 255;
            p[3].r = (43 * p[1].r + 21 * p[0].r + 32) >> 6; p[3].g = (43 * p[1].g + 21 * p[0].g + 32) >> 6;
            p[3].b = (43 * p[1].b + 21 * p[0].b + 32) >> 6; p[3].a = 255;
        } else {
            p[2].r = (p[0].r + p[1].r + 1) / 2; p[2].g = (p[0].g + p[1].g + 1) / 2;
            p[2].b = (p[0].b + p[1].b + 1) / 2; p[2].a = 255;
            p[3] = zero;
        }
    } else {                                                     /* Intel :2846-2874 */
        if (four) {
            p[2].r = (171 * p[0].r + 85 * p[1].r + 128) >> 8; p[2].g = (171 * p[0].g + 85 * p[1].g + 128) >> 8;
            p[2].b = (171 * p[0].b + 85 * p[1].b + 128) >> 8; p[2].a = 255;
            p[3].r = (171 * p[1].r + 85 * p[0].r + 128) >> 8; p[3].g = (171 * p[1].g + 85 * p[0].g + 128) >> 8;
            p[3].b = (171 * p[1].b + 85 * p[0].b + 128) >> 8; p[3].a = 255;
        } else {
            p[2].r = (128 * p[0].r + 128 * p[1].r + 128) >> 8; p[2].g = (128 * p[0].g + 128 * p[1].g + 128) >> 8;
            p[2].b = (128 * p[0].b + 128 * p[1].b + 128) >> 8; p[2].a = 255;
            p[3] = zero;
        }
    }
}

/* evaluate_palette (icbc.h:2876-2881): the 4-colour form when col0 > col1. */
static void eval_palette32(uint16_t u0, uint16_t u1, c32 p[4], int decoder) {
    eval_palette32_form(u0, u1, p, decoder, u0 > u1);
}

/* Float palette (icbc.h:2893-2900). */
static void eval_palette_v3(uint16_t u0, uint16_t u1, v3 p[4], int decoder) {
    c32 p32[4];
    eval_palette32(u0, u1, p32, decoder);
    for (int i = 0; i < 4; i++) p[i] = c32_to_v3(p32[i]);
}

/* ------------------------------------------------------------- tables */

typedef struct {
    uint8_t match5[256][2], match6[256][2];
    float w1_3, w2_3, w1_9, w4_9, w2_9;
} dec_tables;

static dec_tables g_dec[4];
static uint8_t g_four[968][3];
static int g_four_total[16];
static uint8_t g_three[152][2];
static int g_three_total[16];
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

/* Single-colour match tables (icbc.h:3377-3485): best (max, min) endpoint
 * pair per 8-bit value; D3D10 takes the worst of the AMD/NVIDIA/Intel errors. */
static void prepare_match(uint8_t table[256][2], int bits, int decoder) {
    const int levels = 1 << bits;
    int expand[64];
    for (int i = 0; i < levels; i++)
        expand[i] = bits == 5 ? ((i << 3) | (i >> 2)) : ((i << 2) | (i >> 4));
    for (int i = 0; i < 256; i++) {
        int best = 256 * 100;
        for (int mn = 0; mn < levels; mn++) {
            for (int mx = 0; mx < levels; mx++) {
                int mine = expand[mn], maxe = expand[mx];
                int amd = (43 * maxe + 21 * mine + 32) >> 6;
                int nv = bits == 5 ? ((2 * mx + mn) * 22) / 8
                                   : (256 * mine + (maxe - mine) / 4 + 128 + (maxe - mine) * 80) / 256;
                int intel = (171 * maxe + 85 * mine + 128) >> 8;
                int amd_err = abs(amd - i), nv_err = abs(nv - i), intel_err = abs(intel - i);
                int err;
                if (decoder == ORACLE_D3D10) {
                    int m = amd_err > nv_err ? amd_err : nv_err;
                    err = m > intel_err ? m : intel_err;
                } else if (decoder == ORACLE_NVIDIA) err = nv_err;
                else if (decoder == ORACLE_INTEL) err = intel_err;
                else err = amd_err;
                if (err < best) {
                    best = err;
                    table[i][0] = (uint8_t)mx;
                    table[i][1] = (uint8_t)mn;
                }
            }
        }
    }
}

/* Decoder-dependent interpolation weights (icbc.h:3495-3515). */
static void init_weights(dec_tables *t, int decoder) {
    t->w1_3 = 1.0f / 3;
    t->w2_3 = 2.0f / 3;
    if (decoder == ORACLE_AMD) { t->w1_3 = 21.0f / 64; t->w2_3 = 43.0f / 64; }
    else if (decoder == ORACLE_INTEL) { t->w1_3 = 85.0f / 256; t->w2_3 = 171.0f / 256; }
    t->w1_9 = t->w1_3 * t->w1_3;
    t->w4_9 = t->w2_3 * t->w2_3;
    t->w2_9 = t->w1_3 * t->w2_3;
}

/* Cluster boundary enumerations (icbc.h:1965-2034): all cumulative
 * boundaries 0 <= c0 <= c1 <= c2 <= t (except all-zero), grouped by the
 * total t at which they first appear, so a prefix of the list serves n
 * colours. */
static void init_cluster(void) {
    int i = 0;
    for (int t = 1; t <= 16; t++) {
        for (int c0 = 0; c0 <= t; c0++)
            for (int c1 = 0; c1 <= t - c0; c1++)
                for (int c2 = 0; c2 <= t - c0 - c1; c2++) {
                    if (c0 == 0 && c1 == 0 && c2 == 0) continue;
                    int found = 0;
                    if (t > 1)
                        for (int j = 0; j < g_four_total[t - 2]; j++)
                            if (g_four[j][0] == c0 && g_four[j][1] == c0 + c1 && g_four[j][2] == c0 + c1 + c2) { found = 1; break; }
                    if (!found) {
                        g_four[i][0] = (uint8_t)c0; g_four[i][1] = (uint8_t)(c0 + c1); g_four[i][2] = (uint8_t)(c0 + c1 + c2);
                        i++;
                    }
                }
        g_four_total[t - 1] = i;
    }
    i = 0;
    for (int t = 1; t <= 16; t++) {
        for (int c0 = 0; c0 <= t; c0++)
            for (int c1 = 0; c1 <= t - c0; c1++) {
                if (c0 == 0 && c1 == 0) continue;
                int found = 0;
                if (t > 1)
                    for (int j = 0; j < g_three_total[t - 2]; j++)
                        if (g_three[j][0] == c0 && g_three[j][1] == c0 + c1) { found = 1; break; }
                if (!found) { g_three[i][0] = (uint8_t)c0; g_three[i][1] = (uint8_t)(c0 + c1); i++; }
            }
        g_three_total[t - 1] = i;
    }
}

static void init_once(void) {
    for (int d = 0; d < 4; d++) {
        prepare_match(g_dec[d].match5, 5, d);
        prepare_match(g_dec[d].match6, 6, d);
        init_weights(&g_dec[d], d);
    }
    init_cluster();
}

void oracle_init(void) { pthread_once(&g_once, init_once); }

void oracle_tables(int decoder, uint8_t match5[512], uint8_t match6[512], float weights5[5]) {
    oracle_init();
    const dec_tables *t = &g_dec[decoder & 3];
    memcpy(match5, t->match5, 512);
    memcpy(match6, t->match6, 512);
    weights5[0] = t->w1_3; weights5[1] = t->w2_3; weights5[2] = t->w1_9; weights5[3] = t->w4_9; weights5[4] = t->w2_9;
}

int oracle_cluster_tables(uint32_t four[968], int four_total[16], uint32_t three[152], int three_total[16]) {
    oracle_init();
    for (int i = 0; i < 968; i++) four[i] = g_four[i][0] | (g_four[i][1] << 8) | ((uint32_t)g_four[i][2] << 16);
    for (int i = 0; i < 152; i++) three[i] = g_three[i][0] | (g_three[i][1] << 8);
    memcpy(four_total, g_four_total, sizeof(g_four_total));
    memcpy(three_total, g_three_total, sizeof(g_three_total));
    return 0;
}

/* ------------------------------------------------------- input processing */

/* is_black (icbc.h:1673-1680). */
static inline int is_black(v3 c) { return c.x < 1.0f / 8 && c.y < 1.0f / 8 && c.z < 1.0f / 8; }

/* reduce_colors: greedy merge of texels closer than threshold per channel,
 * running weighted mean, weights <= 0 skipped (icbc.h:1683-1728). */
static int reduce_colors(const float *in, const float *in_w, float threshold, v3 *colors,
                         float *weights, int *any_black, oracle_stats *st) {
    *any_black = 0;
    int n = 0;
    for (int i = 0; i < 16; i++) {
        v3 ci = load_xyz(in, i);
        float wi = in_w[i];
        if (wi > 0) {
            int j;
            for (j = 0; j < n; j++) {
                if (st) st->reduce_pairs++;
                if (v3_eq(colors[j], ci, threshold)) {
                    colors[j] = v3_div(v3_add(v3_scale(colors[j], weights[j]), v3_scale(ci, wi)), weights[j] + wi);
                    weights[j] += wi;
                    if (st) st->reduce_merges++;
                    break;
                }
            }
            if (j == n) { colors[n] = ci; weights[n] = wi; n++; }
            if (is_black(ci)) *any_black = 1;
        }
    }
    return n;
}

/* skip_blacks (icbc.h:1730-1748). */
static int skip_blacks(const v3 *in, const float *in_w, int count, v3 *colors, float *weights) {
    int n = 0;
    for (int i = 0; i < count; i++) {
        if (is_black(in[i])) continue;
        colors[n] = in[i];
        weights[n] = in_w[i];
        n++;
    }
    return n;
}

/* ------------------------------------------------------------------ PCA */

/* computeCentroid + computeCovariance (icbc.h:1755-1795): unsquared weights. */
static void covariance(int n, const v3 *p, const float *w, float cov[6]) {
    v3 centroid = {0, 0, 0};
    float total = 0.0f;
    for (int i = 0; i < n; i++) {
        total += w[i];
        centroid = v3_add(centroid, v3_scale(p[i], w[i]));
    }
    centroid = v3_scale(centroid, 1.0f / total);
    for (int i = 0; i < 6; i++) cov[i] = 0.0f;
    for (int i = 0; i < n; i++) {
        v3 a = v3_sub(p[i], centroid);
        v3 b = v3_scale(a, w[i]);
        cov[0] += a.x * b.x; cov[1] += a.x * b.y; cov[2] += a.x * b.z;
        cov[3] += a.y * b.y; cov[4] += a.y * b.z; cov[5] += a.z * b.z;
    }
}

/* estimatePrincipalComponent + firstEigenVector_PowerMethod, 6 iterations
 * normalised by the largest component (icbc.h:1798-1836). */
static v3 principal_axis(const float m[6]) {
    if (m[0] == 0 && m[3] == 0 && m[5] == 0) return v3_make(0, 0, 0);
    v3 row0 = {m[0], m[1], m[2]}, row1 = {m[1], m[3], m[4]}, row2 = {m[2], m[4], m[5]};
    float r0 = v3_dot(row0, row0), r1 = v3_dot(row1, row1), r2 = v3_dot(row2, row2);
    v3 v = (r0 > r1 && r0 > r2) ? row0 : (r1 > r2 ? row1 : row2);
    for (int i = 0; i < 6; i++) {
        float x = v.x * m[0] + v.y * m[1] + v.z * m[2];
        float y = v.x * m[1] + v.y * m[3] + v.z * m[4];
        float z = v.x * m[2] + v.y * m[4] + v.z * m[5];
        float norm = tmax(tmax(x, y), z);
        v = v3_scale(v3_make(x, y, z), 1.0f / norm);
    }
    return v;
}

/* ------------------------------------------------------------------ SAT */

typedef struct { float r[16], g[16], b[16], w[16]; } sat_t;

/* compute_sat: project on the principal axis, stable insertion sort,
 * prefix sums of colour*weight and weight, FLT_MAX fill (icbc.h:1857-1937). */
static int compute_sat(const v3 *colors, const float *weights, int count, sat_t *sat, oracle_stats *st) {
    float cov[6];
    covariance(count, colors, weights, cov);
    v3 axis = principal_axis(cov);
    int order[16];
    float dps[16];
    for (int i = 0; i < count; i++) { order[i] = i; dps[i] = v3_dot(colors[i], axis); }
    for (int i = 0; i < count; i++)
        for (int j = i; j > 0 && dps[j] < dps[j - 1]; j--) {
            float t = dps[j]; dps[j] = dps[j - 1]; dps[j - 1] = t;
            int o = order[j]; order[j] = order[j - 1]; order[j - 1] = o;
        }
    float w = weights[order[0]];
    sat->r[0] = colors[order[0]].x * w;
    sat->g[0] = colors[order[0]].y * w;
    sat->b[0] = colors[order[0]].z * w;
    sat->w[0] = w;
    for (int i = 1; i < count; i++) {
        w = weights[order[i]];
        sat->r[i] = sat->r[i - 1] + colors[order[i]].x * w;
        sat->g[i] = sat->g[i - 1] + colors[order[i]].y * w;
        sat->b[i] = sat->b[i - 1] + colors[order[i]].z * w;
        sat->w[i] = sat->w[i - 1] + w;
    }
    for (int i = count; i < 16; i++) sat->r[i] = sat->g[i] = sat->b[i] = sat->w[i] = FLT_MAX;
    if (st) { st->sat_builds++; st->sat_points += count; }
    return count;
}

/* ---------------------------------------------------------- cluster fit */

/* The cross-lane argmin of the SIMD loops (reduce_min_index, icbc.h:574-586,
 * :812-831, :1031-1039): the smallest per-lane best error, ties to the lowest
 * lane (-0 and +0 compare equal).  Lane l kept the first strict minimum of the
 * combinations l, l + vec, l + 2 vec, ... */
static int lane_argmin(const float *best, int vec) {
    float m = best[0];
    for (int l = 1; l < vec; l++) m = best[l] < m ? best[l] : m;
    for (int l = 0; l < vec; l++)
        if (best[l] <= m) return l;
    return 0;
}

/* cluster_fit_three (icbc.h:2075-2345): every 2-boundary split of the sorted
 * colours, least-squares endpoints with weights 1/2, snapped to 565, the
 * minimum metric-weighted error kept.  The loop runs over whole vectors of
 * the profile's width: the combinations past the count's total come from
 * the table for larger counts (or its zero padding) and read the SAT's
 * FLT_MAX fill, or what the profile's gather reads there (p_gather), as the
 * reference's SIMD builds do. */
static void cluster_fit_three(const sat_t *sat, int count, v3 metric_sqr, const prof_t *pf, v3 *start, v3 *end,
                              oracle_stats *st) {
    const float r_sum = sat->r[count - 1], g_sum = sat->g[count - 1], b_sum = sat->b[count - 1], w_sum = sat->w[count - 1];
    float best[16];
    v3 bs[16], be[16];
    for (int l = 0; l < 16; l++) { best[l] = FLT_MAX; bs[l] = be[l] = v3_make(0, 0, 0); }
    const int total = g_three_total[count - 1];
    const int padded = (total + pf->vec - 1) / pf->vec * pf->vec;
    for (int i = 0; i < padded; i++) {
        const int l = i % pf->vec;
        v3 x0 = {0, 0, 0}, x1 = {0, 0, 0};
        float w0 = 0, w1 = 0;
        int c0 = p_gather(pf, count, (i < 152 ? g_three[i][0] : 0) - 1);
        int c1 = p_gather(pf, count, (i < 152 ? g_three[i][1] : 0) - 1);
        if (c0 >= 0) { x0 = v3_make(sat->r[c0], sat->g[c0], sat->b[c0]); w0 = sat->w[c0]; }
        if (c1 >= 0) { x1 = v3_make(sat->r[c1], sat->g[c1], sat->b[c1]); w1 = sat->w[c1]; }
        float w2 = w_sum - w1;
        x1 = v3_sub(x1, x0);
        w1 = w1 - w0;
        float alphabeta_sum = w1 * 0.25f;
        float alpha2_sum = w0 + alphabeta_sum;
        float beta2_sum = w2 + alphabeta_sum;
        float factor = 1.0f / p_m2sub(pf, alpha2_sum, beta2_sum, alphabeta_sum, alphabeta_sum);
        v3 alphax_sum = v3_add(x0, v3_scale(x1, 0.5f));
        v3 betax_sum = v3_sub(v3_make(r_sum, g_sum, b_sum), alphax_sum);
        v3 a, b;
        a.x = p_m2sub(pf, alphax_sum.x, beta2_sum, betax_sum.x, alphabeta_sum) * factor;
        a.y = p_m2sub(pf, alphax_sum.y, beta2_sum, betax_sum.y, alphabeta_sum) * factor;
        a.z = p_m2sub(pf, alphax_sum.z, beta2_sum, betax_sum.z, alphabeta_sum) * factor;
        b.x = p_m2sub(pf, betax_sum.x, alpha2_sum, alphax_sum.x, alphabeta_sum) * factor;
        b.y = p_m2sub(pf, betax_sum.y, alpha2_sum, alphax_sum.y, alphabeta_sum) * factor;
        b.z = p_m2sub(pf, betax_sum.z, alpha2_sum, alphax_sum.z, alphabeta_sum) * factor;
        a = p_round_ept(pf, a);
        b = p_round_ept(pf, b);
        /* e2 = vm2sub(a, vmsub(b, ab, ax), b, bx) * 2 ; e1 = vmadd(a*a, alpha2, vmadd(b*b, beta2, e2)) */
        v3 e2, e1;
        e2.x = p_m2sub(pf, a.x, p_msub(pf, b.x, alphabeta_sum, alphax_sum.x), b.x, betax_sum.x) * 2.0f;
        e2.y = p_m2sub(pf, a.y, p_msub(pf, b.y, alphabeta_sum, alphax_sum.y), b.y, betax_sum.y) * 2.0f;
        e2.z = p_m2sub(pf, a.z, p_msub(pf, b.z, alphabeta_sum, alphax_sum.z), b.z, betax_sum.z) * 2.0f;
        e1.x = p_madd(pf, a.x * a.x, alpha2_sum, p_madd(pf, b.x * b.x, beta2_sum, e2.x));
        e1.y = p_madd(pf, a.y * a.y, alpha2_sum, p_madd(pf, b.y * b.y, beta2_sum, e2.y));
        e1.z = p_madd(pf, a.z * a.z, alpha2_sum, p_madd(pf, b.z * b.z, beta2_sum, e2.z));
        float error = v3_dot(e1, metric_sqr);
        if (error < best[l]) { best[l] = error; bs[l] = a; be[l] = b; }
    }
    if (st) st->cf3_combos += total;
    const int w = lane_argmin(best, pf->vec);
    *start = bs[w];
    *end = be[w];
}

/* cluster_fit_four (icbc.h:2348-2743) with the decoder's interpolation
 * weights w1_3, w2_3, w1_9, w4_9, w2_9; vector loop as cluster_fit_three. */
static void cluster_fit_four(const sat_t *sat, int count, v3 metric_sqr, const dec_tables *dt, const prof_t *pf,
                             v3 *start, v3 *end, oracle_stats *st) {
    const float r_sum = sat->r[count - 1], g_sum = sat->g[count - 1], b_sum = sat->b[count - 1], w_sum = sat->w[count - 1];
    const float w1_3 = dt->w1_3, w2_3 = dt->w2_3, w1_9 = dt->w1_9, w4_9 = dt->w4_9, w2_9 = dt->w2_9;
    float best[16];
    v3 bs[16], be[16];
    for (int l = 0; l < 16; l++) { best[l] = FLT_MAX; bs[l] = be[l] = v3_make(0, 0, 0); }
    const int total = g_four_total[count - 1];
    const int padded = (total + pf->vec - 1) / pf->vec * pf->vec;
    for (int i = 0; i < padded; i++) {
        const int l = i % pf->vec;
        v3 x0 = {0, 0, 0}, x1 = {0, 0, 0}, x2 = {0, 0, 0};
        float w0 = 0, w1 = 0, w2 = 0;
        int c0 = p_gather(pf, count, (i < 968 ? g_four[i][0] : 0) - 1);
        int c1 = p_gather(pf, count, (i < 968 ? g_four[i][1] : 0) - 1);
        int c2 = p_gather(pf, count, (i < 968 ? g_four[i][2] : 0) - 1);
        if (c0 >= 0) { x0 = v3_make(sat->r[c0], sat->g[c0], sat->b[c0]); w0 = sat->w[c0]; }
        if (c1 >= 0) { x1 = v3_make(sat->r[c1], sat->g[c1], sat->b[c1]); w1 = sat->w[c1]; }
        if (c2 >= 0) { x2 = v3_make(sat->r[c2], sat->g[c2], sat->b[c2]); w2 = sat->w[c2]; }
        float w3 = w_sum - w2;
        x2 = v3_sub(x2, x1);
        x1 = v3_sub(x1, x0);
        w2 = w2 - w1;
        w1 = w1 - w0;
        float alpha2_sum = p_madd(pf, w2, w1_9, p_madd(pf, w1, w4_9, w0));
        float beta2_sum = p_madd(pf, w1, w1_9, p_madd(pf, w2, w4_9, w3));
        float alphabeta_sum = (w1 + w2) * w2_9;
        float factor = 1.0f / p_m2sub(pf, alpha2_sum, beta2_sum, alphabeta_sum, alphabeta_sum);
        v3 alphax_sum;
        alphax_sum.x = p_madd(pf, x2.x, w1_3, p_madd(pf, x1.x, w2_3, x0.x));
        alphax_sum.y = p_madd(pf, x2.y, w1_3, p_madd(pf, x1.y, w2_3, x0.y));
        alphax_sum.z = p_madd(pf, x2.z, w1_3, p_madd(pf, x1.z, w2_3, x0.z));
        v3 betax_sum = v3_sub(v3_make(r_sum, g_sum, b_sum), alphax_sum);
        v3 a, b;
        a.x = p_m2sub(pf, alphax_sum.x, beta2_sum, betax_sum.x, alphabeta_sum) * factor;
        a.y = p_m2sub(pf, alphax_sum.y, beta2_sum, betax_sum.y, alphabeta_sum) * factor;
        a.z = p_m2sub(pf, alphax_sum.z, beta2_sum, betax_sum.z, alphabeta_sum) * factor;
        b.x = p_m2sub(pf, betax_sum.x, alpha2_sum, alphax_sum.x, alphabeta_sum) * factor;
        b.y = p_m2sub(pf, betax_sum.y, alpha2_sum, alphax_sum.y, alphabeta_sum) * factor;
        b.z = p_m2sub(pf, betax_sum.z, alpha2_sum, alphax_sum.z, alphabeta_sum) * factor;
        a = p_round_ept(pf, a);
        b = p_round_ept(pf, b);
        v3 e2, e1;
        e2.x = p_m2sub(pf, a.x, p_msub(pf, b.x, alphabeta_sum, alphax_sum.x), b.x, betax_sum.x) * 2.0f;
        e2.y = p_m2sub(pf, a.y, p_msub(pf, b.y, alphabeta_sum, alphax_sum.y), b.y, betax_sum.y) * 2.0f;
        e2.z = p_m2sub(pf, a.z, p_msub(pf, b.z, alphabeta_sum, alphax_sum.z), b.z, betax_sum.z) * 2.0f;
        e1.x = p_madd(pf, a.x * a.x, alpha2_sum, p_madd(pf, b.x * b.x, beta2_sum, e2.x));
        e1.y = p_madd(pf, a.y * a.y, alpha2_sum, p_madd(pf, b.y * b.y, beta2_sum, e2.y));
        e1.z = p_madd(pf, a.z * a.z, alpha2_sum, p_madd(pf, b.z * b.z, beta2_sum, e2.z));
        float error = v3_dot(e1, metric_sqr);
        if (error < best[l]) { best[l] = error; bs[l] = a; be[l] = b; }
    }
    if (st) st->cf4_combos += total;
    const int w = lane_argmin(best, pf->vec);
    *start = bs[w];
    *end = be[w];
}

/* ------------------------------------------- cluster fit, 4-lane vectors */

/* cluster_fit_four / cluster_fit_three of a 4-lane profile (SSE2, SSE4.1,
 * NEON) run four combinations at a time in GCC vector types, the way the
 * reference's 4-lane builds run them (VFloat, icbc.h:427-668 for SSE,
 * :1121-1235 for NEON): combination i in lane i % 4, each lane keeping its
 * first strict minimum, then lane_argmin.  Every lane operation is the IEEE
 * operation of the scalar-lane loops above, in the same order and without
 * contraction (this file is built with -ffp-contract=off), and the SAT
 * entries come through the same p_gather, so both loops give the same bits;
 * these exist to time a vectorised CPU encoder.  The vector types compile to
 * NEON on aarch64 and to SSE2 on x86-64, with no target intrinsics. */
typedef float f4 __attribute__((vector_size(16)));
typedef int32_t i4 __attribute__((vector_size(16)));

static inline f4 f4_1(float x) { f4 r = {x, x, x, x}; return r; }
static inline f4 f4_sel(i4 m, f4 a, f4 b) { return (f4)(((i4)a & m) | ((i4)b & ~m)); }

/* p_saturate: tmin(tmax(a, 0), 1) with the template's comparisons (a NaN
 * goes to 0), the NaN kept on NEON. */
static inline f4 f4_saturate(const prof_t *p, f4 a) {
    const f4 z = f4_1(0.0f), o = f4_1(1.0f);
    f4 x = f4_sel(z < a, a, z);
    x = f4_sel(x < o, x, o);
    return p->nan ? f4_sel(a != a, a, x) : x;
}

/* p_round01 of 0 <= a <= 63 (or a NaN): half to even through the 2^23
 * addition, exact in that range, or int(a + 0.5f). */
static inline f4 f4_round01(const prof_t *p, f4 a) {
    if (p->rne) return (a + f4_1(8388608.0f)) - f4_1(8388608.0f);
    return __builtin_convertvector(__builtin_convertvector(a + f4_1(0.5f), i4), f4);
}

static inline void f4_round_ept(const prof_t *p, f4 *x, f4 *y, f4 *z) {
    *x = f4_round01(p, f4_saturate(p, *x) * f4_1(31.0f)) * f4_1(1.0f / 31.0f);
    *y = f4_round01(p, f4_saturate(p, *y) * f4_1(63.0f)) * f4_1(1.0f / 63.0f);
    *z = f4_round01(p, f4_saturate(p, *z) * f4_1(31.0f)) * f4_1(1.0f / 31.0f);
}

/* The SAT as 17 (r, g, b, w) vectors indexed by a cluster table entry:
 * entry 0 reads zero, entry e the SAT slot e - 1 as the profile gathers it. */
static void f4_sat_table(const prof_t *p, const sat_t *sat, int count, f4 tt[17]) {
    tt[0] = f4_1(0.0f);
    for (int e = 1; e <= 16; e++) {
        const int c = p_gather(p, count, e - 1);
        if (c < 0) {
            tt[e] = f4_1(0.0f);
        } else {
            f4 v = {sat->r[c], sat->g[c], sat->b[c], sat->w[c]};
            tt[e] = v;
        }
    }
}

/* Four lanes' SAT entries e[0], e[stride], e[2 stride], e[3 stride] as
 * channel vectors (a 4x4 transpose). */
static inline void f4_gather(const f4 *tt, const uint8_t *e, int stride, f4 *r, f4 *g, f4 *b, f4 *w) {
    const f4 A = tt[e[0]], B = tt[e[stride]], C = tt[e[2 * stride]], D = tt[e[3 * stride]];
    const i4 lo = {0, 4, 1, 5}, hi = {2, 6, 3, 7}, l2 = {0, 1, 4, 5}, h2 = {2, 3, 6, 7};
    const f4 t0 = __builtin_shuffle(A, B, lo), t1 = __builtin_shuffle(A, B, hi);
    const f4 t2 = __builtin_shuffle(C, D, lo), t3 = __builtin_shuffle(C, D, hi);
    *r = __builtin_shuffle(t0, t2, l2);
    *g = __builtin_shuffle(t0, t2, h2);
    *b = __builtin_shuffle(t1, t3, l2);
    *w = __builtin_shuffle(t1, t3, h2);
}

/* The least-squares endpoints, their 565 snap and the metric-weighted error
 * of four combinations (the common tail of icbc.h:2299-2323 and
 * :2697-2733); keeps each lane's first strict minimum. */
typedef struct { f4 best, ar, ag, ab, br, bg, bb; } f4_keep;

static inline void f4_fit(const prof_t *p, f4 alpha2, f4 beta2, f4 alphabeta, f4 axr, f4 axg, f4 axb, f4 bxr,
                          f4 bxg, f4 bxb, f4 mr, f4 mg, f4 mb, f4_keep *k) {
    const f4 factor = f4_1(1.0f) / (alpha2 * beta2 - alphabeta * alphabeta);
    f4 ar = (axr * beta2 - bxr * alphabeta) * factor;
    f4 ag = (axg * beta2 - bxg * alphabeta) * factor;
    f4 ab = (axb * beta2 - bxb * alphabeta) * factor;
    f4 br = (bxr * alpha2 - axr * alphabeta) * factor;
    f4 bg = (bxg * alpha2 - axg * alphabeta) * factor;
    f4 bb = (bxb * alpha2 - axb * alphabeta) * factor;
    f4_round_ept(p, &ar, &ag, &ab);
    f4_round_ept(p, &br, &bg, &bb);
    const f4 two = f4_1(2.0f);
    const f4 e2r = (ar * (br * alphabeta - axr) - br * bxr) * two;
    const f4 e2g = (ag * (bg * alphabeta - axg) - bg * bxg) * two;
    const f4 e2b = (ab * (bb * alphabeta - axb) - bb * bxb) * two;
    const f4 e1r = (ar * ar) * alpha2 + ((br * br) * beta2 + e2r);
    const f4 e1g = (ag * ag) * alpha2 + ((bg * bg) * beta2 + e2g);
    const f4 e1b = (ab * ab) * alpha2 + ((bb * bb) * beta2 + e2b);
    const f4 error = e1r * mr + e1g * mg + e1b * mb;
    const i4 m = error < k->best;
    k->best = f4_sel(m, error, k->best);
    k->ar = f4_sel(m, ar, k->ar);
    k->ag = f4_sel(m, ag, k->ag);
    k->ab = f4_sel(m, ab, k->ab);
    k->br = f4_sel(m, br, k->br);
    k->bg = f4_sel(m, bg, k->bg);
    k->bb = f4_sel(m, bb, k->bb);
}

static void f4_keep_init(f4_keep *k) {
    k->best = f4_1(FLT_MAX);
    k->ar = k->ag = k->ab = k->br = k->bg = k->bb = f4_1(0.0f);
}

static void f4_keep_result(const f4_keep *k, v3 *start, v3 *end) {
    float best[4];
    for (int l = 0; l < 4; l++) best[l] = k->best[l];
    const int w = lane_argmin(best, 4);
    *start = v3_make(k->ar[w], k->ag[w], k->ab[w]);
    *end = v3_make(k->br[w], k->bg[w], k->bb[w]);
}

static void cluster_fit_three_v4(const sat_t *sat, int count, v3 metric_sqr, const prof_t *pf, v3 *start, v3 *end,
                                 oracle_stats *st) {
    f4 tt[17];
    f4_sat_table(pf, sat, count, tt);
    const f4 r_sum = f4_1(sat->r[count - 1]), g_sum = f4_1(sat->g[count - 1]), b_sum = f4_1(sat->b[count - 1]);
    const f4 w_sum = f4_1(sat->w[count - 1]);
    const f4 mr = f4_1(metric_sqr.x), mg = f4_1(metric_sqr.y), mb = f4_1(metric_sqr.z);
    const f4 quarter = f4_1(0.25f), half = f4_1(0.5f);
    f4_keep k;
    f4_keep_init(&k);
    const int total = g_three_total[count - 1];
    const int padded = (total + 3) & ~3;
    for (int i = 0; i < padded; i += 4) {
        f4 x0r, x0g, x0b, w0, x1r, x1g, x1b, w1;
        f4_gather(tt, &g_three[i][0], 2, &x0r, &x0g, &x0b, &w0);
        f4_gather(tt, &g_three[i][1], 2, &x1r, &x1g, &x1b, &w1);
        const f4 w2 = w_sum - w1;
        x1r = x1r - x0r;
        x1g = x1g - x0g;
        x1b = x1b - x0b;
        w1 = w1 - w0;
        const f4 alphabeta = w1 * quarter;
        const f4 alpha2 = w0 + alphabeta;
        const f4 beta2 = w2 + alphabeta;
        const f4 axr = x0r + x1r * half, axg = x0g + x1g * half, axb = x0b + x1b * half;
        f4_fit(pf, alpha2, beta2, alphabeta, axr, axg, axb, r_sum - axr, g_sum - axg, b_sum - axb, mr, mg, mb, &k);
    }
    if (st) st->cf3_combos += total;
    f4_keep_result(&k, start, end);
}

static void cluster_fit_four_v4(const sat_t *sat, int count, v3 metric_sqr, const dec_tables *dt, const prof_t *pf,
                                v3 *start, v3 *end, oracle_stats *st) {
    f4 tt[17];
    f4_sat_table(pf, sat, count, tt);
    const f4 r_sum = f4_1(sat->r[count - 1]), g_sum = f4_1(sat->g[count - 1]), b_sum = f4_1(sat->b[count - 1]);
    const f4 w_sum = f4_1(sat->w[count - 1]);
    const f4 w1_3 = f4_1(dt->w1_3), w2_3 = f4_1(dt->w2_3), w1_9 = f4_1(dt->w1_9), w4_9 = f4_1(dt->w4_9);
    const f4 w2_9 = f4_1(dt->w2_9);
    const f4 mr = f4_1(metric_sqr.x), mg = f4_1(metric_sqr.y), mb = f4_1(metric_sqr.z);
    f4_keep k;
    f4_keep_init(&k);
    const int total = g_four_total[count - 1];
    const int padded = (total + 3) & ~3;
    for (int i = 0; i < padded; i += 4) {
        f4 x0r, x0g, x0b, w0, x1r, x1g, x1b, w1, x2r, x2g, x2b, w2;
        f4_gather(tt, &g_four[i][0], 3, &x0r, &x0g, &x0b, &w0);
        f4_gather(tt, &g_four[i][1], 3, &x1r, &x1g, &x1b, &w1);
        f4_gather(tt, &g_four[i][2], 3, &x2r, &x2g, &x2b, &w2);
        const f4 w3 = w_sum - w2;
        x2r = x2r - x1r;
        x2g = x2g - x1g;
        x2b = x2b - x1b;
        x1r = x1r - x0r;
        x1g = x1g - x0g;
        x1b = x1b - x0b;
        w2 = w2 - w1;
        w1 = w1 - w0;
        const f4 alpha2 = w2 * w1_9 + (w1 * w4_9 + w0);
        const f4 beta2 = w1 * w1_9 + (w2 * w4_9 + w3);
        const f4 alphabeta = (w1 + w2) * w2_9;
        const f4 axr = x2r * w1_3 + (x1r * w2_3 + x0r);
        const f4 axg = x2g * w1_3 + (x1g * w2_3 + x0g);
        const f4 axb = x2b * w1_3 + (x1b * w2_3 + x0b);
        f4_fit(pf, alpha2, beta2, alphabeta, axr, axg, axb, r_sum - axr, g_sum - axg, b_sum - axb, mr, mg, mb, &k);
    }
    if (st) st->cf4_combos += total;
    f4_keep_result(&k, start, end);
}

/* ------------------------------------------------------ error evaluation */

/* evaluate_mse(Vector3 p, Vector3 c, Vector3 w) = |((p - c) * w) * 255|^2 (icbc.h:2955-2963). */
static inline float texel_mse(v3 p, v3 c, v3 w) {
    v3 d = v3_scale(v3_mul(v3_sub(p, c), w), 255);
    return v3_dot(d, d);
}

/* Weighted error of a block for given indices, texels summed in order
 * (icbc.h:3006-3028). */
static float block_mse(const float *in, const float *in_w, v3 cw, const v3 pal[4], uint32_t indices) {
    float error = 0.0f;
    for (int i = 0; i < 16; i++) {
        int index = (indices >> (2 * i)) & 3;
        error += in_w[i] * texel_mse(pal[index], load_xyz(in, i), cw);
    }
    return error;
}

static float block_mse_out(const float *in, const float *in_w, v3 cw, const blk *b, int decoder) {
    v3 pal[4];
    eval_palette_v3(b->col0, b->col1, pal, decoder);
    return block_mse(in, in_w, cw, pal, b->indices);
}

static inline int iabs(int x) { return x < 0 ? -x : x; }
static inline int c32_mse(c32 p, c32 c) {
    return (p.r - c.r) * (p.r - c.r) + (p.g - c.g) * (p.g - c.g) + (p.b - c.b) * (p.b - c.b);
}

/* ------------------------------------------------------ index selection */

/* Index bits are assembled as interleave(indices1, indices0) (icbc.h:3079-3095):
 * texel i gets bit 2i = x1, bit 2i+1 = x0. */
static inline uint32_t pack_index(uint32_t x1, uint32_t x0, int i) { return (x1 << (2 * i)) | (x0 << (2 * i + 1)); }

/* compute_indices4 (icbc.h:3097-3131). */
static uint32_t compute_indices4(const float *in, v3 cw, const v3 pal[4]) {
    v3 p0 = v3_mul(pal[0], cw), p1 = v3_mul(pal[1], cw), p2 = v3_mul(pal[2], cw), p3 = v3_mul(pal[3], cw);
    uint32_t out = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = v3_mul(load_xyz(in, i), cw);
        v3 t0 = v3_sub(c, p0), t1 = v3_sub(c, p1), t2 = v3_sub(c, p2), t3 = v3_sub(c, p3);
        float d0 = v3_dot(t0, t0), d1 = v3_dot(t1, t1), d2 = v3_dot(t2, t2), d3 = v3_dot(t3, t3);
        int b1 = d1 > d2, b2 = d0 > d2, b0 = d0 > d3, b3 = d1 > d3, b4 = d2 > d3;
        uint32_t x0 = (uint32_t)((b1 & b2) | (b0 & b3));
        uint32_t x1 = (uint32_t)(b0 & b4);
        out |= pack_index(x1, x0, i);
    }
    return out;
}

/* compute_indices3, with the transparent-black entry when allowed (icbc.h:3133-3176). */
static uint32_t compute_indices3(const float *in, v3 cw, int allow_black, const v3 pal[4]) {
    v3 p0 = v3_mul(pal[0], cw), p1 = v3_mul(pal[1], cw), p2 = v3_mul(pal[2], cw);
    uint32_t out = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = v3_mul(load_xyz(in, i), cw);
        uint32_t x0, x1;
        if (allow_black) {
            v3 t0 = v3_sub(p0, c), t1 = v3_sub(p1, c), t2 = v3_sub(p2, c);
            float d0 = v3_dot(t0, t0), d1 = v3_dot(t1, t1), d2 = v3_dot(t2, t2), d3 = v3_dot(c, c);
            int i1 = d1 < d2, i2 = (d2 <= d0) & (d2 <= d1), i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
            x0 = (uint32_t)(i2 | i3);
            x1 = (uint32_t)(i1 | i3);
        } else {
            v3 t0 = v3_sub(c, p0), t1 = v3_sub(c, p1), t2 = v3_sub(c, p2);
            float d0 = v3_dot(t0, t0), d1 = v3_dot(t1, t1), d2 = v3_dot(t2, t2);
            int i1 = d1 < d2, i2 = (d2 <= d0) & (d2 <= d1);
            x0 = (uint32_t)i2;
            x1 = (uint32_t)i1;
        }
        out |= pack_index(x1, x0, i);
    }
    return out;
}

/* compute_indices, generic nearest-of-four used by refinement (icbc.h:3179-3235). */
static uint32_t compute_indices(const float *in, v3 cw, const v3 pal[4]) {
    v3 p0 = v3_mul(pal[0], cw), p1 = v3_mul(pal[1], cw), p2 = v3_mul(pal[2], cw), p3 = v3_mul(pal[3], cw);
    uint32_t out = 0;
    for (int i = 0; i < 16; i++) {
        v3 c = v3_mul(load_xyz(in, i), cw);
        v3 t0 = v3_sub(c, p0), t1 = v3_sub(c, p1), t2 = v3_sub(c, p2), t3 = v3_sub(c, p3);
        float d0 = v3_dot(t0, t0), d1 = v3_dot(t1, t1), d2 = v3_dot(t2, t2), d3 = v3_dot(t3, t3);
        int i1 = (d1 <= d0) & (d1 < d2) & (d1 < d3);
        int i2 = (d2 <= d0) & (d2 <= d1) & (d2 < d3);
        int i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
        out |= pack_index((uint32_t)(i1 | i3), (uint32_t)(i2 | i3), i);
    }
    return out;
}

/* output_block3 (icbc.h:3238-3255): endpoints ordered col0 <= col1. */
static float output_block3(const float *in, const float *in_w, v3 cw, int allow_black, v3 v0, v3 v1, int decoder, blk *b, oracle_stats *st) {
    uint16_t c0 = vector3_to_color16(v0), c1 = vector3_to_color16(v1);
    if (c0 > c1) { uint16_t t = c0; c0 = c1; c1 = t; }
    v3 pal[4];
    eval_palette_v3(c0, c1, pal, decoder);
    b->col0 = c0;
    b->col1 = c1;
    b->indices = compute_indices3(in, cw, allow_black, pal);
    if (st) st->out3_blocks++;
    return block_mse(in, in_w, cw, pal, b->indices);
}

/* output_block4 (icbc.h:3257-3274): endpoints ordered col0 >= col1. */
static float output_block4(const float *in, const float *in_w, v3 cw, v3 v0, v3 v1, int decoder, blk *b, oracle_stats *st) {
    uint16_t c0 = vector3_to_color16(v0), c1 = vector3_to_color16(v1);
    if (c0 < c1) { uint16_t t = c0; c0 = c1; c1 = t; }
    v3 pal[4];
    eval_palette_v3(c0, c1, pal, decoder);
    b->col0 = c0;
    b->col1 = c1;
    b->indices = compute_indices4(in, cw, pal);
    if (st) st->out4_blocks++;
    return block_mse(in, in_w, cw, pal, b->indices);
}

/* ------------------------------------------------------- endpoint fitting */

/* optimize_end_points4: unweighted least squares over the 16 input texels
 * for fixed indices (icbc.h:3278-3310). */
static int optimize_end_points4(uint32_t indices, const float *in, v3 *a, v3 *b) {
    float alpha2_sum = 0.0f, beta2_sum = 0.0f, alphabeta_sum = 0.0f;
    v3 alphax_sum = {0, 0, 0}, betax_sum = {0, 0, 0};
    for (int i = 0; i < 16; i++) {
        const uint32_t bits = indices >> (2 * i);
        float beta = (float)(bits & 1);
        if (bits & 2) beta = (1 + beta) / 3.0f;
        float alpha = 1.0f - beta;
        alpha2_sum += alpha * alpha;
        beta2_sum += beta * beta;
        alphabeta_sum += alpha * beta;
        alphax_sum = v3_add(alphax_sum, v3_scale(load_xyz(in, i), alpha));
        betax_sum = v3_add(betax_sum, v3_scale(load_xyz(in, i), beta));
    }
    float denom = alpha2_sum * beta2_sum - alphabeta_sum * alphabeta_sum;
    if (feq(denom, 0.0f, 0.0001f)) return 0;
    float factor = 1.0f / denom;
    *a = v3_saturate(v3_scale(v3_sub(v3_scale(alphax_sum, beta2_sum), v3_scale(betax_sum, alphabeta_sum)), factor));
    *b = v3_saturate(v3_scale(v3_sub(v3_scale(betax_sum, alpha2_sum), v3_scale(alphax_sum, alphabeta_sum)), factor));
    return 1;
}

/* fit_colors_bbox (icbc.h:3313-3322). */
static void fit_colors_bbox(const v3 *colors, int count, v3 *c0, v3 *c1) {
    *c0 = v3_make(0, 0, 0);
    *c1 = v3_make(1, 1, 1);
    for (int i = 0; i < count; i++) {
        *c0 = v3_max(*c0, colors[i]);
        *c1 = v3_min(*c1, colors[i]);
    }
}

/* select_diagonal (icbc.h:3324-3360). */
static void select_diagonal(const v3 *colors, int count, v3 *c0, v3 *c1) {
    v3 center = v3_scale(v3_add(*c0, *c1), 0.5f);
    float cov_xz = 0.0f, cov_yz = 0.0f;
    for (int i = 0; i < count; i++) {
        v3 t = v3_sub(colors[i], center);
        cov_xz += t.x * t.z;
        cov_yz += t.y * t.z;
    }
    float x0 = c0->x, y0 = c0->y, x1 = c1->x, y1 = c1->y;
    if (cov_xz < 0) { float t = x0; x0 = x1; x1 = t; }
    if (cov_yz < 0) { float t = y0; y0 = y1; y1 = t; }
    *c0 = v3_make(x0, y0, c0->z);
    *c1 = v3_make(x1, y1, c1->z);
}

/* inset_bbox (icbc.h:3362-3368). */
static void inset_bbox(v3 *c0, v3 *c1) {
    float bias = (8.0f / 255.0f) / 16.0f;
    v3 inset = v3_saturate(v3_sub(v3_div(v3_sub(*c0, *c1), 16.0f), v3_make(bias, bias, bias)));
    *c0 = v3_saturate(v3_sub(*c0, inset));
    *c1 = v3_saturate(v3_add(*c1, inset));
}

/* compress_dxt1_single_color_optimal (icbc.h:3519-3534). */
static void single_color(c32 c, const dec_tables *dt, blk *out) {
    out->col0 = (uint16_t)((dt->match5[c.r][0] << 11) | (dt->match6[c.g][0] << 5) | dt->match5[c.b][0]);
    out->col1 = (uint16_t)((dt->match5[c.r][1] << 11) | (dt->match6[c.g][1] << 5) | dt->match5[c.b][1]);
    out->indices = 0xaaaaaaaau;
    if (out->col0 < out->col1) {
        uint16_t t = out->col0; out->col0 = out->col1; out->col1 = t;
        out->indices ^= 0x55555555u;
    }
}

/* compress_dxt1_cluster_fit (icbc.h:3537-3571). */
static float cluster_fit(const float *in, const float *in_w, const v3 *colors, const float *weights, int count,
                         v3 cw, int three_color_mode, int try_black, int allow_black, int decoder,
                         const dec_tables *dt, const prof_t *pf, blk *out, oracle_stats *st) {
    v3 metric_sqr = v3_mul(cw, cw);
    sat_t sat;
    int sat_count = compute_sat(colors, weights, count, &sat, st);
    v3 start, end;
    if (pf->vx)
        cluster_fit_four_v4(&sat, sat_count, metric_sqr, dt, pf, &start, &end, st);
    else
        cluster_fit_four(&sat, sat_count, metric_sqr, dt, pf, &start, &end, st);
    float best = output_block4(in, in_w, cw, start, end, decoder, out, st);
    if (three_color_mode) {
        if (try_black) {
            v3 tc[16];
            float tw[16];
            int tcount = skip_blacks(colors, weights, count, tc, tw);
            if (!tcount) return best;
            sat_count = compute_sat(tc, tw, tcount, &sat, st);
        }
        if (pf->vx)
            cluster_fit_three_v4(&sat, sat_count, metric_sqr, pf, &start, &end, st);
        else
            cluster_fit_three(&sat, sat_count, metric_sqr, pf, &start, &end, st);
        blk b3;
        float e3 = output_block3(in, in_w, cw, allow_black, start, end, decoder, &b3, st);
        if (e3 < best) { best = e3; *out = b3; }
    }
    return best;
}

/* Refinement deltas (icbc.h:3584-3609). */
static const int8_t k_deltas[16][3] = {
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1},
    {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {-1, -1, 0}, {-1, 0, -1}, {0, -1, -1},
    {-1, 1, 0}, {1, -1, 0}, {0, -1, 1}, {0, 1, -1}};

/* Adds a delta to the 5:6:5 fields of an endpoint with per-field wrap, as
 * the reference's bitfield += does. */
static inline uint16_t add565(uint16_t c, int dr, int dg, int db) {
    int r = (((c >> 11) & 31) + dr) & 31;
    int g = (((c >> 5) & 63) + dg) & 63;
    int b = ((c & 31) + db) & 31;
    return (uint16_t)((r << 11) | (g << 5) | b);
}

/* refine_endpoints (icbc.h:3574-3651): 256 single-step endpoint moves,
 * alternating col1/col0 every 16 steps; indices come from the palette of the
 * current best block, the error from the moved endpoints; stop after 32
 * steps without improvement. */
static float refine_endpoints(const float *in, const float *in_w, v3 cw, int three_color_mode, float input_error,
                              int decoder, blk *out, oracle_stats *st) {
    float best = input_error;
    int last = 0;
    for (int i = 0; i < 256; i++) {
        blk refined = *out;
        const int8_t *d = k_deltas[i % 16];
        if ((i / 16) & 1) refined.col0 = add565(refined.col0, d[0], d[1], d[2]);
        else refined.col1 = add565(refined.col1, d[0], d[1], d[2]);
        if (!three_color_mode) {
            if (refined.col0 == refined.col1) refined.col1 = add565(refined.col1, 0, 1, 0);
            if (refined.col0 < refined.col1) { uint16_t t = refined.col0; refined.col0 = refined.col1; refined.col1 = t; }
        }
        v3 pal[4];
        eval_palette_v3(out->col0, out->col1, pal, decoder);
        refined.indices = compute_indices(in, cw, pal);
        float e = block_mse_out(in, in_w, cw, &refined, decoder);
        if (st) st->refine_steps++;
        if (e < best) { best = e; *out = refined; last = i; }
        if (i - last > 32) break;
    }
    return best;
}

/* ------------------------------------------------------------ top level */

typedef struct {
    float threshold;
    int box_fit, least_squares_fit, cluster_fit, cluster_fit_3, cluster_fit_3_black_only, endpoint_refinement;
} options;

/* setup_options (icbc.h:3663-3731). */
static options setup_options(int level, int three_color_mode, int black) {
    options o = {0.0f, 0, 0, 0, 0, 0, 0};
    switch (level) {
    case 0: o.box_fit = 1; break;
    case 1: o.box_fit = 1; o.least_squares_fit = 1; break;
    case 2: o.box_fit = 1; o.least_squares_fit = 1; o.cluster_fit = 1;
            o.cluster_fit_3_black_only = three_color_mode && black; o.threshold = 1.0f / 24; break;
    case 3: o.box_fit = 1; o.cluster_fit = 1;
            o.cluster_fit_3_black_only = three_color_mode && black; o.threshold = 1.0f / 32; break;
    case 4: o.cluster_fit = 1; o.cluster_fit_3_black_only = three_color_mode && black; o.threshold = 1.0f / 48; break;
    case 5: o.cluster_fit = 1; o.cluster_fit_3_black_only = three_color_mode && black; o.threshold = 1.0f / 64; break;
    case 6: o.cluster_fit = 1; o.cluster_fit_3_black_only = three_color_mode && black; o.threshold = 1.0f / 96; break;
    case 7: o.cluster_fit = 1; o.cluster_fit_3_black_only = three_color_mode && black; o.threshold = 1.0f / 128; break;
    case 8: o.cluster_fit = 1; o.cluster_fit_3 = three_color_mode; o.threshold = 1.0f / 256; break;
    case 9: o.cluster_fit = 1; o.cluster_fit_3 = three_color_mode; o.threshold = 1.0f / 256; o.endpoint_refinement = 1; break;
    default: break;
    }
    return o;
}

static void store_block(const blk *b, void *out) {
    uint8_t *o = (uint8_t *)out;
    o[0] = (uint8_t)(b->col0 & 255); o[1] = (uint8_t)(b->col0 >> 8);
    o[2] = (uint8_t)(b->col1 & 255); o[3] = (uint8_t)(b->col1 >> 8);
    o[4] = (uint8_t)(b->indices & 255); o[5] = (uint8_t)((b->indices >> 8) & 255);
    o[6] = (uint8_t)((b->indices >> 16) & 255); o[7] = (uint8_t)(b->indices >> 24);
}

static void load_block(const void *in, blk *b) {
    const uint8_t *p = (const uint8_t *)in;
    b->col0 = (uint16_t)(p[0] | (p[1] << 8));
    b->col1 = (uint16_t)(p[2] | (p[3] << 8));
    b->indices = (uint32_t)p[4] | ((uint32_t)p[5] << 8) | ((uint32_t)p[6] << 16) | ((uint32_t)p[7] << 24);
}

/* Internal compress_bc1 (icbc.h:3734-3808).  Levels outside 0..9 leave the
 * output untouched and return FLT_MAX, as the reference's switch does. */
float oracle_compress_bc1(int decoder, int level, const float *in, const float *in_w, const float cwa[3],
                          int three_color_mode, int three_color_black, void *outp, oracle_stats *st) {
    oracle_init();
    int profile = (decoder >> ORACLE_PROFILE_SHIFT) & 7;
    prof_t prof = k_prof[profile < 7 ? profile : 0];
    prof.vx = (decoder & ORACLE_VECTOR_LOOPS) && prof.vec == 4;
    const prof_t *pf = &prof;
    decoder &= 3;
    const dec_tables *dt = &g_dec[decoder];
    options opt = setup_options(level, three_color_mode, three_color_black);
    v3 cw = v3_make(cwa[0], cwa[1], cwa[2]);
    v3 colors[16];
    float weights[16];
    int any_black = 0, count;
    blk out;
    load_block(outp, &out);
    if (st) st->blocks++;

    if (opt.cluster_fit) {
        count = reduce_colors(in, in_w, opt.threshold, colors, weights, &any_black, st);
    } else {
        for (int i = 0; i < 16; i++) colors[i] = load_xyz(in, i);
        count = 16;
    }

    if (count == 0) {
        out.col0 = out.col1 = 0;
        out.indices = 0;
        store_block(&out, outp);
        if (st) st->zero_blocks++;
        return 0;
    }
    if (count == 1) {
        single_color(vector3_to_color32(colors[0]), dt, &out);
        store_block(&out, outp);
        if (st) st->single_blocks++;
        return block_mse_out(in, in_w, cw, &out, decoder);
    }

    float error = FLT_MAX;
    if (opt.box_fit) {
        v3 c0, c1;
        fit_colors_bbox(colors, count, &c0, &c1);
        inset_bbox(&c0, &c1);
        select_diagonal(colors, count, &c0, &c1);
        if (st) { st->box_fits++; st->box_points += count; }
        error = output_block4(in, in_w, cw, c0, c1, decoder, &out, st);
        if (opt.least_squares_fit) {
            if (st) st->lsq_fits++;
            if (optimize_end_points4(out.indices, in, &c0, &c1)) {
                blk ob;
                float oe = output_block4(in, in_w, cw, c0, c1, decoder, &ob, st);
                if (oe < error) { error = oe; out = ob; }
            }
        }
    }
    if (opt.cluster_fit) {
        int use_black = any_black && three_color_black;
        int use_three = opt.cluster_fit_3 || (use_black && opt.cluster_fit_3_black_only);
        blk cb;
        float ce = cluster_fit(in, in_w, colors, weights, count, cw, use_three, use_black, three_color_black,
                               decoder, dt, pf, &cb, st);
        if (ce < error) { out = cb; error = ce; }
    }
    if (opt.endpoint_refinement)
        error = refine_endpoints(in, in_w, cw, three_color_mode, error, decoder, &out, st);
    if (opt.box_fit || opt.cluster_fit) store_block(&out, outp);
    return error;
}

/* ------------------------------------------------------ decode/evaluate */

void oracle_decode_bc1(const void *block, uint8_t rgba[64], int decoder) {
    blk b;
    load_block(block, &b);
    c32 pal[4];
    eval_palette32(b.col0, b.col1, pal, decoder & 3);
    for (int i = 0; i < 16; i++) {
        c32 c = pal[(b.indices >> (2 * i)) & 3];
        rgba[4 * i + 0] = (uint8_t)c.r; rgba[4 * i + 1] = (uint8_t)c.g;
        rgba[4 * i + 2] = (uint8_t)c.b; rgba[4 * i + 3] = (uint8_t)c.a;
    }
}

float oracle_evaluate_bc1_error(const uint8_t rgba[64], const void *block, int decoder) {
    blk b;
    load_block(block, &b);
    c32 pal[4];
    eval_palette32(b.col0, b.col1, pal, decoder & 3);
    float error = 0.0f;
    for (int i = 0; i < 16; i++) {
        c32 c = {rgba[4 * i + 0], rgba[4 * i + 1], rgba[4 * i + 2], 255};
        error += (float)c32_mse(pal[(b.indices >> (2 * i)) & 3], c);
    }
    return error;
}

/* icbc::decode_bc3 (icbc.h:2929-2947, :3824-3826): BlockBC3 is the BC4
 * alpha half (alpha0, alpha1, 6 index bytes) then a BC1 block.  The colour
 * palette is always the 4-colour form (evaluate_palette4, icbc.h:2882-2891).
 * The reference's alpha palette only sets entries 0 and 1 and its alpha index
 * is always 0, so every texel's alpha is alpha0. */
void oracle_decode_bc3(const void *block, uint8_t rgba[64], int decoder) {
    const uint8_t *q = (const uint8_t *)block;
    blk b;
    load_block(q + 8, &b);
    c32 pal[4];
    eval_palette32_form(b.col0, b.col1, pal, decoder & 3, 1);
    for (int i = 0; i < 16; i++) {
        c32 c = pal[(b.indices >> (2 * i)) & 3];
        rgba[4 * i + 0] = (uint8_t)c.r; rgba[4 * i + 1] = (uint8_t)c.g;
        rgba[4 * i + 2] = (uint8_t)c.b; rgba[4 * i + 3] = q[0];
    }
}

/* icbc::evaluate_bc3_error (icbc.h:3048-3071, :3841-3843): per texel, in
 * order, the colour error scaled by alpha / 255 when alpha_blend, then the
 * squared difference of alpha0 and the texel's alpha. */
float oracle_evaluate_bc3_error(const uint8_t rgba[64], const void *block, int alpha_blend, int decoder) {
    const uint8_t *q = (const uint8_t *)block;
    blk b;
    load_block(q + 8, &b);
    c32 pal[4];
    eval_palette32_form(b.col0, b.col1, pal, decoder & 3, 1);
    float error = 0.0f;
    for (int i = 0; i < 16; i++) {
        c32 c = {rgba[4 * i + 0], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3]};
        const float scale = alpha_blend ? ((float)c.a * 1.0f) / 255.0f : 1.0f;
        error += scale * (float)c32_mse(pal[(b.indices >> (2 * i)) & 3], c);
        const int da = (int)q[0] - (int)c.a;
        error += (float)(da * da);
    }
    return error;
}

void oracle_fetch_block(const uint8_t *rgba, int w, int h, int64_t pitch, int bx, int by, uint8_t tex[64]) {
    for (int yy = 0; yy < 4; yy++) {
        int y = by * 4 + yy;
        if (y > h - 1) y = h - 1;
        for (int xx = 0; xx < 4; xx++) {
            int x = bx * 4 + xx;
            if (x > w - 1) x = w - 1;
            memcpy(&tex[(yy * 4 + xx) * 4], rgba + (int64_t)y * pitch + (int64_t)x * 4, 4);
        }
    }
}

double oracle_image_sse(const uint8_t *rgba, int w, int h, int64_t pitch, const void *blocks, int decoder) {
    const int bw = (w + 3) / 4, bh = (h + 3) / 4;
    double total = 0.0;
    for (int by = 0; by < bh; by++)
        for (int bx = 0; bx < bw; bx++) {
            uint8_t tex[64], dec[64];
            oracle_fetch_block(rgba, w, h, pitch, bx, by, tex);
            oracle_decode_bc1((const uint8_t *)blocks + 8 * ((int64_t)by * bw + bx), dec, decoder);
            for (int i = 0; i < 16; i++)
                for (int c = 0; c < 3; c++) {
                    double d = (double)dec[4 * i + c] - (double)tex[4 * i + c];
                    total += d * d;
                }
        }
    return total;
}

/* ------------------------------------------------- threaded block loops */

typedef struct {
    int decoder, level, tc, tcb;
    const float *colors, *weights;
    float cw[3];
    uint8_t *out;
    float *errors;
    int64_t n;
    /* image mode */
    const uint8_t *rgba;
    int w, h, bw, weight_mode;
    int64_t pitch;
    const float *plane;
    int64_t next;
    pthread_mutex_t lock;
    oracle_stats stats;
} job_t;

static int64_t take_chunk(job_t *j) {
    return __atomic_fetch_add(&j->next, 32, __ATOMIC_RELAXED);
}

static void merge_stats(job_t *j, const oracle_stats *s) {
    pthread_mutex_lock(&j->lock);
    int64_t *dst = (int64_t *)&j->stats;
    const int64_t *src = (const int64_t *)s;
    for (size_t k = 0; k < sizeof(oracle_stats) / sizeof(int64_t); k++) dst[k] += src[k];
    pthread_mutex_unlock(&j->lock);
}

static void *block_worker(void *arg) {
    job_t *j = (job_t *)arg;
    oracle_stats st;
    memset(&st, 0, sizeof(st));
    static const float ones[16] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
    for (;;) {
        int64_t b0 = take_chunk(j);
        if (b0 >= j->n) break;
        int64_t b1 = b0 + 32 < j->n ? b0 + 32 : j->n;
        for (int64_t b = b0; b < b1; b++) {
            float e;
            if (j->rgba) {
                uint8_t tex[64];
                float col[64], wt[16];
                int bx = (int)(b % j->bw), by = (int)(b / j->bw);
                oracle_fetch_block(j->rgba, j->w, j->h, j->pitch, bx, by, tex);
                for (int t = 0; t < 16; t++) {
                    col[4 * t + 0] = tex[4 * t + 0] / 255.0f;
                    col[4 * t + 1] = tex[4 * t + 1] / 255.0f;
                    col[4 * t + 2] = tex[4 * t + 2] / 255.0f;
                    col[4 * t + 3] = 1.0f;
                    if (j->weight_mode == ORACLE_W_ALPHA) wt[t] = tex[4 * t + 3] / 255.0f;
                    else if (j->weight_mode == ORACLE_W_PLANE) {
                        int x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
                        if (x > j->w - 1) x = j->w - 1;
                        if (y > j->h - 1) y = j->h - 1;
                        wt[t] = j->plane[(int64_t)y * j->w + x];
                    } else wt[t] = 1.0f;
                }
                memset(j->out + 8 * b, 0, 8);
                e = oracle_compress_bc1(j->decoder, j->level, col, wt, j->cw, j->tc, j->tcb, j->out + 8 * b, &st);
            } else {
                e = oracle_compress_bc1(j->decoder, j->level, j->colors + 64 * b,
                                        j->weights ? j->weights + 16 * b : ones, j->cw, j->tc, j->tcb,
                                        j->out + 8 * b, &st);
            }
            if (j->errors) j->errors[b] = e;
        }
    }
    merge_stats(j, &st);
    return NULL;
}

static int run_job(job_t *j, int nthreads, oracle_stats *stats) {
    oracle_init();
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    j->next = 0;
    memset(&j->stats, 0, sizeof(j->stats));
    pthread_mutex_init(&j->lock, NULL);
    pthread_t th[256];
    int started = 0;
    for (int t = 1; t < nthreads; t++)
        if (pthread_create(&th[started], NULL, block_worker, j) == 0) started++;
    block_worker(j);
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&j->lock);
    if (stats) *stats = j->stats;
    return started + 1;
}

int oracle_compress_blocks(int decoder, int level, const float *colors, const float *weights, const float cw[3],
                           int tc, int tcb, void *out, float *errors, int64_t n, int nthreads, oracle_stats *stats) {
    job_t j;
    memset(&j, 0, sizeof(j));
    j.decoder = decoder; j.level = level; j.tc = tc; j.tcb = tcb;
    j.colors = colors; j.weights = weights;
    j.cw[0] = cw[0]; j.cw[1] = cw[1]; j.cw[2] = cw[2];
    j.out = (uint8_t *)out; j.errors = errors; j.n = n;
    return run_job(&j, nthreads, stats);
}

int oracle_encode_image(const uint8_t *rgba, int w, int h, int64_t pitch, int weight_mode, const float *plane,
                        int decoder, int level, const float cw[3], int tc, int tcb, void *out, float *errors,
                        int nthreads, oracle_stats *stats) {
    job_t j;
    memset(&j, 0, sizeof(j));
    j.decoder = decoder; j.level = level; j.tc = tc; j.tcb = tcb;
    j.cw[0] = cw[0]; j.cw[1] = cw[1]; j.cw[2] = cw[2];
    j.out = (uint8_t *)out; j.errors = errors;
    j.rgba = rgba; j.w = w; j.h = h; j.pitch = pitch; j.weight_mode = weight_mode; j.plane = plane;
    j.bw = (w + 3) / 4;
    j.n = (int64_t)j.bw * ((h + 3) / 4);
    return run_job(&j, nthreads, stats);
}
