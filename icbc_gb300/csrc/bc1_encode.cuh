// bc1_encode.cuh -- the BC1 block encoder for one warp of 32 blocks.
//
// Work split inside a warp:
//   * serial stages of icbc's compress_bc1 (reduce_colors, box fit, least
//     squares, PCA + summed-area table, index selection, refinement) run one
//     block per lane;
//   * the 4- and 3-cluster enumerations (the hot loops) run warp-wide: the
//     combinations of every block of the warp that needs a search form one
//     list, cut into 64 ranges walked two per lane; a walker keeps the first
//     strict minimum of its share and folds it into its block's slot with a
//     64-bit atomicMin, ties going to the lowest table index -- the winner
//     the sequential loop of icbc.h:2362-2733 keeps.
//
// Shared memory per warp, one row per block of the warp:
//   in    [32][65]  texels r,g,b (float) + weight, 16 x 4 floats (odd stride:
//                   per-lane scalar accesses are conflict-free)
//   sat   [32][68]  float4 (r, g, b, w) entries: first the reduced colours
//                   (reduce_colors), then, built in place through registers,
//                   the SAT with a leading zero entry, entries 0..16 (17
//                   float4 per row: any 8 lanes' 16-byte accesses to entry k
//                   of their rows, or to different entries of any rows in
//                   the cluster search, spread over the 8 bank groups)
//   slots [32]      u64 per block: best (error, table index) of a cluster search
//   info  [32]      int per block: its first combination | colour count << 24
// 17 KB per warp: three 4-warp CTAs per SM at levels 2..9.
#pragma once

#include "bc1_device.cuh"

namespace icbc_gpu {

constexpr int kWarpsPerCta = 4;
constexpr int kInStride = 65;
constexpr int kSatStride = 68;
constexpr unsigned kFull = 0xffffffffu;

constexpr size_t kWarpFloatsLow = 32 * kInStride;                                  // L0, L1
constexpr size_t kWarpFloatsHigh = 32 * kInStride + 32 * kSatStride + 64 + 32;    // L2..L9

__host__ __device__ constexpr size_t smem_bytes(bool cluster_fit) {
    return sizeof(SharedTables) + kWarpsPerCta * 4 * (cluster_fit ? kWarpFloatsHigh : kWarpFloatsLow);
}
// The RGBA8 image kernels of levels 2..9 keep texels as bytes (ByteRow): 17
// words per lane (odd stride) instead of 65 floats, 11 KB per warp in all --
// small enough for four CTAs per SM.
constexpr int kInWordsByte = 17;
constexpr size_t kWarpFloatsByte = 32 * kInWordsByte + 32 * kSatStride + 64 + 32;
__host__ __device__ constexpr size_t smem_bytes_byte_rows() { return sizeof(SharedTables) + kWarpsPerCta * 4 * kWarpFloatsByte; }

// Options of each quality level (setup_options, icbc.h:3663-3731).
template <int L>
struct Level {
    static constexpr bool box = L <= 3;
    static constexpr bool lsq = L == 1 || L == 2;
    static constexpr bool cluster = L >= 2;
    static constexpr bool cf3_black_only = L >= 2 && L <= 7;
    static constexpr bool cf3_always = L >= 8;
    static constexpr bool refine = L == 9;
    static constexpr float threshold = L == 2 ? 1.0f / 24 : L == 3 ? 1.0f / 32 : L == 4 ? 1.0f / 48
                                     : L == 5 ? 1.0f / 64 : L == 6 ? 1.0f / 96 : L == 7 ? 1.0f / 128
                                     : L >= 8 ? 1.0f / 256 : 0.0f;
};

// Refinement step deltas (icbc.h:3584-3609).
__constant__ int8_t c_deltas[16][3] = {
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1},
    {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {-1, -1, 0}, {-1, 0, -1}, {0, -1, -1},
    {-1, 1, 0}, {1, -1, 0}, {0, -1, 1}, {0, 1, -1}};

struct EncodeParams {
    int decoder;
    int three_color_mode;
    int three_color_black;
    V3 cw;
    // SIMD profile of the reference build reproduced by the profile kernels
    // (bc1_simd.cu): vector width of the cluster loops, fused vmadd/vmsub,
    // vround01 half to even, vsaturate keeping a NaN (NEON), and what the
    // gather of the SAT reads past its table (fill_sat_tail).  The plain
    // kernels ignore these.
    int simd_vec, simd_fma, simd_rne, simd_nan, simd_gather;
};

// Everything one warp needs for a group of 32 blocks.
struct WarpCtx {
    const SharedTables *T;
    const DecoderTables *D;
    float *in;
    float *sat;                  // per block: 17 float4 (r, g, b, w) SAT entries
    unsigned long long *slots;   // per block: the search's argmin key
    int *info;                   // per block: first combination | count << 24
    int lane;
};

// ------------------------------------------------------------ per lane --

// A lane's SAT row holds float4 (r, g, b, w) entries: its reduced colours,
// then its summed-area table.  The row stride (17 float4) puts the 16-byte
// accesses of 8 lanes (one shared-memory phase) in 8 different bank groups,
// whether the lanes read their own rows or the walkers gather across rows.
__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ V3 xyz(float4 v) { return v3(v.x, v.y, v.z); }

// reduce_colors (icbc.h:1683-1728) into rrow (the lane's SAT row, as scratch).
template <class Row>
__device__ __forceinline__ int reduce_colors(const Row &row, float threshold, float *rrow, bool &any_black) {
    int n = 0;
    any_black = false;
    for (int i = 0; i < 16; i++) {
        const V3 ci = row.color(i);
        const float wi = row.weight(i);
        if (wi > 0) {
            int j = 0;
            for (; j < n; j++) {
                const float4 c4 = ld4(rrow + 4 * j);
                const V3 cj = xyz(c4);
                if (near3(cj, ci, threshold)) {
                    const float wj = c4.w;
                    const float s = wj + wi;
                    if (Row::kBounded)
                        st4(rrow + 4 * j, make_float4(div_bounded(cj.x * wj + ci.x * wi, s),
                                                      div_bounded(cj.y * wj + ci.y * wi, s),
                                                      div_bounded(cj.z * wj + ci.z * wi, s), s));
                    else
                        st4(rrow + 4 * j, make_float4((cj.x * wj + ci.x * wi) / s, (cj.y * wj + ci.y * wi) / s,
                                                      (cj.z * wj + ci.z * wi) / s, s));
                    break;
                }
            }
            if (j == n) {
                st4(rrow + 4 * n, make_float4(ci.x, ci.y, ci.z, wi));
                n++;
            }
            if (is_black(ci)) any_black = true;
        }
    }
    return n;
}

// compute_sat (icbc.h:1857-1937) in place: the reduced colours in the lane's
// SAT row are read into registers, then the row is overwritten with the SAT.
// With skip_black the colours skip_blacks (icbc.h:1730-1748) would drop are
// masked out instead of compacted (order among the rest is unchanged, so
// every sum runs in the reference's order).  Returns the number of colours
// in the table (0: nothing left).
//   centroid, covariance, power iterations: icbc.h:1755-1844
//   stable insertion sort along the axis: replaced by stable ranks
//     (position = #smaller + #equal-and-earlier), the same permutation for
//     every non-NaN key; keys containing NaN take a literal insertion sort.
// N: the unrolled width, 16 or, when count <= N, 8 or 12 (the same sums in
// the same order: the entries past count contribute nothing either way).
template <int N = 16>
__device__ __forceinline__ int build_sat_inplace(float *srow, int count, bool skip_black) {
    float cx[N], cy[N], cz[N], cw[N];
    unsigned use = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const bool in = i < count;
        const float4 c = ld4(srow + 4 * i);
        cx[i] = in ? c.x : 0.0f;
        cy[i] = in ? c.y : 0.0f;
        cz[i] = in ? c.z : 0.0f;
        cw[i] = in ? c.w : 0.0f;
        if (in && !(skip_black && is_black(v3(cx[i], cy[i], cz[i])))) use |= 1u << i;
    }
    const int m = __popc(use);
    if (m == 0) return 0;
    V3 centroid = v3(0.0f, 0.0f, 0.0f);
    float total = 0.0f;
#pragma unroll
    for (int i = 0; i < N; i++) {
        if (use & (1u << i)) {
            total += cw[i];
            centroid = centroid + v3(cx[i], cy[i], cz[i]) * cw[i];
        }
    }
    centroid = centroid * (1.0f / total);
    float m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        if (use & (1u << i)) {
            const V3 a = v3(cx[i], cy[i], cz[i]) - centroid;
            const V3 b = a * cw[i];
            m0 += a.x * b.x; m1 += a.x * b.y; m2 += a.x * b.z;
            m3 += a.y * b.y; m4 += a.y * b.z; m5 += a.z * b.z;
        }
    }
    V3 axis = v3(0.0f, 0.0f, 0.0f);
    if (!(m0 == 0 && m3 == 0 && m5 == 0)) {
        const V3 row0 = v3(m0, m1, m2), row1 = v3(m1, m3, m4), row2 = v3(m2, m4, m5);
        const float r0 = dot(row0, row0), r1 = dot(row1, row1), r2 = dot(row2, row2);
        V3 v = (r0 > r1 && r0 > r2) ? row0 : (r1 > r2 ? row1 : row2);
#pragma unroll
        for (int it = 0; it < 6; it++) {
            const float x = v.x * m0 + v.y * m1 + v.z * m2;
            const float y = v.x * m1 + v.y * m3 + v.z * m4;
            const float z = v.x * m2 + v.y * m4 + v.z * m5;
            const float norm = tmax(tmax(x, y), z);
            v = v3(x, y, z) * (1.0f / norm);
        }
        axis = v;
    }
    float dps[N];
    bool has_nan = false;
#pragma unroll
    for (int i = 0; i < N; i++) {
        dps[i] = dot(v3(cx[i], cy[i], cz[i]), axis);
        has_nan |= ((use >> i) & 1) && (dps[i] != dps[i]);
    }
    st4(srow, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (!has_nan) {
        // Stable ranks from the pairs i < j (120 at width 16): j sorts
        // before i iff dps[j] < dps[i]; otherwise i (the earlier one) sorts
        // before j.
        int pos[N];
#pragma unroll
        for (int i = 0; i < N; i++) pos[i] = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
#pragma unroll
            for (int j = i + 1; j < N; j++) {
                const bool both = ((use >> i) & (use >> j) & 1) != 0;
                const bool j_first = dps[j] < dps[i];
                pos[i] += both && j_first;
                pos[j] += both && !j_first;
            }
        }
#pragma unroll
        for (int i = 0; i < N; i++) {
            if (use & (1u << i)) st4(srow + 4 * (pos[i] + 1), make_float4(cx[i] * cw[i], cy[i] * cw[i], cz[i] * cw[i], cw[i]));
        }
    } else {
        // Literal stable insertion sort of the kept colours (NaN keys).  The
        // colours are copied to a local array first so that the dynamic
        // indexing here does not move the register arrays to local memory.
        float lc[4 * N];
#pragma unroll
        for (int i = 0; i < N; i++) {
            lc[4 * i + 0] = cx[i];
            lc[4 * i + 1] = cy[i];
            lc[4 * i + 2] = cz[i];
            lc[4 * i + 3] = cw[i];
        }
        int order[N];
        float key[N];
        int k = 0;
#pragma unroll
        for (int i = 0; i < N; i++)
            if (use & (1u << i)) { order[k] = i; key[k] = dps[i]; k++; }
        for (int i = 0; i < m; i++)
            for (int j = i; j > 0 && key[j] < key[j - 1]; j--) {
                const float t = key[j]; key[j] = key[j - 1]; key[j - 1] = t;
                const int o = order[j]; order[j] = order[j - 1]; order[j - 1] = o;
            }
        for (int q = 0; q < m; q++) {
            const float *c = lc + 4 * order[q];
            st4(srow + 4 * (q + 1), make_float4(c[0] * c[3], c[1] * c[3], c[2] * c[3], c[3]));
        }
    }
    // Prefix sums in sorted order: entry k = entry k - 1 + term k.
    float4 acc = ld4(srow + 4);
    for (int k = 2; k <= m; k++) {
        const float4 t = ld4(srow + 4 * k);
        acc = make_float4(acc.x + t.x, acc.y + t.y, acc.z + t.z, acc.w + t.w);
        st4(srow + 4 * k, acc);
    }
    return m;
}

// output_block4 (icbc.h:3257-3274): endpoints ordered col0 >= col1.
template <class Row>
__device__ __forceinline__ float output_block4(const WarpCtx &w, const Row &row, const EncodeParams &p, V3 v0, V3 v1,
                                               uint32_t &c0, uint32_t &c1, uint32_t &idx) {
    uint32_t a = to565(v0, *w.T), b = to565(v1, *w.T);
    if (a < b) { const uint32_t t = a; a = b; b = t; }
    const PalF pal = palette_f(a, b, p.decoder, w.T->lut255, w.D);
    c0 = a;
    c1 = b;
    return select_indices<4>(row, p.cw, pal, false, idx);
}

// output_block3 (icbc.h:3238-3255): endpoints ordered col0 <= col1.
template <class Row>
__device__ __forceinline__ float output_block3(const WarpCtx &w, const Row &row, const EncodeParams &p, V3 v0, V3 v1,
                                               uint32_t &c0, uint32_t &c1, uint32_t &idx) {
    uint32_t a = to565(v0, *w.T), b = to565(v1, *w.T);
    if (a > b) { const uint32_t t = a; a = b; b = t; }
    const PalF pal = palette_f(a, b, p.decoder, w.T->lut255, w.D);
    c0 = a;
    c1 = b;
    return select_indices<3>(row, p.cw, pal, p.three_color_black != 0, idx);
}

// optimize_end_points4 (icbc.h:3278-3310): unweighted least squares over the
// 16 input texels for fixed indices.
template <class Row>
__device__ __forceinline__ bool optimize_end_points4(const Row &row, uint32_t indices, V3 &a, V3 &b) {
    float alpha2 = 0.0f, beta2 = 0.0f, ab = 0.0f;
    V3 ax = v3(0.0f, 0.0f, 0.0f), bx = v3(0.0f, 0.0f, 0.0f);
#pragma unroll 1
    for (int i = 0; i < 16; i++) {
        const uint32_t bits = indices >> (2 * i);
        // beta = bits & 1, and for bits & 2 (1 + beta) / 3: the two possible
        // quotients are the constants 1/3 and 2/3 as floats.
        float beta = (float)(bits & 1);
        if (bits & 2) beta = (bits & 1) ? 2.0f / 3.0f : 1.0f / 3.0f;
        const float alpha = 1.0f - beta;
        alpha2 += alpha * alpha;
        beta2 += beta * beta;
        ab += alpha * beta;
        const V3 c = row.color(i);
        ax = ax + c * alpha;
        bx = bx + c * beta;
    }
    const float denom = alpha2 * beta2 - ab * ab;
    if (fabsf(denom - 0.0f) < 0.0001f) return false;
    const float factor = 1.0f / denom;
    a = saturate((ax * beta2 - bx * ab) * factor);
    b = saturate((bx * alpha2 - ax * ab) * factor);
    return true;
}

// Box fit: fit_colors_bbox, inset_bbox, select_diagonal (icbc.h:3313-3368).
// `colors`: the reduced colours in a SAT row (SatColors) or a texel row.
struct SatColors {
    const float *p;
    __device__ __forceinline__ V3 color(int i) const { return xyz(ld4(p + 4 * i)); }
};

template <class C>
__device__ __forceinline__ void box_fit(const C &colors, int count, V3 &c0, V3 &c1) {
    c0 = v3(0.0f, 0.0f, 0.0f);
    c1 = v3(1.0f, 1.0f, 1.0f);
    for (int i = 0; i < count; i++) {
        const V3 c = colors.color(i);
        c0 = vmax(c0, c);
        c1 = vmin(c1, c);
    }
    const float bias = (8.0f / 255.0f) / 16.0f;
    const V3 d = c0 - c1;
    const V3 inset = saturate(v3(d.x / 16.0f - bias, d.y / 16.0f - bias, d.z / 16.0f - bias));
    c0 = saturate(c0 - inset);
    c1 = saturate(c1 + inset);
    const V3 center = (c0 + c1) * 0.5f;
    float cov_xz = 0.0f, cov_yz = 0.0f;
    for (int i = 0; i < count; i++) {
        const V3 t = colors.color(i) - center;
        cov_xz += t.x * t.z;
        cov_yz += t.y * t.z;
    }
    float x0 = c0.x, y0 = c0.y, x1 = c1.x, y1 = c1.y;
    if (cov_xz < 0) { const float t = x0; x0 = x1; x1 = t; }
    if (cov_yz < 0) { const float t = y0; y0 = y1; y1 = t; }
    c0 = v3(x0, y0, c0.z);
    c1 = v3(x1, y1, c1.z);
}

// compress_dxt1_single_color_optimal (icbc.h:3519-3534) of vector3_to_color32(c).
__device__ __forceinline__ void single_color(const DecoderTables *D, V3 c, uint32_t &c0, uint32_t &c1, uint32_t &idx) {
    const uint32_t r = (uint32_t)(saturate(c.x) * 255 + 0.5f) & 255;
    const uint32_t g = (uint32_t)(saturate(c.y) * 255 + 0.5f) & 255;
    const uint32_t b = (uint32_t)(saturate(c.z) * 255 + 0.5f) & 255;
    uint32_t a0 = ((uint32_t)D->match5[r][0] << 11) | ((uint32_t)D->match6[g][0] << 5) | D->match5[b][0];
    uint32_t a1 = ((uint32_t)D->match5[r][1] << 11) | ((uint32_t)D->match6[g][1] << 5) | D->match5[b][1];
    uint32_t ix = 0xaaaaaaaau;
    if (a0 < a1) { const uint32_t t = a0; a0 = a1; a1 = t; ix ^= 0x55555555u; }
    c0 = a0;
    c1 = a1;
    idx = ix;
}

__device__ __forceinline__ uint32_t add565(uint32_t c, int dr, int dg, int db) {
    const uint32_t r = (((c >> 11) & 31) + dr) & 31;
    const uint32_t g = (((c >> 5) & 63) + dg) & 63;
    const uint32_t b = ((c & 31) + db) & 31;
    return (r << 11) | (g << 5) | b;
}

// Generic nearest-of-four index of one texel (compute_indices' loop body,
// icbc.h:3179-3235), palette entries already multiplied by the colour weights.
__device__ __forceinline__ uint32_t index_generic(V3 color, V3 cw, V3 p0, V3 p1, V3 p2, V3 p3) {
    const V3 c = color * cw;
    const V3 t0 = c - p0, t1 = c - p1, t2 = c - p2, t3 = c - p3;
    const float d0 = dot(t0, t0), d1 = dot(t1, t1), d2 = dot(t2, t2), d3 = dot(t3, t3);
    const bool i1 = (d1 <= d0) & (d1 < d2) & (d1 < d3);
    const bool i2 = (d2 <= d0) & (d2 <= d1) & (d2 < d3);
    const bool i3 = (d3 <= d0) & (d3 <= d1) & (d3 <= d2);
    return (uint32_t)(i1 | i3) | ((uint32_t)(i2 | i3) << 1);
}

// Generic nearest-of-four indices (compute_indices, icbc.h:3179-3235).
template <int UNROLL = 1, class Row>
__device__ __forceinline__ uint32_t indices_generic(const Row &row, V3 cw, const PalF &pal) {
    const V3 p0 = pal.c[0] * cw, p1 = pal.c[1] * cw, p2 = pal.c[2] * cw, p3 = pal.c[3] * cw;
    uint32_t out = 0;
#pragma unroll UNROLL
    for (int t = 0; t < 16; t++) out |= index_generic(row.color(t), cw, p0, p1, p2, p3) << (2 * t);
    return out;
}

// refine_endpoints (icbc.h:3574-3651).  Indices of a step come from the
// palette of the current best block, so they change only when a step is
// accepted; the step's error uses the moved endpoints' palette.
template <class Row>
__device__ __forceinline__ float refine(const WarpCtx &w, const Row &row, const EncodeParams &p, float input_error,
                                        uint32_t &c0, uint32_t &c1, uint32_t &idx) {
    float best = input_error;
    int last = 0;
    uint32_t base_idx = indices_generic(row, p.cw, palette_f(c0, c1, p.decoder, w.T->lut255, w.D));
    for (int i = 0; i < 256; i++) {
        const int d = i & 15;
        const int dr = c_deltas[d][0], dg = c_deltas[d][1], db = c_deltas[d][2];
        uint32_t r0 = c0, r1 = c1;
        if ((i >> 4) & 1) r0 = add565(r0, dr, dg, db);
        else r1 = add565(r1, dr, dg, db);
        if (!p.three_color_mode) {
            if (r0 == r1) r1 = add565(r1, 0, 1, 0);
            if (r0 < r1) { const uint32_t t = r0; r0 = r1; r1 = t; }
        }
        const PalF pr = palette_f(r0, r1, p.decoder, w.T->lut255, w.D);
        const float e = block_error(row, p.cw, pr, base_idx);
        if (e < best) {
            best = e;
            c0 = r0;
            c1 = r1;
            idx = base_idx;
            last = i;
            base_idx = indices_generic(row, p.cw, pr);
        }
        if (i - last > 32) break;
    }
    return best;
}

// One block's refinement state, for refinement run one step at a time.
struct RefineLane {
    uint32_t c0, c1, idx, base_idx;
    float best;
    int i, last;
};

// `lut`: the exact table of i / 255.0f.
template <class Row>
__device__ __forceinline__ void refine_begin(const WarpCtx &w, const float *lut, const Row &row, const EncodeParams &p,
                                             float error, uint32_t c0, uint32_t c1, uint32_t idx, RefineLane &s) {
    s.c0 = c0;
    s.c1 = c1;
    s.idx = idx;
    s.best = error;
    s.i = 0;
    s.last = 0;
    s.base_idx = indices_generic<4>(row, p.cw, palette_f(c0, c1, p.decoder, lut, w.D));
}

// block_error with the palette in shared memory: entry e of this lane at
// pal[32 * e] (a warp's palettes laid out entry-major, so the 16-byte loads of
// any 8 lanes fall in 8 bank groups whatever their indices).  One load per
// texel instead of a 4-way select; the same floats in the same order.
template <int UNROLL = 1, class Row>
__device__ __forceinline__ float block_error_pal(const Row &row, V3 cw, const PalF &p, float4 *pal,
                                                 uint32_t indices) {
#pragma unroll
    for (int e = 0; e < 4; e++) pal[32 * e] = make_float4(p.c[e].x, p.c[e].y, p.c[e].z, 0.0f);
    float error = 0.0f;
#pragma unroll UNROLL
    for (int t = 0; t < 16; t++) {
        const float4 q = pal[32 * ((indices >> (2 * t)) & 3)];
        error += row.weight(t) * texel_mse(v3(q.x, q.y, q.z), row.color(t), cw);
    }
    return error;
}

// Iteration s.i of refine_endpoints (icbc.h:3614-3648), one trip of
// refine()'s loop but for its index update: when the step is accepted it
// takes the candidate and returns true with the candidate's palette in `pr`,
// and s.base_idx must be set to indices_generic(row, cw, pr) before the next
// iteration (the caller computes it, across lanes).  `stop`: the loop would
// stop after this iteration.  With `pal` (this lane's shared-memory palette
// slot, block_error_pal) the step's error picks entries by a load.
template <class Row>
__device__ __forceinline__ bool refine_try(const WarpCtx &w, const float *lut, const Row &row, const EncodeParams &p,
                                           RefineLane &s, PalF &pr, bool &stop, float4 *pal = nullptr) {
    const int d = s.i & 15;
    const int dr = c_deltas[d][0], dg = c_deltas[d][1], db = c_deltas[d][2];
    uint32_t r0 = s.c0, r1 = s.c1;
    if ((s.i >> 4) & 1) r0 = add565(r0, dr, dg, db);
    else r1 = add565(r1, dr, dg, db);
    if (!p.three_color_mode) {
        if (r0 == r1) r1 = add565(r1, 0, 1, 0);
        if (r0 < r1) { const uint32_t t = r0; r0 = r1; r1 = t; }
    }
    pr = palette_f(r0, r1, p.decoder, lut, w.D);
    const float e = pal ? block_error_pal<4>(row, p.cw, pr, pal, s.base_idx) : block_error<4>(row, p.cw, pr, s.base_idx);
    const bool accept = e < s.best;
    if (accept) {
        s.best = e;
        s.c0 = r0;
        s.c1 = r1;
        s.idx = s.base_idx;
        s.last = s.i;
    }
    s.i++;
    stop = (s.i - 1 - s.last > 32) || s.i == 256;
    return accept;
}

// Per-block hand-over from the encode kernel to the refinement kernel.
struct RefineSlot {
    float error;       // compress_bc1's error before refinement
    uint32_t pending;  // 1: refinement applies (two or more distinct colours)
};

// ---------------------------------------------------------- cluster fit --

// Per-block sums of a SAT (its last entry) and the warp-uniform weights.
struct FitSums {
    float r_sum, g_sum, b_sum, w_sum;
};

struct FitWeights {
    float w1_3, w2_3, w1_9, w4_9, w2_9;
    V3 metric;
};

__device__ __forceinline__ FitSums fit_sums(const float *S, int count) {
    const float4 v = ld4(S + 4 * count);
    FitSums k;
    k.r_sum = v.x;
    k.g_sum = v.y;
    k.b_sum = v.z;
    k.w_sum = v.w;
    return k;
}

__device__ __forceinline__ FitWeights fit_weights(const DecoderTables *D, V3 metric) {
    FitWeights k;
    k.w1_3 = D->w1_3; k.w2_3 = D->w2_3; k.w1_9 = D->w1_9; k.w4_9 = D->w4_9; k.w2_9 = D->w2_9;
    k.metric = metric;
    return k;
}

// The metric-weighted error of a combination's snapped endpoints
// (icbc.h:2317-2323, :2715-2722): e2 = (a * (b * ab - ax) - b * bx) * 2,
// e1 = (a * a) * alpha2 + ((b * b) * beta2 + e2), dot(e1, metric).  BND:
// the product by 2 folds into the sum as one fused multiply-add (exact).
template <bool BND>
__device__ __forceinline__ float fit_error(V3 a, V3 b, V3 ax, V3 bx, float alpha2, float beta2, float ab, V3 metric) {
    const V3 t = v3(a.x * (b.x * ab - ax.x) - b.x * bx.x, a.y * (b.y * ab - ax.y) - b.y * bx.y,
                    a.z * (b.z * ab - ax.z) - b.z * bx.z);
    V3 e1;
    if (BND) {
        e1 = v3((a.x * a.x) * alpha2 + __fmaf_rn(t.x, 2.0f, (b.x * b.x) * beta2),
                (a.y * a.y) * alpha2 + __fmaf_rn(t.y, 2.0f, (b.y * b.y) * beta2),
                (a.z * a.z) * alpha2 + __fmaf_rn(t.z, 2.0f, (b.z * b.z) * beta2));
    } else {
        e1 = v3((a.x * a.x) * alpha2 + ((b.x * b.x) * beta2 + t.x * 2.0f),
                (a.y * a.y) * alpha2 + ((b.y * b.y) * beta2 + t.y * 2.0f),
                (a.z * a.z) * alpha2 + ((b.z * b.z) * beta2 + t.z * 2.0f));
    }
    return dot(e1, metric);
}

// One cluster_fit_four iteration (icbc.h:2650-2722), scalar arithmetic order.
// BND (inputs of a kBounded row): e2 = t * 2 enters e1 only through
// (b * b) * beta2 + e2, and t * 2 is exact when t cannot overflow, so the
// product and that sum are one fused multiply-add with the same bits; and
// the determinant is +0 or of magnitude between 2^-100 and 2^100 (weights
// are 0 or at least 1/255, sums at most 16), where rcp_bounded is 1 / d.
template <bool BND = false>
__device__ __forceinline__ float cf4_combo(const float *S, uint32_t packed, const FitSums &k, const FitWeights &q,
                                          V3 &a, V3 &b) {
    const int i0 = packed & 0xff, i1 = (packed >> 8) & 0xff, i2 = packed >> 16;
    const float4 s0 = ld4(S + 4 * i0), s1 = ld4(S + 4 * i1), s2 = ld4(S + 4 * i2);
    V3 x0 = xyz(s0), x1 = xyz(s1), x2 = xyz(s2);
    const float w0 = s0.w;
    float w1 = s1.w, w2 = s2.w;
    const float w3 = k.w_sum - w2;
    x2 = x2 - x1;
    x1 = x1 - x0;
    w2 = w2 - w1;
    w1 = w1 - w0;
    const float alpha2 = w2 * q.w1_9 + (w1 * q.w4_9 + w0);
    const float beta2 = w1 * q.w1_9 + (w2 * q.w4_9 + w3);
    const float ab = (w1 + w2) * q.w2_9;
    const float factor = BND ? rcp_bounded(alpha2 * beta2 - ab * ab) : 1.0f / (alpha2 * beta2 - ab * ab);
    const V3 ax = v3(x2.x * q.w1_3 + (x1.x * q.w2_3 + x0.x), x2.y * q.w1_3 + (x1.y * q.w2_3 + x0.y),
                     x2.z * q.w1_3 + (x1.z * q.w2_3 + x0.z));
    const V3 bx = v3(k.r_sum - ax.x, k.g_sum - ax.y, k.b_sum - ax.z);
    a = round_ept(v3((ax.x * beta2 - bx.x * ab) * factor, (ax.y * beta2 - bx.y * ab) * factor,
                     (ax.z * beta2 - bx.z * ab) * factor));
    b = round_ept(v3((bx.x * alpha2 - ax.x * ab) * factor, (bx.y * alpha2 - ax.y * ab) * factor,
                     (bx.z * alpha2 - ax.z * ab) * factor));
    return fit_error<BND>(a, b, ax, bx, alpha2, beta2, ab, q.metric);
}

// One cluster_fit_three iteration (icbc.h:2273-2323).  BND: as cf4_combo,
// and x1 * 0.5 is exact (never denormal), so alphax_sum = x0 + x1 * 0.5 is
// one fused multiply-add.
template <bool BND = false>
__device__ __forceinline__ float cf3_combo(const float *S, uint32_t packed, const FitSums &k, const FitWeights &q,
                                          V3 &a, V3 &b) {
    const int i0 = packed & 0xff, i1 = (packed >> 8) & 0xff;
    const float4 s0 = ld4(S + 4 * i0), s1 = ld4(S + 4 * i1);
    const V3 x0 = xyz(s0);
    V3 x1 = xyz(s1);
    const float w0 = s0.w;
    float w1 = s1.w;
    const float w2 = k.w_sum - w1;
    x1 = x1 - x0;
    w1 = w1 - w0;
    const float ab = w1 * 0.25f;
    const float alpha2 = w0 + ab;
    const float beta2 = w2 + ab;
    const float factor = BND ? rcp_bounded(alpha2 * beta2 - ab * ab) : 1.0f / (alpha2 * beta2 - ab * ab);
    const V3 ax = BND ? v3(__fmaf_rn(x1.x, 0.5f, x0.x), __fmaf_rn(x1.y, 0.5f, x0.y), __fmaf_rn(x1.z, 0.5f, x0.z))
                      : x0 + x1 * 0.5f;
    const V3 bx = v3(k.r_sum - ax.x, k.g_sum - ax.y, k.b_sum - ax.z);
    a = round_ept(v3((ax.x * beta2 - bx.x * ab) * factor, (ax.y * beta2 - bx.y * ab) * factor,
                     (ax.z * beta2 - bx.z * ab) * factor));
    b = round_ept(v3((bx.x * alpha2 - ax.x * ab) * factor, (bx.y * alpha2 - ax.y * ab) * factor,
                     (bx.z * alpha2 - ax.z * ab) * factor));
    return fit_error<BND>(a, b, ax, bx, alpha2, beta2, ab, q.metric);
}

// ----------------------------------------------- SIMD-profile cluster fit --
//
// The reference's SIMD builds (ICBC_SIMD 1..5 and -1, icbc.h:427-1235) run the
// same cluster loops with vmadd / vmsub fused on AVX2 and AVX-512
// (icbc.h:734-752, :970-976), vround01 rounding half to even from SSE4.1 on
// and on NEON (icbc.h:518-524, :764-766, :988-990, :1159-1162), and, on NEON
// only, a vsaturate that keeps a NaN (vmaxq_f32 / vminq_f32 return NaN for a
// NaN operand, icbc.h:1155-1157; the x86 max / min return the other operand).
// These are cf4_combo / cf3_combo with those three choices.
__device__ __forceinline__ float pm_madd(bool f, float a, float b, float c) {
    return f ? __fmaf_rn(a, b, c) : a * b + c;
}
__device__ __forceinline__ float pm_msub(bool f, float a, float b, float c) {
    return f ? __fmaf_rn(a, b, -c) : a * b - c;
}
// vm2sub(a, b, c, d) = vmsub(a, b, c * d) (icbc.h:415, :754-756, :978-980).
__device__ __forceinline__ float pm_m2sub(bool f, float a, float b, float c, float d) { return pm_msub(f, a, b, c * d); }
// vround5 / vround6 of a saturated value: int(t + 0.5f) or round-half-even
// of t = x * n, both exact for 0 <= t < 2^23 through the 2^23 addition (a
// NaN, kept by NEON's vsaturate, stays NaN through both).
__device__ __forceinline__ float pm_round(float x, float n, float inv_n, bool rne, bool nan) {
    const float t = ((nan && x != x) ? x : __saturatef(x)) * n;
    const float r = rne ? __fsub_rn(__fadd_rn(t, 8388608.0f), 8388608.0f) : snap_floor(t + 0.5f);
    return r * inv_n;
}
__device__ __forceinline__ V3 pm_round_ept(V3 v, bool rne, bool nan) {
    return v3(pm_round(v.x, 31.0f, 1.0f / 31.0f, rne, nan), pm_round(v.y, 63.0f, 1.0f / 63.0f, rne, nan),
              pm_round(v.z, 31.0f, 1.0f / 31.0f, rne, nan));
}

// cluster_fit_four's iteration (icbc.h:2685-2733) under a SIMD profile.
__device__ __forceinline__ float cf4_combo_simd(const float *S, uint32_t packed, const FitSums &k, const FitWeights &q,
                                               bool f, bool rne, bool nan, V3 &a, V3 &b) {
    const int i0 = packed & 0xff, i1 = (packed >> 8) & 0xff, i2 = packed >> 16;
    const float4 s0 = ld4(S + 4 * i0), s1 = ld4(S + 4 * i1), s2 = ld4(S + 4 * i2);
    V3 x0 = xyz(s0), x1 = xyz(s1), x2 = xyz(s2);
    const float w0 = s0.w;
    float w1 = s1.w, w2 = s2.w;
    const float w3 = k.w_sum - w2;
    x2 = x2 - x1;
    x1 = x1 - x0;
    w2 = w2 - w1;
    w1 = w1 - w0;
    const float alpha2 = pm_madd(f, w2, q.w1_9, pm_madd(f, w1, q.w4_9, w0));
    const float beta2 = pm_madd(f, w1, q.w1_9, pm_madd(f, w2, q.w4_9, w3));
    const float ab = (w1 + w2) * q.w2_9;
    const float factor = 1.0f / pm_m2sub(f, alpha2, beta2, ab, ab);
    const V3 ax = v3(pm_madd(f, x2.x, q.w1_3, pm_madd(f, x1.x, q.w2_3, x0.x)),
                     pm_madd(f, x2.y, q.w1_3, pm_madd(f, x1.y, q.w2_3, x0.y)),
                     pm_madd(f, x2.z, q.w1_3, pm_madd(f, x1.z, q.w2_3, x0.z)));
    const V3 bx = v3(k.r_sum - ax.x, k.g_sum - ax.y, k.b_sum - ax.z);
    a = pm_round_ept(v3(pm_m2sub(f, ax.x, beta2, bx.x, ab) * factor, pm_m2sub(f, ax.y, beta2, bx.y, ab) * factor,
                        pm_m2sub(f, ax.z, beta2, bx.z, ab) * factor), rne, nan);
    b = pm_round_ept(v3(pm_m2sub(f, bx.x, alpha2, ax.x, ab) * factor, pm_m2sub(f, bx.y, alpha2, ax.y, ab) * factor,
                        pm_m2sub(f, bx.z, alpha2, ax.z, ab) * factor), rne, nan);
    const V3 e2 = v3(pm_m2sub(f, a.x, pm_msub(f, b.x, ab, ax.x), b.x, bx.x) * 2.0f,
                     pm_m2sub(f, a.y, pm_msub(f, b.y, ab, ax.y), b.y, bx.y) * 2.0f,
                     pm_m2sub(f, a.z, pm_msub(f, b.z, ab, ax.z), b.z, bx.z) * 2.0f);
    const V3 e1 = v3(pm_madd(f, a.x * a.x, alpha2, pm_madd(f, b.x * b.x, beta2, e2.x)),
                     pm_madd(f, a.y * a.y, alpha2, pm_madd(f, b.y * b.y, beta2, e2.y)),
                     pm_madd(f, a.z * a.z, alpha2, pm_madd(f, b.z * b.z, beta2, e2.z)));
    return dot(e1, q.metric);
}

// cluster_fit_three's iteration (icbc.h:2299-2323) under a SIMD profile.
__device__ __forceinline__ float cf3_combo_simd(const float *S, uint32_t packed, const FitSums &k, const FitWeights &q,
                                               bool f, bool rne, bool nan, V3 &a, V3 &b) {
    const int i0 = packed & 0xff, i1 = (packed >> 8) & 0xff;
    const float4 s0 = ld4(S + 4 * i0), s1 = ld4(S + 4 * i1);
    const V3 x0 = xyz(s0);
    V3 x1 = xyz(s1);
    const float w0 = s0.w;
    float w1 = s1.w;
    const float w2 = k.w_sum - w1;
    x1 = x1 - x0;
    w1 = w1 - w0;
    const float ab = w1 * 0.25f;
    const float alpha2 = w0 + ab;
    const float beta2 = w2 + ab;
    const float factor = 1.0f / pm_m2sub(f, alpha2, beta2, ab, ab);
    const V3 ax = x0 + x1 * 0.5f;
    const V3 bx = v3(k.r_sum - ax.x, k.g_sum - ax.y, k.b_sum - ax.z);
    a = pm_round_ept(v3(pm_m2sub(f, ax.x, beta2, bx.x, ab) * factor, pm_m2sub(f, ax.y, beta2, bx.y, ab) * factor,
                        pm_m2sub(f, ax.z, beta2, bx.z, ab) * factor), rne, nan);
    b = pm_round_ept(v3(pm_m2sub(f, bx.x, alpha2, ax.x, ab) * factor, pm_m2sub(f, bx.y, alpha2, ax.y, ab) * factor,
                        pm_m2sub(f, bx.z, alpha2, ax.z, ab) * factor), rne, nan);
    const V3 e2 = v3(pm_m2sub(f, a.x, pm_msub(f, b.x, ab, ax.x), b.x, bx.x) * 2.0f,
                     pm_m2sub(f, a.y, pm_msub(f, b.y, ab, ax.y), b.y, bx.y) * 2.0f,
                     pm_m2sub(f, a.z, pm_msub(f, b.z, ab, ax.z), b.z, bx.z) * 2.0f);
    const V3 e1 = v3(pm_madd(f, a.x * a.x, alpha2, pm_madd(f, b.x * b.x, beta2, e2.x)),
                     pm_madd(f, a.y * a.y, alpha2, pm_madd(f, b.y * b.y, beta2, e2.y)),
                     pm_madd(f, a.z * a.z, alpha2, pm_madd(f, b.z * b.z, beta2, e2.z)));
    return dot(e1, q.metric);
}

// What the SIMD loops read for their padding lanes past a SAT of m colours
// (row entry k holds SAT slot k - 1): compute_sat's FLT_MAX fill
// (icbc.h:1931-1936), except where the build's gather reads something else.
// kGatherTbl: NEON's table lookups cover the first 8, 12 or 16 slots by count
// (vqtbl2q / vqtbl3q / vqtbl4q, icbc.h:2586-2650, :2224-2270) and read zero
// past them.  kGatherPerm8: AVX2 with m <= 8 permutes the first 8 slots
// (permutevar8x32, icbc.h:2428-2445, :2128-2145, :867-870), index modulo 8.
constexpr int kGatherFull = 0, kGatherTbl = 1, kGatherPerm8 = 2;
__device__ __forceinline__ void fill_sat_tail(float *srow, int m, int gather) {
    const int lim = gather == kGatherTbl ? (m <= 8 ? 8 : m <= 12 ? 12 : 16) : 16;
    for (int k = m + 1; k <= 16; k++)
        st4(srow + 4 * k, k - 1 < lim ? make_float4(FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX) : make_float4(0, 0, 0, 0));
    if (gather == kGatherPerm8 && m <= 8)
        for (int k = 9; k <= 16; k++) st4(srow + 4 * k, ld4(srow + 4 * (k - 8)));
}

// In a SIMD build, combination k of a block is evaluated in lane k % vec;
// each lane keeps its first strict minimum and the cross-lane reduction
// (reduce_min_index, icbc.h:574-586, :812-831, :1031-1039) takes the smallest
// error, ties to the lowest lane.  So the winner is the smallest
// (error, k % vec, k / vec); the rank below orders the last two.
// vec is a power of two (1, 4, 8 or 16).
__device__ __forceinline__ int simd_rank(int k, int vec) { return ((k & (vec - 1)) << 10) | (k >> (__ffs(vec) - 1)); }
__device__ __forceinline__ int simd_unrank(int r, int vec) { return (r & 1023) * vec + (r >> 10); }

// Warp-cooperative search of the cluster combinations of every block of the
// warp that needs one.  The warp's whole work -- the concatenation of each
// block's combination list -- is cut into 64 equal contiguous ranges; lane l
// walks ranges l and l + 32 side by side (two independent dependency
// chains).  A walker keeps the first strict minimum of its share of a block
// and, when it leaves the block, folds (error, table index) into the block's
// slot with a 64-bit atomicMin on an order-preserving key.  The minimum key
// is the smallest error with ties to the lowest table index: the combination
// the sequential loop of icbc.h:2089-2344 / :2362-2742 keeps.  Errors equal
// to zero are keyed as +0 because the loop's strict < treats -0 and +0 alike.
struct Walker {
    int g, gend;      // global combination range still to do
    int b, k, total;  // current block, its combination index, its count
    const float *S;
    FitSums sums;
    float best;
    int best_k;
};

// A block's search info word: its first combination in the group's list
// (bits 0-23) and its colour count (bits 24-28; 0: no search).
constexpr int kInfoShift = 24;
constexpr int kInfoMask = (1 << kInfoShift) - 1;
__device__ __forceinline__ int block_info(const WarpCtx &w, int b) { return w.info[b]; }

// With SIMD, a block's combinations run to a whole number of vectors of
// `vec` lanes (icbc.h:2089, :2362: the padding lanes read table entries of
// larger counts, or zeros, against the SAT's FLT_MAX fill).
__device__ __forceinline__ int padded_total(int t, int vec) { return (t + vec - 1) / vec * vec; }

template <bool FOUR, bool SIMD = false>
__device__ __forceinline__ void walker_enter(const WarpCtx &w, Walker &v, int b, int k, int vec = 1) {
    const float *S = w.sat + b * kSatStride;
    const int cnt = w.info[b] >> kInfoShift;
    v.b = b;
    v.k = k;
    v.S = S;
    v.total = FOUR ? w.T->four_total[cnt - 1] : w.T->three_total[cnt - 1];
    if (SIMD) v.total = padded_total(v.total, vec);
    v.sums = fit_sums(S, cnt);
    v.best = FLT_MAX;
    v.best_k = 0x7fffffff;
}

__device__ __forceinline__ void walker_flush(const WarpCtx &w, const Walker &v) {
    if (v.best_k != 0x7fffffff) {
        const float f = v.best == 0.0f ? 0.0f : v.best;
        uint32_t u = __float_as_uint(f);
        u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        atomicMin(&w.slots[v.b], ((unsigned long long)u << 32) | (uint32_t)v.best_k);
    }
}

// Starts a walker at global combination g (if any work is left for it),
// over a search group of NB blocks.
template <bool FOUR, int NB, bool SIMD = false>
__device__ __forceinline__ void walker_start_n(const WarpCtx &w, Walker &v, int g, int gend, int vec = 1) {
    v.g = g;
    v.gend = gend;
    v.S = w.sat;
    v.k = 0;
    v.total = 1;
    v.sums = FitSums{0.0f, 0.0f, 0.0f, 0.0f};
    v.best = FLT_MAX;
    v.best_k = 0x7fffffff;
    v.b = 0;
    if (g < gend) {
        // The last block whose first combination is <= g always has work.
        int lo = 0, hi = NB;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if ((block_info(w, mid) & kInfoMask) <= g) lo = mid;
            else hi = mid;
        }
        walker_enter<FOUR, SIMD>(w, v, lo, g - (block_info(w, lo) & kInfoMask), vec);
    }
}

template <bool FOUR, bool SIMD = false>
__device__ __forceinline__ void walker_start(const WarpCtx &w, Walker &v, int g, int gend, int vec = 1) {
    walker_start_n<FOUR, 32, SIMD>(w, v, g, gend, vec);
}

// One step: fold the error of combination k in, move to k + 1, and cross
// into the next block with work when this one is done.  `next` is the table
// entry of the following combination, loaded one iteration ahead; a block
// change reloads it.
// One step, in two parts: walker_fold folds the error of combination k in
// and moves to k + 1; walker_cross, when the walker has left its block with
// work still to do, flushes it and enters the next block with work (`next`,
// the table entry loaded one iteration ahead, is reloaded).  The search
// checks for crossings once per iteration for the whole warp, so the rare
// divergent crossing code stays off the common path.
// With SIMD the walker keeps the smallest (error, simd_rank) of its share
// in best / best_k (best_k holds the rank), never an error of FLT_MAX.
template <bool SIMD = false>
__device__ __forceinline__ void walker_fold(Walker &v, float e, int vec = 1) {
    const bool live = v.g < v.gend;
    bool better;
    int rk = v.k;
    if (SIMD) {
        rk = simd_rank(v.k, vec);
        better = live && (e < v.best || (e == v.best && v.best_k != 0x7fffffff && rk < v.best_k));
    } else {
        better = live && e < v.best;
    }
    v.best = better ? e : v.best;
    v.best_k = better ? rk : v.best_k;
    v.g += live;
    v.k += live;
}

__device__ __forceinline__ bool walker_crossing(const Walker &v) { return v.k == v.total && v.g < v.gend; }

template <bool FOUR, bool SIMD = false>
__device__ __forceinline__ void walker_cross(const WarpCtx &w, Walker &v, uint32_t &next, int vec = 1) {
    walker_flush(w, v);
    int nb = v.b + 1;
    while ((block_info(w, nb) >> kInfoShift) == 0) nb++;
    walker_enter<FOUR, SIMD>(w, v, nb, 0, vec);
    next = (FOUR ? w.T->four : w.T->three)[0];
}

// Returns this lane's winning table index, or -1 (no search, or no error
// below FLT_MAX: the reference then keeps zero endpoints).
template <bool FOUR, bool SIMD = false, bool BND = false>
__device__ __forceinline__ int flat_search(const WarpCtx &w, bool need, int count, const FitWeights &q,
                                           const EncodeParams *p = nullptr) {
    const int lane = w.lane;
    const int vec = SIMD ? p->simd_vec : 1;
    int T = need ? (FOUR ? w.T->four_total[count - 1] : w.T->three_total[count - 1]) : 0;
    if (SIMD) T = padded_total(T, vec);
    int incl = T;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += y;
    }
    const int W = __shfl_sync(kFull, incl, 31);
    w.info[lane] = (incl - T) | ((need ? count : 0) << kInfoShift);
    w.slots[lane] = ~0ull;
    __syncwarp();
    if (W == 0) return -1;
    const int per = (W + 63) / 64;
    Walker A, B;
    walker_start<FOUR, SIMD>(w, A, min(lane * per, W), min(lane * per + per, W), vec);
    walker_start<FOUR, SIMD>(w, B, min((lane + 32) * per, W), min((lane + 32) * per + per, W), vec);
    const uint32_t *table = FOUR ? w.T->four : w.T->three;
    // The padded SIMD range reaches the last table entry; its look-ahead
    // index is clamped to the table (that entry is then never used).
    const int last = FOUR ? 991 : 159;
    uint32_t pa = table[A.k], pb = table[B.k];
    for (int it = 0; it < per; it++) {
        // Entry k + 1 of each walker is fetched before this step's arithmetic
        // (the tables are padded past their last used entry).
        uint32_t na = table[SIMD ? min(A.k + 1, last) : A.k + 1], nb = table[SIMD ? min(B.k + 1, last) : B.k + 1];
        V3 a, b;
        float ea, eb;
        if (SIMD) {
            const bool f = p->simd_fma != 0, rne = p->simd_rne != 0, nan = p->simd_nan != 0;
            ea = FOUR ? cf4_combo_simd(A.S, pa, A.sums, q, f, rne, nan, a, b)
                      : cf3_combo_simd(A.S, pa, A.sums, q, f, rne, nan, a, b);
            eb = FOUR ? cf4_combo_simd(B.S, pb, B.sums, q, f, rne, nan, a, b)
                      : cf3_combo_simd(B.S, pb, B.sums, q, f, rne, nan, a, b);
        } else {
            ea = FOUR ? cf4_combo<BND>(A.S, pa, A.sums, q, a, b) : cf3_combo<BND>(A.S, pa, A.sums, q, a, b);
            eb = FOUR ? cf4_combo<BND>(B.S, pb, B.sums, q, a, b) : cf3_combo<BND>(B.S, pb, B.sums, q, a, b);
        }
        walker_fold<SIMD>(A, ea, vec);
        walker_fold<SIMD>(B, eb, vec);
        const bool xa = walker_crossing(A), xb = walker_crossing(B);
        if (__any_sync(kFull, xa || xb)) {
            if (xa) walker_cross<FOUR, SIMD>(w, A, na, vec);
            if (xb) walker_cross<FOUR, SIMD>(w, B, nb, vec);
        }
        pa = na;
        pb = nb;
    }
    walker_flush(w, A);
    walker_flush(w, B);
    __syncwarp();
    const unsigned long long key = w.slots[lane];
    if (!need || key == ~0ull) return -1;
    return SIMD ? simd_unrank((int)(uint32_t)key, vec) : (int)(uint32_t)key;
}

// The same search over a group of NW warps (the whole CTA): the combinations
// of the group's 32 * NW blocks form one list cut into 64 * NW equal ranges,
// two per thread.  `g` is the group's context: its sat / info / slots hold
// the rows of all the group's blocks, block j = warp * 32 + lane, and
// g.lane = threadIdx.x.  `sums` is NW ints of shared memory.  Every thread of
// the CTA must call it together (it synchronises the CTA) with the same fit
// weights `q`: every thread walks combinations of any of the group's blocks.
// Same winner rule as flat_search: per block the smallest (error, table index).
// Every walker of the group search runs exactly `per` steps: a walker that
// passes the end of the list walks on into a sentinel block after the last
// one (index 32 * NW: 16 colours, a SAT row of NaNs, set up by the kernel),
// whose errors are NaN and never fold in, and a walker with no range starts
// there.  So no step tests whether its walker is live.  The sentinel has 968
// (or 152) combinations, more than a walker's `per` <= 484 (or 76) steps, so
// no walker crosses out of it.
template <bool FOUR, int NB>
__device__ __forceinline__ void walker_start_s(const WarpCtx &w, Walker &v, int g, int W) {
    int b = NB, k = 0;
    if (g < W) {
        int lo = 0, hi = NB;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if ((block_info(w, mid) & kInfoMask) <= g) lo = mid;
            else hi = mid;
        }
        b = lo;
        k = g - (block_info(w, lo) & kInfoMask);
    }
    walker_enter<FOUR>(w, v, b, k);
}

__device__ __forceinline__ void walker_fold_s(Walker &v, float e) {
    const bool better = e < v.best;
    v.best = better ? e : v.best;
    v.best_k = better ? v.k : v.best_k;
    v.k++;
}

// RUNS: step in runs between block crossings (levels 8-9, whose blocks have
// hundreds of combinations); otherwise test for crossings after every step
// (at levels 2-7 a warp's 64 walkers leave a block every step or two).
template <bool FOUR, int NW, bool BND = false, bool RUNS = true>
__device__ __forceinline__ int flat_search_group(const WarpCtx &g, int *sums, bool need, int count,
                                                 const FitWeights &q) {
    const int j = threadIdx.x;
    const int lane = j & 31, warp = j >> 5;
    const int T = need ? (FOUR ? g.T->four_total[count - 1] : g.T->three_total[count - 1]) : 0;
    int incl = T;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) sums[warp] = incl;
    __syncthreads();
    int before = 0, W = 0;
#pragma unroll
    for (int k = 0; k < NW; k++) {
        const int v = sums[k];
        before += k < warp ? v : 0;
        W += v;
    }
    g.info[j] = (before + incl - T) | ((need ? count : 0) << kInfoShift);
    g.slots[j] = ~0ull;
    __syncthreads();
    if (W == 0) return -1;
    const int per = (W + 64 * NW - 1) / (64 * NW);
    Walker A, B;
    walker_start_s<FOUR, 32 * NW>(g, A, j * per, W);
    walker_start_s<FOUR, 32 * NW>(g, B, (j + 32 * NW) * per, W);
    const uint32_t *table = FOUR ? g.T->four : g.T->three;
    uint32_t pa = table[A.k], pb = table[B.k];
    for (int it = 0; it < per;) {
        // The warp runs, without crossing tests, as many steps as its first
        // walker to reach the end of its block needs (at least one: a walker
        // is never at its block's end here), then moves the walkers that
        // reached it into their next block.
        const int run = RUNS ? __reduce_min_sync(kFull, min(min(A.total - A.k, B.total - B.k), per - it)) : 1;
        for (int r = 0; r < run; r++) {
            const uint32_t na = table[A.k + 1], nb = table[B.k + 1];
            V3 a, b;
            const float ea = FOUR ? cf4_combo<BND>(A.S, pa, A.sums, q, a, b) : cf3_combo<BND>(A.S, pa, A.sums, q, a, b);
            const float eb = FOUR ? cf4_combo<BND>(B.S, pb, B.sums, q, a, b) : cf3_combo<BND>(B.S, pb, B.sums, q, a, b);
            walker_fold_s(A, ea);
            walker_fold_s(B, eb);
            pa = na;
            pb = nb;
        }
        it += run;
        const bool xa = A.k == A.total, xb = B.k == B.total;
        if (RUNS || __any_sync(kFull, xa || xb)) {
            if (xa) walker_cross<FOUR>(g, A, pa);
            if (xb) walker_cross<FOUR>(g, B, pb);
        }
    }
    walker_flush(g, A);
    walker_flush(g, B);
    __syncthreads();
    const unsigned long long key = g.slots[j];
    if (!need || key == ~0ull) return -1;
    return (int)(uint32_t)key;
}

// ------------------------------------------------------------- encoder --

// Encodes the warp's 32 blocks, whose texels are in w.in.  `active` marks
// the lanes that own a real block.  c0/c1/idx hold the caller's prior output
// bytes on entry (levels 4..9 keep them when nothing is accepted) and the
// encoded block on return; the return value is compress_bc1's error.
//
// With DEFER the refinement of level 9 is not run here: `refine_next` is set
// for the blocks it applies to (the caller hands them to k_refine), and the
// returned error is the one refinement starts from.
__device__ __forceinline__ FloatRow float_row(const WarpCtx &w) { return FloatRow{w.in + w.lane * kInStride}; }

// reduce_colors (icbc.h:1683-1728) followed only while at most one colour is
// kept: true when the block reduces to 0 or 1 colours (`count`, and `c` the
// colour -- reduce_colors' arithmetic, every texel merged into the first
// colour), false as soon as a second colour appears.  Unrolled: a row over a
// register array stays in registers.
template <class Row>
__device__ __forceinline__ bool reduce_to_one(const Row &row, float threshold, V3 &c, int &count) {
    c = v3(0.0f, 0.0f, 0.0f);
    float wc = 0.0f;
    count = 0;
    bool other = false;
#pragma unroll
    for (int t = 0; t < 16; t++) {
        const V3 ct = row.color(t);
        const float wt = row.weight(t);
        if (!other && wt > 0) {
            if (count == 0) {
                c = ct;
                wc = wt;
                count = 1;
            } else if (near3(c, ct, threshold)) {
                const float s = wc + wt;
                if (Row::kBounded)
                    c = v3(div_bounded(c.x * wc + ct.x * wt, s), div_bounded(c.y * wc + ct.y * wt, s),
                           div_bounded(c.z * wc + ct.z * wt, s));
                else
                    c = v3((c.x * wc + ct.x * wt) / s, (c.y * wc + ct.y * wt) / s, (c.z * wc + ct.z * wt) / s);
                wc = s;
            } else {
                other = true;
            }
        }
    }
    return !other;
}

// The reduce_colors threshold of a level given at run time (Level<L>::threshold).
__device__ __forceinline__ float level_threshold(int level) {
    switch (level) {
        case 2: return Level<2>::threshold;
        case 3: return Level<3>::threshold;
        case 4: return Level<4>::threshold;
        case 5: return Level<5>::threshold;
        case 6: return Level<6>::threshold;
        case 7: return Level<7>::threshold;
        case 8: return Level<8>::threshold;
        default: return Level<9>::threshold;
    }
}

// The blocks of 0 or 1 reduced colours (icbc.h:3752-3764): the zero block, or
// the optimal single-colour endpoints of `color` with their error.
template <int UNROLL = 1, class Row>
__device__ __forceinline__ float trivial_block(const DecoderTables *D, const float *lut255, const Row &row,
                                               const EncodeParams &p, V3 color, int count, uint32_t &c0,
                                               uint32_t &c1, uint32_t &idx) {
    if (count == 0) {
        c0 = c1 = idx = 0;
        return 0.0f;
    }
    single_color(D, color, c0, c1, idx);
    return block_error<UNROLL>(row, p.cw, palette_f(c0, c1, p.decoder, lut255, D), idx);
}

// With NW > 1 the cluster searches run over the whole CTA of NW warps
// (flat_search_group on the group context *g, NW ints of shared memory at
// gsums): every thread of the CTA must make the call together.  The group
// search shares one set of fit weights, so it needs every thread's decoder
// and colour weights alike; `group` false (the same for the whole CTA) makes
// each warp search its own blocks instead.
template <int L, bool DEFER, bool SIMD = false, int NW = 1, class Row>
__device__ __forceinline__ float encode_warp_ex(const WarpCtx &w, const Row &row, const EncodeParams &p, bool active,
                                                uint32_t &c0, uint32_t &c1, uint32_t &idx, bool &refine_next,
                                                const WarpCtx *g = nullptr, int *gsums = nullptr, bool group = true) {
    using O = Level<L>;
    refine_next = false;
    const int lane = w.lane;
    float *srow = w.sat + lane * kSatStride;
    float err = 0.0f;
    int count = 16;
    bool any_black = false, live = false, need4 = false;

    if (active && O::cluster) count = reduce_colors(row, O::threshold, srow, any_black);
    // The SAT build unrolled no wider than the warp's largest colour count
    // needs: 8, 12 or 16 entries (warp-uniform; levels 2-7, where most
    // blocks reduce to a few colours; at levels 8-9 the extra builds' code
    // cost 0.4%).
    const int wmax = O::cluster && L <= 7 && !SIMD ? __reduce_max_sync(kFull, active ? count : 0) : 16;
    const int width = wmax <= 8 ? 8 : wmax <= 12 ? 12 : 16;
    if (active) {
        if (O::cluster && count <= 1) {
            err = trivial_block(w.D, w.T->lut255, row, p, xyz(ld4(srow)), count, c0, c1, idx);
        } else {
            live = true;
            err = FLT_MAX;
            if (O::box) {
                V3 e0, e1;
                if (O::cluster) box_fit(SatColors{srow}, count, e0, e1);
                else box_fit(row, count, e0, e1);
                err = output_block4(w, row, p, e0, e1, c0, c1, idx);
                if (O::lsq && optimize_end_points4(row, idx, e0, e1)) {
                    uint32_t o0, o1, oi;
                    const float oe = output_block4(w, row, p, e0, e1, o0, o1, oi);
                    if (oe < err) { err = oe; c0 = o0; c1 = o1; idx = oi; }
                }
            }
            if (O::cluster) {
                if (width == 8) build_sat_inplace<8>(srow, count, false);
                else if (width == 12) build_sat_inplace<12>(srow, count, false);
                else build_sat_inplace(srow, count, false);
                if (SIMD) fill_sat_tail(srow, count, p.simd_gather);
                need4 = true;
            }
        }
    }

    if (O::cluster) {
        const V3 metric = p.cw * p.cw;
        __syncwarp();
        // 4-colour cluster fit of every block that needs one, across the warp.
        const FitWeights q = fit_weights(w.D, metric);
        int my4;
        if (NW > 1 && group) my4 = flat_search_group<true, NW, Row::kBounded, (L >= 8)>(*g, gsums, need4, count, q);
        else my4 = flat_search<true, SIMD, Row::kBounded && !SIMD>(w, need4, count, q, &p);
        uint32_t f0 = 0, f1 = 0, fi = 0;
        float ferr = 0.0f;
        bool need3 = false;
        int count3 = count;
        if (need4) {
            V3 a = v3(0.0f, 0.0f, 0.0f), b = a;
            if (my4 >= 0) {
                if (SIMD)
                    cf4_combo_simd(srow, w.T->four[my4], fit_sums(srow, count), q, p.simd_fma, p.simd_rne, p.simd_nan,
                                   a, b);
                else cf4_combo(srow, w.T->four[my4], fit_sums(srow, count), q, a, b);
            }
            ferr = output_block4(w, row, p, a, b, f0, f1, fi);
            const bool use_black = any_black && p.three_color_black;
            const bool use_three = (O::cf3_always && p.three_color_mode) ||
                                   (O::cf3_black_only && p.three_color_mode && p.three_color_black && use_black);
            if (use_three) {
                if (use_black) {
                    // The reduced colours were overwritten by the SAT: reduce again,
                    // then build the table of the non-black ones.
                    bool ab;
                    reduce_colors(row, O::threshold, srow, ab);
                    count3 = width == 8    ? build_sat_inplace<8>(srow, count, true)
                             : width == 12 ? build_sat_inplace<12>(srow, count, true)
                                           : build_sat_inplace(srow, count, true);
                    if (SIMD) fill_sat_tail(srow, count3, p.simd_gather);
                    need3 = count3 > 0;
                } else {
                    need3 = true;
                }
            }
        }
        __syncwarp();
        int my3;
        if (NW > 1 && group) my3 = flat_search_group<false, NW, Row::kBounded, (L >= 8)>(*g, gsums, need3, count3, q);
        else my3 = flat_search<false, SIMD, Row::kBounded && !SIMD>(w, need3, count3, q, &p);
        if (need3) {
            V3 a = v3(0.0f, 0.0f, 0.0f), b = a;
            if (my3 >= 0) {
                if (SIMD)
                    cf3_combo_simd(srow, w.T->three[my3], fit_sums(srow, count3), q, p.simd_fma, p.simd_rne,
                                   p.simd_nan, a, b);
                else cf3_combo(srow, w.T->three[my3], fit_sums(srow, count3), q, a, b);
            }
            uint32_t t0, t1, ti;
            const float e3 = output_block3(w, row, p, a, b, t0, t1, ti);
            if (e3 < ferr) { ferr = e3; f0 = t0; f1 = t1; fi = ti; }
        }
        if (need4 && ferr < err) { c0 = f0; c1 = f1; idx = fi; err = ferr; }
    }

    if (O::refine && live) {
        if (DEFER) refine_next = true;
        else err = refine(w, row, p, err, c0, c1, idx);
    }
    return err;
}

// encode_warp_ex on the warp's float texel rows, refinement inline.
template <int L>
__device__ __forceinline__ float encode_warp(const WarpCtx &w, const EncodeParams &p, bool active, uint32_t &c0,
                                             uint32_t &c1, uint32_t &idx) {
    bool unused;
    return encode_warp_ex<L, false>(w, float_row(w), p, active, c0, c1, idx, unused);
}

}  // namespace icbc_gpu
