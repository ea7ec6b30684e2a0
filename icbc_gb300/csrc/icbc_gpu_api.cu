// icbc_gpu_api.cu -- host side of the C ABI declared in include/icbc_gpu.h.
//
// Owns the init-time tables (built here on the host, uploaded once per
// device), validates every argument before a launch, plans batched work and
// runs the host-buffer end-to-end path.  No exceptions cross the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/icbc_gpu.h"
#include "bc1_kernels.h"

using namespace icbc_gpu;

namespace {

std::mutex g_mutex;
int g_decoder = -1;
bool g_tables_built = false;
GlobalTables g_host_tables;
GlobalTables *g_dev_tables[64] = {};
thread_local std::string t_last_error;

int set_cuda_error(cudaError_t e) {
    t_last_error = cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? ICBC_GPU_ERR_OUT_OF_MEMORY : ICBC_GPU_ERR_CUDA;
}

// Rounding thresholds between adjacent expanded 5- and 6-bit values
// (icbc.h:1560-1570).  They are data of the BC1 encoding and must match the
// reference literally, including the FLT_MAX sentinels.
const float kMid5[32] = {
    0.015686f, 0.047059f, 0.078431f, 0.111765f, 0.145098f, 0.176471f, 0.207843f, 0.241176f,
    0.274510f, 0.305882f, 0.337255f, 0.370588f, 0.403922f, 0.435294f, 0.466667f, 0.5f,
    0.533333f, 0.564706f, 0.596078f, 0.629412f, 0.662745f, 0.694118f, 0.725490f, 0.758824f,
    0.792157f, 0.823529f, 0.854902f, 0.888235f, 0.921569f, 0.952941f, 0.984314f, FLT_MAX};
const float kMid6[64] = {
    0.007843f, 0.023529f, 0.039216f, 0.054902f, 0.070588f, 0.086275f, 0.101961f, 0.117647f,
    0.133333f, 0.149020f, 0.164706f, 0.180392f, 0.196078f, 0.211765f, 0.227451f, 0.245098f,
    0.262745f, 0.278431f, 0.294118f, 0.309804f, 0.325490f, 0.341176f, 0.356863f, 0.372549f,
    0.388235f, 0.403922f, 0.419608f, 0.435294f, 0.450980f, 0.466667f, 0.482353f, 0.500000f,
    0.517647f, 0.533333f, 0.549020f, 0.564706f, 0.580392f, 0.596078f, 0.611765f, 0.627451f,
    0.643137f, 0.658824f, 0.674510f, 0.690196f, 0.705882f, 0.721569f, 0.737255f, 0.754902f,
    0.772549f, 0.788235f, 0.803922f, 0.819608f, 0.835294f, 0.850980f, 0.866667f, 0.882353f,
    0.898039f, 0.913725f, 0.929412f, 0.945098f, 0.960784f, 0.976471f, 0.992157f, FLT_MAX};

// Best (max, min) endpoint pair reproducing each 8-bit value under a decoder's
// interpolation, the error measure of PrepareOptTable5/6 (icbc.h:3377-3485):
// D3D10 takes the worst of the AMD, NVIDIA and Intel reconstructions.  Ties
// keep the first pair in (min, max) scan order.
void build_match(uint8_t table[256][2], int bits, int decoder) {
    const int levels = 1 << bits;
    for (int v = 0; v < 256; v++) {
        int best = 25600;
        for (int lo = 0; lo < levels; lo++) {
            for (int hi = 0; hi < levels; hi++) {
                const int elo = bits == 5 ? (lo << 3) | (lo >> 2) : (lo << 2) | (lo >> 4);
                const int ehi = bits == 5 ? (hi << 3) | (hi >> 2) : (hi << 2) | (hi >> 4);
                const int amd = std::abs(((43 * ehi + 21 * elo + 32) >> 6) - v);
                const int nv = std::abs((bits == 5 ? ((2 * hi + lo) * 22) / 8
                                                   : (256 * elo + (ehi - elo) / 4 + 128 + (ehi - elo) * 80) / 256) - v);
                const int intel = std::abs(((171 * ehi + 85 * elo + 128) >> 8) - v);
                int err;
                switch (decoder) {
                    case 1: err = nv; break;
                    case 2: err = amd; break;
                    case 3: err = intel; break;
                    default: err = std::max(std::max(amd, nv), intel); break;
                }
                if (err < best) {
                    best = err;
                    table[v][0] = (uint8_t)hi;
                    table[v][1] = (uint8_t)lo;
                }
            }
        }
    }
}

// All tables, built once.  The cluster enumerations list every boundary
// triple 0 <= c0 <= c1 <= c2 <= t (pairs c0 <= c1 <= t for three clusters),
// except all-zero, grouped by t = 1..16 and ordered by (c0, c1) inside a
// group -- the order icbc.h:1965-2034 produces, so a prefix serves n colours.
void build_tables(GlobalTables &G) {
    std::memset(&G, 0, sizeof(G));
    SharedTables &S = G.s;
    int i4 = 0, i3 = 0;
    for (int t = 1; t <= 16; t++) {
        for (int c0 = 0; c0 <= t; c0++)
            for (int c1 = c0; c1 <= t; c1++) S.four[i4++] = (uint32_t)c0 | ((uint32_t)c1 << 8) | ((uint32_t)t << 16);
        S.four_total[t - 1] = i4;
        for (int c0 = 0; c0 <= t; c0++) S.three[i3++] = (uint32_t)c0 | ((uint32_t)t << 8);
        S.three_total[t - 1] = i3;
    }
    for (int i = 0; i < 256; i++) S.lut255[i] = (float)i / 255.0f;
    std::memcpy(S.mid5, kMid5, sizeof(kMid5));
    std::memcpy(S.mid6, kMid6, sizeof(kMid6));
    for (int d = 0; d < 4; d++) {
        DecoderTables &D = G.dec[d];
        // init_decoder_weights (icbc.h:3495-3515).
        float w1_3 = 1.0f / 3, w2_3 = 2.0f / 3;
        if (d == 2) { w1_3 = 21.0f / 64; w2_3 = 43.0f / 64; }
        if (d == 3) { w1_3 = 85.0f / 256; w2_3 = 171.0f / 256; }
        D.w1_3 = w1_3;
        D.w2_3 = w2_3;
        D.w1_9 = w1_3 * w1_3;
        D.w4_9 = w2_3 * w2_3;
        D.w2_9 = w1_3 * w2_3;
        build_match(D.match5, 5, d);
        build_match(D.match6, 6, d);
        // Linear palette forms (entries 2/3 of icbc.h:2752-2874), NVIDIA unused.
        static const int kLin[4][8] = {
            {87382, 43691, 0, 17, 1, 1, 0, 1},   // D3D10: (2a+b)/3 exact for a, b <= 255; (a+b)/2
            {0, 0, 0, 0, 0, 0, 0, 0},            // NVIDIA: own formulas
            {43, 21, 32, 6, 1, 1, 1, 1},         // AMD: (43a+21b+32)>>6; (a+b+1)/2
            {171, 85, 128, 8, 128, 128, 128, 8}  // Intel: (171a+85b+128)>>8; (128a+128b+128)>>8
        };
        std::memcpy(D.lin, kLin[d], sizeof(D.lin));
    }
}

// Makes sure the current device holds the tables; returns them in *out.
// The first call on a device allocates and uploads them (synchronously).
int ensure_device_tables(const GlobalTables **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e);
    if (dev < 0 || dev >= 64) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_decoder < 0) return ICBC_GPU_ERR_NOT_INITIALIZED;
    if (!g_dev_tables[dev]) {
        GlobalTables *d = nullptr;
        e = cudaMalloc(&d, sizeof(GlobalTables));
        if (e == cudaSuccess) e = cudaMemcpy(d, &g_host_tables, sizeof(GlobalTables), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (d) cudaFree(d);
            return set_cuda_error(e);
        }
        g_dev_tables[dev] = d;
    }
    if (out) *out = g_dev_tables[dev];
    return ICBC_GPU_OK;
}

const BlocksLauncher kBlocksLaunch[10] = {launch_blocks_l0, launch_blocks_l1, launch_blocks_l2, launch_blocks_l3,
                                          launch_blocks_l4, launch_blocks_l5, launch_blocks_l6, launch_blocks_l7,
                                          launch_blocks_l8, launch_blocks_l9};
const ImageLauncher kImageLaunch[10] = {launch_image_l0, launch_image_l1, launch_image_l2, launch_image_l3,
                                        launch_image_l4, launch_image_l5, launch_image_l6, launch_image_l7,
                                        launch_image_l8, launch_image_l9};
const ImageLauncherExt kImageLaunchExt[10] = {launch_image_ext_l0, launch_image_ext_l1, launch_image_ext_l2,
                                              launch_image_ext_l3, launch_image_ext_l4, launch_image_ext_l5,
                                              launch_image_ext_l6, launch_image_ext_l7, launch_image_ext_l8,
                                              launch_image_ext_l9};
const BatchLevelLauncher kBatchLevelLaunch[10] = {launch_batch_level_l0, launch_batch_level_l1, launch_batch_level_l2,
                                                  launch_batch_level_l3, launch_batch_level_l4, launch_batch_level_l5,
                                                  launch_batch_level_l6, launch_batch_level_l7, launch_batch_level_l8,
                                                  launch_batch_level_l9};

// An image of at least this many blocks (a 4096 x 4096 image) fills the GPU
// for many waves on its own: inside a batch it gets its level's own kernel,
// whose code is one level's, rather than a share of the all-levels batch
// kernel, which gains it nothing and fetches instructions from a larger body.
constexpr int64_t kOwnLaunchBlocks = int64_t(1) << 20;

int sm_count() {
    static int sms[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!sms[dev]) {
        int n = 1;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        sms[dev] = n > 0 ? n : 1;
    }
    return sms[dev];
}

int resolve_decoder(int decoder, int *out) {
    if (decoder == ICBC_GPU_DECODER_DEFAULT) {
        std::lock_guard<std::mutex> lock(g_mutex);
        decoder = g_decoder;
        if (decoder < 0) return ICBC_GPU_ERR_NOT_INITIALIZED;
    }
    if (decoder < 0 || decoder > 3) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    *out = decoder;
    return ICBC_GPU_OK;
}

bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

EncodeParams make_params(int decoder, int tc, int tcb, const float cw[3]) {
    EncodeParams p;
    p.decoder = decoder;
    p.three_color_mode = tc ? 1 : 0;
    p.three_color_black = tcb ? 1 : 0;
    p.cw = V3{cw[0], cw[1], cw[2]};
    p.simd_vec = 1;
    p.simd_fma = 0;
    p.simd_rne = 0;
    p.simd_nan = 0;
    p.simd_gather = kGatherFull;
    return p;
}

// Cluster-loop parameters of the reference's SIMD builds (ICBC_SIMD 0..5 and
// -1 = NEON, icbc.h:59-66): vector width, fused vmadd/vmsub, vround01 half to
// even, vsaturate keeping a NaN, the SAT gather's reads past its table
// (AVX2's permutevar8x32, NEON's table lookups).  Index = ICBC_SIMD, NEON last.
struct SimdProfile {
    int vec, fma, rne, nan, gather;
};
constexpr SimdProfile kSimdProfiles[7] = {{1, 0, 0, 0, kGatherFull},  {4, 0, 0, 0, kGatherFull},
                                          {4, 0, 1, 0, kGatherFull},  {8, 0, 1, 0, kGatherFull},
                                          {8, 1, 1, 0, kGatherPerm8}, {16, 1, 1, 0, kGatherFull},
                                          {4, 0, 1, 1, kGatherTbl}};
constexpr int kSimdNeonIndex = 6;

// Table index of an ICBC_GPU_SIMD_* value, or -1 when it is not one.
static int simd_index(int profile) {
    if (profile == ICBC_GPU_SIMD_NEON) return kSimdNeonIndex;
    return profile >= 0 && profile <= 5 ? profile : -1;
}

static void set_simd(EncodeParams &p, int index) {
    p.simd_vec = kSimdProfiles[index].vec;
    p.simd_fma = kSimdProfiles[index].fma;
    p.simd_rne = kSimdProfiles[index].rne;
    p.simd_nan = kSimdProfiles[index].nan;
    p.simd_gather = kSimdProfiles[index].gather;
}

// Validates an image descriptor and resolves it for the kernels.
int resolve_image(const icbc_gpu_image &im, ImageDesc &d) {
    if (!im.rgba || !im.out || im.width < 1 || im.height < 1) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (im.level < 0 || im.level > 9) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (im.weight_mode < 0 || im.weight_mode > 2) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (im.pitch < 4 * (int64_t)im.width) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(im.rgba, 4) || im.pitch % 4 || !aligned(im.out, 8)) return ICBC_GPU_ERR_MISALIGNED;
    if (im.weight_mode == ICBC_GPU_WEIGHTS_PLANE) {
        if (!im.weight_plane || im.weight_pitch < im.width) return ICBC_GPU_ERR_INVALID_ARGUMENT;
        if (!aligned(im.weight_plane, 4)) return ICBC_GPU_ERR_MISALIGNED;
    }
    if (im.errors && !aligned(im.errors, 4)) return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(im.decoder, &dec);
    if (st) return st;
    d.rgba = im.rgba;
    d.pitch = im.pitch;
    d.weight_plane = im.weight_plane;
    d.weight_pitch = im.weight_pitch;
    d.out = reinterpret_cast<uint2 *>(im.out);
    d.errors = im.errors;
    d.width = im.width;
    d.height = im.height;
    d.bw = (im.width + 3) / 4;
    d.nblocks = (int64_t)d.bw * ((im.height + 3) / 4);
    d.weight_mode = im.weight_mode;
    d.vec16 = aligned(im.rgba, 16) && im.pitch % 16 == 0;
    d.level = im.level;
    d.decoder = dec;
    d.three_color_mode = im.three_color_mode ? 1 : 0;
    d.three_color_black = im.three_color_black ? 1 : 0;
    d.cw[0] = im.color_weights[0];
    d.cw[1] = im.color_weights[1];
    d.cw[2] = im.color_weights[2];
    return ICBC_GPU_OK;
}

}  // namespace

namespace icbc_gpu {

// Host-side services shared with other translation units of the library.
const GlobalTables &host_tables() {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_tables_built) {
        build_tables(g_host_tables);
        g_tables_built = true;
    }
    return g_host_tables;
}

int resolve_image_desc(const icbc_gpu_image &image, ImageDesc &desc) { return resolve_image(image, desc); }

int resolve_image_desc_checked(const icbc_gpu_image &image, ImageDesc &desc) { return resolve_image(image, desc); }

int ensure_tables_on_device(const GlobalTables **out) { return ensure_device_tables(out); }

int current_sm_count() { return sm_count(); }

}  // namespace icbc_gpu

// Relative cost of a 32-block task per level, used to order batched work
// most-expensive first (cluster fit dominates from level 2 on).
static const int kLevelCost[10] = {1, 2, 6, 8, 12, 14, 16, 17, 20, 26};

namespace icbc_gpu {
int level_cost(int level) { return kLevelCost[level < 0 ? 0 : level > 9 ? 9 : level]; }

// Per-level launch shapes of the plain kernels (see icbc_gpu_launch_config).
static icbc_gpu_launch_config g_launch[10] = {{1, 1, 0, 0}, {1, 1, 0, 0}, {2, 0, 0, 0}, {2, 0, 0, 0}, {2, 0, 0, 0},
                                             {2, 0, 0, 0}, {2, 0, 0, 0}, {2, 0, 0, 0}, {2, 0, 0, 0}, {2, 0, 0, 0}};

LaunchShape launch_shape(int level) {
    const icbc_gpu_launch_config c = g_launch[level < 0 ? 0 : level > 9 ? 9 : level];
    return LaunchShape{c.groups_per_warp, c.persistent != 0, c.cta_warps, c.batch_cta_warps};
}
}  // namespace icbc_gpu

struct icbc_gpu_batch {
    ImageDesc *d_images = nullptr;
    BatchTask *d_tasks = nullptr;
    int *d_counter = nullptr;
    int ntasks = 0;
    int grid = 0;
    // Level-9 images refine in a second launch (k_refine's batch mode):
    // per-image slot base (-1: none), the refinement map, the slots, a counter.
    int64_t *d_refine_base = nullptr;
    int64_t *d_map_start = nullptr;
    uint32_t *d_map_image = nullptr;
    RefineSlot *d_slots = nullptr;
    unsigned long long *d_refine_counter = nullptr;
    int64_t refine_total = 0;
    int map_n = 0;
    // Two passes (byte rows): per-image list regions of the level-2..9
    // images (base -1: none), their counts, and how many leading tasks are
    // those images' (the planner puts them first).
    uint32_t *d_list = nullptr;
    unsigned int *d_listed = nullptr;
    int64_t *d_list_base = nullptr;
    int ntasks_listed = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

int icbc_gpu_init(int decoder) {
    if (decoder < 0 || decoder > 3) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_tables_built) {
            build_tables(g_host_tables);
            g_tables_built = true;
        }
        g_decoder = decoder;
    }
    return ensure_device_tables(nullptr);
}

int icbc_gpu_get_decoder(void) {
    std::lock_guard<std::mutex> lock(g_mutex);
    return g_decoder;
}

const char *icbc_gpu_status_string(int status) {
    switch (status) {
        case ICBC_GPU_OK: return "ok";
        case ICBC_GPU_ERR_INVALID_ARGUMENT: return "invalid argument";
        case ICBC_GPU_ERR_NOT_INITIALIZED: return "not initialized (call icbc_gpu_init)";
        case ICBC_GPU_ERR_CUDA: return "CUDA error";
        case ICBC_GPU_ERR_OUT_OF_MEMORY: return "out of memory";
        case ICBC_GPU_ERR_MISALIGNED: return "misaligned pointer or pitch";
        case ICBC_GPU_ERR_BUDGET: return "request exceeds the memory budget";
        case ICBC_GPU_ERR_NOT_READY: return "not ready";
        case ICBC_GPU_ERR_CANCELLED: return "cancelled";
        case ICBC_GPU_ERR_NOT_FOUND: return "not found";
        default: return "unknown status";
    }
}

const char *icbc_gpu_last_error(void) { return t_last_error.c_str(); }

int icbc_gpu_sm_count(void) { return sm_count(); }

int icbc_gpu_set_launch_config(int level, const icbc_gpu_launch_config *config) {
    if (level < 0 || level > 9 || !config || config->groups_per_warp < 1 || config->groups_per_warp > 64 ||
        !(config->cta_warps == 0 || config->cta_warps == 4 || config->cta_warps == 8 || config->cta_warps == 16) ||
        !(config->batch_cta_warps == 0 || config->batch_cta_warps == 4 || config->batch_cta_warps == 8 ||
          config->batch_cta_warps == 16))
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    g_launch[level] = *config;
    g_launch[level].persistent = config->persistent ? 1 : 0;
    return ICBC_GPU_OK;
}

int icbc_gpu_get_launch_config(int level, icbc_gpu_launch_config *config) {
    if (level < 0 || level > 9 || !config) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    *config = g_launch[level];
    return ICBC_GPU_OK;
}

int icbc_gpu_debug_tables(int decoder, uint8_t match5[512], uint8_t match6[512], float weights[5], uint32_t four[968],
                          int32_t four_total[16], uint32_t three[152], int32_t three_total[16]) {
    if (decoder < 0 || decoder > 3) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_tables_built) {
        build_tables(g_host_tables);
        g_tables_built = true;
    }
    const DecoderTables &D = g_host_tables.dec[decoder];
    if (match5) std::memcpy(match5, D.match5, 512);
    if (match6) std::memcpy(match6, D.match6, 512);
    if (weights) {
        weights[0] = D.w1_3; weights[1] = D.w2_3; weights[2] = D.w1_9; weights[3] = D.w4_9; weights[4] = D.w2_9;
    }
    if (four) std::memcpy(four, g_host_tables.s.four, 968 * sizeof(uint32_t));
    if (four_total) std::memcpy(four_total, g_host_tables.s.four_total, sizeof(g_host_tables.s.four_total));
    if (three) std::memcpy(three, g_host_tables.s.three, 152 * sizeof(uint32_t));
    if (three_total) std::memcpy(three_total, g_host_tables.s.three_total, sizeof(g_host_tables.s.three_total));
    return ICBC_GPU_OK;
}

int icbc_gpu_compress_bc1_blocks(int level, const float *d_colors, const float *d_weights, const float color_weights[3],
                                 int three_color_mode, int three_color_black, int decoder, void *d_out,
                                 float *d_errors, int64_t n_blocks, void *stream) {
    if (level < 0 || level > 9 || n_blocks < 0 || !color_weights) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return ICBC_GPU_OK;
    if (!d_colors || !d_out) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(d_colors, 16) || (d_weights && !aligned(d_weights, 16)) || !aligned(d_out, 8) ||
        (d_errors && !aligned(d_errors, 4)))
        return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(decoder, &dec);
    if (st) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const GlobalTables *G = nullptr;
    st = ensure_device_tables(&G);
    if (st) return st;
    BlocksSrc src{d_colors, d_weights};
    cudaError_t e = kBlocksLaunch[level](G, src, make_params(dec, three_color_mode, three_color_black, color_weights),
                                         d_out, d_errors, n_blocks, s, sm_count());
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_compress_bc1_blocks_simd(int simd_profile, int level, const float *d_colors, const float *d_weights,
                                      const float color_weights[3], int three_color_mode, int three_color_black,
                                      int decoder, void *d_out, float *d_errors, int64_t n_blocks, void *stream) {
    const int si = simd_index(simd_profile);
    if (si < 0) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    // The scalar profile, and levels without a cluster fit, are the plain path.
    if (simd_profile == 0 || level == 0 || level == 1)
        return icbc_gpu_compress_bc1_blocks(level, d_colors, d_weights, color_weights, three_color_mode,
                                            three_color_black, decoder, d_out, d_errors, n_blocks, stream);
    if (level < 0 || level > 9 || n_blocks < 0 || !color_weights) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return ICBC_GPU_OK;
    if (!d_colors || !d_out) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(d_colors, 16) || (d_weights && !aligned(d_weights, 16)) || !aligned(d_out, 8) ||
        (d_errors && !aligned(d_errors, 4)))
        return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(decoder, &dec);
    if (st) return st;
    const GlobalTables *G = nullptr;
    st = ensure_device_tables(&G);
    if (st) return st;
    EncodeParams p = make_params(dec, three_color_mode, three_color_black, color_weights);
    set_simd(p, si);
    BlocksSrc src{d_colors, d_weights};
    cudaError_t e = launch_simd(G, nullptr, &src, p, reinterpret_cast<uint2 *>(d_out), d_errors, n_blocks, level,
                                reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_compress_bc1_image_simd(int simd_profile, const icbc_gpu_image *image, void *stream) {
    const int si = simd_index(simd_profile);
    if (si < 0 || !image) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (simd_profile == 0 || image->level == 0 || image->level == 1) return icbc_gpu_compress_bc1_image(image, stream);
    ImageDesc d;
    int st = resolve_image(*image, d);
    if (st) return st;
    const GlobalTables *G = nullptr;
    st = ensure_device_tables(&G);
    if (st) return st;
    if (d.nblocks == 0) return ICBC_GPU_OK;
    EncodeParams p = make_params(d.decoder, d.three_color_mode, d.three_color_black, d.cw);
    set_simd(p, si);
    cudaError_t e = launch_simd(G, &d, nullptr, p, d.out, d.errors, d.nblocks, d.level,
                                reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_compress_bc1_image(const icbc_gpu_image *image, void *stream) {
    if (!image) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    ImageDesc d;
    int st = resolve_image(*image, d);
    if (st) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const GlobalTables *G = nullptr;
    st = ensure_device_tables(&G);
    if (st) return st;
    cudaError_t e = kImageLaunch[d.level](G, d, make_params(d.decoder, d.three_color_mode, d.three_color_black, d.cw),
                                          s, sm_count());
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_batch_create(const icbc_gpu_image *images, int n_images, icbc_gpu_batch **batch) {
    if (!batch || n_images < 0 || (n_images > 0 && !images)) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    *batch = nullptr;
    std::vector<ImageDesc> descs((size_t)n_images);
    for (int i = 0; i < n_images; i++) {
        int st = resolve_image(images[i], descs[i]);
        if (st) return st;
        if (descs[i].nblocks > 0xffffffffLL - 32) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    }
    const GlobalTables *G = nullptr;
    int st = ensure_device_tables(&G);
    if (st) return st;
    // Tasks of 32 blocks, most expensive level first; inside a level the
    // images with the same decoder and colour weights together (the CTA-wide
    // kernels search a round's blocks together only when its tasks share
    // them), larger images first, so the tail of each launch is cheap work.
    std::vector<int> order((size_t)n_images);
    for (int i = 0; i < n_images; i++) order[i] = i;
    auto cw_key = [&](int i) {
        uint64_t k = 0;
        for (int c = 0; c < 3; c++) {
            uint32_t u;
            std::memcpy(&u, &descs[i].cw[c], 4);
            k = k * 0x9e3779b97f4a7c15ull + u;
        }
        return k;
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (kLevelCost[descs[a].level] != kLevelCost[descs[b].level])
            return kLevelCost[descs[a].level] > kLevelCost[descs[b].level];
        if (descs[a].decoder != descs[b].decoder) return descs[a].decoder < descs[b].decoder;
        const uint64_t ka = cw_key(a), kb = cw_key(b);
        if (ka != kb) return ka < kb;
        return descs[a].nblocks > descs[b].nblocks;
    });
    std::vector<int> own;  // images that get their level's own launch
    std::vector<BatchTask> tasks;
    for (int i : order) {
        if (descs[i].nblocks >= kOwnLaunchBlocks) {
            own.push_back(i);
            continue;
        }
        for (int64_t b = 0; b < descs[i].nblocks; b += 32) tasks.push_back(BatchTask{(uint32_t)i, (uint32_t)b});
    }
    if (tasks.size() > 0x7fffffff) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    // Refinement slots of the level-9 images, in task order; then those of
    // the level-9 images with their own launch, one counter each.
    std::vector<int64_t> refine_base((size_t)n_images, -1), map_start, own_base;
    std::vector<uint32_t> map_image;
    int64_t refine_total = 0;
    for (int i : order) {
        if (descs[i].level != 9 || descs[i].nblocks == 0 || descs[i].nblocks >= kOwnLaunchBlocks) continue;
        refine_base[i] = refine_total;
        map_start.push_back(refine_total);
        map_image.push_back((uint32_t)i);
        refine_total += descs[i].nblocks;
    }
    map_start.push_back(refine_total);
    int64_t slots_total = refine_total;
    for (int i : own) {
        own_base.push_back(descs[i].level == 9 ? slots_total : -1);
        if (descs[i].level == 9) slots_total += descs[i].nblocks;
    }
    icbc_gpu_batch *B = new icbc_gpu_batch();
    B->ntasks = (int)tasks.size();
    // Byte texel rows (four CTAs per SM) unless an image brings a weight plane.
    bool byte_rows = true;
    for (int i = 0; i < n_images; i++) byte_rows &= descs[i].weight_mode != ICBC_GPU_WEIGHTS_PLANE;
    B->grid = sm_count() * batch_ctas_per_sm(byte_rows);
    B->refine_total = refine_total;
    B->map_n = (int)map_image.size();
    // Byte-row batches run in two passes: the blocks of 0 or 1 reduced
    // colours of the level-2..9 images are finished by a register-only pass,
    // which lists the others per image for the encoder.  Those images' tasks
    // are the leading ones (their levels cost the most).
    std::vector<int64_t> list_base((size_t)n_images, -1);
    int64_t list_total = 0;
    if (byte_rows) {
        for (const BatchTask &t : tasks) {
            if (descs[t.image].level < 2) break;
            B->ntasks_listed++;
        }
        for (int i : order) {
            if (descs[i].level < 2 || descs[i].nblocks == 0 || descs[i].nblocks >= kOwnLaunchBlocks) continue;
            list_base[i] = list_total;
            list_total += descs[i].nblocks;
        }
    }
    cudaError_t e = cudaMalloc(&B->d_images, sizeof(ImageDesc) * std::max(1, n_images));
    if (e == cudaSuccess) e = cudaMalloc(&B->d_tasks, sizeof(BatchTask) * std::max<size_t>(1, tasks.size()));
    // counter 0: the all-levels kernel's queue; 1 + L: level L's kernel's
    if (e == cudaSuccess) e = cudaMalloc(&B->d_counter, sizeof(int) * 11);
    if (e == cudaSuccess && n_images)
        e = cudaMemcpy(B->d_images, descs.data(), sizeof(ImageDesc) * n_images, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !tasks.empty())
        e = cudaMemcpy(B->d_tasks, tasks.data(), sizeof(BatchTask) * tasks.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && slots_total) {
        e = cudaMalloc(&B->d_slots, sizeof(RefineSlot) * (size_t)slots_total);
        // counter 0: the batch's refinement queue; 1..: one per own-launch image
        if (e == cudaSuccess) e = cudaMalloc(&B->d_refine_counter, sizeof(unsigned long long) * (1 + own.size()));
    }
    if (e == cudaSuccess && refine_total) {
        e = cudaMalloc(&B->d_refine_base, sizeof(int64_t) * n_images);
        if (e == cudaSuccess) e = cudaMalloc(&B->d_map_start, sizeof(int64_t) * map_start.size());
        if (e == cudaSuccess) e = cudaMalloc(&B->d_map_image, sizeof(uint32_t) * map_image.size());
        if (e == cudaSuccess)
            e = cudaMemcpy(B->d_refine_base, refine_base.data(), sizeof(int64_t) * n_images, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(B->d_map_start, map_start.data(), sizeof(int64_t) * map_start.size(),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(B->d_map_image, map_image.data(), sizeof(uint32_t) * map_image.size(),
                           cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && list_total) {
        e = cudaMalloc(&B->d_list, sizeof(uint32_t) * (size_t)list_total);
        if (e == cudaSuccess) e = cudaMalloc(&B->d_listed, sizeof(unsigned int) * n_images);
        if (e == cudaSuccess) e = cudaMalloc(&B->d_list_base, sizeof(int64_t) * n_images);
        if (e == cudaSuccess)
            e = cudaMemcpy(B->d_list_base, list_base.data(), sizeof(int64_t) * n_images, cudaMemcpyHostToDevice);
    }
    const BatchLists lists{B->d_list, B->d_listed, B->d_list_base};
    // Byte-row batches run one kernel per level (each level's own code), on
    // parallel branches of the graph so one level's tail overlaps the next
    // level's start; the planner's order keeps each level's tasks together.
    int lv_begin[10], lv_end[10];
    for (int l = 0; l < 10; l++) lv_begin[l] = lv_end[l] = -1;
    bool per_level = byte_rows && !tasks.empty();
    for (size_t t = 0; t < tasks.size() && per_level; t++) {
        const int l = descs[tasks[t].image].level;
        if (lv_begin[l] < 0) lv_begin[l] = (int)t;
        else if (lv_end[l] != (int)t) per_level = false;
        lv_end[l] = (int)t + 1;
    }
    cudaStream_t lv_stream[10] = {};
    cudaEvent_t fork = nullptr, lv_done[10] = {};
    if (e == cudaSuccess && per_level) {
        e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        for (int l = 0; l < 10 && e == cudaSuccess; l++) {
            if (lv_begin[l] < 0) continue;
            e = cudaStreamCreateWithFlags(&lv_stream[l], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&lv_done[l], cudaEventDisableTiming);
        }
    }
    // Capture "reset the queue counter, run the persistent kernel" (after
    // the first pass, when there is one; the level-9 refinement pass after
    // it) once.
    cudaStream_t cs = nullptr;
    // The launches of images with their own kernels take stream-ordered
    // scratch (captured as allocation nodes); its pool must exist first.
    if (e == cudaSuccess && !own.empty()) e = scratch_prepare();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e1 = cudaMemsetAsync(B->d_counter, 0, sizeof(int) * 11, cs);
        if (e1 == cudaSuccess && B->d_list) {
            e1 = cudaMemsetAsync(B->d_listed, 0, sizeof(unsigned int) * n_images, cs);
            if (e1 == cudaSuccess)
                e1 = launch_batch_trivial(G, B->d_images, B->d_tasks, nullptr, n_images, B->ntasks_listed, lists,
                                          B->d_refine_base, B->d_slots, cs, sm_count());
        }
        cudaError_t e2 = e1;
        if (e2 == cudaSuccess && B->ntasks && per_level) {
            e2 = cudaEventRecord(fork, cs);
            for (int l = 9; l >= 0 && e2 == cudaSuccess; l--) {
                if (lv_begin[l] < 0) continue;
                const int n = lv_end[l] - lv_begin[l];
                const int grid = std::min(B->grid, (n + kWarpsPerCta - 1) / kWarpsPerCta);  // a task per warp at most
                e2 = cudaStreamWaitEvent(lv_stream[l], fork, 0);
                if (e2 == cudaSuccess)
                    e2 = kBatchLevelLaunch[l](G, B->d_images, B->d_tasks, lv_begin[l], n, B->d_counter + 1 + l,
                                              lv_stream[l], grid, B->d_refine_base, B->d_slots, lists);
                if (e2 == cudaSuccess) e2 = cudaEventRecord(lv_done[l], lv_stream[l]);
                if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(cs, lv_done[l], 0);
            }
        } else if (e2 == cudaSuccess && B->ntasks) {
            e2 = launch_encode_batch(G, B->d_images, B->d_tasks, nullptr, n_images, B->ntasks, B->d_counter, cs,
                                     B->grid, B->d_refine_base, B->d_slots, byte_rows, lists);
        }
        if (e2 == cudaSuccess && refine_total) {
            e2 = cudaMemsetAsync(B->d_refine_counter, 0, sizeof(unsigned long long), cs);
            if (e2 == cudaSuccess)
                e2 = launch_refine_batch(G, B->d_images, RefineMap{B->d_map_start, B->d_map_image, B->map_n},
                                         B->d_slots, refine_total, B->d_refine_counter, cs, sm_count());
        }
        for (size_t j = 0; j < own.size() && e2 == cudaSuccess; j++) {
            const ImageDesc &d = descs[own[j]];
            RefineSlot *st = own_base[j] >= 0 ? B->d_slots + own_base[j] : nullptr;
            unsigned long long *counter = own_base[j] >= 0 ? B->d_refine_counter + 1 + j : nullptr;
            e2 = kImageLaunchExt[d.level](G, d, make_params(d.decoder, d.three_color_mode, d.three_color_black, d.cw),
                                          cs, sm_count(), st, counter);
        }
        e = cudaStreamEndCapture(cs, &B->graph);
        if (e1 != cudaSuccess) e = e1;
        else if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&B->exec, B->graph, 0);
    if (cs) cudaStreamDestroy(cs);
    for (int l = 0; l < 10; l++) {
        if (lv_stream[l]) cudaStreamDestroy(lv_stream[l]);
        if (lv_done[l]) cudaEventDestroy(lv_done[l]);
    }
    if (fork) cudaEventDestroy(fork);
    if (e != cudaSuccess) {
        int r = set_cuda_error(e);
        icbc_gpu_batch_destroy(B);
        return r;
    }
    *batch = B;
    return ICBC_GPU_OK;
}

int icbc_gpu_batch_launch(icbc_gpu_batch *batch, void *stream) {
    if (!batch || !batch->exec) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaGraphLaunch(batch->exec, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_batch_destroy(icbc_gpu_batch *batch) {
    if (!batch) return ICBC_GPU_OK;
    if (batch->exec) cudaGraphExecDestroy(batch->exec);
    if (batch->graph) cudaGraphDestroy(batch->graph);
    if (batch->d_images) cudaFree(batch->d_images);
    if (batch->d_tasks) cudaFree(batch->d_tasks);
    if (batch->d_counter) cudaFree(batch->d_counter);
    if (batch->d_refine_base) cudaFree(batch->d_refine_base);
    if (batch->d_map_start) cudaFree(batch->d_map_start);
    if (batch->d_map_image) cudaFree(batch->d_map_image);
    if (batch->d_slots) cudaFree(batch->d_slots);
    if (batch->d_refine_counter) cudaFree(batch->d_refine_counter);
    if (batch->d_list) cudaFree(batch->d_list);
    if (batch->d_listed) cudaFree(batch->d_listed);
    if (batch->d_list_base) cudaFree(batch->d_list_base);
    delete batch;
    return ICBC_GPU_OK;
}

int icbc_gpu_compress_bc1_images(const icbc_gpu_image *images, int n_images, void *stream) {
    icbc_gpu_batch *B = nullptr;
    int st = icbc_gpu_batch_create(images, n_images, &B);
    if (st) return st;
    st = icbc_gpu_batch_launch(B, stream);
    if (!st) {
        cudaError_t e = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) st = set_cuda_error(e);
    }
    icbc_gpu_batch_destroy(B);
    return st;
}

int icbc_gpu_compress_bc1_images_each(const icbc_gpu_image *images, int n_images, void *stream) {
    if (n_images < 0 || (n_images > 0 && !images)) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n_images; i++) {
        const int st = icbc_gpu_compress_bc1_image(&images[i], stream);
        if (st) return st;
    }
    return ICBC_GPU_OK;
}

int icbc_gpu_decode_bc1(const void *d_blocks, uint8_t *d_rgba, int64_t n_blocks, int decoder, void *stream) {
    if (n_blocks < 0) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return ICBC_GPU_OK;
    if (!d_blocks || !d_rgba) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(d_blocks, 8) || !aligned(d_rgba, 16)) return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(decoder, &dec);
    if (st) return st;
    cudaError_t e = launch_decode(d_blocks, d_rgba, n_blocks, dec, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_evaluate_bc1_error(const uint8_t *d_rgba, const void *d_blocks, float *d_errors, int64_t n_blocks,
                                int decoder, void *stream) {
    if (n_blocks < 0) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return ICBC_GPU_OK;
    if (!d_blocks || !d_rgba || !d_errors) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(d_blocks, 8) || !aligned(d_rgba, 16) || !aligned(d_errors, 4)) return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(decoder, &dec);
    if (st) return st;
    cudaError_t e = launch_evaluate(d_rgba, d_blocks, d_errors, n_blocks, dec, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_decode_bc3(const void *d_blocks, uint8_t *d_rgba, int64_t n_blocks, int decoder, void *stream) {
    if (n_blocks < 0) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return ICBC_GPU_OK;
    if (!d_blocks || !d_rgba) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(d_blocks, 16) || !aligned(d_rgba, 16)) return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(decoder, &dec);
    if (st) return st;
    cudaError_t e = launch_decode_bc3(d_blocks, d_rgba, n_blocks, dec, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

int icbc_gpu_evaluate_bc3_error(const uint8_t *d_rgba, const void *d_blocks, float *d_errors, int64_t n_blocks,
                                int alpha_blend, int decoder, void *stream) {
    if (n_blocks < 0) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return ICBC_GPU_OK;
    if (!d_blocks || !d_rgba || !d_errors) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!aligned(d_blocks, 16) || !aligned(d_rgba, 16) || !aligned(d_errors, 4)) return ICBC_GPU_ERR_MISALIGNED;
    int dec = 0;
    int st = resolve_decoder(decoder, &dec);
    if (st) return st;
    cudaError_t e = launch_evaluate_bc3(d_rgba, d_blocks, d_errors, n_blocks, alpha_blend != 0, dec,
                                        reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e);
}

// Device buffers of the host-buffer path, grown on demand and reused.
namespace {
// The host-buffer path works in bands of block rows: band i's texels go up
// on `in` while earlier bands encode and their blocks come down on `out`.
// Bands encode on two streams in turn, so consecutive bands' kernels overlap
// on the GPU and one band's tail is filled by the next band's CTAs.
constexpr int kMaxBands = 8;
struct HostPath {
    std::mutex m;
    cudaStream_t stream = nullptr, stream2 = nullptr, in = nullptr, out = nullptr;
    cudaEvent_t uploaded[kMaxBands] = {}, encoded[kMaxBands] = {};
    void *d_img = nullptr;
    size_t img_bytes = 0;
    void *d_out = nullptr;
    size_t out_bytes = 0;
    float *d_err = nullptr;
    size_t err_bytes = 0;
    float *d_plane = nullptr;
    size_t plane_bytes = 0;
};
HostPath g_host_path;

cudaError_t grow(void **p, size_t *have, size_t need) {
    if (*have >= need) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(p, need);
    if (e == cudaSuccess) *have = need;
    return e;
}
}  // namespace

int icbc_gpu_compress_bc1_image_host(const uint8_t *rgba, int32_t width, int32_t height, int64_t pitch,
                                     int32_t weight_mode, const float *weight_plane, int32_t level, int32_t decoder,
                                     int32_t three_color_mode, int32_t three_color_black, const float color_weights[3],
                                     void *out, float *errors) {
    if (!rgba || !out || !color_weights || width < 1 || height < 1 || pitch < 4 * (int64_t)width)
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (weight_mode == ICBC_GPU_WEIGHTS_PLANE && !weight_plane) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    HostPath &H = g_host_path;
    std::lock_guard<std::mutex> lock(H.m);
    cudaError_t e = cudaSuccess;
    if (!H.stream) e = cudaStreamCreateWithFlags(&H.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && !H.stream2) e = cudaStreamCreateWithFlags(&H.stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess && !H.in) e = cudaStreamCreateWithFlags(&H.in, cudaStreamNonBlocking);
    if (e == cudaSuccess && !H.out) e = cudaStreamCreateWithFlags(&H.out, cudaStreamNonBlocking);
    for (int i = 0; i < kMaxBands && e == cudaSuccess; i++) {
        if (!H.uploaded[i]) e = cudaEventCreateWithFlags(&H.uploaded[i], cudaEventDisableTiming);
        if (e == cudaSuccess && !H.encoded[i]) e = cudaEventCreateWithFlags(&H.encoded[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return set_cuda_error(e);
    const int64_t bw = (width + 3) / 4, bh = (height + 3) / 4, nb = bw * bh;
    const int64_t dpitch = ((4 * (int64_t)width + 15) / 16) * 16;
    e = grow(&H.d_img, &H.img_bytes, (size_t)(dpitch * height));
    if (e == cudaSuccess) e = grow(&H.d_out, &H.out_bytes, (size_t)(nb * 8));
    if (e == cudaSuccess && errors) e = grow(reinterpret_cast<void **>(&H.d_err), &H.err_bytes, (size_t)(nb * 4));
    if (e == cudaSuccess && weight_mode == ICBC_GPU_WEIGHTS_PLANE)
        e = grow(reinterpret_cast<void **>(&H.d_plane), &H.plane_bytes, sizeof(float) * (size_t)width * height);
    if (e != cudaSuccess) return set_cuda_error(e);
    // Bands of whole block rows (each band is an independent image whose
    // last band alone meets the bottom edge), at most kLevelBands[level] of
    // at least 512 / that many block rows each.  The light levels take eight
    // (their upload is most of the call, and eight bands overlap it with the
    // encode); levels 6-7 four and 8-9 two: a band of an eighth of the image
    // is too small for the listed pass's 16-warp CTAs and leaves a tail per
    // band, and level 9's refinement queue needs many blocks per lane.
    static const int kLevelBands[10] = {8, 8, 8, 8, 8, 8, 4, 4, 2, 2};
    const int cap_bands = std::min(kMaxBands, kLevelBands[level < 0 ? 0 : level > 9 ? 9 : level]);
    const int bands = (int)std::max<int64_t>(1, std::min<int64_t>(cap_bands, bh / (512 / cap_bands)));
    const int64_t rows_per = (bh + bands - 1) / bands;
    int st = ICBC_GPU_OK;
    for (int i = 0; i < bands && st == ICBC_GPU_OK; i++) {
        const int64_t by0 = i * rows_per, by1 = std::min<int64_t>(bh, by0 + rows_per);
        if (by0 >= by1) break;
        const int64_t y0 = 4 * by0, y1 = std::min<int64_t>(height, 4 * by1);
        const int64_t b0 = by0 * bw, nbb = (by1 - by0) * bw;
        uint8_t *dimg = static_cast<uint8_t *>(H.d_img) + y0 * dpitch;
        e = cudaMemcpy2DAsync(dimg, (size_t)dpitch, rgba + y0 * pitch, (size_t)pitch, 4 * (size_t)width,
                              (size_t)(y1 - y0), cudaMemcpyHostToDevice, H.in);
        if (e == cudaSuccess && weight_mode == ICBC_GPU_WEIGHTS_PLANE)
            e = cudaMemcpyAsync(H.d_plane + y0 * width, weight_plane + y0 * width,
                                sizeof(float) * (size_t)width * (size_t)(y1 - y0), cudaMemcpyHostToDevice, H.in);
        if (e == cudaSuccess && level >= 4)  // prior blocks, kept where no candidate is finite
            e = cudaMemcpyAsync(static_cast<uint8_t *>(H.d_out) + 8 * b0, static_cast<const uint8_t *>(out) + 8 * b0,
                                (size_t)nbb * 8, cudaMemcpyHostToDevice, H.in);
        cudaStream_t cs = (i & 1) ? H.stream2 : H.stream;
        if (e == cudaSuccess) e = cudaEventRecord(H.uploaded[i], H.in);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, H.uploaded[i], 0);
        if (e != cudaSuccess) {
            st = set_cuda_error(e);
            break;
        }
        icbc_gpu_image im;
        std::memset(&im, 0, sizeof(im));
        im.rgba = dimg;
        im.width = width;
        im.height = (int32_t)(y1 - y0);
        im.pitch = dpitch;
        im.weight_mode = weight_mode;
        im.weight_plane = weight_mode == ICBC_GPU_WEIGHTS_PLANE ? H.d_plane + y0 * width : nullptr;
        im.weight_pitch = width;
        im.level = level;
        im.decoder = decoder;
        im.three_color_mode = three_color_mode;
        im.three_color_black = three_color_black;
        im.color_weights[0] = color_weights[0];
        im.color_weights[1] = color_weights[1];
        im.color_weights[2] = color_weights[2];
        im.out = static_cast<uint8_t *>(H.d_out) + 8 * b0;
        im.errors = errors ? H.d_err + b0 : nullptr;
        st = icbc_gpu_compress_bc1_image(&im, cs);
        if (st) break;
        e = cudaEventRecord(H.encoded[i], cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(H.out, H.encoded[i], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<uint8_t *>(out) + 8 * b0, static_cast<uint8_t *>(H.d_out) + 8 * b0,
                                (size_t)nbb * 8, cudaMemcpyDeviceToHost, H.out);
        if (e == cudaSuccess && errors)
            e = cudaMemcpyAsync(errors + b0, H.d_err + b0, (size_t)nbb * 4, cudaMemcpyDeviceToHost, H.out);
        if (e != cudaSuccess) st = set_cuda_error(e);
    }
    // Every stream drains before the buffers can be reused or returned.
    const cudaError_t e1 = cudaStreamSynchronize(H.in);
    const cudaError_t e2 = cudaStreamSynchronize(H.stream);
    const cudaError_t e4 = cudaStreamSynchronize(H.stream2);
    const cudaError_t e3 = cudaStreamSynchronize(H.out);
    if (st) return st;
    if (e1 != cudaSuccess) return set_cuda_error(e1);
    if (e2 != cudaSuccess) return set_cuda_error(e2);
    if (e4 != cudaSuccess) return set_cuda_error(e4);
    return e3 == cudaSuccess ? ICBC_GPU_OK : set_cuda_error(e3);
}

}  // extern "C"
