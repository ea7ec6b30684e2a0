// icbc_compat.hpp -- icbc's public C++ interface, served by the GPU library.
//
// Same namespace, enum values and function signatures as icbc.h (v1.05,
// icbc.h:10-52), so code written against icbc compiles and links unchanged
// against libicbc_gpu.so: the symbols are the ones icbc.h declares.  Each call
// encodes, decodes or evaluates one block with one synchronous round trip to
// the GPU -- results identical to the reference, at per-call latency; batch
// work goes through the C ABI in icbc_gpu.h instead.
//
// Like icbc::init, init() selects the decoder compress_bc1 uses; it must not
// run concurrently with compress_bc1.  The other functions are thread-safe.
// BC3 behaves as the reference's does: decode_bc3 and evaluate_bc3_error use
// the colour half's 4-colour palette and alpha0 for every texel (the
// reference's alpha index is always 0, icbc.h:2929-2947, :3048-3071), and
// compress_bc3 returns 0 without writing the block (icbc.h:3850-3853).
#ifndef ICBC_COMPAT_HPP
#define ICBC_COMPAT_HPP

namespace icbc {

enum Decoder {
    Decoder_D3D10 = 0,
    Decoder_NVIDIA = 1,
    Decoder_AMD = 2,
    Decoder_Intel = 3
};

void init(Decoder decoder = Decoder_D3D10);

enum Quality {
    Quality_Level0,
    Quality_Level1,
    Quality_Level2,
    Quality_Level3,
    Quality_Level4,
    Quality_Level5,
    Quality_Level6,
    Quality_Level7,
    Quality_Level8,
    Quality_Level9,

    Quality_Fast = Quality_Level1,
    Quality_Default = Quality_Level8,
    Quality_Max = Quality_Level9,
};

void decode_bc1(const void *block, unsigned char rgba_block[16 * 4], Decoder decoder = Decoder_D3D10);
void decode_bc3(const void *block, unsigned char rgba_block[16 * 4], Decoder decoder = Decoder_D3D10);

float evaluate_bc1_error(const unsigned char rgba_block[16 * 4], const void *block, Decoder decoder = Decoder_D3D10);
float evaluate_bc3_error(const unsigned char rgba_block[16 * 4], const void *block, bool alpha_blend,
                         Decoder decoder = Decoder_D3D10);

float compress_bc1(Quality level, const float *input_colors, const float *input_weights, const float color_weights[3],
                   bool three_color_mode, bool three_color_black, void *output);
float compress_bc3(Quality level, const float *input_colors, const float *input_weights, const float color_weights[3],
                   bool six_alpha_mode, void *output);

}  // namespace icbc

#endif
