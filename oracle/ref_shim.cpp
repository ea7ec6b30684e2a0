// ref_shim.cpp -- extern "C" entry points over the reference's own icbc.h.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file against
// the unmodified reference header where it lies (scalar profile: ICBC_SIMD=0,
// no FP contraction) into oracle/_ref/libicbc_ref.so.  Tests use it to pin
// the C restatement in icbc_oracle.c, and tests/golden/make_golden.py uses it
// to produce the committed golden vectors.  Nothing in the product loads it.
#define ICBC_IMPLEMENTATION
#include "icbc.h"

#include <stdint.h>
#include <string.h>

extern "C" {

// icbc::init (icbc.h:19, :3813-3818).
void ref_init(int decoder) { icbc::init((icbc::Decoder)decoder); }

// icbc::compress_bc1 (icbc.h:48, :3846-3848) over n blocks, in order, on the
// calling thread, with the decoder of the last ref_init.
void ref_compress_blocks(int level, const float *colors, const float *weights, const float *cw,
                         int three_color_mode, int three_color_black, void *out, float *errors, int64_t n) {
    for (int64_t b = 0; b < n; b++) {
        float e = icbc::compress_bc1((icbc::Quality)level, colors + 64 * b, weights + 16 * b, cw,
                                     three_color_mode != 0, three_color_black != 0, (uint8_t *)out + 8 * b);
        if (errors) errors[b] = e;
    }
}

// icbc::decode_bc1 (icbc.h:38, :3820-3822).
void ref_decode_bc1(const void *block, unsigned char *rgba, int decoder) {
    icbc::decode_bc1(block, rgba, (icbc::Decoder)decoder);
}

// icbc::evaluate_bc1_error (icbc.h:43, :3837-3839).
float ref_evaluate_bc1_error(const unsigned char *rgba, const void *block, int decoder) {
    return icbc::evaluate_bc1_error(rgba, block, (icbc::Decoder)decoder);
}

// icbc::decode_bc3 (icbc.h:39, :3824-3826).
void ref_decode_bc3(const void *block, unsigned char *rgba, int decoder) {
    icbc::decode_bc3(block, rgba, (icbc::Decoder)decoder);
}

// icbc::evaluate_bc3_error (icbc.h:44, :3841-3843).
float ref_evaluate_bc3_error(const unsigned char *rgba, const void *block, int alpha_blend, int decoder) {
    return icbc::evaluate_bc3_error(rgba, block, alpha_blend != 0, (icbc::Decoder)decoder);
}

}
