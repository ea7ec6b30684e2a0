// Test driver for the C++ drop-in: reads blocks, calls icbc:: functions the
// way a reference caller would, writes the results.  Built by
// tests/test_compat.py against include/icbc_compat.hpp and libicbc_gpu.so.
//
// input:  int32 n, decoder, nlevels, levels[nlevels], float cw[3],
//         n x (64 floats colors, 16 floats weights, 64 bytes rgba)
// output: per level, n x (8 bytes block, float error); then for the last
//         level n x (64 bytes decoded, float evaluate_bc1_error); then per
//         block the 16-byte BC3 block {alpha0 = i, alpha1 = 255 - i, 6 index
//         bytes = i, the BC1 block} x (64 bytes decode_bc3, float
//         evaluate_bc3_error with alpha_blend, float compress_bc3's return,
//         1 byte: compress_bc3 left the block as it was)
#include <cstdio>
#include <cstdint>
#include <vector>

#include "icbc_compat.hpp"

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int32_t n = 0, decoder = 0, nlevels = 0;
    if (std::fread(&n, 4, 1, f) != 1 || std::fread(&decoder, 4, 1, f) != 1 || std::fread(&nlevels, 4, 1, f) != 1) return 4;
    std::vector<int32_t> levels(nlevels);
    float cw[3];
    if (std::fread(levels.data(), 4, nlevels, f) != (size_t)nlevels || std::fread(cw, 4, 3, f) != 3) return 4;
    std::vector<float> colors(64 * (size_t)n), weights(16 * (size_t)n);
    std::vector<unsigned char> rgba(64 * (size_t)n);
    for (int i = 0; i < n; i++) {
        if (std::fread(&colors[64 * i], 4, 64, f) != 64 || std::fread(&weights[16 * i], 4, 16, f) != 16 ||
            std::fread(&rgba[64 * i], 1, 64, f) != 64)
            return 4;
    }
    std::fclose(f);
    icbc::init((icbc::Decoder)decoder);
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 5;
    std::vector<unsigned char> blocks(8 * (size_t)n);
    for (int l : levels) {
        for (int i = 0; i < n; i++) {
            unsigned char *out = &blocks[8 * i];
            for (int k = 0; k < 8; k++) out[k] = 0;
            float e = icbc::compress_bc1((icbc::Quality)l, &colors[64 * i], &weights[16 * i], cw, true, true, out);
            std::fwrite(out, 1, 8, o);
            std::fwrite(&e, 4, 1, o);
        }
    }
    for (int i = 0; i < n; i++) {
        unsigned char dec[64];
        icbc::decode_bc1(&blocks[8 * i], dec, (icbc::Decoder)decoder);
        float e = icbc::evaluate_bc1_error(&rgba[64 * i], &blocks[8 * i], (icbc::Decoder)decoder);
        std::fwrite(dec, 1, 64, o);
        std::fwrite(&e, 4, 1, o);
    }
    for (int i = 0; i < n; i++) {
        unsigned char bc3[16], before[16], dec[64];
        bc3[0] = (unsigned char)i;
        bc3[1] = (unsigned char)(255 - i);
        for (int k = 2; k < 8; k++) bc3[k] = (unsigned char)i;
        for (int k = 0; k < 8; k++) bc3[8 + k] = blocks[8 * i + k];
        icbc::decode_bc3(bc3, dec, (icbc::Decoder)decoder);
        float e = icbc::evaluate_bc3_error(&rgba[64 * i], bc3, true, (icbc::Decoder)decoder);
        for (int k = 0; k < 16; k++) before[k] = bc3[k];
        float c = icbc::compress_bc3(icbc::Quality_Default, &colors[64 * i], &weights[16 * i], cw, false, bc3);
        unsigned char same = 1;
        for (int k = 0; k < 16; k++) same &= (unsigned char)(before[k] == bc3[k]);
        std::fwrite(dec, 1, 64, o);
        std::fwrite(&e, 4, 1, o);
        std::fwrite(&c, 4, 1, o);
        std::fwrite(&same, 1, 1, o);
    }
    std::fclose(o);
    return 0;
}
