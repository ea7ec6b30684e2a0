/* CPU checks of the encoder's fused arithmetic forms against the unfused
 * IEEE sequences they replace (built and run by tests/test_fused_forms.py,
 * without FP contraction; fmaf is the C library's correctly rounded fused
 * multiply-add).
 *   snap: floor(fma(s, n, 0.5f)) == floor(fl(fl(s * n) + 0.5f)) for every
 *         float s in [0, 1], n = 31 and 63 (round5 / round6).
 *   div:  div_bounded's sequence, with the IEEE reciprocal in place of
 *         rcp_bounded (equal to it on its whole domain, checked on the GPU),
 *         against a / b for every STEP-th float b in [2^-9, 64] with 16
 *         dividends each: 0, seven spread over the bit patterns of
 *         [2^-24, 64], eight uniform in [0, 64).
 * Prints the number of mismatches. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static uint32_t mix(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    long bad = 0;
    if (!strcmp(argv[1], "snap")) {
        const float ns[2] = {31.0f, 63.0f};
        for (int k = 0; k < 2; k++) {
            volatile float n = ns[k];
            for (uint32_t u = 0; u <= f2u(1.0f); u++) {
                const float s = u2f(u);
                volatile float p = s * n;
                volatile float t = p + 0.5f;
                const float a = floorf(t), b = floorf(fmaf(s, n, 0.5f));
                bad += f2u(a) != f2u(b);
            }
        }
    } else if (!strcmp(argv[1], "div")) {
        const uint32_t step = argc > 2 ? (uint32_t)strtoul(argv[2], NULL, 0) : 1;
        const uint32_t low = f2u(0x1p-24f), top = f2u(64.0f);
        for (uint32_t ub = f2u(0x1p-9f); ub <= top; ub += step) {
            const float b = u2f(ub);
            volatile float one = 1.0f;
            const float y = one / b;
            for (uint32_t k = 0; k < 16; k++) {
                const uint32_t r = mix(ub * 16u + k);
                const float a = k == 7 ? 0.0f : k < 7 ? u2f(low + r % (top - low + 1))
                                                      : (float)(r >> 8) * (64.0f / 16777216.0f);
                volatile float av = a, bv = b;
                const float e = av / bv;
                const float q0 = a * y;
                const float q1 = fmaf(fmaf(-b, q0, a), y, q0);
                const float q2 = fmaf(fmaf(-b, q1, a), y, q1);
                bad += f2u(q2) != f2u(e);
            }
        }
    } else {
        return 2;
    }
    printf("%ld\n", bad);
    return 0;
}
