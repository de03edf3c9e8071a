/* Exhaustive check of the pressure solve's division by a neighbour count (pressure_stream.cu,
 * div_count): for every 32-bit pattern x and every count d in 1 .. 6, the FMA-corrected quotient
 * q0 = x * RN(1/d), q = fma(fma(-q0, d, x), RN(1/d), q0), taken when x = +0 or
 * 2^-100 <= |x| <= FLT_MAX (IEEE division otherwise), must equal the IEEE quotient x / d bit for
 * bit (NaN results compare as NaN). Prints one line per divisor and exits non-zero on a mismatch.
 * Built without FMA contraction (-ffp-contract=off) so that only the explicit fmaf calls fuse. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static float div_count(float x, int cn) {
    const float d = (float)cn, r = 1.0f / d;
    const uint32_t b = u_of(x);
    if ((b & 0x7fffffffu) - 0x0d800000u <= 0x7f7fffffu - 0x0d800000u || b == 0u) {
        const float q0 = x * r;
        return fmaf(fmaf(-q0, d, x), r, q0);
    }
    return x / d;
}

int main(void) {
    int bad_any = 0;
    for (int d = 1; d <= 6; d++) {
        unsigned long long bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
        for (long long i = 0; i < (1LL << 32); i++) {
            const float x = f_of((uint32_t)i);
            const float want = x / (float)d, got = div_count(x, d);
            if (u_of(got) != u_of(want) && !(isnan(got) && isnan(want))) bad++;
        }
        printf("count %d: %llu mismatches\n", d, bad);
        if (bad) bad_any = 1;
    }
    return bad_any;
}
