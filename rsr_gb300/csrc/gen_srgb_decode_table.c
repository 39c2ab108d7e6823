/*
 * gen_srgb_decode_table.c -- writes srgb_decode_table.inc, the 256-entry
 * sRGB8 -> linear float table the device texture upload uses.
 *
 * rsr converts texture bytes with ryg::srgb8_to_float
 * (3rdparty/ryg-srgb/ryg-srgb.h:33-56, called from
 * src/rgl/rglr/rglr_texture_load.cxx:52-54): c = i * (1/255) in float;
 * c / 12.92 for c <= 0.04045, else ((c + 0.055) / 1.055) ^ 2.4, every
 * constant a float and the power taken with the float exponent 2.4f.  Here
 * the power is evaluated in double precision and rounded once to float, so
 * the table does not depend on the host's powf; tests check it against the
 * reference function's own output (tests/golden/srgb8_to_float.bin).
 *
 *   gcc -O2 -ffp-contract=off -o gen gen_srgb_decode_table.c -lm && ./gen > srgb_decode_table.inc
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

int main(void) {
    for (int i = 0; i < 256; ++i) {
        const float c = (float)i * (1.0f / 255.0f);
        float v;
        if (c <= 0.04045f) v = c / 12.92f;
        else v = (float)pow((double)((c + 0.055f) / 1.055f), (double)2.4f);
        uint32_t u;
        memcpy(&u, &v, 4);
        printf("0x%08xu,%s", u, (i % 8 == 7) ? "\n" : " ");
    }
    return 0;
}
