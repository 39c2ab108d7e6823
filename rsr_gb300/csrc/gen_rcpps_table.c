/*
 * gen_rcpps_table.c -- measures the host CPU's RCPPS (SSE approximate
 * reciprocal) and writes the 2048-entry table that reproduces it.
 *
 * rsr divides by w with rmlv::oneover (src/rml/rmlv/rmlv_mvec4.hxx:631-651):
 * r = rcpps(a); r = (r + r) - a*(r*r).  RCPPS is implementation-defined, so
 * bit-exact parity with the reference needs the exact table of the CPU that
 * produced the reference's results.  On Intel cores the result depends only
 * on the top 11 mantissa bits and scales exactly with the exponent; this
 * program checks that property over all 2^32 inputs before writing:
 *   rcp(x) = sign | ((e0 - (e - 127)) << 23) | mant(T[m >> 12])  (normal x)
 * with 0 / denormal -> inf, inf -> 0, NaN -> quiet NaN, and a result exponent
 * <= 0 flushed to signed zero.  x86-64 only; the generated table is
 * committed so non-x86 builds use the same numbers.
 *
 *   gcc -O2 -msse2 gen_rcpps_table.c -o gen && ./gen > rcpps_table.inc
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <xmmintrin.h>

static uint32_t T[2048];

static uint32_t hw(uint32_t x) {
    float f, r;
    memcpy(&f, &x, 4);
    r = _mm_cvtss_f32(_mm_rcp_ss(_mm_set_ss(f)));
    memcpy(&x, &r, 4);
    return x;
}

static uint32_t model(uint32_t x) {
    uint32_t s = x & 0x80000000u, e = (x >> 23) & 255u, m = x & 0x7fffffu;
    if (e == 255u) return m ? (x | 0x00400000u) : s;
    if (e == 0u) return s | 0x7f800000u;
    uint32_t t = T[m >> 12];
    int er = (int)((t >> 23) & 255u) - ((int)e - 127);
    if (er <= 0) return s;
    return s | ((uint32_t)er << 23) | (t & 0x7fffffu);
}

int main(void) {
    for (uint32_t i = 0; i < 2048; ++i) T[i] = hw((127u << 23) | (i << 12));
    uint64_t bad = 0;
    uint32_t x = 0;
    do { if (hw(x) != model(x)) ++bad; ++x; } while (x != 0);
    if (bad) { fprintf(stderr, "rcpps model mismatch on %llu inputs\n", (unsigned long long)bad); return 1; }
    printf("/* RCPPS results for inputs 1.0 + i/2048 (i = 0..2047), measured on the\n"
           " * host by gen_rcpps_table.c and verified against all 2^32 inputs. */\n");
    for (int i = 0; i < 2048; ++i) printf("0x%08xu,%s", T[i], (i % 8 == 7) ? "\n" : " ");
    return 0;
}
