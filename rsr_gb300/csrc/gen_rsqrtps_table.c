/*
 * gen_rsqrtps_table.c -- measures the host CPU's RSQRTPS (SSE approximate
 * reciprocal square root) and writes the 4096-entry table that reproduces it.
 *
 * rsr normalises vectors with rmlv::normalize (src/rml/rmlv/rmlv_soa.hxx:
 * 242-248): v * rsqrtps(dot(v, v)), used by OBJ1Program's per-vertex light
 * vector (src/viewer/shaders.hxx:664-676).  RSQRTPS is implementation-defined,
 * so bit-exact parity with the reference needs the table of the CPU that
 * produced the reference's results.  For a normal positive x = 2^k * 1.m the
 * result depends only on the parity of k and the top 11 mantissa bits, and
 * scales exactly by 2^-(k - (k & 1))/2; this program checks that property
 * over all 2^32 inputs before writing:
 *   rsqrt(x) = T[(k & 1) * 2048 + (m >> 12)] * 2^-((k - (k & 1)) / 2)
 * with +-0 and denormals -> inf of the same sign, +inf -> +0, negative
 * normals and -inf -> the default NaN, NaN -> the quiet NaN.  x86-64 only;
 * the generated table is committed so non-x86 builds use the same numbers.
 *
 *   gcc -O2 -msse2 gen_rsqrtps_table.c -o gen && ./gen > rsqrtps_table.inc
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <xmmintrin.h>

static uint32_t T[4096];

static uint32_t hw(uint32_t x) {
    float f, r;
    memcpy(&f, &x, 4);
    r = _mm_cvtss_f32(_mm_rsqrt_ss(_mm_set_ss(f)));
    memcpy(&x, &r, 4);
    return x;
}

static uint32_t model(uint32_t x) {
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 255u, m = x & 0x7fffffu;
    if (e == 255u) {
        if (m) return x | 0x00400000u;           /* NaN: quieted */
        return s ? 0xffc00000u : 0u;             /* -inf: default NaN, +inf: +0 */
    }
    if (e == 0u) return s | 0x7f800000u;         /* zero and denormals: inf */
    if (s) return 0xffc00000u;                   /* negative: default NaN */
    const int k = (int)e - 127, p = k & 1;
    const uint32_t t = T[(uint32_t)p * 2048u + (m >> 12)];
    const int er = (int)((t >> 23) & 255u) - (k - p) / 2;
    return ((uint32_t)er << 23) | (t & 0x7fffffu);
}

int main(void) {
    for (uint32_t p = 0; p < 2; ++p)
        for (uint32_t i = 0; i < 2048; ++i) T[p * 2048 + i] = hw(((127u + p) << 23) | (i << 12));
    uint64_t bad = 0;
    uint32_t x = 0, first = 0;
    do {
        if (hw(x) != model(x)) { if (!bad) first = x; ++bad; }
        ++x;
    } while (x != 0);
    if (bad) {
        fprintf(stderr, "rsqrtps model mismatch on %llu inputs (first 0x%08x: hw 0x%08x model 0x%08x)\n",
                (unsigned long long)bad, first, hw(first), model(first));
        return 1;
    }
    printf("/* RSQRTPS results for inputs 2^p * (1.0 + i/2048) (p = 0, 1; i = 0..2047),\n"
           " * measured on the host by gen_rsqrtps_table.c and verified against all 2^32 inputs. */\n");
    for (int i = 0; i < 4096; ++i) printf("0x%08xu,%s", T[i], (i % 8 == 7) ? "\n" : " ");
    return 0;
}
