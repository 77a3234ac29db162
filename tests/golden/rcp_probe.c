// Fixture probe (x86-64 only, never built for the product or on an Arm host):
// prints the SSE RCPPS reciprocal estimate of 1 + t/2048 for t = 0..2047 as
// 32-bit patterns, one per line. The reference's release build (gcc -O3
// -ffast-math -march=native) quantizes with this estimate plus one Newton step
// (src/vc/vc.c:299, vectorised); on the host that produced the golden archives
// the estimate depends only on the top 11 mantissa bits and scales exactly
// with the exponent, so these 2048 values reproduce it for every normal input.
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#if defined(__x86_64__)
#include <xmmintrin.h>
int main(void) {
    for (uint32_t t = 0; t < 2048; ++t) {
        uint32_t b = (127u << 23) | (t << 12);
        float x, r;
        memcpy(&x, &b, 4);
        r = _mm_cvtss_f32(_mm_rcp_ps(_mm_set1_ps(x)));
        uint32_t rb;
        memcpy(&rb, &r, 4);
        printf("%u\n", rb);
    }
    return 0;
}
#else
int main(void) { fprintf(stderr, "rcp_probe: x86-64 only\n"); return 1; }
#endif
