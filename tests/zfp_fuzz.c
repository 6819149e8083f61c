/* Fuzz driver for the host ZFP codec (csrc/rtm_zfp.c), built with AddressSanitizer and
 * UBSan by tests/test_zfp_decode.py: every truncation of a stream in an exact-size buffer,
 * random streams, and the threaded encoder at exact output capacity.  Exit status 0 when the
 * codec stays in bounds and the large field decodes within its tolerance. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rtm_gpu.h"

static unsigned long long state = 88172645463325252ULL;

static unsigned next_u32(void)
{
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (unsigned)state;
}

static float *random_field(int n)
{
    float *f = (float *)malloc(sizeof(float) * (size_t)n);
    for (int i = 0; i < n; ++i) f[i] = (float)((int)(next_u32() % 2001) - 1000) * 1e-3f;
    return f;
}

int main(void)
{
    const int nx = 37, ny = 41;
    float *f = random_field(nx * ny), *o = (float *)malloc(sizeof(float) * nx * ny);
    const size_t cap = rtm_zfp_encode_bound(nx, ny);
    unsigned char *s = (unsigned char *)malloc(cap);
    size_t used = 0;
    if (rtm_zfp_encode_float2d(f, nx, ny, 1e-4, s, cap, &used) != RTM_OK) return 1;
    for (size_t cut = 0; cut <= used; ++cut) {
        unsigned char *b = (unsigned char *)malloc(cut ? cut : 1);
        memcpy(b, s, cut);
        (void)rtm_zfp_decode_float2d(b, cut, 1e-4, nx, ny, o);
        free(b);
    }
    for (int t = 0; t < 2000; ++t) {
        const size_t n = next_u32() % 300;
        unsigned char *b = (unsigned char *)malloc(n ? n : 1);
        for (size_t i = 0; i < n; ++i) b[i] = (unsigned char)next_u32();
        (void)rtm_zfp_decode_float2d(b, n, (t & 1) ? 0.0 : 1e-4, nx, ny, o);
        free(b);
    }
    const int gx = 64, gy = 1200;          /* 300 block rows: the threaded encoder */
    float *g = random_field(gx * gy), *g2 = (float *)malloc(sizeof(float) * gx * gy);
    const size_t cap2 = rtm_zfp_encode_bound(gx, gy);
    unsigned char *s2 = (unsigned char *)malloc(cap2);
    size_t used2 = 0;
    if (rtm_zfp_encode_float2d(g, gx, gy, 1e-4, s2, cap2, &used2) != RTM_OK) return 2;
    unsigned char *exact = (unsigned char *)malloc(used2);
    memcpy(exact, s2, used2);
    if (rtm_zfp_decode_float2d(exact, used2, 1e-4, gx, gy, g2) != RTM_OK) return 3;
    double mx = 0.0;
    for (int i = 0; i < gx * gy; ++i) {
        const double d = g2[i] > g[i] ? g2[i] - g[i] : g[i] - g2[i];
        if (d > mx) mx = d;
    }
    free(f); free(o); free(s); free(g); free(g2); free(s2); free(exact);
    return mx <= 1e-4 ? 0 : 4;
}
