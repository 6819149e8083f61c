/*
 * rtm_zfp.c -- host decoder for the seismogram streams of the migration path: ZFP 0.5.5
 * fixed-accuracy streams of a 2-D float field, as SRC/compression_tools.c:78-135
 * (zfp2d_lossyDecompression) reads them.
 *
 * The stream is header-less: the reader knows the field (nx = receivers, fastest; ny =
 * time samples, over the flat [irec][t] buffer -- compression_tools.c:94) and the
 * tolerance (compression_tools.c:102).  This file restates the published ZFP algorithm
 * (P. Lindstrom, "Fixed-Rate Compressed Floating-Point Arrays", IEEE TVCG 2014, and the
 * zfp 0.5.5 stream format) for that one case:
 *
 *   - the field is cut into 4 x 4 blocks, x fastest; edge blocks are decoded whole and
 *     only their in-range values kept;
 *   - bits are read least-significant first from 64-bit little-endian stream words;
 *   - per block: 1 bit "block has values"; if set, an 8-bit biased common exponent emax,
 *     then the 16 integer coefficients as bit planes from the most significant down to
 *     plane kmin = max(0, 32 - maxprec), maxprec = min(64, max(0, emax - minexp + 6)),
 *     minexp = floor(log2(tolerance)) (the smallest double exponent for tolerance 0);
 *     each plane sends the bits of the coefficients already significant verbatim, then
 *     group-tests the rest (a 1 means another coefficient becomes significant; it is
 *     found by a unary scan, the last position implied);
 *   - coefficients are negabinary, stored in sequency order (perm below), decorrelated
 *     by the ZFP lifting transform (inverse: along y, then along x), and scaled by
 *     2^(emax - 30) into floats.
 *
 * Fixed-accuracy streams have variable-length blocks and no block index, so one stream
 * decodes serially; the engine overlaps it with the GPU forward propagation.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "rtm_gpu.h"

/* ---- bit reader (LSB first; bytes past the end read as zero and are counted) ---------- */
typedef struct {
    const unsigned char *p, *end;
    uint64_t buf;        /* unread bits, next bit in bit 0 */
    unsigned n;          /* valid bits in buf */
    size_t past;         /* bytes supplied beyond the end of the stream */
} zreader;

static void zr_fill(zreader *r)
{
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
    if (r->end - r->p >= 8) {             /* whole bytes up to 57..64 valid bits, one load */
        uint64_t w;
        memcpy(&w, r->p, 8);
        const unsigned k = (64 - r->n) >> 3;
        if (k == 8) {
            r->buf = w;
        } else {
            r->buf |= (w & ((UINT64_C(1) << (8 * k)) - 1)) << r->n;
        }
        r->p += k;
        r->n += 8 * k;
        return;
    }
#endif
    while (r->n <= 56) {
        uint64_t byte = 0;
        if (r->p < r->end) byte = *r->p++;
        else r->past++;
        r->buf |= byte << r->n;
        r->n += 8;
    }
}

static unsigned zr_bit(zreader *r)
{
    if (r->n == 0) zr_fill(r);
    const unsigned b = (unsigned)(r->buf & 1u);
    r->buf >>= 1;
    r->n--;
    return b;
}

/* m <= 32 bits, first bit read in bit 0 of the result */
static uint64_t zr_bits(zreader *r, unsigned m)
{
    if (m == 0) return 0;
    if (r->n < m) zr_fill(r);
    const uint64_t v = r->buf & ((UINT64_C(1) << m) - 1);
    r->buf >>= m;
    r->n -= m;
    return v;
}

/* Drops m <= n buffered bits. */
static void zr_skip(zreader *r, unsigned m)
{
    r->buf = m < 64 ? r->buf >> m : 0;
    r->n -= m;
}

/* bits consumed beyond the stream's end (the stream was truncated or corrupt) */
static int zr_overrun(const zreader *r)
{
    return (uint64_t)r->past * 8 > (uint64_t)r->n;
}

/* ---- block transform ------------------------------------------------------------------ */
/* Sequency order of the 16 coefficients of a 4 x 4 block: by i + j, then by i*i + j*j,
 * then larger i first; entry = i + 4 j (i along x). */
static const unsigned char zfp_perm2[16] = {
    0,                 /* (0,0) */
    1, 4,              /* (1,0) (0,1) */
    5,                 /* (1,1) */
    2, 8,              /* (2,0) (0,2) */
    6, 9,              /* (2,1) (1,2) */
    3, 12,             /* (3,0) (0,3) */
    10,                /* (2,2) */
    7, 13,             /* (3,1) (1,3) */
    11, 14,            /* (3,2) (2,3) */
    15                 /* (3,3) */
};

/* wrap-around arithmetic on the 32-bit coefficients */
static inline int32_t w_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t w_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t w_dbl(int32_t a) { return (int32_t)((uint32_t)a << 1); }
static inline int32_t a_half(int32_t a) { return a >> 1; }   /* arithmetic shift (gcc) */

/* Inverse of ZFP's non-orthogonal decorrelating lift on 4 values at stride s. */
static void inv_lift4(int32_t *v, int s)
{
    int32_t x = v[0], y = v[s], z = v[2 * s], w = v[3 * s];
    y = w_add(y, a_half(w)); w = w_sub(w, a_half(y));
    y = w_add(y, w); w = w_dbl(w); w = w_sub(w, y);
    z = w_add(z, x); x = w_dbl(x); x = w_sub(x, z);
    y = w_add(y, z); z = w_dbl(z); z = w_sub(z, y);
    w = w_add(w, x); x = w_dbl(x); x = w_sub(x, w);
    v[0] = x; v[s] = y; v[2 * s] = z; v[3 * s] = w;
}

/* ---- one block -------------------------------------------------------------------------- */
static void decode_block_f2(zreader *r, int minexp, float out[16])
{
    if (!zr_bit(r)) {                       /* no values above the tolerance */
        for (int i = 0; i < 16; ++i) out[i] = 0.0f;
        return;
    }
    const int emax = (int)zr_bits(r, 8) - 127;
    int maxprec = emax - minexp + 6;        /* 2 * (dims + 1) guard planes, dims = 2 */
    if (maxprec < 0) maxprec = 0;
    if (maxprec > 64) maxprec = 64;
    const unsigned kmin = maxprec < 32 ? (unsigned)(32 - maxprec) : 0u;

    /* bit planes, most significant first */
    uint32_t u[16];
    memset(u, 0, sizeof u);
    unsigned n = 0;                         /* coefficients known to be significant */
    for (unsigned k = 32; k-- > kmin;) {
        uint64_t x = zr_bits(r, n);         /* plane k of the first n coefficients */
        while (n < 16 && zr_bit(r)) {       /* group test: one more becomes significant */
            if (n < 15) {
                /* a run of zeros ends at the next significant coefficient, or at the 15th
                 * after which the last one is implied: count the run in one step */
                if (r->n < 16) zr_fill(r);
                const unsigned lim = 15 - n;
                const unsigned z = r->buf ? (unsigned)__builtin_ctzll(r->buf) : 64u;
                if (z >= lim) {
                    zr_skip(r, lim);
                    n = 15;
                } else {
                    zr_skip(r, z + 1);
                    n += z;
                }
            }
            x |= UINT64_C(1) << n;
            ++n;
        }
        while (x) {                          /* set bits of the plane into the coefficients */
            u[__builtin_ctzll(x)] |= UINT32_C(1) << k;
            x &= x - 1;
        }
    }
    /* negabinary -> two's complement, sequency order -> block order */
    int32_t q[16];
    for (int i = 0; i < 16; ++i)
        q[zfp_perm2[i]] = (int32_t)((u[i] ^ 0xaaaaaaaau) - 0xaaaaaaaau);
    for (int x = 0; x < 4; ++x) inv_lift4(q + x, 4);        /* along y */
    for (int y = 0; y < 4; ++y) inv_lift4(q + 4 * y, 1);    /* along x */
    /* q * 2^(emax-30): one rounding either way, so a multiply by the normal power of two
     * equals ldexpf, which remains for scales outside the normal range */
    const int e = emax - 30;
    if (e >= -126 && e <= 127) {
        const uint32_t bits = (uint32_t)(e + 127) << 23;
        float sc;
        memcpy(&sc, &bits, sizeof sc);
        for (int i = 0; i < 16; ++i) out[i] = (float)q[i] * sc;
    } else {
        for (int i = 0; i < 16; ++i) out[i] = ldexpf((float)q[i], e);
    }
}

/* minexp of zfp's fixed-accuracy mode for `tolerance` (0: the smallest double exponent) */
static int zfp_minexp(double tolerance)
{
    if (tolerance > 0.0) {
        int e = 0;
        (void)frexp(tolerance, &e);
        return e - 1;
    }
    return -1074;
}

int rtm_zfp_decode_float2d(const void *stream, size_t bytes, double tolerance, int nx, int ny,
                           float *out)
{
    if ((!stream && bytes) || !out || nx < 0 || ny < 0) return RTM_ERR_INVALID;
    zreader r;
    r.p = (const unsigned char *)stream;
    r.end = r.p + bytes;
    r.buf = 0;
    r.n = 0;
    r.past = 0;
    const int minexp = zfp_minexp(tolerance);
    float blk[16];
    for (int by = 0; by < ny; by += 4)
        for (int bx = 0; bx < nx; bx += 4) {
            decode_block_f2(&r, minexp, blk);
            if (zr_overrun(&r)) return RTM_ERR_DECODE;
            const int mx = nx - bx < 4 ? nx - bx : 4, my = ny - by < 4 ? ny - by : 4;
            for (int j = 0; j < my; ++j)
                for (int i = 0; i < mx; ++i)
                    out[(size_t)(by + j) * (size_t)nx + (size_t)(bx + i)] = blk[i + 4 * j];
        }
    return RTM_OK;
}

/* ---- encoder (the seismogram generator's side, compression_tools.c:10-71) ---------------
 * The inverse of the decode above: block-floating-point quantisation to 30 fraction bits
 * below the block's exponent, the forward lift (along x, then along y), sequency order and
 * negabinary, bit planes with group tests; edge blocks padded by ZFP's partial-block rule
 * (a row of n < 4 values continues v0 v0 v1 v0 / ... v1 v2 v0 -- see pad4).  The stream
 * is flushed to whole 64-bit words, as zfp_compress returns it. */
typedef struct {
    unsigned char *p, *end;
    uint64_t buf;        /* pending bits, first in bit 0 */
    unsigned n;          /* pending bit count (< 64) */
    int full;            /* the output buffer was too small */
} zwriter;

static void zw_word(zwriter *w, uint64_t v)
{
    for (int i = 0; i < 8; ++i) {
        if (w->p < w->end) *w->p++ = (unsigned char)(v >> (8 * i));
        else w->full = 1;
    }
}

static void zw_bits(zwriter *w, uint64_t v, unsigned m)     /* m <= 32 */
{
    if (m == 0) return;
    v &= (UINT64_C(1) << m) - 1;
    w->buf |= v << w->n;
    if (w->n + m >= 64) {
        zw_word(w, w->buf);
        const unsigned used = 64 - w->n;
        w->buf = used < 64 ? v >> used : 0;
        w->n = w->n + m - 64;
    } else {
        w->n += m;
    }
}

static void zw_bit(zwriter *w, unsigned b) { zw_bits(w, b & 1u, 1); }

static void zw_flush(zwriter *w)
{
    if (w->n) zw_word(w, w->buf);
    w->buf = 0;
    w->n = 0;
}

/* ZFP's padding of a partial row (stride s) holding n < 4 valid values */
static void pad4(float *v, int n, int s)
{
    switch (n) {
    case 0: v[0] = 0.0f; /* fall through */
    case 1: v[s] = v[0]; /* fall through */
    case 2: v[2 * s] = v[s]; /* fall through */
    case 3: v[3 * s] = v[0]; /* fall through */
    default: break;
    }
}

/* Forward of inv_lift4. */
static void fwd_lift4(int32_t *v, int s)
{
    int32_t x = v[0], y = v[s], z = v[2 * s], w = v[3 * s];
    x = w_add(x, w); x = a_half(x); w = w_sub(w, x);
    z = w_add(z, y); z = a_half(z); y = w_sub(y, z);
    x = w_add(x, z); x = a_half(x); z = w_sub(z, x);
    w = w_add(w, y); w = a_half(w); y = w_sub(y, w);
    w = w_add(w, a_half(y)); y = w_sub(y, a_half(w));
    v[0] = x; v[s] = y; v[2 * s] = z; v[3 * s] = w;
}

static int block_exponent(const float v[16])
{
    float mx = 0.0f;
    for (int i = 0; i < 16; ++i) {
        const float a = fabsf(v[i]);
        if (mx < a) mx = a;
    }
    if (mx > 0.0f) {
        int e = 0;
        (void)frexpf(mx, &e);
        return e < 1 - 127 ? 1 - 127 : e;
    }
    return -127;
}

static void encode_block_f2(zwriter *w, int minexp, const float v[16])
{
    const int emax = block_exponent(v);
    int maxprec = emax - minexp + 6;
    if (maxprec < 0) maxprec = 0;
    if (maxprec > 64) maxprec = 64;
    const unsigned e = maxprec ? (unsigned)(emax + 127) : 0u;
    if (!e) {
        zw_bit(w, 0);
        return;
    }
    zw_bit(w, 1);
    zw_bits(w, e, 8);
    int32_t q[16];
    const float scale = ldexpf(1.0f, 30 - emax);
    for (int i = 0; i < 16; ++i) q[i] = (int32_t)(scale * v[i]);
    for (int y = 0; y < 4; ++y) fwd_lift4(q + 4 * y, 1);    /* along x */
    for (int x = 0; x < 4; ++x) fwd_lift4(q + x, 4);        /* along y */
    uint32_t u[16];
    for (int i = 0; i < 16; ++i)
        u[i] = ((uint32_t)q[zfp_perm2[i]] + 0xaaaaaaaau) ^ 0xaaaaaaaau;
    const unsigned kmin = maxprec < 32 ? (unsigned)(32 - maxprec) : 0u;
    unsigned n = 0;
    for (unsigned k = 32; k-- > kmin;) {
        uint64_t x = 0;
        for (unsigned i = 0; i < 16; ++i) x |= (uint64_t)((u[i] >> k) & 1u) << i;
        zw_bits(w, x, n);
        x = n < 64 ? x >> n : 0;
        while (n < 16) {
            zw_bit(w, x != 0);               /* group test */
            if (!x) break;
            /* unary run to the next significant coefficient: its zeros and its one, or 15 - n
             * zeros when it is the 16th (implied), written at once */
            const unsigned z = (unsigned)__builtin_ctzll(x);
            if (n + z < 15) {
                zw_bits(w, UINT64_C(1) << z, z + 1);
                x >>= z + 1;
                n += z + 1;
            } else {
                zw_bits(w, 0, 15 - n);
                x = 0;                       /* the implied 16th was x's last bit */
                n = 16;
            }
        }
    }
}

size_t rtm_zfp_encode_bound(int nx, int ny)
{
    if (nx <= 0 || ny <= 0) return 8;
    const size_t blocks = (size_t)((nx + 3) / 4) * (size_t)((ny + 3) / 4);
    return blocks * 200 + 8;                 /* < 1 + 8 + 32 * 48 bits per block, whole words */
}

/* Blocks of block rows [r0, r1) into w (the serial order within the rows). */
static void encode_rows(zwriter *w, const float *in, int nx, int ny, int minexp, int r0, int r1)
{
    float blk[16];
    for (int by = 4 * r0; by < ny && by < 4 * r1; by += 4)
        for (int bx = 0; bx < nx; bx += 4) {
            const int mx = nx - bx < 4 ? nx - bx : 4, my = ny - by < 4 ? ny - by : 4;
            for (int j = 0; j < my; ++j)
                for (int i = 0; i < mx; ++i)
                    blk[i + 4 * j] = in[(size_t)(by + j) * (size_t)nx + (size_t)(bx + i)];
            if (mx < 4 || my < 4) {
                for (int j = 0; j < my; ++j) pad4(blk + 4 * j, mx, 1);
                for (int i = 0; i < 4; ++i) pad4(blk + i, my, 4);
            }
            encode_block_f2(w, minexp, blk);
        }
}

/* One thread's share of a parallel encode: its block rows into a private buffer. */
typedef struct {
    const float *in;
    int nx, ny, minexp, r0, r1;
    unsigned char *buf;
    size_t cap;
    uint64_t nbits;         /* bits written (before the final word flush) */
    int full;
} enc_chunk;

static void *encode_chunk(void *arg)
{
    enc_chunk *c = (enc_chunk *)arg;
    zwriter w;
    w.p = c->buf;
    w.end = c->buf + c->cap;
    w.buf = 0;
    w.n = 0;
    w.full = 0;
    encode_rows(&w, c->in, c->nx, c->ny, c->minexp, c->r0, c->r1);
    c->nbits = (uint64_t)(w.p - c->buf) * 8 + w.n;
    zw_flush(&w);
    c->full = w.full;
    return NULL;
}

/* Appends the first nbits bits of a chunk's buffer (LSB first) to w. */
static void append_bits(zwriter *w, const unsigned char *src, uint64_t nbits)
{
    for (; nbits >= 64; nbits -= 64, src += 8) {
        uint64_t v;
        memcpy(&v, src, 8);
        zw_bits(w, v & 0xffffffffu, 32);
        zw_bits(w, v >> 32, 32);
    }
    if (nbits) {
        uint64_t v = 0;
        for (unsigned i = 0; i < 8; ++i) v |= (uint64_t)src[i] << (8 * i);
        const unsigned m = (unsigned)nbits;
        zw_bits(w, v & 0xffffffffu, m < 32 ? m : 32);
        if (m > 32) zw_bits(w, v >> 32, m - 32);
    }
}

int rtm_zfp_encode_float2d(const float *in, int nx, int ny, double tolerance, void *out,
                           size_t capacity, size_t *bytes)
{
    if (!in || !out || nx < 0 || ny < 0) return RTM_ERR_INVALID;
    zwriter w;
    w.p = (unsigned char *)out;
    w.end = w.p + capacity;
    w.buf = 0;
    w.n = 0;
    w.full = 0;
    const int minexp = zfp_minexp(tolerance);
    const int rows = (ny + 3) / 4;
    /* Large fields: block rows in chunks on host threads, their bit streams concatenated
     * bit for bit -- the serial stream, as ZFP's OpenMP mode also produces it. */
    enum { kMaxThreads = 16, kRowsPerThread = 64 };
    long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
    int nthr = rows / kRowsPerThread;
    if (nthr > kMaxThreads) nthr = kMaxThreads;
    if (ncpu > 0 && nthr > ncpu) nthr = (int)ncpu;
    enc_chunk ch[kMaxThreads];
    pthread_t th[kMaxThreads];
    int started = 0;
    if (nthr >= 2) {
        for (int k = 0; k < nthr; ++k) {
            enc_chunk *c = &ch[k];
            c->in = in; c->nx = nx; c->ny = ny; c->minexp = minexp;
            c->r0 = (int)((long)rows * k / nthr);
            c->r1 = (int)((long)rows * (k + 1) / nthr);
            c->cap = (size_t)(c->r1 - c->r0) * (size_t)((nx + 3) / 4) * 200 + 16;
            c->buf = (unsigned char *)malloc(c->cap);
            c->nbits = 0;
            c->full = 0;
            if (!c->buf) break;
            if (pthread_create(&th[k], NULL, encode_chunk, c) != 0) {
                free(c->buf);
                break;
            }
            ++started;
        }
        for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
        int ok = started == nthr;
        for (int k = 0; k < started && ok; ++k) ok = !ch[k].full;
        if (ok)
            for (int k = 0; k < nthr; ++k) append_bits(&w, ch[k].buf, ch[k].nbits);
        for (int k = 0; k < started; ++k) free(ch[k].buf);
        if (!ok) {                           /* fall back to one thread */
            w.p = (unsigned char *)out;
            w.buf = 0;
            w.n = 0;
            w.full = 0;
            encode_rows(&w, in, nx, ny, minexp, 0, rows);
        }
    } else {
        encode_rows(&w, in, nx, ny, minexp, 0, rows);
    }
    zw_flush(&w);
    if (w.full) return RTM_ERR_INVALID;
    if (bytes) *bytes = (size_t)(w.p - (unsigned char *)out);
    return RTM_OK;
}

int rtm_zfp_decode_file(const char *path, float *array, int nx, int ny, float tolerance)
{
    if (!path || !array) return RTM_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return RTM_ERR_IO;
    if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return RTM_ERR_IO; }
    const long len = ftell(f);
    if (len < 0 || fseek(f, 0, SEEK_SET) != 0) { fclose(f); return RTM_ERR_IO; }
    unsigned char *buf = (unsigned char *)malloc(len > 0 ? (size_t)len : 1);
    if (!buf) { fclose(f); return RTM_ERR_NOMEM; }
    const size_t got = fread(buf, 1, (size_t)len, f);
    fclose(f);
    int st = got == (size_t)len ? rtm_zfp_decode_float2d(buf, got, (double)tolerance, nx, ny, array)
                                : RTM_ERR_IO;
    free(buf);
    return st;
}
