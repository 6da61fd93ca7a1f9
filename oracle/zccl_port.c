/*
 * zccl_port.c -- CPU restatement of ZCCL's fastmode1 float32 codec.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle.  tests/ use it as the checker,
 * bench.py times it as the CPU baseline.  The GPU product never links it.
 *
 * Stream layout (the reference writes it at ZCCL/src/ZCCL_float.c:529-791):
 *   header : T little-endian uint64 chunk offsets, relative to the end of the
 *            header (header[0] == 0)                     (ZCCL_float.c:777-790)
 *   chunk t: segment t; the last chunk also carries segment T when
 *            N % T != 0                                  (ZCCL_float.c:672-772)
 *   segment: raw int32 quantized head, then blocks of L deltas, the last one
 *            shortened to (len-1) % L elements           (ZCCL_float.c:563-670)
 *   block  : 1 width byte b; if b > 0: ceil(n/8) sign bytes (MSB first),
 *            n * (b/8) high bytes (little-endian per element), then the low
 *            b%8 bits of every element as an MSB-first bit stream
 *                                                        (ZCCL_TypeManager.c:12-91,
 *                                                         :118-421, :824-848)
 * Quantization truncates toward zero: q = (int)((double)x * (double)(1.0f/eb))
 * (ZCCL_float.c:540,580).  Widths use the host libm: (int)log2f(max) + 1
 * (ZCCL_float.c:606).  Deltas chain across the blocks of a segment
 * (ZCCL_float.c:581-582) and wrap as int32.
 */
#include "zccl_port.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- geometry -------------------------------------------------------- */

/* The magnitude layout of a block of width b: B whole bytes per element,
 * then r bits per element.  fmt 0 is fastmode1 (B = b/8, r = b%8); fmt 1 is
 * the fixed-rate appendix codec, which keeps whole bytes only:
 * B = b/8 + 1 (at most 4), r = 0 (ZCCL/src/ZCCL_appendix.c:18-39). */
static void split(int fmt, int b, int *B, int *r)
{
    if (fmt) {
        *B = b / 8 + 1 > 4 ? 4 : b / 8 + 1;
        *r = 0;
    } else {
        *B = b / 8;
        *r = b % 8;
    }
}

/* Bytes of one encoded block of n elements at width b. */
static size_t block_bytes_f(int b, size_t n, int fmt)
{
    if (b == 0) return 1;
    int B, r;
    split(fmt, b, &B, &r);
    return 1 + (n + 7) / 8 + (size_t)B * n + ((size_t)r * n + 7) / 8;
}

static size_t block_bytes(int b, size_t n) { return block_bytes_f(b, n, 0); }

/* Largest possible encoding of a segment of len elements (every block at
 * width 32). */
static size_t segment_worst_bytes(size_t len, size_t L)
{
    size_t nfull = (len - 1) / L, ntail = (len - 1) % L;
    size_t s = 4 + nfull * block_bytes(32, L);
    if (ntail) s += block_bytes(32, ntail);
    return s;
}

int port_width(uint32_t m)
{
    if (m == 0) return 0;
    return (int)log2f((float)m) + 1; /* ZCCL_float.c:606, host libm */
}

static inline int32_t quantize(float x, double inv)
{
    /* float * double is computed in double and exact; (int) truncates. */
    return (int32_t)(x * inv);
}

static inline uint32_t magnitude(int32_t d)
{
    return d < 0 ? 0u - (uint32_t)d : (uint32_t)d;
}

/* ---- block coder ----------------------------------------------------- */

/* Encode n deltas into o; returns bytes written. */
static size_t encode_block_f(unsigned char *o, const int32_t *d, size_t n, int fmt)
{
    uint32_t m = 0;
    for (size_t j = 0; j < n; j++) {
        uint32_t v = magnitude(d[j]);
        if (v > m) m = v;
    }
    if (m == 0) {
        o[0] = 0;
        return 1;
    }
    int b = port_width(m);
    int B, r;
    split(fmt, b, &B, &r);
    unsigned char *p = o;
    *p++ = (unsigned char)b;

    size_t ns = (n + 7) / 8;
    memset(p, 0, ns);
    for (size_t j = 0; j < n; j++)
        if (d[j] < 0) p[j / 8] |= (unsigned char)(0x80u >> (j % 8));
    p += ns;

    for (size_t j = 0; j < n; j++) {
        uint32_t v = magnitude(d[j]) >> r;
        for (int k = 0; k < B; k++) *p++ = (unsigned char)(v >> (8 * k));
    }
    if (r) {
        uint32_t mask = (1u << r) - 1u;
        uint32_t acc = 0;
        int nacc = 0;
        for (size_t j = 0; j < n; j++) {
            acc = (acc << r) | (magnitude(d[j]) & mask);
            nacc += r;
            if (nacc >= 8) {
                nacc -= 8;
                *p++ = (unsigned char)(acc >> nacc);
            }
        }
        if (nacc) *p++ = (unsigned char)(acc << (8 - nacc));
    }
    return (size_t)(p - o);
}

/* Decode one block of n deltas from s into d; returns bytes consumed. */
static size_t decode_block_f(const unsigned char *s, size_t n, int32_t *d, int fmt)
{
    int b = s[0];
    if (b == 0) {
        memset(d, 0, n * sizeof(int32_t));
        return 1;
    }
    int B, r;
    split(fmt, b, &B, &r);
    const unsigned char *sg = s + 1;
    const unsigned char *hi = sg + (n + 7) / 8;
    const unsigned char *lo = hi + (size_t)B * n;
    uint32_t acc = 0;
    int nacc = 0;
    for (size_t j = 0; j < n; j++) {
        uint32_t v = 0;
        for (int k = 0; k < B; k++) v |= (uint32_t)hi[j * B + k] << (8 * k);
        v <<= r;
        if (r) {
            while (nacc < r) {
                acc = (acc << 8) | *lo++;
                nacc += 8;
            }
            nacc -= r;
            v |= (acc >> nacc) & ((1u << r) - 1u);
        }
        int neg = (sg[j / 8] >> (7 - j % 8)) & 1;
        d[j] = (int32_t)(neg ? 0u - v : v);
    }
    return block_bytes_f(b, n, fmt);
}

static size_t encode_block(unsigned char *o, const int32_t *d, size_t n) { return encode_block_f(o, d, n, 0); }
static size_t decode_block(const unsigned char *s, size_t n, int32_t *d) { return decode_block_f(s, n, d, 0); }

/* ---- per-segment passes ---------------------------------------------- */

static size_t encode_segment(unsigned char *o, const float *x, size_t len, double inv, size_t L,
                             int32_t *d, int fmt)
{
    unsigned char *p = o;
    int32_t prior = quantize(x[0], inv);
    memcpy(p, &prior, 4);
    p += 4;
    for (size_t i = 1; i < len; i += L) {
        size_t n = len - i < L ? len - i : L;
        for (size_t j = 0; j < n; j++) {
            int32_t q = quantize(x[i + j], inv);
            d[j] = (int32_t)((uint32_t)q - (uint32_t)prior);
            prior = q;
        }
        p += encode_block_f(p, d, n, fmt);
    }
    return (size_t)(p - o);
}

static size_t decode_segment(float *y, const unsigned char *s, size_t len, float eb, size_t L,
                             int32_t *d, int fmt)
{
    const unsigned char *p = s;
    int32_t prior;
    memcpy(&prior, p, 4);
    p += 4;
    y[0] = (float)prior * eb;
    for (size_t i = 1; i < len; i += L) {
        size_t n = len - i < L ? len - i : L;
        p += decode_block_f(p, n, d, fmt);
        for (size_t j = 0; j < n; j++) {
            prior = (int32_t)((uint32_t)prior + (uint32_t)d[j]);
            y[i + j] = (float)prior * eb;
        }
    }
    return (size_t)(p - s);
}

/* Homomorphic add of one segment pair (ZCCLd_float.c:1072-1221): heads add
 * as int32; a block pair with one zero-width side copies the other block;
 * otherwise both are decoded, added and re-encoded. */
static void homadd_segment(unsigned char **po, const unsigned char **pa, const unsigned char **pb,
                           size_t len, size_t L, int32_t *d1, int32_t *d2)
{
    unsigned char *o = *po;
    const unsigned char *a = *pa, *b = *pb;
    int32_t h1, h2, hs;
    memcpy(&h1, a, 4);
    memcpy(&h2, b, 4);
    hs = (int32_t)((uint32_t)h1 + (uint32_t)h2);
    memcpy(o, &hs, 4);
    a += 4;
    b += 4;
    o += 4;
    for (size_t i = 1; i < len; i += L) {
        size_t n = len - i < L ? len - i : L;
        int w1 = a[0], w2 = b[0];
        if (w1 == 0 && w2 == 0) {
            *o++ = 0;
            a++;
            b++;
        } else if (w1 == 0) {
            size_t s2 = block_bytes(w2, n);
            memcpy(o, b, s2);
            o += s2;
            b += s2;
            a++;
        } else if (w2 == 0) {
            size_t s1 = block_bytes(w1, n);
            memcpy(o, a, s1);
            o += s1;
            a += s1;
            b++;
        } else {
            a += decode_block(a, n, d1);
            b += decode_block(b, n, d2);
            for (size_t j = 0; j < n; j++) d1[j] = (int32_t)((uint32_t)d1[j] + (uint32_t)d2[j]);
            o += encode_block(o, d1, n);
        }
    }
    *po = o;
    *pa = a;
    *pb = b;
}

/* ---- stream-level entry points --------------------------------------- */

void port_compress_f(unsigned char *out, const float *in, size_t *outSize, float absErrBound,
                     size_t nbEle, int blockSize, int T, int fmt)
{
    const size_t L = (size_t)blockSize;
    const size_t tbs = nbEle / (size_t)T, rem = nbEle % (size_t)T;
    const double inv = (double)(1.0f / absErrBound); /* float division, ZCCL_float.c:540 */
    unsigned char **bufs = (unsigned char **)malloc((size_t)T * sizeof(*bufs));
    size_t *sizes = (size_t *)malloc((size_t)T * sizeof(size_t));

#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; t++) {
        size_t lo = (size_t)t * tbs;
        int has_rm = (t == T - 1 && rem != 0);
        size_t cap = segment_worst_bytes(tbs, L) + (has_rm ? segment_worst_bytes(rem, L) : 0);
        unsigned char *buf = (unsigned char *)malloc(cap);
        int32_t *d = (int32_t *)malloc(L * sizeof(int32_t));
        size_t s = encode_segment(buf, in + lo, tbs, inv, L, d, fmt);
        if (has_rm) s += encode_segment(buf + s, in + lo + tbs, rem, inv, L, d, fmt);
        bufs[t] = buf;
        sizes[t] = s;
        free(d);
    }

    uint64_t off = 0;
    for (int t = 0; t < T; t++) {
        memcpy(out + 8 * (size_t)t, &off, 8);
        off += sizes[t];
    }
    *outSize = 8 * (size_t)T + off;

#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; t++) {
        uint64_t o;
        memcpy(&o, out + 8 * (size_t)t, 8);
        memcpy(out + 8 * (size_t)T + o, bufs[t], sizes[t]);
        free(bufs[t]);
    }
    free(bufs);
    free(sizes);
}

void port_decompress_f(float *out, size_t nbEle, float absErrBound, int blockSize,
                       const unsigned char *cmp, int T, int fmt)
{
    const size_t L = (size_t)blockSize;
    const size_t tbs = nbEle / (size_t)T, rem = nbEle % (size_t)T;
    const unsigned char *data = cmp + 8 * (size_t)T;

#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; t++) {
        uint64_t o;
        memcpy(&o, cmp + 8 * (size_t)t, 8);
        int32_t *d = (int32_t *)malloc(L * sizeof(int32_t));
        size_t lo = (size_t)t * tbs;
        size_t used = decode_segment(out + lo, data + o, tbs, absErrBound, L, d, fmt);
        if (t == T - 1 && rem != 0)
            decode_segment(out + lo + tbs, data + o + used, rem, absErrBound, L, d, fmt);
        free(d);
    }
}

void port_compress(unsigned char *out, const float *in, size_t *outSize, float absErrBound,
                   size_t nbEle, int blockSize, int T)
{
    port_compress_f(out, in, outSize, absErrBound, nbEle, blockSize, T, 0);
}

void port_decompress(float *out, size_t nbEle, float absErrBound, int blockSize,
                     const unsigned char *cmp, int T)
{
    port_decompress_f(out, nbEle, absErrBound, blockSize, cmp, T, 0);
}

void port_homadd(unsigned char *out, size_t *outSize, size_t nbEle, float absErrBound,
                 int blockSize, const unsigned char *cmp1, const unsigned char *cmp2, int T)
{
    (void)absErrBound;
    const size_t L = (size_t)blockSize;
    const size_t tbs = nbEle / (size_t)T, rem = nbEle % (size_t)T;
    unsigned char **bufs = (unsigned char **)malloc((size_t)T * sizeof(*bufs));
    size_t *sizes = (size_t *)malloc((size_t)T * sizeof(size_t));

#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; t++) {
        uint64_t o1, o2;
        memcpy(&o1, cmp1 + 8 * (size_t)t, 8);
        memcpy(&o2, cmp2 + 8 * (size_t)t, 8);
        const unsigned char *a = cmp1 + 8 * (size_t)T + o1;
        const unsigned char *b = cmp2 + 8 * (size_t)T + o2;
        int has_rm = (t == T - 1 && rem != 0);
        size_t cap = segment_worst_bytes(tbs, L) + (has_rm ? segment_worst_bytes(rem, L) : 0);
        unsigned char *buf = (unsigned char *)malloc(cap);
        unsigned char *o = buf;
        int32_t *d1 = (int32_t *)malloc(L * sizeof(int32_t));
        int32_t *d2 = (int32_t *)malloc(L * sizeof(int32_t));
        homadd_segment(&o, &a, &b, tbs, L, d1, d2);
        if (has_rm) homadd_segment(&o, &a, &b, rem, L, d1, d2);
        bufs[t] = buf;
        sizes[t] = (size_t)(o - buf);
        free(d1);
        free(d2);
    }
    /* Every input byte has been read; out may now overwrite cmp2. */
    uint64_t off = 0;
    for (int t = 0; t < T; t++) {
        memcpy(out + 8 * (size_t)t, &off, 8);
        off += sizes[t];
    }
    *outSize += 8 * (size_t)T + off;

#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; t++) {
        uint64_t o;
        memcpy(&o, out + 8 * (size_t)t, 8);
        memcpy(out + 8 * (size_t)T + o, bufs[t], sizes[t]);
        free(bufs[t]);
    }
    free(bufs);
    free(sizes);
}

/* ======================================================================
 * SZp 3-D codec, serial form (SZp_compress3D_fast / SZp_compress3D,
 * ZCCL/src/ZCCL_float.c:1706-1860; SZp_decompress3D, ZCCL/src/ZCCLd_float.c:2801-2871).
 *
 *   q(i,j,k) = (int)floor((double)x * (0.5 / eb) + 0.5)            (ZCCL_float.h:57-61)
 *   e = the 3-D mixed difference of q, zero outside the volume     (ZCCL_float.h:63-73)
 *   stream = one rate byte per block (blocks of bs^3 in x, y, z order, edge
 *            blocks cut short), then per block of non-zero rate: its sign
 *            bits and fixed-length magnitude bits, the fastmode1 packers'
 *            layout (signs MSB-first, B = rate/8 high bytes little-endian,
 *            r = rate%8 low bits MSB-first); rate = bit length of the
 *            block's largest |e| (no log2f)
 *   x' = (float)((double)q * (2 eb)), q the 3-D prefix sum of e   (ZCCLd_float.c:2807,2855-2857)
 * Integer arithmetic wraps modulo 2^32 like the reference's int.
 * ====================================================================== */

static size_t pack_payload(unsigned char *o, const int32_t *e, size_t n, int b)
{
    int B = b / 8, r = b % 8;
    unsigned char *p = o;
    size_t ns = (n + 7) / 8;
    memset(p, 0, ns);
    for (size_t j = 0; j < n; j++)
        if (e[j] < 0) p[j / 8] |= (unsigned char)(0x80u >> (j % 8));
    p += ns;
    for (size_t j = 0; j < n; j++) {
        uint32_t v = magnitude(e[j]) >> r;
        for (int k = 0; k < B; k++) *p++ = (unsigned char)(v >> (8 * k));
    }
    if (r) {
        uint32_t mask = (1u << r) - 1u, acc = 0;
        int nacc = 0;
        for (size_t j = 0; j < n; j++) {
            acc = (acc << r) | (magnitude(e[j]) & mask);
            nacc += r;
            if (nacc >= 8) {
                nacc -= 8;
                *p++ = (unsigned char)(acc >> nacc);
            }
        }
        if (nacc) *p++ = (unsigned char)(acc << (8 - nacc));
    }
    return (size_t)(p - o);
}

static size_t unpack_payload(const unsigned char *s, size_t n, int b, int32_t *e)
{
    int B = b / 8, r = b % 8;
    const unsigned char *sg = s, *hi = s + (n + 7) / 8, *lo = hi + (size_t)B * n;
    uint32_t acc = 0;
    int nacc = 0;
    for (size_t j = 0; j < n; j++) {
        uint32_t v = 0;
        for (int k = 0; k < B; k++) v |= (uint32_t)hi[j * B + k] << (8 * k);
        v <<= r;
        if (r) {
            while (nacc < r) {
                acc = (acc << 8) | *lo++;
                nacc += 8;
            }
            nacc -= r;
            v |= (acc >> nacc) & ((1u << r) - 1u);
        }
        int neg = (sg[j / 8] >> (7 - j % 8)) & 1;
        e[j] = (int32_t)(neg ? 0u - v : v);
    }
    return (n + 7) / 8 + (size_t)B * n + ((size_t)r * n + 7) / 8;
}

static int bit_length(uint32_t m)
{
    int b = 0;
    while (m) {
        b++;
        m >>= 1;
    }
    return b;
}

/* q over the volume with a zero plane before each axis: index (i+1, j+1, k+1). */
#define ZP3(i, j, k) ((((size_t)(i)) * (d2 + 1) + (size_t)(j)) * (d3 + 1) + (size_t)(k))

void port_szp3d_compress(const float *x, unsigned char *out, size_t d1, size_t d2, size_t d3, int bs,
                         double eb, size_t *cmpSize)
{
    const double inv = 0.5 / eb;
    uint32_t *q = (uint32_t *)calloc((d1 + 1) * (d2 + 1) * (d3 + 1), sizeof(uint32_t));
    for (size_t i = 0; i < d1; i++)
        for (size_t j = 0; j < d2; j++)
            for (size_t k = 0; k < d3; k++) {
                double v = floor((double)x[(i * d2 + j) * d3 + k] * inv + 0.5);
                q[ZP3(i + 1, j + 1, k + 1)] = (uint32_t)(int32_t)v;
            }
    const size_t nb1 = (d1 - 1) / bs + 1, nb2 = (d2 - 1) / bs + 1, nb3 = (d3 - 1) / bs + 1;
    int32_t *e = (int32_t *)malloc((size_t)bs * bs * bs * sizeof(int32_t));
    unsigned char *p = out + nb1 * nb2 * nb3;
    size_t blk = 0;
    for (size_t bx = 0; bx < nb1; bx++)
        for (size_t by = 0; by < nb2; by++)
            for (size_t bz = 0; bz < nb3; bz++) {
                size_t n = 0;
                uint32_t m = 0;
                for (size_t i = bx * bs; i < d1 && i < (bx + 1) * bs; i++)
                    for (size_t j = by * bs; j < d2 && j < (by + 1) * bs; j++)
                        for (size_t k = bz * bs; k < d3 && k < (bz + 1) * bs; k++) {
                            uint32_t v = q[ZP3(i + 1, j + 1, k + 1)] - q[ZP3(i + 1, j + 1, k)] -
                                         q[ZP3(i + 1, j, k + 1)] + q[ZP3(i + 1, j, k)] -
                                         q[ZP3(i, j + 1, k + 1)] + q[ZP3(i, j + 1, k)] +
                                         q[ZP3(i, j, k + 1)] - q[ZP3(i, j, k)];
                            e[n++] = (int32_t)v;
                            uint32_t a = magnitude((int32_t)v);
                            if (a > m) m = a;
                        }
                int b = bit_length(m);
                out[blk++] = (unsigned char)b;
                if (b) p += pack_payload(p, e, n, b);
            }
    *cmpSize = (size_t)(p - out);
    free(e);
    free(q);
}

void port_szp3d_decompress(float *y, const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs,
                           double eb)
{
    const double twice = eb * 2;
    uint32_t *q = (uint32_t *)calloc((d1 + 1) * (d2 + 1) * (d3 + 1), sizeof(uint32_t));
    const size_t nb1 = (d1 - 1) / bs + 1, nb2 = (d2 - 1) / bs + 1, nb3 = (d3 - 1) / bs + 1;
    int32_t *e = (int32_t *)malloc((size_t)bs * bs * bs * sizeof(int32_t));
    const unsigned char *p = cmp + nb1 * nb2 * nb3;
    size_t blk = 0;
    for (size_t bx = 0; bx < nb1; bx++)
        for (size_t by = 0; by < nb2; by++)
            for (size_t bz = 0; bz < nb3; bz++) {
                const size_t sx = (bx + 1) * bs < d1 ? bs : d1 - bx * bs;
                const size_t sy = (by + 1) * bs < d2 ? bs : d2 - by * bs;
                const size_t sz = (bz + 1) * bs < d3 ? bs : d3 - bz * bs;
                const size_t n = sx * sy * sz;
                int b = cmp[blk++];
                if (b)
                    p += unpack_payload(p, n, b, e);
                else
                    memset(e, 0, n * sizeof(int32_t));
                size_t t = 0;
                for (size_t i = bx * bs; i < bx * bs + sx; i++)
                    for (size_t j = by * bs; j < by * bs + sy; j++)
                        for (size_t k = bz * bs; k < bz * bs + sz; k++)
                            q[ZP3(i + 1, j + 1, k + 1)] = (uint32_t)e[t++];
            }
    /* the 3-D prefix sum, one axis at a time */
    for (size_t i = 1; i <= d1; i++)
        for (size_t j = 1; j <= d2; j++)
            for (size_t k = 1; k <= d3; k++) q[ZP3(i, j, k)] += q[ZP3(i, j, k - 1)];
    for (size_t i = 1; i <= d1; i++)
        for (size_t j = 1; j <= d2; j++)
            for (size_t k = 1; k <= d3; k++) q[ZP3(i, j, k)] += q[ZP3(i, j - 1, k)];
    for (size_t i = 1; i <= d1; i++)
        for (size_t j = 1; j <= d2; j++)
            for (size_t k = 1; k <= d3; k++) {
                q[ZP3(i, j, k)] += q[ZP3(i - 1, j, k)];
                y[((i - 1) * d2 + (j - 1)) * d3 + (k - 1)] = (float)((double)(int32_t)q[ZP3(i, j, k)] * twice);
            }
    free(e);
    free(q);
}
#undef ZP3

/* ======================================================================
 * The counts the reference's _record variants return.
 * ====================================================================== */

/* Walks the blocks of a segment of len elements starting at p (after its
 * raw head): adds the bytes of the blocks to *bytes and the elements of the
 * blocks of non-zero width to *nz; returns the byte after the segment. */
static const unsigned char *walk_segment(const unsigned char *p, size_t len, size_t L, size_t *bytes, size_t *nz)
{
    if (len == 0) return p;
    p += 4;
    for (size_t left = len - 1; left > 0;) {
        const size_t m = left < L ? left : L;
        const int b = p[0];
        const size_t s = block_bytes(b, m);
        *bytes += s;
        if (b) *nz += m;
        p += s;
        left -= m;
    }
    return p;
}

void port_record_counts(const unsigned char *cmp, size_t n, int L, size_t *compress_count,
                        size_t *decompress_count)
{
    size_t bytes = 0, nz = 0;
    walk_segment(cmp + 8, n, (size_t)L, &bytes, &nz);
    const size_t C = 8 + 4 + bytes;
    /* ZCCL_float_single_thread_arg_record (ZCCL/src/ZCCL_float.c:990-1209):
     * 20 bytes around the head; 12 per element of every block (the float
     * read and two 4-byte stores whatever the delta's sign); per block its
     * bytes, plus 8 per element (the sign and magnitude arrays read by the
     * packers) when its width is not 0; 56 for the offset table and the
     * copies' bookkeeping; the chunk copied out, read and written. */
    *compress_count = 20 + 12 * (n - 1) + bytes + 8 * nz + 56 + 2 * (C - 8);
    /* ZCCL_float_decompress_single_thread_arg_record
     * (ZCCL/src/ZCCLd_float.c:376-536): 24 bytes around the head; per block
     * its bytes, plus 8 per element for a constant block (a float read and
     * written) or 20 per element otherwise (the unpacked sign and magnitude
     * arrays, the delta read, the float written and read). */
    *decompress_count = 24 + bytes + 8 * (n - 1) + 12 * nz;
}

/* Classifies the block pairs of one segment of two streams. */
static void cases_segment(const unsigned char **pa, const unsigned char **pb, size_t len, size_t L,
                          unsigned long long c[4])
{
    if (len == 0) return;
    const unsigned char *a = *pa + 4, *b = *pb + 4;
    for (size_t left = len - 1; left > 0;) {
        const size_t m = left < L ? left : L;
        const int wa = a[0], wb = b[0];
        c[!wa && !wb ? 0 : !wa ? 1 : !wb ? 2 : 3]++;
        a += block_bytes(wa, m);
        b += block_bytes(wb, m);
        left -= m;
    }
    *pa = a;
    *pb = b;
}

void port_homadd_cases(const unsigned char *cmp1, const unsigned char *cmp2, size_t nbEle, int blockSize, int T,
                       unsigned long long counts[4])
{
    /* ZCCL_float_homomophic_add_openmp_threadblock_record
     * (ZCCL/src/ZCCLd_float.c:2067-2800): counter_1 both widths 0,
     * counter_2 only the first 0, counter_3 only the second 0, counter_4
     * neither, over every block pair of every segment. */
    const size_t L = (size_t)blockSize, tbs = nbEle / (size_t)T, rem = nbEle % (size_t)T;
    counts[0] = counts[1] = counts[2] = counts[3] = 0;
    for (int t = 0; t < T; t++) {
        uint64_t o1, o2;
        memcpy(&o1, cmp1 + 8 * (size_t)t, 8);
        memcpy(&o2, cmp2 + 8 * (size_t)t, 8);
        const unsigned char *a = cmp1 + 8 * (size_t)T + o1, *b = cmp2 + 8 * (size_t)T + o2;
        cases_segment(&a, &b, tbs, L, counts);
        if (t == T - 1 && rem) cases_segment(&a, &b, rem, L, counts);
    }
}

/* ======================================================================
 * SZp 3-D codec, OpenMP form (SZp_compress3D_fast_openmp,
 * ZCCL/src/ZCCL_float.c:1862-2048; SZp_decompress3D_fast_openmp,
 * ZCCL/src/ZCCLd_float.c:2873-3034): the volume is split among T threads
 * by a 3-D grid of tdims[0] x tdims[1] x tdims[2] sub-volumes; the stream
 * is T little-endian size_t offsets (relative to the end of the offsets)
 * followed by every sub-volume's serial-form stream in thread order.
 * ====================================================================== */

static int cmp_int_desc(const void *a, const void *b)
{
    const int x = *(const int *)a, y = *(const int *)b;
    return (x < y) - (x > y);
}

/* My_Dims_create(n, 3, {0, 0, 0}) (ZCCL/src/ZCCL_multidim.c:100-140): the
 * prime factors of n, largest first, each multiplied into the currently
 * smallest dimension (the first of equals), the result sorted descending. */
void port_dims3(int n, int d[3])
{
    int f[64], nf = 0;
    d[0] = d[1] = d[2] = 1;
    for (int i = 2, rem = n; i <= rem; i++)
        while (rem % i == 0) {
            f[nf++] = i;
            rem /= i;
        }
    qsort(f, (size_t)nf, sizeof(int), cmp_int_desc);
    for (int i = 0; i < nf; i++) {
        int m = 0;
        for (int j = 1; j < 3; j++)
            if (d[j] < d[m]) m = j;
        d[m] *= f[i];
    }
    qsort(d, 3, sizeof(int), cmp_int_desc);
}

/* Sub-volume of thread r: origin o[3] and extent s[3] (ZCCL_float.c:1904-1933:
 * extents base + 1 for the first `rem` parts of each axis, thread order
 * x-major). */
static void split_meta(size_t d1, size_t d2, size_t d3, const int td[3], int r, size_t o[3], size_t s[3])
{
    const size_t dim[3] = {d1, d2, d3};
    int c[3];
    c[0] = r / (td[1] * td[2]);
    c[1] = (r / td[2]) % td[1];
    c[2] = r % td[2];
    for (int a = 0; a < 3; a++) {
        const size_t base = dim[a] / (size_t)td[a], rem = dim[a] % (size_t)td[a];
        o[a] = (size_t)c[a] * base + ((size_t)c[a] < rem ? (size_t)c[a] : rem);
        s[a] = base + ((size_t)c[a] < rem ? 1u : 0u);
    }
}

void port_szp3d_compress_split(const float *x, unsigned char *out, size_t d1, size_t d2, size_t d3, int bs,
                               double eb, int T, size_t *cmpSize)
{
    int td[3];
    port_dims3(T, td);
    size_t off = 0;
    for (int r = 0; r < T; r++) {
        size_t o[3], s[3];
        split_meta(d1, d2, d3, td, r, o, s);
        float *sub = (float *)malloc((s[0] * s[1] * s[2] + 1) * sizeof(float));
        for (size_t i = 0; i < s[0]; i++)
            for (size_t j = 0; j < s[1]; j++)
                memcpy(sub + (i * s[1] + j) * s[2], x + ((o[0] + i) * d2 + o[1] + j) * d3 + o[2], s[2] * sizeof(float));
        size_t sz = 0;
        memcpy(out + 8 * (size_t)r, &off, 8);
        port_szp3d_compress(sub, out + 8 * (size_t)T + off, s[0], s[1], s[2], bs, eb, &sz);
        off += sz;
        free(sub);
    }
    *cmpSize = 8 * (size_t)T + off;
}

void port_szp3d_decompress_split(float *y, const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs,
                                 double eb, int T)
{
    int td[3];
    port_dims3(T, td);
    for (int r = 0; r < T; r++) {
        size_t o[3], s[3];
        split_meta(d1, d2, d3, td, r, o, s);
        uint64_t off;
        memcpy(&off, cmp + 8 * (size_t)r, 8);
        float *sub = (float *)malloc((s[0] * s[1] * s[2] + 1) * sizeof(float));
        port_szp3d_decompress(sub, cmp + 8 * (size_t)T + off, s[0], s[1], s[2], bs, eb);
        for (size_t i = 0; i < s[0]; i++)
            for (size_t j = 0; j < s[1]; j++)
                memcpy(y + ((o[0] + i) * d2 + o[1] + j) * d3 + o[2], sub + (i * s[1] + j) * s[2], s[2] * sizeof(float));
        free(sub);
    }
}
