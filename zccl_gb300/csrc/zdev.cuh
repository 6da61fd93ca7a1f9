/*
 * zdev.cuh -- device building blocks shared by the codec kernels.
 *
 *   quantize*()          bit-exact stand-ins for (int)((double)x * (double)inv)
 *   width_of()           bit-exact stand-in for (int)log2f((float)m) + 1
 *   encode_full/decode_full   one 32-element block, registers <-> packed bytes
 *   encode_small/decode_small/decode_add_full   the same for widths below 16
 *   encode_mid/decode_mid     the same for widths 16..23 (two high bytes)
 *   encode_block32/decode_block32   the fastest of these for a block's width
 *   encode_any/decode_any     any block, one element at a time
 *   Packer / Reader      MSB-first bit streams in shared memory
 *   tma_load_superset()  TMA bulk copy global -> shared
 *   store_realign()      shared -> global at any byte alignment
 *   cta_excl_scan()      block-wide exclusive scan
 *   lb_publish/resolve   single-pass decoupled look-back across tiles
 */
#ifndef ZCCL_GB300_ZDEV_CUH
#define ZCCL_GB300_ZDEV_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "zccl_err.h"
#include "zgeom.h"

/* ---------------------------------------------------------------------
 * Exact arithmetic
 * ------------------------------------------------------------------- */

/* Width thresholds, filled on the host from the host's libm: thr[w] is the
 * smallest m of bit length w whose (int)log2f((float)m) equals w (so its
 * width is w + 1), or 0xFFFFFFFF when none exists.  glibc rounds log2f of
 * 5,876 integers just below a power of two up to that power. */
struct ZWidthTable {
    uint32_t thr[33];
};

/* zg_block_bytes for a full 32-element fastmode1 block of width b <= 32: the
 * header, four sign bytes and 4 b bytes of magnitudes; a zero-width block is
 * its header alone. */
__device__ __forceinline__ uint32_t block32_bytes(uint32_t b) { return b ? 4u * b + 5u : 1u; }

/* (int)log2f((float)m) + 1 for m > 0 and 0 for m == 0, as the reference
 * computes it with the host libm (ZCCL/src/ZCCL_float.c:606). */
__device__ __forceinline__ uint32_t width_of(uint32_t m, const ZWidthTable &wt)
{
    uint32_t w = 32u - __clz(m); /* bit length; 0 for m == 0 */
    return w + (m >= wt.thr[w] ? 1u : 0u);
}

/* (int)((double)x * (double)inv) without FP64.
 *
 * The product of two floats is exact in double, and the reference truncates
 * it toward zero.  mul.rz returns the float nearest the exact product on the
 * side of zero; while |P| < 2^24 every integer is a float, so truncating the
 * rz product gives trunc(P).  Above that, the TwoProduct error-free
 * transformation (Ogita, Rump, Oishi 2005) splits P = p + e exactly with p
 * an integer-valued float, and trunc(P) = p + floor(e) (P > 0) or
 * p + ceil(e) (P < 0).  Non-finite values or |P| >= 2^31 (undefined in the
 * reference) set ZERR_RANGE in *bad. */
__device__ __forceinline__ int32_t quantize(float x, float inv, uint32_t &bad)
{
    float pz = __fmul_rz(x, inv);
    if (fabsf(pz) < 16777216.0f) return __float2int_rz(pz);
    float p = __fmul_rn(x, inv);
    float e = __fmaf_rn(x, inv, -p);
    if (!(fabsf(p) < 2147483648.0f)) {
        bad |= ZERR_RANGE;
        return 0;
    }
    float c = p > 0.0f ? floorf(e) : ceilf(e);
    return (int32_t)((uint32_t)__float2int_rz(p) + (uint32_t)__float2int_rz(c));
}

/* The same truncation when the caller knows |x * inv| < 2^24 (see
 * tile_fast_ok()): one rounded-toward-zero multiply and a truncating
 * conversion. */
__device__ __forceinline__ int32_t quantize_fast(float x, float inv)
{
    return __float2int_rz(__fmul_rz(x, inv));
}

/* max over |x| as raw float bits: NaN ranks above +inf, so a NaN also fails
 * the fast-quantization test. */
__device__ __forceinline__ uint32_t abs_bits(float x) { return __float_as_uint(x) & 0x7FFFFFFFu; }

/* Fast quantization is exact for the whole tile when the rounded-toward-
 * zero product of its largest magnitude stays below 2^24. */
__device__ __forceinline__ bool tile_fast_ok(uint32_t amax_bits, float inv)
{
    float am = __uint_as_float(amax_bits);
    return am == am && fabsf(__fmul_rz(am, inv)) < 16777216.0f;
}

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

/* ---------------------------------------------------------------------
 * Bit streams in shared memory.  A block is a sequence of bytes; bits go
 * MSB first within a byte, which is how the reference packs sign bits and
 * the low r bits of every magnitude (ZCCL/src/ZCCL_TypeManager.c:118-421,
 * :824-848).  Whole bytes put as 8k-bit values keep their order.
 * ------------------------------------------------------------------- */

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* OR a finished word into shared memory (the packing buffer starts zeroed,
 * so neighbouring blocks that share a boundary word need no coordination). */
__device__ __forceinline__ void sh_or(uint32_t saddr, uint32_t v)
{
    asm volatile("red.shared.or.b32 [%0], %1;" ::"r"(saddr), "r"(v) : "memory");
}

/* Packs MSB-first bits into a zeroed shared buffer from byte offset o.  The
 * 64-bit accumulator holds nacc pending bits right-aligned; callers keep
 * nacc < 32 before a put of up to 32 bits by calling flush(). */
struct Packer {
    uint32_t wa, nacc; /* shared address of the current word; pending bits */
    uint64_t acc;

    __device__ __forceinline__ void init(uint32_t sbase, uint32_t o)
    {
        wa = sbase + (o & ~3u);
        nacc = (o & 3u) * 8u;
        acc = 0;
    }
    __device__ __forceinline__ void put(uint32_t v, uint32_t n) /* v < 2^n, n <= 32 */
    {
        acc = (acc << n) | v;
        nacc += n;
    }
    __device__ __forceinline__ void flush()
    {
        if (nacc >= 32u) {
            nacc -= 32u;
            sh_or(wa, bswap32((uint32_t)(acc >> nacc)));
            wa += 4;
        }
    }
    __device__ __forceinline__ void finish()
    {
        flush();
        if (nacc) sh_or(wa, bswap32((uint32_t)acc << (32u - nacc)));
    }
};

/* Reads MSB-first bits from byte offset o of a shared word array.  After
 * refill() at least 33 bits are buffered.  Loads whole aligned words, so it
 * may read up to 8 bytes past the last bit it returns (buffers carry slack). */
struct Reader {
    const uint32_t *w;
    uint32_t wi, nacc;
    uint64_t acc; /* valid bits left-aligned */

    __device__ __forceinline__ void init(const uint32_t *words, uint32_t o)
    {
        w = words;
        wi = o >> 2;
        const uint32_t skip = (o & 3u) * 8u;
        acc = ((uint64_t)bswap32(w[wi]) << 32) << skip;
        nacc = 32u - skip;
        wi++;
        refill();
    }
    __device__ __forceinline__ void refill()
    {
        if (nacc <= 32u) {
            acc |= (uint64_t)bswap32(w[wi]) << (32u - nacc);
            wi++;
            nacc += 32u;
        }
    }
    __device__ __forceinline__ uint32_t get(uint32_t n) /* 1 <= n <= 32 */
    {
        uint32_t v = (uint32_t)(acc >> 32) >> (32u - n);
        acc <<= n;
        nacc -= n;
        return v;
    }
};

/* One full block of 32 elements: magnitudes m[] (m[j] >> b == 0), the sign
 * mask (element j at bit 31 - j) and the width b, packed at byte o of the
 * zeroed shared buffer at sbase.  Straight-line code: the header and the 32
 * sign bits, then the B = b/8 high bytes of each element (little-endian per
 * element, four elements per word when B == 1), then the r = b%8 low bits of
 * each element (four r-bit fields merged per put).  A zero-width block is a
 * single 0x00 byte, already in the buffer. */
__device__ __forceinline__ void encode_full(uint32_t sbase, uint32_t o, uint32_t b, uint32_t smask,
                                            const uint32_t (&m)[32], uint32_t fmt = ZG_FASTMODE1)
{
    if (b == 0) return;
    uint32_t B, r;
    zg_split(fmt, b, &B, &r);
    Packer pk;
    pk.init(sbase, o);
    pk.put(b, 8);
    pk.flush();
    pk.put(smask, 32);
    pk.flush();
    if (B == 1) {
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
            uint32_t h = (((m[j] >> r) * 256u + (m[j + 1] >> r)) * 256u + (m[j + 2] >> r)) * 256u +
                         (m[j + 3] >> r);
            pk.put(h, 32);
            pk.flush();
        }
    } else if (B > 1) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
            pk.put(bswap32(m[j] >> r) >> (32u - 8u * B), 8u * B);
            pk.flush();
        }
    }
    if (r) {
        const uint32_t p = 1u << r, mask = p - 1u;
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
            uint32_t v0 = m[j], v1 = m[j + 1], v2 = m[j + 2], v3 = m[j + 3];
            if (B) {
                v0 &= mask;
                v1 &= mask;
                v2 &= mask;
                v3 &= mask;
            }
            pk.put(((v0 * p + v1) * p + v2) * p + v3, 4u * r);
            pk.flush();
        }
    }
    pk.finish();
}

/* The width byte and the four sign bytes of a 32-element fastmode1 block as
 * one 40-bit little-endian value placed at byte o of the zeroed packing
 * buffer (two word ORs). */
__device__ __forceinline__ void put_head(uint32_t sbase, uint32_t o, uint32_t b, uint32_t smask)
{
    const uint32_t q = o >> 2, s8 = (o & 3u) * 8u;
    const uint64_t v = ((uint64_t)bswap32(smask) << 8 | b) << s8; /* at most 40 + 24 bits */
    sh_or(sbase + 4u * q, (uint32_t)v);
    sh_or(sbase + 4u * q + 4u, (uint32_t)(v >> 32));
}

/* The r low bits of the 32 magnitudes m, MSB-first from byte lb (four r-bit
 * fields merged per put). */
__device__ __forceinline__ void put_low_bits(uint32_t sbase, uint32_t lb, uint32_t r, const uint32_t (&m)[32])
{
    const uint32_t p = 1u << r, mask = p - 1u;
    Packer pk;
    pk.init(sbase, lb);
#pragma unroll
    for (int j = 0; j < 32; j += 4) {
        const uint32_t v0 = m[j] & mask, v1 = m[j + 1] & mask, v2 = m[j + 2] & mask, v3 = m[j + 3] & mask;
        pk.put(((v0 * p + v1) * p + v2) * p + v3, 4u * r);
        pk.flush();
    }
    pk.finish();
}

/* encode_full for a width of 1..15 bits (B = b/8 <= 1 whole byte per
 * magnitude), the common case at the error bounds the collectives use, with
 * whole words instead of the bit packer where the layout allows: the header
 * and the four sign bytes by put_head, and for B = 1 the 32 high bytes as
 * eight little-endian words realigned to their byte offset by funnel shifts
 * (nine word ORs); the low bits go through the packer as in encode_full.
 * Same bytes as encode_full in the fastmode1 layout. */
__device__ __forceinline__ void encode_small(uint32_t sbase, uint32_t o, uint32_t b, uint32_t smask,
                                             const uint32_t (&m)[32])
{
    const uint32_t B = b >> 3, r = b & 7u;
    put_head(sbase, o, b, smask);
    const uint32_t hb = o + 5u;
    if (B) {
        const uint32_t q = hb >> 2, sh = (hb & 3u) * 8u;
        uint32_t prev = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t lo2 = __byte_perm(m[4 * k] >> r, m[4 * k + 1] >> r, 0x0040u);
            const uint32_t hi2 = __byte_perm(m[4 * k + 2] >> r, m[4 * k + 3] >> r, 0x0040u);
            const uint32_t W = __byte_perm(lo2, hi2, 0x5410u); /* bytes of elements 4k .. 4k + 3 */
            sh_or(sbase + 4u * (q + (uint32_t)k), __funnelshift_l(prev, W, sh));
            prev = W;
        }
        if (sh) sh_or(sbase + 4u * (q + 8u), prev >> (32u - sh));
    }
    if (r) put_low_bits(sbase, hb + 32u * B, r, m);
}

/* encode_full for a width of 16..23 bits (B = 2 whole bytes per magnitude):
 * the header by put_head, the 32 two-byte high parts (little-endian per
 * element) as sixteen words of two elements each, realigned to their byte
 * offset by funnel shifts (seventeen word ORs), the low bits through the
 * packer.  Same bytes as encode_full in the fastmode1 layout. */
__device__ __forceinline__ void encode_mid(uint32_t sbase, uint32_t o, uint32_t b, uint32_t smask,
                                           const uint32_t (&m)[32])
{
    const uint32_t r = b & 7u;
    put_head(sbase, o, b, smask);
    const uint32_t hb = o + 5u, q = hb >> 2, sh = (hb & 3u) * 8u;
    uint32_t prev = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const uint32_t W = __byte_perm(m[2 * k] >> r, m[2 * k + 1] >> r, 0x5410u); /* elements 2k, 2k + 1 */
        sh_or(sbase + 4u * (q + (uint32_t)k), __funnelshift_l(prev, W, sh));
        prev = W;
    }
    if (sh) sh_or(sbase + 4u * (q + 16u), prev >> (32u - sh));
    if (r) put_low_bits(sbase, hb + 64u, r, m);
}

/* The fastmode1 encoder for a full 32-element block of width b: the word
 * forms for widths 1..23, encode_full otherwise. */
__device__ __forceinline__ void encode_block32(uint32_t sbase, uint32_t o, uint32_t b, uint32_t smask,
                                               const uint32_t (&m)[32])
{
    if (__builtin_expect(b - 1u < 15u, 1))
        encode_small(sbase, o, b, smask, m);
    else if (b >= 16 && b < 24)
        encode_mid(sbase, o, b, smask, m);
    else
        encode_full(sbase, o, b, smask, m);
}

/* Bytes a .. a + 7 of the shared words w as a 64-bit big-endian value
 * (hi: bytes a .. a + 3).  Reads the three words that hold them. */
__device__ __forceinline__ void be64_at(const uint32_t *w, uint32_t a, uint32_t &hi, uint32_t &lo)
{
    const uint32_t k = a >> 2, sh = (a & 3u) * 8u;
    const uint32_t w0 = bswap32(w[k]), w1 = bswap32(w[k + 1]), w2 = bswap32(w[k + 2]);
    hi = __funnelshift_l(w1, w0, sh);
    lo = __funnelshift_l(w2, w1, sh);
}

/* prmt.b32 with a selector whose nibbles may ask for the sign of a byte
 * replicated (nibble bit 3), which __byte_perm does not offer. */
__device__ __forceinline__ uint32_t prmt_sign(uint32_t a, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(a), "r"(sel));
    return r;
}

/* Inverse of encode_full for a block of width b at byte o of the shared
 * words w: d[j] = the int32 delta of element j (as uint32).  Returns the
 * wrapped sum of the deltas.  Branch-free in the width's low part, so the
 * threads of a warp stay together whatever their blocks' widths:
 *   - the high bytes (B = b / 8 == 1, the common case) come from nine
 *     aligned words realigned by funnel shifts, one byte per element;
 *   - the r = b % 8 low bits of eight consecutive elements fill r whole
 *     bytes (byte g r on for group g), read as one big-endian window whose
 *     two 4r-bit halves give four fields each;
 *   - element j's sign (bit 31 - j of the sign word) becomes a mask by
 *     replicating the sign of byte j / 8 of the sign word shifted by j % 8.
 * Reads up to 12 bytes past the block (buffers carry slack). */
__device__ __forceinline__ uint32_t decode_full(const uint32_t *w, uint32_t o, uint32_t b,
                                                uint32_t (&d)[32], uint32_t fmt = ZG_FASTMODE1)
{
    if (b == 0) {
#pragma unroll
        for (int j = 0; j < 32; j++) d[j] = 0;
        return 0;
    }
    uint32_t B, r;
    zg_split(fmt, b, &B, &r);
    uint32_t sg, unused;
    be64_at(w, o + 1, sg, unused);
    const uint32_t hb = o + 5, lb = hb + 32u * B;
    if (B == 1) {
        const uint32_t k0 = hb >> 2, sh = (hb & 3u) * 8u;
        uint32_t prev = w[k0];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t next = w[k0 + k + 1];
            const uint32_t A = __funnelshift_r(prev, next, sh); /* bytes hb + 4k .. hb + 4k + 3 */
            prev = next;
#pragma unroll
            for (int i = 0; i < 4; i++) d[4 * k + i] = __byte_perm(A, 0, 0x4440 | i) << r;
        }
    } else if (B > 1) {
        Reader rd;
        rd.init(w, hb);
#pragma unroll
        for (int j = 0; j < 32; j++) {
            rd.refill();
            d[j] = bswap32(rd.get(8u * B) << (32u - 8u * B)) << r;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; j++) d[j] = 0;
    }
    if (r) {
        const uint32_t mask = (1u << r) - 1u;
        const uint32_t s1 = 32u - r, s2 = s1 - r, s3 = s2 - r, s4 = s3 - r; /* >= 4 */
#pragma unroll
        for (int g = 0; g < 4; g++) {
            uint32_t hi, lo;
            be64_at(w, lb + (uint32_t)g * r, hi, lo);
            const uint32_t h2 = __funnelshift_l(lo, hi, 4u * r); /* fields 4 .. 7 on top */
            d[8 * g + 0] |= (hi >> s1) & mask;
            d[8 * g + 1] |= (hi >> s2) & mask;
            d[8 * g + 2] |= (hi >> s3) & mask;
            d[8 * g + 3] |= (hi >> s4) & mask;
            d[8 * g + 4] |= (h2 >> s1) & mask;
            d[8 * g + 5] |= (h2 >> s2) & mask;
            d[8 * g + 6] |= (h2 >> s3) & mask;
            d[8 * g + 7] |= (h2 >> s4) & mask;
        }
    }
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t t = sg << k; /* element 8m + k's sign is the top bit of byte 3 - m */
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const uint32_t s = prmt_sign(t, 0x1111u * (8u | (3u - (uint32_t)m))); /* all ones when negative */
            const int j = 8 * m + k;
            d[j] = (d[j] ^ s) - s;
            sum += d[j];
        }
    }
    return sum;
}

/* decode_full for a fastmode1 block of width 0..15 (B <= 1), the same
 * instructions for every such width so that a warp whose blocks mix one- and
 * zero-byte magnitudes does not split: the high byte of element 8g + k is
 * byte k of the realigned words of group g, replaced by zero when B = 0; its
 * r low bits are field k of the group's r-byte window; the sign mask comes as
 * in decode_full.  Returns the wrapped sum of the deltas. */
__device__ __forceinline__ uint32_t decode_small(const uint32_t *w, uint32_t o, uint32_t b, uint32_t (&d)[32])
{
    if (b == 0) {
#pragma unroll
        for (int j = 0; j < 32; j++) d[j] = 0;
        return 0;
    }
    const uint32_t B = b >> 3, r = b & 7u;
    uint32_t sg, unused;
    be64_at(w, o + 1, sg, unused);
    const uint32_t hb = o + 5, lb = hb + 32u * B;
    const uint32_t k0 = hb >> 2, sh = (hb & 3u) * 8u;
    const uint32_t zsel = B ? 0u : 4u; /* selector nibble 4..7: a byte of the zero operand */
    uint32_t tk[8];
#pragma unroll
    for (int k = 0; k < 8; k++) tk[k] = sg << k; /* element 8g + k's sign: top bit of byte 3 - g */
    const uint32_t r1 = r, r2 = 2u * r, r3 = 3u * r;
    uint32_t prev = w[k0], sum = 0;
#pragma unroll
    for (int g = 0; g < 4; g++) {
        const uint32_t n1 = w[k0 + 2 * g + 1], n2 = w[k0 + 2 * g + 2];
        const uint32_t A0 = __funnelshift_r(prev, n1, sh), A1 = __funnelshift_r(n1, n2, sh);
        prev = n2;
        uint32_t hi, lo;
        be64_at(w, lb + (uint32_t)g * r, hi, lo);
        const uint32_t h2 = __funnelshift_l(lo, hi, 4u * r); /* fields 4 .. 7 on top */
        const uint32_t sel = 0x1111u * (8u | (3u - (uint32_t)g));
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t A = k < 4 ? A0 : A1;
            const uint32_t H = __byte_perm(A, 0, 0x4440u | (uint32_t)(k & 3) | zsel);
            const uint32_t src = k < 4 ? hi : h2;
            const uint32_t s1 = (k & 3) == 0 ? 0u : (k & 3) == 1 ? r1 : (k & 3) == 2 ? r2 : r3;
            const uint32_t m = __funnelshift_l(src << s1, H, r);
            const uint32_t s = prmt_sign(tk[k], sel); /* all ones when negative */
            d[8 * g + k] = (m ^ s) - s;
            sum += d[8 * g + k];
        }
    }
    return sum;
}

/* decode_full for a fastmode1 block of width 16..23 (B = 2), the form of
 * decode_small with two bytes per magnitude: group g's sixteen high bytes are
 * four realigned words, two elements each (little-endian halves); the low
 * bits and signs come as in decode_small.  ADD: d[j] += delta j (the
 * homomorphic add's accumulation, returns 0); otherwise d[j] = delta j and
 * the wrapped sum of the deltas is returned. */
template <bool ADD>
__device__ __forceinline__ uint32_t decode_mid(const uint32_t *w, uint32_t o, uint32_t b, uint32_t (&d)[32])
{
    const uint32_t r = b & 7u;
    uint32_t sg, unused;
    be64_at(w, o + 1, sg, unused);
    const uint32_t hb = o + 5, lb = hb + 64u;
    const uint32_t k0 = hb >> 2, sh = (hb & 3u) * 8u;
    uint32_t tk[8];
#pragma unroll
    for (int k = 0; k < 8; k++) tk[k] = sg << k; /* element 8g + k's sign: top bit of byte 3 - g */
    const uint32_t r1 = r, r2 = 2u * r, r3 = 3u * r;
    uint32_t prev = w[k0], sum = 0;
#pragma unroll
    for (int g = 0; g < 4; g++) {
        uint32_t A[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t nx = w[k0 + 4 * g + i + 1];
            A[i] = __funnelshift_r(prev, nx, sh); /* bytes hb + 16g + 4i .. + 3: elements 8g + 2i, 8g + 2i + 1 */
            prev = nx;
        }
        uint32_t hi, lo;
        be64_at(w, lb + (uint32_t)g * r, hi, lo);
        const uint32_t h2 = __funnelshift_l(lo, hi, 4u * r); /* fields 4 .. 7 on top */
        const uint32_t sel = 0x1111u * (8u | (3u - (uint32_t)g));
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t H = __byte_perm(A[k >> 1], 0, (k & 1) ? 0x4432u : 0x4410u);
            const uint32_t src = k < 4 ? hi : h2;
            const uint32_t s1 = (k & 3) == 0 ? 0u : (k & 3) == 1 ? r1 : (k & 3) == 2 ? r2 : r3;
            const uint32_t m = __funnelshift_l(src << s1, H, r);
            const uint32_t s = prmt_sign(tk[k], sel); /* all ones when negative */
            const uint32_t v = (m ^ s) - s;
            if (ADD) {
                d[8 * g + k] += v;
            } else {
                d[8 * g + k] = v;
                sum += v;
            }
        }
    }
    return sum;
}

/* The fastmode1 decoder for a full 32-element block of width b: the word
 * forms for widths 0..23, decode_full otherwise.  Returns the wrapped sum. */
__device__ __forceinline__ uint32_t decode_block32(const uint32_t *w, uint32_t o, uint32_t b, uint32_t (&d)[32])
{
    if (b < 16) return decode_small(w, o, b, d);
    if (b < 24) return decode_mid<false>(w, o, b, d);
    return decode_full(w, o, b, d);
}

/* The deltas of a fastmode1 block of width b at byte o added into acc
 * (acc[j] += delta j), for the homomorphic add.  Widths 1..15 take the
 * width-uniform path of decode_small, 16..23 decode_mid; 24..32 read three
 * or four whole bytes per magnitude group by group, so that no second array
 * of 32 values is live. */
__device__ __forceinline__ void decode_add_full(const uint32_t *w, uint32_t o, uint32_t b, uint32_t (&acc)[32])
{
    if (b == 0) return;
    const uint32_t B = b >> 3, r = b & 7u;
    uint32_t sg, unused;
    if (__builtin_expect(b >= 16, 0)) { /* rare at the bounds the collectives use: out of the hot path */
        if (b < 24) {
            decode_mid<true>(w, o, b, acc);
            return;
        }
        be64_at(w, o + 1, sg, unused);
        const uint32_t hb = o + 5, lb = hb + 32u * B;
        const uint32_t bmask = B >= 4 ? 0xFFFFFFFFu : (1u << (8u * B)) - 1u;
#pragma unroll
        for (int g = 0; g < 4; g++) {
            uint32_t hi = 0, lo = 0;
            be64_at(w, lb + (uint32_t)g * r, hi, lo);
            const uint32_t h2 = __funnelshift_l(lo, hi, 4u * r);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t a = hb + (uint32_t)(8 * g + k) * B; /* element 8g + k's little-endian bytes */
                const uint32_t H = __funnelshift_r(w[a >> 2], w[(a >> 2) + 1], (a & 3u) * 8u) & bmask;
                const uint32_t src = k < 4 ? hi : h2;
                const uint32_t m = __funnelshift_l(src << ((uint32_t)(k & 3) * r), H, r);
                const uint32_t s = (uint32_t)((int32_t)(sg << (8 * g + k)) >> 31); /* all ones when negative */
                acc[8 * g + k] += (m ^ s) - s;
            }
        }
        return;
    }
    be64_at(w, o + 1, sg, unused);
    const uint32_t hb = o + 5, lb = hb + 32u * B;
    const uint32_t k0 = hb >> 2, sh = (hb & 3u) * 8u;
    const uint32_t zsel = B ? 0u : 4u;
    uint32_t tk[8];
#pragma unroll
    for (int k = 0; k < 8; k++) tk[k] = sg << k;
    const uint32_t r1 = r, r2 = 2u * r, r3 = 3u * r;
    uint32_t prev = w[k0];
#pragma unroll
    for (int g = 0; g < 4; g++) {
        const uint32_t n1 = w[k0 + 2 * g + 1], n2 = w[k0 + 2 * g + 2];
        const uint32_t A0 = __funnelshift_r(prev, n1, sh), A1 = __funnelshift_r(n1, n2, sh);
        prev = n2;
        uint32_t hi, lo;
        be64_at(w, lb + (uint32_t)g * r, hi, lo);
        const uint32_t h2 = __funnelshift_l(lo, hi, 4u * r);
        const uint32_t sel = 0x1111u * (8u | (3u - (uint32_t)g));
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t A = k < 4 ? A0 : A1;
            const uint32_t H = __byte_perm(A, 0, 0x4440u | (uint32_t)(k & 3) | zsel);
            const uint32_t src = k < 4 ? hi : h2;
            const uint32_t s1 = (k & 3) == 0 ? 0u : (k & 3) == 1 ? r1 : (k & 3) == 2 ? r2 : r3;
            const uint32_t m = __funnelshift_l(src << s1, H, r);
            const uint32_t s = prmt_sign(tk[k], sel);
            acc[8 * g + k] += (m ^ s) - s;
        }
    }
}

/* Any block (n elements, any width), one element at a time: separate
 * streams for the header, the sign bits, the high bytes and the low bits.
 * Used for short tail blocks, block sizes above 32 and tiles that need the
 * exact slow quantization path.  elem(j, neg, mag) gives element j. */
template <class Elem>
__device__ __forceinline__ void encode_any(uint32_t sbase, uint32_t o, uint32_t b, uint32_t n,
                                           Elem elem, uint32_t fmt = ZG_FASTMODE1)
{
    if (b == 0) return;
    uint32_t B, r;
    zg_split(fmt, b, &B, &r);
    const uint32_t ns = (n + 7) >> 3;
    const uint32_t mask = r ? (1u << r) - 1u : 0u;
    Packer ph, ps, pb, pl;
    ph.init(sbase, o);
    ph.put(b, 8);
    ph.finish();
    ps.init(sbase, o + 1);
    pb.init(sbase, o + 1 + ns);
    pl.init(sbase, o + 1 + ns + B * n);
    for (uint32_t j = 0; j < n; j++) {
        uint32_t neg, mg;
        elem(j, neg, mg);
        ps.put(neg, 1);
        ps.flush();
        if (B) {
            pb.put(bswap32(mg >> r) >> (32u - 8u * B), 8u * B);
            pb.flush();
        }
        if (r) {
            pl.put(mg & mask, r);
            pl.flush();
        }
    }
    ps.finish();
    if (B) pb.finish();
    if (r) pl.finish();
}

/* Element-at-a-time decoder for any block; sink(j, delta). */
template <class Sink>
__device__ __forceinline__ void decode_any(const uint32_t *w, uint32_t o, uint32_t b, uint32_t n,
                                           Sink sink, uint32_t fmt = ZG_FASTMODE1)
{
    if (b == 0) {
        for (uint32_t j = 0; j < n; j++) sink(j, 0u);
        return;
    }
    uint32_t B, r;
    zg_split(fmt, b, &B, &r);
    const uint32_t ns = (n + 7) >> 3;
    Reader rs, rh, rl;
    rs.init(w, o + 1);
    rh.init(w, o + 1 + ns);
    rl.init(w, o + 1 + ns + B * n);
    for (uint32_t j = 0; j < n; j++) {
        rs.refill();
        rh.refill();
        rl.refill();
        uint32_t v = B ? bswap32(rh.get(8u * B) << (32u - 8u * B)) << r : 0u;
        if (r) v |= rl.get(r);
        if (rs.get(1)) v = 0u - v;
        sink(j, v);
    }
}

/* v[j] and v[j] += x for a runtime j, as selects and predicated adds so
 * that the register array stays in registers (short tail blocks only). */
__device__ __forceinline__ uint32_t pick(const uint32_t (&v)[32], uint32_t j)
{
    uint32_t r = v[0];
#pragma unroll
    for (int k = 1; k < 32; k++) r = (uint32_t)k == j ? v[k] : r;
    return r;
}

__device__ __forceinline__ void add_at(uint32_t (&v)[32], uint32_t j, uint32_t x)
{
#pragma unroll
    for (int k = 0; k < 32; k++)
        if ((uint32_t)k == j) v[k] += x;
}

/* Barrier `id` (1..15) over the first n threads of the CTA (a multiple of
 * 32), for kernels whose warps split into groups; id 0 is __syncthreads. */
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

/* ---------------------------------------------------------------------
 * TMA (cp.async.bulk) global -> shared, completion on an mbarrier
 * ------------------------------------------------------------------- */

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

/* One arrival on a barrier (release at CTA scope: the caller's earlier
 * shared-memory writes are visible to whoever sees the phase complete). */
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

/* `n` arrivals at once (release at CTA scope). */
__device__ __forceinline__ void mbar_arrive_n(uint64_t *bar, uint32_t n)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(n) : "memory");
}

/* Wait for phase `parity` of the barrier to complete.  Gives up after about
 * 2^32 SM clock cycles (two seconds or more) and reports ZERR_TIMEOUT
 * instead of hanging; a wait that spans other stages of a pipeline (which
 * may themselves wait on other CTAs) stays well inside that limit. */
__device__ __forceinline__ void mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *err)
{
    uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    for (uint32_t it = 0; it < (1u << 30); it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return;
        if (clock64() - t0 > (1ll << 32)) break;
    }
    atomicOr(err, ZERR_TIMEOUT);
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(sdst)),
        "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

/* Shared stores by address (a swizzled layout computes its own). */
__device__ __forceinline__ void st_shared_v4(uint32_t sa, float x, float y, float z, float w)
{
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(sa), "f"(x), "f"(y), "f"(z), "f"(w)
                 : "memory");
}
__device__ __forceinline__ void st_shared_f32(uint32_t sa, float x)
{
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(sa), "f"(x) : "memory");
}

__device__ __forceinline__ float4 ld_shared_v4(uint32_t sa)
{
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(sa)
                 : "memory");
    return v;
}
__device__ __forceinline__ float ld_shared_f32(uint32_t sa)
{
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(sa) : "memory");
    return v;
}

/* TMA tensor load of the box at (c0, c1) of a 2-D map into shared memory,
 * completing on the mbarrier (whose byte count the caller arms). */
__device__ __forceinline__ void tma_load_2d(uint32_t sa, const void *map, int32_t c0, int32_t c1, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(sa),
        "l"((uint64_t)(uintptr_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

/* TMA tensor store of the box at (c0, c1) of a 2-D map from shared memory,
 * in the issuing thread's bulk group.  The writers of the shared box run
 * fence_proxy_async_smem() and a barrier before it. */
__device__ __forceinline__ void tma_store_2d(const void *map, uint32_t sa, int32_t c0, int32_t c1)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     (uint64_t)(uintptr_t)map),
                 "r"(sa), "r"(c0), "r"(c1)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
/* The issuing thread's bulk stores have read their shared source (the
 * buffer may be written again) / have completed. */
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

/* Thread 0 only: TMA bulk copy of the 16-byte-aligned superset
 * [floor16(g), ceil16(g + nbytes)) into the 16-byte-aligned buffer s, arming
 * the barrier with its byte count.  The superset only adds bytes of 16-byte
 * chunks that already contain bytes of the range, so it never touches a page
 * the range does not.  The range starts at s + (g & 15). */
__device__ __forceinline__ void tma_load_superset(uint8_t *s, const uint8_t *g, uint32_t nbytes,
                                                  uint64_t *bar)
{
    uintptr_t a0 = (uintptr_t)g & ~(uintptr_t)15u;
    uintptr_t a1 = ((uintptr_t)g + nbytes + 15u) & ~(uintptr_t)15u;
    fence_proxy_async_smem(); /* earlier generic accesses of s before the async write */
    mbar_expect_tx(bar, (uint32_t)(a1 - a0));
    if (a1 > a0) bulk_g2s(s, (const void *)a0, (uint32_t)(a1 - a0), bar);
}

/* Write shared bytes s[0, nbytes) to global [g, g + nbytes) for any
 * alignment of g.  16-byte-aligned global chunks get one vector store each,
 * assembled from two aligned shared loads and funnel shifts; the ragged
 * ends (shared with neighbouring tiles) are stored byte by byte.  s must be
 * 16-byte aligned with 32 readable bytes of slack.  Called by all threads. */
__device__ __forceinline__ void store_realign(uint8_t *g, const uint8_t *s, uint32_t nbytes, uint32_t tid,
                                              uint32_t nt)
{
    const uintptr_t g0 = (uintptr_t)g, g1 = g0 + nbytes;
    const uintptr_t a0 = (g0 + 15u) & ~(uintptr_t)15u, a1 = g1 & ~(uintptr_t)15u;
    if (a1 <= a0) {
        for (uint32_t i = tid; i < nbytes; i += nt) g[i] = s[i];
        return;
    }
    const uint32_t d = (uint32_t)(a0 - g0); /* shared offset of the first aligned chunk */
    const uint32_t tail = (uint32_t)(g1 - a1);
    for (uint32_t i = tid; i < d + tail; i += nt) { /* ragged ends, any thread count */
        const uint32_t k = i < d ? i : (uint32_t)(a1 - g0) + (i - d);
        g[k] = s[k];
    }
    const uint32_t nch = (uint32_t)((a1 - a0) >> 4), q = d >> 2, sh = (d & 3u) * 8u;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(s);
    uint4 *g4 = reinterpret_cast<uint4 *>(a0);
    for (uint32_t c = tid; c < nch; c += nt) {
        uint4 lo = s4[c], hi = s4[c + 1];
        uint32_t o0, o1, o2, o3, o4;
        /* q is the same for every thread of the tile: a uniform branch */
        switch (q) {
        case 0: o0 = lo.x; o1 = lo.y; o2 = lo.z; o3 = lo.w; o4 = hi.x; break;
        case 1: o0 = lo.y; o1 = lo.z; o2 = lo.w; o3 = hi.x; o4 = hi.y; break;
        case 2: o0 = lo.z; o1 = lo.w; o2 = hi.x; o3 = hi.y; o4 = hi.z; break;
        default: o0 = lo.w; o1 = hi.x; o2 = hi.y; o3 = hi.z; o4 = hi.w; break;
        }
        uint4 v;
        v.x = __funnelshift_r(o0, o1, sh);
        v.y = __funnelshift_r(o1, o2, sh);
        v.z = __funnelshift_r(o2, o3, sh);
        v.w = __funnelshift_r(o3, o4, sh);
        g4[c] = v;
    }
}

__device__ __forceinline__ void store_realign(uint8_t *g, const uint8_t *s, uint32_t nbytes)
{
    store_realign(g, s, nbytes, threadIdx.x, blockDim.x);
}

/* ---------------------------------------------------------------------
 * Block-wide exclusive scans (blockDim.x <= 1024, multiple of 32).
 * `wsum` is shared scratch of 33 words.
 * ------------------------------------------------------------------- */
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
    uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

/* Exclusive scan of v over the first n threads of the CTA, synchronised
 * on barrier `id` (wrapping uint32 add, so it also serves int32 sums);
 * *total receives the sum of all v. */
__device__ __forceinline__ uint32_t grp_excl_scan(uint32_t v, uint32_t *wsum, uint32_t *total, uint32_t n,
                                                  uint32_t id)
{
    uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = n >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) wsum[warp] = inc;
    named_sync(id, n);
    if (warp == 0) {
        uint32_t t = lane < nw ? wsum[lane] : 0u;
        uint32_t ti = warp_incl_scan(t);
        if (lane < nw) wsum[lane] = ti - t;
        if (lane == 31) wsum[32] = ti;
    }
    named_sync(id, n);
    uint32_t r = wsum[warp] + inc - v;
    *total = wsum[32];
    named_sync(id, n);
    return r;
}

/* The same with one barrier: every warp reads all warp sums.  Callers
 * alternate between two scratch arrays on consecutive calls, so that a
 * warp's next write cannot overtake a slower warp's read. */
__device__ __forceinline__ uint32_t grp_excl_scan1(uint32_t v, uint32_t *ws, uint32_t *total, uint32_t n,
                                                   uint32_t id)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = n >> 5;
    const uint32_t inc = warp_incl_scan(v);
    if (lane == 31) ws[warp] = inc;
    named_sync(id, n);
    const uint32_t t = lane < nw ? ws[lane] : 0u;
    *total = __reduce_add_sync(0xffffffffu, t);
    return __reduce_add_sync(0xffffffffu, lane < warp ? t : 0u) + inc - v;
}

/* Two exclusive scans at once (v0 with scratch ws0, v1 with ws1, 33 words
 * each) over the first n threads, with one barrier: every warp reads all
 * warp sums.  Callers alternate between two pairs of scratch arrays on
 * consecutive calls, as for grp_excl_scan1. */
__device__ __forceinline__ void grp_excl_scan2_1(uint32_t v0, uint32_t v1, uint32_t *ws0, uint32_t *ws1,
                                                 uint32_t &r0, uint32_t &r1, uint32_t &t0, uint32_t &t1,
                                                 uint32_t n, uint32_t id)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = n >> 5;
    const uint32_t i0 = warp_incl_scan(v0), i1 = warp_incl_scan(v1);
    if (lane == 31) {
        ws0[warp] = i0;
        ws1[warp] = i1;
    }
    named_sync(id, n);
    const uint32_t a = lane < nw ? ws0[lane] : 0u, b = lane < nw ? ws1[lane] : 0u;
    t0 = __reduce_add_sync(0xffffffffu, a);
    t1 = __reduce_add_sync(0xffffffffu, b);
    r0 = __reduce_add_sync(0xffffffffu, lane < warp ? a : 0u) + i0 - v0;
    r1 = __reduce_add_sync(0xffffffffu, lane < warp ? b : 0u) + i1 - v1;
}

/* The same over the whole CTA. */
__device__ __forceinline__ uint32_t cta_excl_scan(uint32_t v, uint32_t *wsum, uint32_t *total)
{
    return grp_excl_scan(v, wsum, total, blockDim.x, 0);
}

/* ---------------------------------------------------------------------
 * Decoupled look-back (Merrill & Garland 2016).  status[t] packs a 2-bit
 * flag (1 = aggregate of tile t only, 2 = inclusive prefix through t) over
 * a 62-bit value; values add modulo 2^62.  Tiles are taken in ticket order,
 * so every tile a CTA waits on belongs to a CTA that is already running and
 * never waits on a later tile.
 * ------------------------------------------------------------------- */
/* Polls of a predecessor's word before the look-back gives up (about a
 * second at the 32 ns back-off; callers may pass a smaller limit). */
#define LB_SPIN_LIMIT (1u << 22)
#define LB_FLAG_A (1ull << 62)
#define LB_FLAG_P (2ull << 62)
#define LB_VAL (LB_FLAG_A - 1ull)

/* A status word carries its flag and its value together, and a reader
 * uses nothing else that the writer produced, so relaxed device-scope
 * accesses suffice: no acquire (which would keep a lane's eight loads from
 * overlapping) and no release (which would hold the store until the
 * thread's earlier output stores complete). */
__device__ __forceinline__ void st_flag(uint64_t *p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t ld_flag(const uint64_t *p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* Any lane of the publishing warp may call it; lane 0 stores: this tile's
 * aggregate, or, for a first tile (no predecessor in its scan), its
 * inclusive value start + agg. */
__device__ __forceinline__ void lb_publish(uint64_t *status, uint64_t tile, uint64_t agg, bool first,
                                           uint64_t start)
{
    if ((threadIdx.x & 31u) == 0)
        st_flag(status + tile, first ? (LB_FLAG_P | ((start + agg) & LB_VAL))
                                        : (LB_FLAG_A | (agg & LB_VAL)));
}

/* Called by all lanes of one warp after lb_publish: returns the exclusive
 * prefix of the tile (the sum of every tile back to and including the
 * nearest one that published an inclusive value, or `start` for a first
 * tile) and publishes the tile's inclusive value.  Each round inspects 256
 * predecessors (lane l reads tiles pos - l - 32k, k < 8, all loads in flight
 * together): with a persistent grid several hundred tiles are in flight at
 * once, and the nearest inclusive value is typically that far back.  A
 * predecessor that never publishes makes the wait give up after a bounded
 * number of polls: ZERR_TIMEOUT is set, the missing value counts as 0 and
 * the inclusive value is still published, so successors never hang. */
static __device__ __noinline__ uint64_t lb_resolve(uint64_t *status, uint64_t tile, uint64_t agg,
                                                   bool first, uint64_t start, uint32_t *err,
                                                   uint32_t spin_limit = LB_SPIN_LIMIT)
{
    const uint32_t lane = threadIdx.x & 31u;
    if (first) return start;
    uint64_t prefix = 0;
    int64_t pos = (int64_t)tile - 1;
    uint32_t spins = 0;
    for (;;) {
        uint64_t v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int64_t idx = pos - (int64_t)(lane + 32u * k);
            v[k] = idx >= 0 ? ld_flag(status + idx) : LB_FLAG_P; /* before tile 0: value 0 */
        }
        /* nearest inclusive value: smallest distance lane + 32k flagged P */
        uint32_t kp = 8, fp = 31, pending = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t flag = (uint32_t)(v[k] >> 62);
            const uint32_t pm = __ballot_sync(0xffffffffu, flag == 2u);
            const uint32_t xm = __ballot_sync(0xffffffffu, flag == 0u);
            if (kp == 8) {
                if (pm) {
                    kp = k;
                    fp = (uint32_t)(__ffs(pm) - 1);
                    pending |= xm & ((1u << fp) - 1u);
                } else {
                    pending |= xm;
                }
            }
        }
        if (pending) {
            if (++spins < spin_limit) {
                __nanosleep(32);
                continue;
            }
            /* give up: missing values count as 0 */
            if (lane == 0) atomicOr(err, ZERR_TIMEOUT);
        }
        uint64_t c = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const bool ready = (v[k] >> 62) != 0;
            if ((uint32_t)k < kp || ((uint32_t)k == kp && lane <= fp))
                c += ready ? (v[k] & LB_VAL) : 0ull;
        }
        prefix += warp_sum_u64(c);
        if (kp < 8) break;
        pos -= 256;
        spins = 0;
    }
    if (lane == 0) st_flag(status + tile, LB_FLAG_P | ((prefix + agg) & LB_VAL));
    return prefix & LB_VAL;
}

#endif
