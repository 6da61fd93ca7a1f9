/*
 * zk_szp3d.cu -- the SZp 3-D Lorenzo codec, serial stream form.
 *
 * Replaces SZp_compress3D_fast / SZp_compress3D (ZCCL/src/ZCCL_float.c:1706-1860)
 * and SZp_decompress3D (ZCCL/src/ZCCLd_float.c:2801-2871) and produces the
 * same bytes and floats.  The reference walks the volume block by block and
 * carries its Lorenzo state from block to block; the quantity it encodes is
 * the 3-D mixed difference of the quantized values with zeros outside the
 * volume (ZCCL_float.h:63-73), which every element can form on its own, and
 * its inverse is the 3-D prefix sum.  So here every step is data parallel:
 *
 * quantization  q = (int)floor((double)x * (0.5 / eb) + 0.5) (ZCCL_float.h:57-61)
 *                with the reference's double rounding: float pairs where that
 *                is provably the same, FP64 for the rest;
 * compress   K1  the rate of every block (the bit length of its largest
 *                difference magnitude) into the rate table at the stream's
 *                start, and its payload size;
 *            K2  an exclusive scan of the payload sizes (three kernels);
 *            K3  every block packed at its offset: sign bits, then B =
 *                rate/8 high bytes per element, then the r = rate%8 low bits
 *                (the fastmode1 packers' layout,
 *                ZCCL/src/ZCCL_TypeManager.c:12-91,824-848);
 * decompress K1  payload sizes from the rate table, K2 the same scan,
 *            K3  every block's differences into the output buffer, viewed
 *                as int32;
 *            K4-K6 inclusive prefix sums along z (a warp per row), y and x
 *                (a thread per column, rows loaded in batches), the last one
 *                writing (float)((double)q * (2 eb)) in place
 *                (ZCCLd_float.c:2855-2857).
 * Block sides 2, 4 and 8 (row-mapped kernels): a warp takes a run of 32 / bs
 * blocks along z and walks their rows, coalesced, with the neighbours in
 * registers; compress is one pass (K1-K3 together, quantizing as it loads,
 * the run's place in the stream by decoupled look-back; no quantized
 * volume); decompress K3 stages each run's bytes in shared memory and
 * writes whole rows.  Other block sides: a quantized volume, then
 * a warp (up to 512 elements) or a CTA per block.
 * Integer sums wrap modulo 2^32 like the reference's int.
 */
#include "zkern.cuh"

namespace {

constexpr uint32_t SZ_THREADS = 256;
constexpr uint32_t SZ_CHUNK = 2048; /* sizes per CTA in the scan */
constexpr uint32_t SZ_SCAN_BATCH = 8; /* rows loaded together in the y and x prefix sums */

struct Sz3Dims {
    uint64_t d1, d2, d3;
    uint32_t bs;
    uint64_t nb1, nb2, nb3, nblocks;
};

__host__ __device__ inline Sz3Dims sz3_dims(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t bs)
{
    Sz3Dims g;
    g.d1 = d1;
    g.d2 = d2;
    g.d3 = d3;
    g.bs = bs;
    g.nb1 = (d1 - 1) / bs + 1;
    g.nb2 = (d2 - 1) / bs + 1;
    g.nb3 = (d3 - 1) / bs + 1;
    g.nblocks = g.nb1 * g.nb2 * g.nb3;
    return g;
}

/* Block b's first element and extent on each axis. */
struct Sz3Block {
    uint64_t x0, y0, z0;
    uint32_t sx, sy, sz, n;
};

__device__ __forceinline__ Sz3Block sz3_block(const Sz3Dims &g, uint64_t b)
{
    Sz3Block k;
    const uint64_t bz = b % g.nb3, by = (b / g.nb3) % g.nb2, bx = b / (g.nb3 * g.nb2);
    k.x0 = bx * g.bs;
    k.y0 = by * g.bs;
    k.z0 = bz * g.bs;
    k.sx = (uint32_t)min((uint64_t)g.bs, g.d1 - k.x0);
    k.sy = (uint32_t)min((uint64_t)g.bs, g.d2 - k.y0);
    k.sz = (uint32_t)min((uint64_t)g.bs, g.d3 - k.z0);
    k.n = k.sx * k.sy * k.sz;
    return k;
}

/* Payload bytes of a block of n elements at rate b (0 for rate 0). */
__host__ __device__ inline uint32_t sz3_payload(uint32_t b, uint32_t n)
{
    if (!b) return 0;
    return (n + 7) / 8 + (b >> 3) * n + ((b & 7u) * n + 7) / 8;
}

/* A double as a pair of floats, hi = RN(d), lo = RN(d - hi), so that
 * hi + lo is within 2^-48 of d; ok only where both are normal floats
 * (2^-90 <= d <= 2^90), else the kernels take the double steps. */
struct Sz3Split {
    double d;
    float hi, lo;
    int ok;
};

Sz3Split sz3_split(double d)
{
    Sz3Split s;
    s.d = d;
    s.hi = (float)d;
    s.lo = (float)(d - (double)s.hi);
    s.ok = d >= 0x1p-90 && d <= 0x1p90;
    return s;
}

/* (int)floor((double)x * inv + 0.5), each step rounded as double
 * arithmetic rounds it (ZCCL_float.h:57-61).  FP64 is slow on this GPU, so
 * small products take one FMA (below); larger ones are first formed as a
 * float pair: hi = x*ih, its exact error
 * by FMA, plus x*il, within 2^-19 of x*inv + 0.5 when |x*ih| < 2^26.  When
 * the fractional part of that sum is more than 2^-12 from an integer, no
 * rounding of the exact product (at most 2^-27 here) can move it across
 * one, so its floor is the reference's; otherwise (about one element in
 * two thousand, or out of range, or not finite) the double steps run as
 * they are.  *bad is set where the reference is undefined. */
__device__ __forceinline__ int32_t sz3_quantize(float x, const Sz3Split &inv, uint32_t &bad)
{
    /* Below 2^11 one FMA suffices: x * ih + 0.5 rounded once is within
     * 2^-12.4 of x * inv + 0.5 (x * il and half an ulp), so a fraction more
     * than 2^-12 from an integer floors like the exact value. */
    const float t1 = __fmaf_rn(x, inv.hi, 0.5f);
    if (inv.ok && fabsf(t1) < 2048.0f) { /* NaN fails */
        const float n1 = floorf(t1), f1 = __fsub_rn(t1, n1);
        if (f1 > 2.44140625e-4f && f1 < 0.999755859375f) return (int32_t)n1;
    }
    const float th = __fmul_rn(x, inv.hi);
    if (inv.ok && fabsf(th) < 67108864.0f) { /* 2^26; NaN takes the double path */
        const float tl = __fmaf_rn(x, inv.lo, __fmaf_rn(x, inv.hi, -th));
        const float s = __fadd_rn(th, 0.5f); /* th + 0.5 = s + e exactly (TwoSum) */
        const float bb = __fsub_rn(s, th);
        const float e = __fadd_rn(__fsub_rn(th, __fsub_rn(s, bb)), __fsub_rn(0.5f, bb));
        const float n = floorf(s);
        float fr = __fadd_rn(__fsub_rn(s, n), __fadd_rn(e, tl));
        const float m = floorf(fr);
        fr = __fsub_rn(fr, m);
        if (fr > 2.44140625e-4f && fr < 0.999755859375f) return (int32_t)n + (int32_t)m;
    }
    const double v = floor(__dadd_rn(__dmul_rn((double)x, inv.d), 0.5));
    if (!(v >= -2147483648.0 && v < 2147483648.0)) { /* not finite, or outside int: undefined in the reference */
        bad = 1;
        return 0;
    }
    return (int32_t)v;
}

/* (float)((double)q * twice) (ZCCLd_float.c:2857): with the product as a
 * float pair (within 2^-22 of an ulp of the result for |q| < 2^24), its
 * nearest float is the reference's unless the pair lies within 2^-18 of
 * half an ulp from it (a midpoint the double rounding could decide) or the
 * result is a power of two or tiny; those take the double steps. */
__device__ __forceinline__ float sz3_value(int32_t q, const Sz3Split &tw)
{
    if (tw.ok && q == 0) return 0.0f;
    if (tw.ok && q > -16777216 && q < 16777216) {
        const float qf = (float)q;
        const float hi = __fmul_rn(qf, tw.hi);
        const float lo = __fmaf_rn(qf, tw.lo, __fmaf_rn(qf, tw.hi, -hi));
        const float r = __fadd_rn(hi, lo);
        const uint32_t rb = __float_as_uint(r) & 0x7FFFFFFFu, ex = rb >> 23;
        if (ex > 24u && ex < 254u && (rb & 0x7FFFFFu) != 0u) {
            const float half = __uint_as_float((ex - 24u) << 23); /* half an ulp of r */
            const float d = __fadd_rn(__fsub_rn(hi, r), lo);      /* (hi + lo) - r */
            if (fabsf(d) < __fmul_rn(half, 0.999996185302734375f)) return r; /* 1 - 2^-18 */
        }
    }
    return (float)__dmul_rn((double)q, tw.d);
}

/* ---- K0: quantization -------------------------------------------------- */
__global__ void k_sz3_quant(const float *__restrict__ x, int32_t *__restrict__ q, uint64_t n, Sz3Split inv,
                            uint32_t *err)
{
    uint32_t bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        q[i] = sz3_quantize(x[i], inv, bad);
    if (bad) atomicOr(err, ZERR_RANGE);
}

/* The mixed difference at (i, j, k), zeros outside the volume. */
__device__ __forceinline__ uint32_t sz3_diff(const int32_t *q, const Sz3Dims &g, uint64_t i, uint64_t j, uint64_t k)
{
    const uint64_t s0 = g.d2 * g.d3, s1 = g.d3, p = i * s0 + j * s1 + k;
    auto at = [&](bool ok, uint64_t o) -> uint32_t { return ok ? (uint32_t)q[o] : 0u; };
    const bool bi = i > 0, bj = j > 0, bk = k > 0;
    return at(true, p) - at(bk, p - 1) - at(bj, p - s1) + at(bj && bk, p - s1 - 1) - at(bi, p - s0) +
           at(bi && bk, p - s0 - 1) + at(bi && bj, p - s0 - s1) - at(bi && bj && bk, p - s0 - s1 - 1);
}

/* Element t of a block (i slowest, k fastest), as in the reference. */
__device__ __forceinline__ void sz3_elem(const Sz3Block &k, uint32_t t, uint64_t &i, uint64_t &j, uint64_t &z)
{
    const uint32_t kz = t % k.sz, jy = (t / k.sz) % k.sy, ix = t / (k.sz * k.sy);
    i = k.x0 + ix;
    j = k.y0 + jy;
    z = k.z0 + kz;
}

__device__ __forceinline__ uint32_t mag(uint32_t v) { return (int32_t)v < 0 ? 0u - v : v; }

/* Blocks go to groups of G threads: a warp per block (G = 32) up to
 * 512 elements, the whole CTA (G = SZ_THREADS) above. */
template <uint32_t G>
__device__ __forceinline__ void group_sync()
{
    if (G == 32)
        __syncwarp();
    else
        __syncthreads();
}

/* ---- K1: rates and payload sizes (a group per block) -------------------- */
template <uint32_t G>
__global__ void __launch_bounds__(SZ_THREADS) k_sz3_rates(const int32_t *q, Sz3Dims g, uint8_t *out, uint32_t *sizes)
{
    __shared__ uint32_t wmax[SZ_THREADS / 32];
    const uint32_t per = SZ_THREADS / G, sub = threadIdx.x / G, gt = threadIdx.x % G;
    for (uint64_t b0 = (uint64_t)blockIdx.x * per; b0 < g.nblocks; b0 += (uint64_t)gridDim.x * per) {
        const uint64_t b = b0 + sub;
        const bool live = b < g.nblocks; /* uniform over the group */
        uint32_t m = 0;
        Sz3Block k = {};
        if (live) {
            k = sz3_block(g, b);
            for (uint32_t t = gt; t < k.n; t += G) {
                uint64_t i, j, z;
                sz3_elem(k, t, i, j, z);
                m = max(m, mag(sz3_diff(q, g, i, j, z)));
            }
        }
        m = __reduce_max_sync(0xffffffffu, m);
        if (G == 32) {
            if (live && gt == 0) {
                const uint32_t rate = 32u - __clz(m);
                out[b] = (uint8_t)rate;
                sizes[b] = sz3_payload(rate, k.n);
            }
        } else {
            if ((threadIdx.x & 31u) == 0) wmax[threadIdx.x >> 5] = m;
            __syncthreads();
            if (threadIdx.x == 0 && live) {
                for (uint32_t w = 0; w < blockDim.x / 32; w++) m = max(m, wmax[w]);
                const uint32_t rate = 32u - __clz(m);
                out[b] = (uint8_t)rate;
                sizes[b] = sz3_payload(rate, k.n);
            }
            __syncthreads();
        }
    }
}

/* ---- decompress K1: payload sizes from the rate table ------------------- */
__global__ void k_sz3_sizes(const uint8_t *in, uint64_t avail, Sz3Dims g, uint32_t *sizes, uint32_t *err)
{
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < g.nblocks; b += (uint64_t)gridDim.x * blockDim.x) {
        if (b >= avail) {
            atomicOr(err, ZERR_BOUNDS);
            sizes[b] = 0;
            continue;
        }
        const uint32_t rate = in[b];
        if (rate > 32) atomicOr(err, ZERR_CORRUPT);
        const Sz3Block k = sz3_block(g, b);
        sizes[b] = rate > 32 ? 0 : sz3_payload(rate, k.n);
    }
}

/* ---- K2: exclusive scan of the sizes into 64-bit offsets ---------------- */
__global__ void __launch_bounds__(1024) k_sz3_chunk_sums(const uint32_t *sizes, uint64_t nb, uint64_t *sums)
{
    __shared__ uint64_t ws[32];
    const uint64_t c = blockIdx.x, lo = c * SZ_CHUNK;
    uint64_t s = 0;
    for (uint64_t i = lo + threadIdx.x; i < nb && i < lo + SZ_CHUNK; i += blockDim.x) s += sizes[i];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31u) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; w++) t += ws[w];
        sums[c] = t;
    }
}

/* One CTA: exclusive scan of the chunk sums in place; *total = all bytes. */
__global__ void __launch_bounds__(1024) k_sz3_scan_sums(uint64_t *sums, uint64_t nchunks, uint64_t head, uint64_t *total)
{
    __shared__ uint64_t ws[33];
    uint64_t carry = 0;
    for (uint64_t c0 = 0; c0 < nchunks; c0 += blockDim.x) {
        const uint64_t c = c0 + threadIdx.x;
        const uint64_t v = c < nchunks ? sums[c] : 0;
        uint64_t inc = v;
        const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (uint32_t)o) inc += u;
        }
        if (lane == 31) ws[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const uint64_t t = lane < blockDim.x / 32 ? ws[lane] : 0;
            uint64_t ti = t;
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t u = __shfl_up_sync(0xffffffffu, ti, o);
                if (lane >= (uint32_t)o) ti += u;
            }
            ws[lane] = ti - t;
            if (lane == 31) ws[32] = ti;
        }
        __syncthreads();
        if (c < nchunks) sums[c] = carry + ws[warp] + inc - v;
        carry += ws[32];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = head + carry;
}

__global__ void __launch_bounds__(1024) k_sz3_offsets(const uint32_t *sizes, uint64_t nb, const uint64_t *sums,
                                                      uint64_t *offs)
{
    __shared__ uint64_t ws[33];
    const uint64_t c = blockIdx.x, lo = c * SZ_CHUNK;
    const uint32_t per = SZ_CHUNK / blockDim.x; /* consecutive sizes per thread */
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint64_t v[SZ_CHUNK / 1024 > 0 ? SZ_CHUNK / 1024 : 1];
    uint64_t s = 0;
    for (uint32_t r = 0; r < per; r++) {
        const uint64_t i = lo + (uint64_t)threadIdx.x * per + r;
        v[r] = i < nb ? sizes[i] : 0;
        s += v[r];
    }
    uint64_t inc = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += u;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint64_t t = lane < blockDim.x / 32 ? ws[lane] : 0;
        uint64_t ti = t;
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= (uint32_t)o) ti += u;
        }
        ws[lane] = ti - t;
    }
    __syncthreads();
    uint64_t run = sums[c] + ws[warp] + inc - s;
    for (uint32_t r = 0; r < per; r++) {
        const uint64_t i = lo + (uint64_t)threadIdx.x * per + r;
        if (i < nb) offs[i] = run;
        run += v[r];
    }
}

/* One block's n differences e[] (element order) packed at o with rate
 * `rate` > 0: sign bits (bit 7 - t % 8 of byte t / 8), B = rate/8 high
 * bytes per element (little-endian), then the r = rate%8 low bits, eight
 * elements to r bytes, MSB first; every byte by one of G threads (gt). */
template <uint32_t G>
__device__ __forceinline__ void sz3_pack_block(const uint32_t *e, uint32_t n, uint32_t rate, uint8_t *o, uint32_t gt)
{
    const uint32_t B = rate >> 3, r = rate & 7u, ns = (n + 7) / 8;
    for (uint32_t c = gt; c < ns; c += G) {
        uint32_t v = 0;
        for (uint32_t u = 0; u < 8 && 8 * c + u < n; u++) v |= ((e[8 * c + u] >> 31) & 1u) << (7 - u);
        o[c] = (uint8_t)v;
    }
    uint8_t *h = o + ns;
    if (B == 1) {
        for (uint32_t t = gt; t < n; t += G) h[t] = (uint8_t)(mag(e[t]) >> r);
    } else {
        for (uint32_t c = gt; c < B * n; c += G) {
            const uint32_t t = c / B, byte = c % B;
            h[c] = (uint8_t)((mag(e[t]) >> r) >> (8 * byte));
        }
    }
    if (r) {
        uint8_t *l = h + B * n;
        const uint32_t mask = (1u << r) - 1u, ng = (n + 7) / 8, tail = (r * n + 7) / 8;
        for (uint32_t gi = gt; gi < ng; gi += G) {
            uint64_t acc = 0;
            for (uint32_t u = 0; u < 8; u++) {
                const uint32_t t = 8 * gi + u;
                acc = (acc << r) | (t < n ? (mag(e[t]) & mask) : 0u);
            }
            for (uint32_t m = 0; m < r; m++) {
                const uint32_t at = gi * r + m;
                if (at < tail) l[at] = (uint8_t)(acc >> (8 * (r - 1 - m)));
            }
        }
    }
}

/* Element t of a block packed at `sg` with rate <= 32 (0: all zero). */
__device__ __forceinline__ uint32_t sz3_unpack_elem(const uint8_t *sg, uint32_t rate, uint32_t n, uint32_t t)
{
    if (!rate) return 0u;
    const uint32_t B = rate >> 3, r = rate & 7u, ns = (n + 7) / 8;
    const uint8_t *h = sg + ns, *l = h + B * n;
    uint32_t v = 0;
    for (uint32_t byte = 0; byte < B; byte++) v |= (uint32_t)h[t * B + byte] << (8 * byte);
    v <<= r;
    if (r) { /* bits [t r, t r + r) of the low section, MSB first */
        const uint64_t bit = (uint64_t)t * r;
        const uint64_t by = bit >> 3;
        const uint32_t w = ((uint32_t)l[by] << 8) | (by + 1 < (r * (uint64_t)n + 7) / 8 ? l[by + 1] : 0u);
        v |= (w >> (16 - (uint32_t)(bit & 7u) - r)) & ((1u << r) - 1u);
    }
    if ((sg[t >> 3] >> (7 - (t & 7u))) & 1u) v = 0u - v;
    return v;
}

/* ---- compress K3: pack every block at its offset (a group per block) ---- */
template <uint32_t G>
__global__ void __launch_bounds__(SZ_THREADS) k_sz3_pack(const int32_t *q, Sz3Dims g, uint8_t *out, uint64_t cap,
                                                         const uint64_t *offs, uint32_t *err)
{
    extern __shared__ uint32_t e_all[]; /* bs^3 differences per group */
    const uint32_t per = SZ_THREADS / G, sub = threadIdx.x / G, gt = threadIdx.x % G;
    uint32_t *e = e_all + sub * (g.bs * g.bs * g.bs);
    for (uint64_t b0 = (uint64_t)blockIdx.x * per; b0 < g.nblocks; b0 += (uint64_t)gridDim.x * per) {
        const uint64_t b = b0 + sub;
        /* every exit below is uniform over the group; a CTA-wide group meets
         * its barriers in every case */
        uint32_t rate = b < g.nblocks ? out[b] : 0u;
        const Sz3Block k = rate ? sz3_block(g, b) : Sz3Block{};
        const uint32_t n = k.n;
        const uint64_t base = rate ? g.nblocks + offs[b] : 0;
        if (rate && base + sz3_payload(rate, n) > cap) {
            if (gt == 0) atomicOr(err, ZERR_CAPACITY);
            rate = 0;
        }
        if (rate) {
            for (uint32_t t = gt; t < n; t += G) {
                uint64_t i, j, z;
                sz3_elem(k, t, i, j, z);
                e[t] = sz3_diff(q, g, i, j, z);
            }
        }
        group_sync<G>();
        if (rate) sz3_pack_block<G>(e, n, rate, out + base, gt);
        group_sync<G>();
    }
}

/* ---- decompress K3: every block's differences into the volume (a group per block) */
template <uint32_t G>
__global__ void __launch_bounds__(SZ_THREADS) k_sz3_unpack(const uint8_t *in, uint64_t avail, Sz3Dims g,
                                                           const uint64_t *offs, uint32_t *vol, uint32_t *err)
{
    const uint64_t s0 = g.d2 * g.d3, s1 = g.d3;
    const uint32_t per = SZ_THREADS / G, sub = threadIdx.x / G, gt = threadIdx.x % G;
    for (uint64_t b0 = (uint64_t)blockIdx.x * per; b0 < g.nblocks; b0 += (uint64_t)gridDim.x * per) {
        const uint64_t b = b0 + sub;
        if (b >= g.nblocks) continue; /* no barrier below */
        const Sz3Block k = sz3_block(g, b);
        uint32_t rate = b < avail ? in[b] : 0u;
        const uint64_t base = g.nblocks + offs[b];
        const uint32_t n = k.n;
        if (rate > 32 || base + sz3_payload(rate, n) > avail) { /* uniform over the CTA */
            if (gt == 0) atomicOr(err, rate > 32 ? ZERR_CORRUPT : ZERR_BOUNDS);
            rate = 0;
        }
        const uint8_t *sg = in + base;
        for (uint32_t t = gt; t < n; t += G) {
            const uint32_t v = sz3_unpack_elem(sg, rate, n, t);
            uint64_t i, j, z;
            sz3_elem(k, t, i, j, z);
            vol[i * s0 + j * s1 + z] = v;
        }
    }
}

/* ---- block sides 2, 4 and 8: row-mapped kernels -------------------------
 * A warp takes a unit of U = 32 / BS consecutive blocks along z with the
 * same block row and plane: lane l owns z = z0 + l, in block l / BS.  It
 * walks the unit's rows plane by plane, row by row (the order of the
 * elements in a block), loads each row of x once, coalesced, quantizes it
 * and forms the mixed difference from neighbours it holds: the z neighbour
 * by a shuffle (lane 0 loads its own), the previous row's z-difference and
 * the previous plane's 2-D differences in registers.  The row and plane
 * before the unit come in once more for that (zeros outside the volume).
 * So compress reads x twice (rates, then packing) and keeps no quantized
 * volume; decompress writes whole rows. */
struct Sz3Unit {
    uint64_t bi, bj, bk0, i0, j0, z0;
    uint32_t sx, sy;
};

template <uint32_t BS>
__host__ __device__ inline uint64_t sz3_units(const Sz3Dims &g)
{
    return g.nb1 * g.nb2 * ((g.nb3 + 32 / BS - 1) / (32 / BS));
}

template <uint32_t BS>
__device__ __forceinline__ Sz3Unit sz3_unit(const Sz3Dims &g, uint64_t u)
{
    constexpr uint32_t U = 32 / BS;
    const uint64_t nzc = (g.nb3 + U - 1) / U;
    Sz3Unit k;
    k.bj = (u / nzc) % g.nb2;
    k.bi = u / (nzc * g.nb2);
    k.bk0 = (u % nzc) * U;
    k.i0 = k.bi * BS;
    k.j0 = k.bj * BS;
    k.z0 = k.bk0 * BS;
    k.sx = (uint32_t)min((uint64_t)BS, g.d1 - k.i0);
    k.sy = (uint32_t)min((uint64_t)BS, g.d2 - k.j0);
    return k;
}

/* Extent along z of the unit's block c (0 past the volume). */
template <uint32_t BS>
__device__ __forceinline__ uint32_t sz3_unit_sz(const Sz3Dims &g, const Sz3Unit &k, uint32_t c)
{
    const uint64_t bk = k.bk0 + c;
    return bk < g.nb3 ? (uint32_t)min((uint64_t)BS, g.d3 - bk * BS) : 0u;
}

/* row(di, dj, e): the difference at (i0 + di, j0 + dj, z0 + lane) for every
 * lane (meaningless where z0 + lane >= d3); called by the whole warp. */
template <uint32_t BS, class Row>
__device__ __forceinline__ void sz3_walk(const float *__restrict__ x, const Sz3Dims &g, const Sz3Split &inv,
                                         const Sz3Unit &k, uint32_t &bad, Row row)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t s0 = g.d2 * g.d3, s1 = g.d3, z = k.z0 + lane;
    const bool zin = z < g.d3;
    auto live = [&](uint32_t r) { return r == 0 ? k.j0 > 0 : r - 1 < k.sy; }; /* row j0 - 1 + r */
    /* plane i's rows j0 - 1 .. j0 + BS - 1 (v), and in lane r the element
     * before z0 of row r (l), which lane 0 needs; all loads issued before
     * any is used; rows outside read as 0 */
    auto load = [&](uint64_t i, float (&v)[BS + 1], float &l) {
#pragma unroll
        for (uint32_t r = 0; r <= BS; r++) {
            const uint64_t o = i * s0 + (k.j0 + r - 1) * s1; /* wraps only where not live */
            v[r] = live(r) && zin ? x[o + z] : 0.0f;
        }
        const uint64_t o = i * s0 + (k.j0 + lane - 1) * s1;
        l = lane <= BS && live(lane) && k.z0 ? x[o + k.z0 - 1] : 0.0f;
    };
    uint32_t dp[BS]; /* the previous plane's 2-D differences, row by row */
#pragma unroll
    for (uint32_t dj = 0; dj < BS; dj++) dp[dj] = 0;
    int di = k.i0 ? -1 : 0;
    float cv[BS + 1], nv[BS + 1], cl, nl = 0.0f;
    load((uint64_t)((int64_t)k.i0 + di), cv, cl);
    for (; di < (int)k.sx; di++) {
        if (di + 1 < (int)k.sx) load(k.i0 + (uint64_t)(di + 1), nv, nl); /* the next plane, in flight meanwhile */
        const uint32_t qleft = (uint32_t)sz3_quantize(cl, inv, bad); /* 0 where cl is */
        auto zdiff = [&](uint32_t r) -> uint32_t {                   /* q(z) - q(z - 1) of row r */
            const uint32_t q = zin ? (uint32_t)sz3_quantize(cv[r], inv, bad) : 0u;
            const uint32_t up = __shfl_up_sync(0xffffffffu, q, 1), l0 = __shfl_sync(0xffffffffu, qleft, r);
            return q - (lane ? up : l0);
        };
        uint32_t rp = k.j0 ? zdiff(0) : 0u;
#pragma unroll
        for (uint32_t dj = 0; dj < BS; dj++) {
            if (dj < k.sy) {
                const uint32_t rc = zdiff(dj + 1);
                const uint32_t d = rc - rp;
                rp = rc;
                if (di >= 0) row((uint32_t)di, dj, d - dp[dj]);
                dp[dj] = d;
            }
        }
#pragma unroll
        for (uint32_t r = 0; r <= BS; r++) cv[r] = nv[r];
        cl = nl;
    }
}

/* compress, one pass (quantization included): warps take units in ticket
 * order; a unit's differences go to shared memory in element order while
 * their largest magnitudes give the blocks' rates and payload sizes; the
 * unit's place in the stream comes from a decoupled look-back over the
 * units before it (the unit's bytes are its blocks', consecutive), then
 * its blocks are packed (all at once, BS lanes each, for BS up to 4; else
 * one after another by the whole warp).  The last unit records the
 * stream's size. */
template <uint32_t BS>
__global__ void __launch_bounds__(SZ_THREADS, BS <= 4 ? 4 : 3) k_sz3_compress_rows(const float *__restrict__ x, Sz3Dims g, Sz3Split inv,
                                                                  uint8_t *out, uint64_t cap, uint64_t *status,
                                                                  uint32_t *ticket, uint64_t *total, uint32_t *err)
{
    constexpr uint32_t U = 32 / BS, NB = BS * BS * BS;
    extern __shared__ uint32_t e_all[]; /* U blocks per warp */
    const uint32_t lane = threadIdx.x & 31u, dz = lane % BS;
    uint32_t *e = e_all + (threadIdx.x >> 5) * (U * NB);
    const uint64_t units = sz3_units<BS>(g);
    uint32_t bad = 0, full = 0;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(ticket, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= units) break; /* uniform */
        const Sz3Unit k = sz3_unit<BS>(g, u);
        const uint32_t sz = sz3_unit_sz<BS>(g, k, lane / BS);
        const bool zin = k.z0 + lane < g.d3;
        uint32_t *eb = e + (lane / BS) * NB;
        uint32_t m = 0;
        __syncwarp(); /* the previous unit is packed */
        sz3_walk<BS>(x, g, inv, k, bad, [&](uint32_t di, uint32_t dj, uint32_t v) {
            if (zin) {
                eb[(di * k.sy + dj) * sz + dz] = v;
                m = max(m, mag(v));
            }
        });
#pragma unroll
        for (uint32_t o = 1; o < BS; o <<= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        /* lane c < U: block c's rate and size */
        const uint32_t mc = __shfl_sync(0xffffffffu, m, (lane % U) * BS);
        const uint32_t szc = lane < U ? sz3_unit_sz<BS>(g, k, lane) : 0u;
        const uint32_t rate = szc ? 32u - __clz(mc) : 0u, size = szc ? sz3_payload(rate, k.sx * k.sy * szc) : 0u;
        const uint32_t inc = warp_incl_scan(size), agg = __shfl_sync(0xffffffffu, inc, 31);
        lb_publish(status, u, agg, u == 0, 0);
        const uint64_t prefix = lb_resolve(status, u, agg, u == 0, 0, err);
        const uint64_t base = g.nblocks + prefix + (inc - size);
        if (szc) out[(k.bi * g.nb2 + k.bj) * g.nb3 + k.bk0 + lane] = (uint8_t)rate;
        if (u == units - 1 && lane == 0) *total = g.nblocks + prefix + agg;
        __syncwarp();
        if constexpr (BS <= 4) { /* all blocks of the unit at once, BS lanes each */
            const uint32_t c = lane / BS;
            const uint32_t rc = __shfl_sync(0xffffffffu, rate, c);
            const uint64_t bc = __shfl_sync(0xffffffffu, base, c);
            const uint32_t n = k.sx * k.sy * sz;
            if (rc && n) {
                if (bc + sz3_payload(rc, n) > cap)
                    full = 1;
                else
                    sz3_pack_block<BS>(e + c * NB, n, rc, out + bc, dz);
            }
        } else { /* blocks of 512 elements: one after another, the whole warp on each */
            for (uint32_t c = 0; c < U; c++) {
                const uint32_t rc = __shfl_sync(0xffffffffu, rate, c);
                const uint64_t bc = __shfl_sync(0xffffffffu, base, c);
                const uint32_t n = k.sx * k.sy * sz3_unit_sz<BS>(g, k, c);
                if (!rc || !n) continue; /* uniform */
                if (bc + sz3_payload(rc, n) > cap) {
                    full = 1;
                    continue;
                }
                sz3_pack_block<32>(e + c * NB, n, rc, out + bc, lane);
            }
        }
    }
    if (bad) atomicOr(err, ZERR_RANGE);
    if (full) atomicOr(err, ZERR_CAPACITY);
}

/* Bytes that hold a unit's blocks at most (every block at rate 32). */
template <uint32_t BS>
__host__ __device__ constexpr uint32_t sz3_unit_stage()
{
    return ((32 / BS) * ((BS * BS * BS + 7) / 8 + 4 * BS * BS * BS) + 15) & ~15u;
}

/* decompress K3: a warp per unit; the unit's blocks, consecutive in the
 * stream, come into shared memory in one coalesced copy, then every lane
 * decodes its own elements straight into whole rows of the output */
template <uint32_t BS>
__global__ void __launch_bounds__(SZ_THREADS) k_sz3_unpack_rows(const uint8_t *__restrict__ in, uint64_t avail,
                                                                Sz3Dims g, const uint64_t *__restrict__ offs,
                                                                uint32_t *__restrict__ vol, uint32_t *err)
{
    constexpr uint32_t U = 32 / BS, STAGE = sz3_unit_stage<BS>();
    extern __shared__ __align__(16) uint8_t st_all[];
    const uint32_t lane = threadIdx.x & 31u, dz = lane % BS, c = lane / BS;
    uint8_t *stg = st_all + (threadIdx.x >> 5) * STAGE;
    const uint64_t units = sz3_units<BS>(g), s0 = g.d2 * g.d3, s1 = g.d3;
    uint32_t flag = 0;
    for (uint64_t u = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < units;
         u += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const Sz3Unit k = sz3_unit<BS>(g, u);
        uint32_t rate = 0;
        uint64_t base = 0, end = 0;
        if (lane < U && k.bk0 + lane < g.nb3) { /* lane c: block c's rate and place */
            const uint64_t b = (k.bi * g.nb2 + k.bj) * g.nb3 + k.bk0 + lane;
            const uint32_t n = k.sx * k.sy * sz3_unit_sz<BS>(g, k, lane);
            rate = b < avail ? in[b] : 0u;
            base = g.nblocks + offs[b];
            if (rate > 32 || base + sz3_payload(rate, n) > avail) {
                flag |= rate > 32 ? ZERR_CORRUPT : ZERR_BOUNDS;
                rate = 0;
            }
            end = rate ? base + sz3_payload(rate, n) : 0;
        }
        /* blocks follow one another in the stream: the unit's bytes are
         * [block 0's place, the last end), at most STAGE of them (the places
         * come from the same rates; checked all the same) */
        const uint64_t first = __shfl_sync(0xffffffffu, base, 0);
        if (rate && (base < first || end - first > STAGE)) {
            flag |= ZERR_CORRUPT;
            rate = 0;
            end = 0;
        }
#pragma unroll
        for (uint32_t o = 16; o; o >>= 1) end = max(end, __shfl_xor_sync(0xffffffffu, end, o));
        const uint32_t nbytes = end > first ? (uint32_t)min(end - first, (uint64_t)STAGE) : 0u;
        __syncwarp(); /* the previous unit is decoded */
#pragma unroll 8
        for (uint32_t t = lane; t < nbytes; t += 32) stg[t] = in[first + t];
        __syncwarp();
        const uint32_t rl = __shfl_sync(0xffffffffu, rate, c);
        const uint64_t bl = __shfl_sync(0xffffffffu, base, c);
        const uint32_t sz = sz3_unit_sz<BS>(g, k, c), n = k.sx * k.sy * sz;
        if (k.z0 + lane < g.d3) {
            const uint8_t *sg = stg + (rl ? bl - first : 0);
            uint32_t *o = vol + k.i0 * s0 + k.j0 * s1 + k.z0 + lane;
            for (uint32_t di = 0; di < k.sx; di++)
#pragma unroll
                for (uint32_t dj = 0; dj < BS; dj++)
                    if (dj < k.sy) o[di * s0 + dj * s1] = sz3_unpack_elem(sg, rl, n, (di * k.sy + dj) * sz + dz);
        }
    }
    if (flag) atomicOr(err, flag);
}

/* ---- decompress K4-K6: the 3-D prefix sum ------------------------------ */
__global__ void k_sz3_scan_z(uint32_t *vol, uint64_t rows, uint64_t d3)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= rows) return;
    uint32_t *p = vol + row * d3;
    uint32_t run = 0;
    for (uint64_t k0 = 0; k0 < d3; k0 += 32) {
        const uint64_t k = k0 + lane;
        const uint32_t v = k < d3 ? p[k] : 0u;
        const uint32_t inc = warp_incl_scan(v);
        if (k < d3) p[k] = run + inc;
        run += __shfl_sync(0xffffffffu, inc, 31);
    }
}

/* y: a thread per (i, k), j sequential */
__global__ void k_sz3_scan_y(uint32_t *vol, uint64_t d1, uint64_t d2, uint64_t d3)
{
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d1 * d3) return;
    const uint64_t i = t / d3, k = t % d3;
    uint32_t *p = vol + i * d2 * d3 + k;
    uint32_t run = 0;
    for (uint64_t j0 = 0; j0 < d2; j0 += SZ_SCAN_BATCH) { /* the loads of a batch ahead of its stores */
        uint32_t v[SZ_SCAN_BATCH];
#pragma unroll
        for (uint32_t u = 0; u < SZ_SCAN_BATCH; u++) v[u] = j0 + u < d2 ? p[(j0 + u) * d3] : 0u;
#pragma unroll
        for (uint32_t u = 0; u < SZ_SCAN_BATCH; u++) {
            run += v[u];
            if (j0 + u < d2) p[(j0 + u) * d3] = run;
        }
    }
}

/* x: a thread per (j, k), i sequential; writes the floats in place */
__global__ void k_sz3_scan_x(uint32_t *vol, uint64_t d1, uint64_t plane, Sz3Split twice)
{
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane) return;
    uint32_t run = 0;
    for (uint64_t i0 = 0; i0 < d1; i0 += SZ_SCAN_BATCH) {
        uint32_t v[SZ_SCAN_BATCH];
#pragma unroll
        for (uint32_t u = 0; u < SZ_SCAN_BATCH; u++) v[u] = i0 + u < d1 ? vol[(i0 + u) * plane + t] : 0u;
#pragma unroll
        for (uint32_t u = 0; u < SZ_SCAN_BATCH; u++) {
            run += v[u];
            if (i0 + u < d1) reinterpret_cast<float *>(vol)[(i0 + u) * plane + t] = sz3_value((int32_t)run, twice);
        }
    }
}

unsigned grid_for(uint64_t items, unsigned per_cta)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    uint64_t g = (items + per_cta - 1) / per_cta, cap = (uint64_t)(nsm > 0 ? nsm : 1) * 16;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

/* Scratch layout: err[4] | sizes[nb] | offs[nb] | sums[nchunks] | total | q volume (compress). */
struct Sz3Ws {
    uint32_t *err, *sizes;
    uint64_t *offs, *sums, *total;
    int32_t *q;
};

Sz3Ws sz3_bind(void *ws, const Sz3Dims &g)
{
    uint8_t *p = static_cast<uint8_t *>(ws);
    const uint64_t nch = (g.nblocks + SZ_CHUNK - 1) / SZ_CHUNK;
    Sz3Ws w;
    w.err = reinterpret_cast<uint32_t *>(p);
    size_t o = 16;
    w.sizes = reinterpret_cast<uint32_t *>(p + o);
    o = (o + 4 * g.nblocks + 15) & ~(size_t)15;
    w.offs = reinterpret_cast<uint64_t *>(p + o);
    o += 8 * g.nblocks;
    w.sums = reinterpret_cast<uint64_t *>(p + o);
    o += 8 * nch;
    w.total = reinterpret_cast<uint64_t *>(p + o);
    o = (o + 8 + 255) & ~(size_t)255;
    w.q = reinterpret_cast<int32_t *>(p + o);
    return w;
}

cudaError_t sz3_scan(const Sz3Dims &g, const Sz3Ws &w, cudaStream_t st)
{
    const uint64_t nch = (g.nblocks + SZ_CHUNK - 1) / SZ_CHUNK;
    k_sz3_chunk_sums<<<(unsigned)nch, 1024, 0, st>>>(w.sizes, g.nblocks, w.sums);
    k_sz3_scan_sums<<<1, 1024, 0, st>>>(w.sums, nch, g.nblocks, w.total);
    k_sz3_offsets<<<(unsigned)nch, 1024, 0, st>>>(w.sizes, g.nblocks, w.sums, w.offs);
    return cudaGetLastError();
}

/* Block sides with the row-mapped kernels. */
bool sz3_rows(uint32_t bs) { return bs == 2 || bs == 4 || bs == 8; }

/* One pass; the units' look-back flags use the offsets array (8 bytes a
 * block, at least 8 a unit) and the ticket the third of the four scratch
 * words before it (the first two are error words the status check reads),
 * both zeroed first. */
template <uint32_t BS>
cudaError_t sz3_compress_rows(uint8_t *out, uint64_t cap, const float *x, const Sz3Dims &g, const Sz3Ws &w,
                              const Sz3Split &inv, cudaStream_t st)
{
    const uint64_t units = sz3_units<BS>(g);
    if (units >> 32) return cudaErrorInvalidValue; /* tickets are 32-bit */
    uint64_t *status = w.offs;
    cudaError_t e = cudaMemsetAsync(status, 0, 8 * units, st);
    if (e != cudaSuccess) return e;
    const size_t smem = 4ull * 32 * BS * BS * (SZ_THREADS / 32);
    const void *fn = (const void *)k_sz3_compress_rows<BS>;
    if (smem > 48 * 1024 && (e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
                                cudaSuccess)
        return e;
    int dev = 0, nsm = 0, per = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, SZ_THREADS, smem)) != cudaSuccess)
        return e;
    const uint64_t want = (units + SZ_THREADS / 32 - 1) / (SZ_THREADS / 32), most = (uint64_t)nsm * (per > 0 ? per : 1);
    const unsigned grid = (unsigned)(want < most ? want : most);
    k_sz3_compress_rows<BS><<<grid, SZ_THREADS, smem, st>>>(x, g, inv, out, cap, status, w.err + 2, w.total, w.err);
    return cudaGetLastError();
}

template <uint32_t BS>
cudaError_t sz3_unpack_rows(const uint8_t *in, uint64_t avail, const Sz3Dims &g, const Sz3Ws &w, uint32_t *vol,
                            cudaStream_t st)
{
    const size_t smem = (size_t)sz3_unit_stage<BS>() * (SZ_THREADS / 32);
    cudaError_t e;
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_sz3_unpack_rows<BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
        return e;
    k_sz3_unpack_rows<BS><<<grid_for(sz3_units<BS>(g), SZ_THREADS / 32), SZ_THREADS, smem, st>>>(in, avail, g, w.offs,
                                                                                                 vol, w.err);
    return cudaGetLastError();
}

} // namespace

size_t sz3_workspace_bytes(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t bs, bool compress)
{
    const Sz3Dims g = sz3_dims(d1, d2, d3, bs);
    Sz3Ws w = sz3_bind(nullptr, g);
    const size_t head = (size_t)reinterpret_cast<uintptr_t>(w.q);
    return head + (compress && !sz3_rows(bs) ? 4 * (size_t)(d1 * d2 * d3) : 0) + 256;
}

size_t sz3_max_stream_bytes(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t bs)
{
    const Sz3Dims g = sz3_dims(d1, d2, d3, bs);
    return (size_t)(g.nblocks + (size_t)sz3_payload(32, bs * bs * bs) * g.nblocks);
}

cudaError_t sz3_compress(uint8_t *out, uint64_t cap, const float *x, uint64_t d1, uint64_t d2, uint64_t d3,
                         uint32_t bs, double eb, void *ws, uint64_t *d_size, cudaStream_t st)
{
    const Sz3Dims g = sz3_dims(d1, d2, d3, bs);
    const Sz3Ws w = sz3_bind(ws, g);
    cudaError_t e = cudaMemsetAsync(w.err + 2, 0, 8, st); /* the ticket; status words stay until checked */
    if (e != cudaSuccess) return e;
    /* the rate table is part of the stream: cap must hold it */
    if (cap < g.nblocks) return cudaErrorInvalidValue;
    const Sz3Split inv = sz3_split(0.5 / eb);
    if (sz3_rows(bs)) {
        e = bs == 2 ? sz3_compress_rows<2>(out, cap, x, g, w, inv, st)
                    : bs == 4 ? sz3_compress_rows<4>(out, cap, x, g, w, inv, st) : sz3_compress_rows<8>(out, cap, x, g, w, inv, st);
        if (e != cudaSuccess) return e;
        return d_size ? cudaMemcpyAsync(d_size, w.total, 8, cudaMemcpyDeviceToDevice, st) : cudaSuccess;
    }
    const uint64_t n = d1 * d2 * d3;
    k_sz3_quant<<<grid_for(n, 1024), 256, 0, st>>>(x, w.q, n, inv, w.err);
    const bool wb = bs * bs * bs <= 512; /* a warp per block */
    if (wb)
        k_sz3_rates<32><<<grid_for(g.nblocks, SZ_THREADS / 32), SZ_THREADS, 0, st>>>(w.q, g, out, w.sizes);
    else
        k_sz3_rates<SZ_THREADS><<<grid_for(g.nblocks, 1), SZ_THREADS, 0, st>>>(w.q, g, out, w.sizes);
    if ((e = sz3_scan(g, w, st)) != cudaSuccess) return e;
    if (wb) {
        k_sz3_pack<32><<<grid_for(g.nblocks, SZ_THREADS / 32), SZ_THREADS, 4ull * bs * bs * bs * (SZ_THREADS / 32), st>>>(
            w.q, g, out, cap, w.offs, w.err);
    } else {
        const size_t smem = 4ull * bs * bs * bs;
        if (smem > 48 * 1024 && (e = cudaFuncSetAttribute(k_sz3_pack<SZ_THREADS>,
                                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
                                    cudaSuccess)
            return e;
        k_sz3_pack<SZ_THREADS><<<grid_for(g.nblocks, 1), SZ_THREADS, smem, st>>>(w.q, g, out, cap, w.offs, w.err);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return d_size ? cudaMemcpyAsync(d_size, w.total, 8, cudaMemcpyDeviceToDevice, st) : cudaSuccess;
}

cudaError_t sz3_decompress(float *y, const uint8_t *in, uint64_t avail, uint64_t d1, uint64_t d2, uint64_t d3,
                           uint32_t bs, double eb, void *ws, cudaStream_t st)
{
    const Sz3Dims g = sz3_dims(d1, d2, d3, bs);
    const Sz3Ws w = sz3_bind(ws, g);
    cudaError_t e = cudaMemsetAsync(w.err + 2, 0, 8, st); /* the ticket; status words stay until checked */
    if (e != cudaSuccess) return e;
    k_sz3_sizes<<<grid_for(g.nblocks, 256), 256, 0, st>>>(in, avail, g, w.sizes, w.err);
    if ((e = sz3_scan(g, w, st)) != cudaSuccess) return e;
    uint32_t *vol = reinterpret_cast<uint32_t *>(y);
    if (sz3_rows(bs)) {
        e = bs == 2 ? sz3_unpack_rows<2>(in, avail, g, w, vol, st)
                    : bs == 4 ? sz3_unpack_rows<4>(in, avail, g, w, vol, st) : sz3_unpack_rows<8>(in, avail, g, w, vol, st);
        if (e != cudaSuccess) return e;
    } else if (bs * bs * bs <= 512)
        k_sz3_unpack<32><<<grid_for(g.nblocks, SZ_THREADS / 32), SZ_THREADS, 0, st>>>(in, avail, g, w.offs, vol, w.err);
    else
        k_sz3_unpack<SZ_THREADS><<<grid_for(g.nblocks, 1), SZ_THREADS, 0, st>>>(in, avail, g, w.offs, vol, w.err);
    const uint64_t rows = d1 * d2;
    k_sz3_scan_z<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, st>>>(vol, rows, d3);
    k_sz3_scan_y<<<(unsigned)((d1 * d3 + 255) / 256), 256, 0, st>>>(vol, d1, d2, d3);
    k_sz3_scan_x<<<(unsigned)((d2 * d3 + 255) / 256), 256, 0, st>>>(vol, d1, d2 * d3, sz3_split(eb * 2));
    return cudaGetLastError();
}
