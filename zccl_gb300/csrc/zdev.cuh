/*
 * zdev.cuh -- device building blocks shared by the codec kernels.
 *
 *   quantize()      bit-exact stand-in for (int)((double)x * (double)inv)
 *   width_of()      bit-exact stand-in for (int)log2f((float)m) + 1
 *   BitWriter/Reader MSB-first byte streams in shared memory
 *   stage_in/out()  TMA bulk copies between global memory and shared memory
 *   lookback()      single-pass decoupled look-back scan over tiles
 *   cta_scan*()     block-wide exclusive scans
 */
#ifndef ZCCL_GB300_ZDEV_CUH
#define ZCCL_GB300_ZDEV_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "zgeom.h"
#include "zccl_err.h"

/* Width thresholds, filled on the host from the host's libm: thr[w] is the
 * smallest m of bit length w whose (int)log2f((float)m) equals w (so its
 * width is w + 1), or 0xFFFFFFFF when none exists.  glibc rounds log2f of
 * 5,876 integers just below a power of two up to that power. */
struct ZWidthTable {
    uint32_t thr[33];
};

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

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

/* ---------------------------------------------------------------------
 * Bit streams in shared memory.  A stream is a sequence of bytes; bits go
 * MSB first within a byte, which is how the reference packs sign bits and
 * the low r bits of every magnitude (ZCCL/src/ZCCL_TypeManager.c:118-421,
 * :824-848).  Whole bytes written through put(v, 8k) keep their order.
 * ------------------------------------------------------------------- */

/* Packs MSB-first bits into a ZEROED shared buffer starting at byte offset
 * o.  Finished 32-bit words are OR-ed in, so blocks that share a boundary
 * word (or several tiny blocks sharing one word) need no coordination and
 * the leading bits of a block's first word stay untouched.  The 64-bit
 * accumulator holds `nacc` pending bits right-aligned; flush() must run
 * before it passes 64 bits (puts of up to 32 bits with nacc < 32 are safe). */
struct Packer {
    uint32_t *w;
    uint32_t wi, nacc;
    uint64_t acc;

    __device__ __forceinline__ void init(uint32_t *words, uint32_t o)
    {
        w = words;
        wi = o >> 2;
        nacc = (o & 3u) * 8u;
        acc = 0;
    }
    /* append the low n bits of v (1 <= n <= 32, v < 2^n) */
    __device__ __forceinline__ void put(uint32_t v, uint32_t n)
    {
        acc = (n < 32u ? acc << n : acc << 32) | v;
        nacc += n;
    }
    __device__ __forceinline__ void flush()
    {
        if (nacc >= 32u) {
            nacc -= 32u;
            atomicOr(&w[wi++], bswap32((uint32_t)(acc >> nacc)));
        }
    }
    __device__ __forceinline__ void finish()
    {
        flush();
        if (nacc) atomicOr(&w[wi], bswap32((uint32_t)(acc << (32u - nacc))));
    }
};

/* Reads MSB-first bits from byte offset o of a shared buffer.  refill()
 * guarantees at least 32 valid bits; gets totalling up to 32 bits may follow
 * one refill.  Loads whole aligned words, so it may read up to 8 bytes past
 * the last bit it returns (buffers carry slack). */
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
    /* next n bits, 1 <= n <= 32 */
    __device__ __forceinline__ uint32_t get(uint32_t n)
    {
        uint32_t v = (uint32_t)(acc >> 32) >> (32u - n);
        acc = n < 32u ? acc << n : acc << 32;
        nacc -= n;
        return v;
    }
};

/* The r-bit fields of a block, MSB first: the 32 elements of a full block
 * are r words exactly.  Four r-bit values are merged with multiply-adds into
 * one 4r-bit group (4r <= 28) before they enter the packer. */
__device__ __forceinline__ void put_low_bits(Packer &pk, const uint32_t *m, uint32_t n, uint32_t r,
                                             bool masked)
{
    const uint32_t mask = (1u << r) - 1u, p = 1u << r;
#pragma unroll
    for (uint32_t j = 0; j < 32; j += 4) {
        if (j < n) {
            uint32_t v0 = m[j], v1 = m[j + 1], v2 = m[j + 2], v3 = m[j + 3];
            if (masked) {
                v0 &= mask;
                v1 &= mask;
                v2 &= mask;
                v3 &= mask;
            }
            if (j + 4 <= n) {
                pk.put(((v0 * p + v1) * p + v2) * p + v3, 4 * r);
            } else { /* the ragged group of a short block */
                pk.put(v0, r);
                if (j + 1 < n) pk.put(v1, r);
                if (j + 2 < n) pk.put(v2, r);
            }
            pk.flush();
        }
    }
}

/* Inverse of put_low_bits: ORs the r-bit fields into m[]. */
__device__ __forceinline__ void get_low_bits(Reader &rd, uint32_t *m, uint32_t n, uint32_t r)
{
    const uint32_t mask = (1u << r) - 1u;
#pragma unroll
    for (uint32_t j = 0; j < 32; j += 4) {
        if (j < n) {
            rd.refill();
            if (j + 4 <= n) {
                uint32_t q = rd.get(4 * r);
                m[j] |= q >> (3 * r);
                m[j + 1] |= (q >> (2 * r)) & mask;
                m[j + 2] |= (q >> r) & mask;
                m[j + 3] |= q & mask;
            } else {
                m[j] |= rd.get(r);
                if (j + 1 < n) m[j + 1] |= rd.get(r);
                if (j + 2 < n) m[j + 2] |= rd.get(r);
            }
        }
    }
}

/* The B = b/8 high bytes of every element, little-endian per element
 * (ZCCL/src/ZCCL_TypeManager.c:34-47).  With B == 1 four elements fill one
 * word, merged with multiply-adds. */
__device__ __forceinline__ void put_high_bytes(Packer &pk, const uint32_t *m, uint32_t n, uint32_t B,
                                               uint32_t r)
{
    if (B == 1) {
#pragma unroll
        for (uint32_t j = 0; j < 32; j += 4) {
            if (j < n) {
                uint32_t h0 = m[j] >> r, h1 = m[j + 1] >> r, h2 = m[j + 2] >> r, h3 = m[j + 3] >> r;
                if (j + 4 <= n) {
                    pk.put(((h0 * 256u + h1) * 256u + h2) * 256u + h3, 32);
                } else {
                    pk.put(h0, 8);
                    if (j + 1 < n) pk.put(h1, 8);
                    if (j + 2 < n) pk.put(h2, 8);
                }
                pk.flush();
            }
        }
    } else {
#pragma unroll
        for (uint32_t j = 0; j < 32; j++) {
            if (j < n) {
                pk.put(bswap32(m[j] >> r) >> (32 - 8 * B), 8 * B);
                pk.flush();
            }
        }
    }
}

/* Inverse of put_high_bytes: m[j] = high part << r. */
__device__ __forceinline__ void get_high_bytes(Reader &rd, uint32_t *m, uint32_t n, uint32_t B,
                                               uint32_t r)
{
    if (B == 1) {
#pragma unroll
        for (uint32_t j = 0; j < 32; j += 4) {
            if (j < n) {
                rd.refill();
                if (j + 4 <= n) {
                    uint32_t q = rd.get(32);
                    m[j] = (q >> 24) << r;
                    m[j + 1] = ((q >> 16) & 0xFFu) << r;
                    m[j + 2] = ((q >> 8) & 0xFFu) << r;
                    m[j + 3] = (q & 0xFFu) << r;
                } else {
                    m[j] = rd.get(8) << r;
                    if (j + 1 < n) m[j + 1] = rd.get(8) << r;
                    if (j + 2 < n) m[j + 2] = rd.get(8) << r;
                }
            }
        }
    } else {
#pragma unroll
        for (uint32_t j = 0; j < 32; j++) {
            if (j < n) {
                rd.refill();
                m[j] = bswap32(rd.get(8 * B) << (32 - 8 * B)) << r;
            }
        }
    }
}

/* Zero shared bytes [0, nbytes) (rounded up to 16) of a 16-byte-aligned buffer. */
__device__ __forceinline__ void smem_zero(uint8_t *s, uint32_t nbytes)
{
    uint4 *s4 = reinterpret_cast<uint4 *>(s);
    const uint4 z = make_uint4(0, 0, 0, 0);
    for (uint32_t i = threadIdx.x; i < (nbytes + 15u) >> 4; i += blockDim.x) s4[i] = z;
}

/* max over |x| as raw float bits: NaN ranks above +inf, so a NaN also fails
 * the fast-quantization test. */
__device__ __forceinline__ uint32_t abs_bits(float x) { return __float_as_uint(x) & 0x7FFFFFFFu; }

/* Fast quantization is exact for the whole tile when the rounded-toward-
 * zero product of its largest magnitude stays below 2^24 (see quantize()). */
__device__ __forceinline__ bool tile_fast_ok(uint32_t amax_bits, float inv)
{
    float am = __uint_as_float(amax_bits);
    return am == am && fabsf(__fmul_rz(am, inv)) < 16777216.0f;
}

/* ---------------------------------------------------------------------
 * TMA (cp.async.bulk) staging between global and shared memory.
 * The shared copy of a global byte range keeps the range's 16-byte phase:
 * global byte g lands at smem[phase + (g - start)], phase = start & 15, so
 * the 16-byte-aligned middle of the range moves with one bulk copy and the
 * ragged ends (< 16 bytes each) with plain byte accesses.
 * ------------------------------------------------------------------- */

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

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

/* Wait for phase `parity` of the barrier to complete.  Gives up after a
 * bounded number of polls and reports ZERR_TIMEOUT instead of hanging. */
__device__ __forceinline__ void mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *err)
{
    uint32_t addr = smem_u32(bar);
    for (uint32_t it = 0; it < (1u << 21); it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return;
    }
    atomicOr(err, ZERR_TIMEOUT);
}

__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(sdst)),
        "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_s2g(void *gdst, const void *ssrc, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
                 "r"(smem_u32(ssrc)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit_and_wait()
{
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

/* Stage global bytes [g, g + nbytes) into the 16-byte-aligned buffer s.
 * Called by every thread of the CTA; thread 0 issues the bulk copy and the
 * barrier arrival, threads 0..31 copy the ragged ends.  Returns the phase
 * (g & 15); the copy is complete after stage_in_wait(). */
__device__ __forceinline__ uint32_t stage_in(uint8_t *s, const uint8_t *g, uint32_t nbytes,
                                             uint64_t *bar)
{
    uintptr_t ga = (uintptr_t)g, ge = ga + nbytes;
    uint32_t phase = (uint32_t)(ga & 15u);
    uintptr_t a0 = (ga + 15u) & ~(uintptr_t)15u, a1 = ge & ~(uintptr_t)15u;
    uint32_t tid = threadIdx.x;
    if (a1 > a0) {
        if (tid == 0) {
            fence_proxy_async_smem(); /* earlier generic accesses of s before the async write */
            mbar_expect_tx(bar, (uint32_t)(a1 - a0));
            bulk_g2s(s + phase + (a0 - ga), (const void *)a0, (uint32_t)(a1 - a0), bar);
        }
        if (tid < 32) {
            if (ga + tid < a0) s[phase + tid] = g[tid];
            uintptr_t t = a1 + tid;
            if (t < ge) s[phase + (t - ga)] = *(const uint8_t *)t;
        }
    } else {
        if (tid == 0) mbar_expect_tx(bar, 0);
        for (uint32_t i = tid; i < nbytes; i += blockDim.x) s[phase + i] = g[i];
    }
    return phase;
}

__device__ __forceinline__ void stage_in_wait(uint64_t *bar, uint32_t parity, uint32_t *err)
{
    mbar_wait(bar, parity, err);
    __syncthreads();
}

/* Write shared bytes s[phase .. phase + nbytes) to global [g, g + nbytes),
 * where phase == (g & 15).  Every thread calls it after its last write to s;
 * returns once the bulk copy has completed. */
__device__ __forceinline__ void stage_out(uint8_t *g, const uint8_t *s, uint32_t nbytes)
{
    fence_proxy_async_smem();
    __syncthreads();
    uintptr_t ga = (uintptr_t)g, ge = ga + nbytes;
    uint32_t phase = (uint32_t)(ga & 15u);
    uintptr_t a0 = (ga + 15u) & ~(uintptr_t)15u, a1 = ge & ~(uintptr_t)15u;
    uint32_t tid = threadIdx.x;
    if (a1 > a0) {
        if (tid < 32) {
            if (ga + tid < a0) g[tid] = s[phase + tid];
            uintptr_t t = a1 + tid;
            if (t < ge) *(uint8_t *)t = s[phase + (t - ga)];
        }
        if (tid == 0) {
            bulk_s2g((void *)a0, s + phase + (a0 - ga), (uint32_t)(a1 - a0));
            bulk_commit_and_wait();
        }
    } else {
        for (uint32_t i = tid; i < nbytes; i += blockDim.x) g[i] = s[phase + i];
    }
}

/* Issue (thread 0 only) a TMA bulk copy of the 16-byte-aligned superset
 * [floor16(g), ceil16(g + nbytes)) into the 16-byte-aligned buffer s and
 * arm the barrier; returns g & 15, the offset of g inside s.  The superset
 * only adds bytes of 16-byte chunks that already contain bytes of the range,
 * so it never touches a page the range does not.  Every thread may call it
 * to learn the phase; only thread 0 issues. */
__device__ __forceinline__ uint32_t tma_load_superset(uint8_t *s, const uint8_t *g, uint32_t nbytes,
                                                      uint64_t *bar)
{
    uintptr_t a0 = (uintptr_t)g & ~(uintptr_t)15u;
    uintptr_t a1 = ((uintptr_t)g + nbytes + 15u) & ~(uintptr_t)15u;
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        mbar_expect_tx(bar, (uint32_t)(a1 - a0));
        if (a1 > a0) bulk_g2s(s, (const void *)a0, (uint32_t)(a1 - a0), bar);
    }
    return (uint32_t)((uintptr_t)g & 15u);
}

/* Write shared bytes s[0, nbytes) to global [g, g + nbytes) for any
 * alignment of g.  16-byte-aligned global chunks get one vector store each,
 * assembled from two aligned shared loads and a funnel shift; the ragged
 * ends (shared with neighbouring tiles) are stored byte by byte.  s must be
 * 16-byte aligned with 32 readable bytes of slack.  Called by all threads;
 * ends with the data written (no trailing barrier). */
__device__ __forceinline__ void store_realign(uint8_t *g, const uint8_t *s, uint32_t nbytes)
{
    const uintptr_t g0 = (uintptr_t)g, g1 = g0 + nbytes;
    const uintptr_t a0 = (g0 + 15u) & ~(uintptr_t)15u, a1 = g1 & ~(uintptr_t)15u;
    const uint32_t tid = threadIdx.x;
    if (a1 <= a0) {
        for (uint32_t i = tid; i < nbytes; i += blockDim.x) g[i] = s[i];
        return;
    }
    const uint32_t d = (uint32_t)(a0 - g0); /* shared offset of the first aligned chunk */
    if (tid < d) g[tid] = s[tid];
    const uint32_t tail = (uint32_t)(g1 - a1);
    if (tid >= 32 && tid - 32 < tail) {
        uint32_t i = (uint32_t)(a1 - g0) + (tid - 32);
        g[i] = s[i];
    }
    const uint32_t nch = (uint32_t)((a1 - a0) >> 4), q = d >> 2, sh = (d & 3u) * 8u;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(s);
    uint4 *g4 = reinterpret_cast<uint4 *>(a0);
    for (uint32_t c = tid; c < nch; c += blockDim.x) {
        uint4 lo = s4[c], hi = s4[c + 1];
        uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        uint32_t o[5];
        /* q is the same for every thread of the tile: a uniform branch */
        switch (q) {
        case 0: o[0] = w[0]; o[1] = w[1]; o[2] = w[2]; o[3] = w[3]; o[4] = w[4]; break;
        case 1: o[0] = w[1]; o[1] = w[2]; o[2] = w[3]; o[3] = w[4]; o[4] = w[5]; break;
        case 2: o[0] = w[2]; o[1] = w[3]; o[2] = w[4]; o[3] = w[5]; o[4] = w[6]; break;
        default: o[0] = w[3]; o[1] = w[4]; o[2] = w[5]; o[3] = w[6]; o[4] = w[7]; break;
        }
        uint4 v;
        v.x = __funnelshift_r(o[0], o[1], sh);
        v.y = __funnelshift_r(o[1], o[2], sh);
        v.z = __funnelshift_r(o[2], o[3], sh);
        v.w = __funnelshift_r(o[3], o[4], sh);
        g4[c] = v;
    }
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

/* Exclusive scan of v over the CTA (wrapping uint32 add, so it also serves
 * int32 sums); *total receives the sum of all v. */
__device__ __forceinline__ uint32_t cta_excl_scan(uint32_t v, uint32_t *wsum, uint32_t *total)
{
    uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < nw ? wsum[lane] : 0u;
        uint32_t ti = warp_incl_scan(t);
        if (lane < nw) wsum[lane] = ti - t;
        if (lane == 31) wsum[32] = ti;
    }
    __syncthreads();
    uint32_t r = wsum[warp] + inc - v;
    *total = wsum[32];
    __syncthreads();
    return r;
}

/* ---------------------------------------------------------------------
 * Decoupled look-back (Merrill & Garland 2016).  status[t] packs a 2-bit
 * flag (1 = aggregate of tile t only, 2 = inclusive prefix through t) over
 * a 62-bit value.  Tiles are taken in ticket order, so every tile a CTA
 * waits on belongs to a CTA that is already running.
 * ------------------------------------------------------------------- */
#define LB_FLAG_A (1ull << 62)
#define LB_FLAG_P (2ull << 62)
#define LB_VAL (LB_FLAG_A - 1ull)

__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p)
{
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* Lane 0 of the publishing warp: make this tile's aggregate (or, for a
 * first tile, its inclusive value start + agg) visible to successors. */
__device__ __forceinline__ void lb_publish(uint64_t *status, uint64_t tile, uint64_t agg, bool first,
                                           uint64_t start)
{
    if ((threadIdx.x & 31u) == 0)
        st_release(status + tile, first ? (LB_FLAG_P | ((start + agg) & LB_VAL))
                                        : (LB_FLAG_A | (agg & LB_VAL)));
}

/* Called by all lanes of one warp after lb_publish: returns the exclusive
 * prefix of the tile and publishes its inclusive value.  Same semantics as
 * lookback(). */
static __device__ __noinline__ uint64_t lb_resolve(uint64_t *status, uint64_t tile, uint64_t agg,
                                                   bool first, uint64_t start, uint32_t *err)
{
    uint32_t lane = threadIdx.x & 31u;
    if (first) return start;
    uint64_t prefix = 0;
    int64_t pos = (int64_t)tile - 1;
    uint32_t spins = 0;
    for (;;) {
        int64_t idx = pos - (int64_t)lane;
        uint64_t v = idx >= 0 ? ld_acquire(status + idx) : LB_FLAG_P;
        uint32_t flag = (uint32_t)(v >> 62);
        uint32_t pm = __ballot_sync(0xffffffffu, flag == 2u);
        uint32_t xm = __ballot_sync(0xffffffffu, flag == 0u);
        uint32_t fp = pm ? (uint32_t)(__ffs(pm) - 1) : 32u;
        uint32_t need = fp >= 31u ? 0xffffffffu : ((2u << fp) - 1u);
        if (xm & need) {
            if (++spins < (1u << 22)) {
                __nanosleep(32);
                continue;
            }
            if (lane == 0) atomicOr(err, ZERR_TIMEOUT);
            if (flag == 0u) {
                v = 0;
                flag = 1u;
            }
        }
        uint64_t c = (lane <= fp && flag != 0u) ? (v & LB_VAL) : 0ull;
        prefix += warp_sum_u64(c);
        if (fp < 32u) break;
        pos -= 32;
        spins = 0;
    }
    if (lane == 0) st_release(status + tile, LB_FLAG_P | ((prefix + agg) & LB_VAL));
    return prefix & LB_VAL;
}

/* Called by all lanes of one warp.  Publishes this tile's aggregate `agg`
 * (or, when `first`, the inclusive value start + agg) and returns the
 * exclusive prefix: the sum of every tile back to and including the nearest
 * tile that published an inclusive value (or `start` when first).  Values
 * add modulo 2^62.  A predecessor that never publishes makes the wait give
 * up after a bounded number of polls: ZERR_TIMEOUT is set, the missing value
 * counts as 0 and the inclusive value is still published, so successors
 * never hang. */
static __device__ __noinline__ uint64_t lookback(uint64_t *status, uint64_t tile, uint64_t agg, bool first,
                                          uint64_t start, uint32_t *err)
{
    uint32_t lane = threadIdx.x & 31u;
    if (first) {
        if (lane == 0) st_release(status + tile, LB_FLAG_P | ((start + agg) & LB_VAL));
        return start;
    }
    if (lane == 0) st_release(status + tile, LB_FLAG_A | (agg & LB_VAL));
    uint64_t prefix = 0;
    int64_t pos = (int64_t)tile - 1;
    uint32_t spins = 0;
    for (;;) {
        int64_t idx = pos - (int64_t)lane;
        uint64_t v = idx >= 0 ? ld_acquire(status + idx) : LB_FLAG_P;
        uint32_t flag = (uint32_t)(v >> 62);
        uint32_t pm = __ballot_sync(0xffffffffu, flag == 2u);
        uint32_t xm = __ballot_sync(0xffffffffu, flag == 0u);
        uint32_t fp = pm ? (uint32_t)(__ffs(pm) - 1) : 32u;
        uint32_t need = fp >= 31u ? 0xffffffffu : ((2u << fp) - 1u);
        if (xm & need) {
            if (++spins < (1u << 22)) {
                __nanosleep(64);
                continue;
            }
            if (lane == 0) atomicOr(err, ZERR_TIMEOUT);
            if (flag == 0u) {
                v = 0;
                flag = 1u;
            }
        }
        uint64_t c = (lane <= fp && flag != 0u) ? (v & LB_VAL) : 0ull;
        prefix += warp_sum_u64(c);
        if (fp < 32u) break;
        pos -= 32;
        spins = 0;
    }
    if (lane == 0) st_release(status + tile, LB_FLAG_P | ((prefix + agg) & LB_VAL));
    return prefix & LB_VAL;
}

#endif
