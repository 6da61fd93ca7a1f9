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

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

/* ---------------------------------------------------------------------
 * Bit streams in shared memory.  A stream is a sequence of bytes; bits go
 * MSB first within a byte, which is how the reference packs sign bits and
 * the low r bits of every magnitude (ZCCL/src/ZCCL_TypeManager.c:118-421,
 * :824-848).  Whole bytes written through put(v, 8k) keep their order.
 * ------------------------------------------------------------------- */

/* Writes the byte range [lo, hi) of a 16-byte-aligned shared buffer.  Words
 * entirely inside the range are stored whole; the (at most two) words shared
 * with neighbouring blocks are stored byte by byte, so neighbours may write
 * concurrently. */
struct BitWriter {
    uint32_t *w;
    uint32_t wi, lo, hi, nacc;
    uint64_t acc; /* pending bits, left aligned */

    __device__ __forceinline__ void init(uint32_t *words, uint32_t o, uint32_t size)
    {
        w = words;
        lo = o;
        hi = o + size;
        wi = o >> 2;
        nacc = (o & 3u) * 8u;
        acc = 0;
    }
    __device__ __forceinline__ void store(uint32_t be)
    {
        uint32_t mem = bswap32(be);
        uint32_t b0 = wi * 4u;
        if (b0 >= lo && b0 + 4u <= hi) {
            w[wi] = mem;
        } else {
            uint8_t *p = reinterpret_cast<uint8_t *>(w);
#pragma unroll
            for (uint32_t k = 0; k < 4; k++)
                if (b0 + k >= lo && b0 + k < hi) p[b0 + k] = (uint8_t)(mem >> (8 * k));
        }
        wi++;
    }
    /* append the low n bits of v (1 <= n <= 32, v < 2^n) */
    __device__ __forceinline__ void put(uint32_t v, uint32_t n)
    {
        acc |= (uint64_t)v << (64u - nacc - n);
        nacc += n;
        if (nacc >= 32u) {
            store((uint32_t)(acc >> 32));
            acc <<= 32;
            nacc -= 32u;
        }
    }
    __device__ __forceinline__ void finish()
    {
        if (nacc) store((uint32_t)(acc >> 32));
    }
};

/* Reads forward from byte offset o of a 16-byte-aligned shared buffer; may
 * load the word after the last byte it returns (buffers carry slack). */
struct BitReader {
    const uint32_t *w;
    uint32_t wi, nacc;
    uint64_t acc;

    __device__ __forceinline__ void init(const uint32_t *words, uint32_t o)
    {
        w = words;
        wi = o >> 2;
        uint32_t skip = (o & 3u) * 8u;
        acc = ((uint64_t)bswap32(w[wi]) << 32) << skip;
        nacc = 32u - skip;
        wi++;
    }
    /* next n bits (1 <= n <= 32) as an unsigned value */
    __device__ __forceinline__ uint32_t get(uint32_t n)
    {
        if (nacc < n) {
            acc |= (uint64_t)bswap32(w[wi]) << (32u - nacc);
            wi++;
            nacc += 32u;
        }
        uint32_t v = (uint32_t)(acc >> (64u - n));
        acc <<= n;
        nacc -= n;
        return v;
    }
};

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
