/*
 * zk_decompress.cu -- decompressor.
 *
 * Replaces ZCCL_float_decompress_openmp_threadblock_arg
 * (ZCCL/src/ZCCLd_float.c:538-754) and produces the same floats.  One CTA
 * per tile, one thread per block, mirroring the compressor:
 *   1. block sizes come from the width index, a block-wide scan gives every
 *      block's byte offset inside the tile, and the tile's bytes arrive in
 *      shared memory with one TMA bulk copy;
 *   2. every thread unpacks its block (sign bits, high bytes, low-bit
 *      stream, ZCCL/src/ZCCL_TypeManager.c:423-950) into int32 deltas;
 *   3. a block-wide scan of the per-block delta sums, started from the
 *      quantized value before the tile, restores the running values
 *      (ZCCLd_float.c:617-628); the starting value comes from the index when
 *      the stream was produced on the device, otherwise from a decoupled
 *      look-back over tile delta sums that restarts at every segment head,
 *      and is then written back into the index;
 *   4. x = (float)q * eb (ZCCLd_float.c:624) into padded rows, written out
 *      row by row with coalesced stores.
 */
#include "zkern.cuh"

namespace {

template <bool FAST>
__global__ void __launch_bounds__(128) k_decompress(const DecompressArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);
    uint64_t *bcast = reinterpret_cast<uint64_t *>(smem + 160);
    float *rows = reinterpret_cast<float *>(smem + a.sm.rows);
    uint8_t *stage = smem + a.sm.stage;

    const ZGeom &g = a.g;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nw = blockDim.x >> 5;
    const uint32_t L = g.L, stride = zg_row_stride(L);
    uint32_t bad = 0;
    /* The index walk ran to completion before this launch, so every CTA sees
     * the same word: after a failed walk no CTA touches the stream and no
     * CTA waits on another. */
    if (*(volatile const uint32_t *)a.w.walk_err) return;

    if (tid == 0) {
        bcast[0] = a.qprev_valid ? (uint64_t)blockIdx.x : (uint64_t)atomicAdd(a.w.ticket, 1u);
        mbar_init(bar, 1);
    }
    __syncthreads();
    const uint64_t tile = bcast[0];
    ZTile z;
    zg_tile(&g, tile, &z);

    /* 1. block sizes and the tile's bytes */
    uint32_t b = 0, n = 0, size = 0;
    if (tid < z.nblk) {
        n = zg_block_len(z.seg_len, L, z.blk0 + tid);
        b = a.idx.widths[z.gblk0 + tid];
        if (b > 32) {
            bad |= ZERR_CORRUPT;
            b = 0;
        }
        size = zg_block_bytes(b, n);
    }
    const uint32_t headb = z.has_head ? 4u : 0u;
    uint32_t total;
    const uint32_t off = cta_excl_scan(size, wsum, &total);
    total += headb;
    const uint64_t base = a.idx.tile_off[tile];
    uint32_t nload = total;
    /* overflow-safe: base comes from the index and is not trusted */
    if (base > a.avail || total > a.avail - base) {
        bad |= ZERR_BOUNDS;
        nload = base < a.avail ? (uint32_t)min((uint64_t)total, a.avail - base) : 0u;
    }
    const uint32_t ph = stage_in(stage, a.in + base, nload, bar);
    stage_in_wait(bar, 0, a.w.err);
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(stage);

    int32_t head = 0;
    if (z.has_head) {
        uint32_t h = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) h |= (uint32_t)stage[ph + k] << (8 * k);
        head = (int32_t)h;
    }

    /* 2. unpack deltas */
    const uint32_t o = ph + headb + off;
    uint32_t d[FAST ? 32 : 1];
    uint32_t bsum = 0;
    if (tid < z.nblk) {
        if (stage[o] != b) bad |= ZERR_CORRUPT;
        if (FAST) {
#pragma unroll
            for (uint32_t j = 0; j < 32; j++) d[j] = 0;
            if (b) {
                const uint32_t B = b >> 3, r = b & 7u, ns = (n + 7) >> 3;
                BitReader br;
                br.init(sw, o + 1);
                const uint32_t sg = br.get(8 * ns) << (32 - 8 * ns);
                if (B) {
#pragma unroll
                    for (uint32_t j = 0; j < 32; j++)
                        if (j < n) d[j] = bswap32(br.get(8 * B) << (32 - 8 * B)) << r;
                }
                if (r) {
#pragma unroll
                    for (uint32_t j = 0; j < 32; j++)
                        if (j < n) d[j] |= br.get(r);
                }
#pragma unroll
                for (uint32_t j = 0; j < 32; j++) {
                    if ((sg >> (31 - j)) & 1u) d[j] = 0u - d[j];
                    bsum += d[j];
                }
            }
        } else if (b) {
            const uint32_t B = b >> 3, r = b & 7u, ns = (n + 7) >> 3;
            BitReader rs, rh, rl;
            rs.init(sw, o + 1);
            rh.init(sw, o + 1 + ns);
            rl.init(sw, o + 1 + ns + B * n);
            for (uint32_t j = 0; j < n; j++) {
                uint32_t v = B ? bswap32(rh.get(8 * B) << (32 - 8 * B)) << r : 0u;
                if (r) v |= rl.get(r);
                if (rs.get(1)) v = 0u - v;
                bsum += v;
            }
        }
    }

    /* 3. starting value of every block */
    uint32_t tsum;
    const uint32_t pre = cta_excl_scan(bsum, wsum, &tsum);
    if (a.qprev_valid) {
        if (tid == 0) bcast[1] = (uint32_t)(z.has_head ? head : a.idx.tile_qprev[tile]);
    } else if (warp == 0) {
        uint64_t q0 = lookback(a.w.status, tile, tsum, z.has_head != 0, (uint32_t)head, a.w.err);
        if (lane == 0) {
            bcast[1] = (uint32_t)q0;
            a.idx.tile_qprev[tile] = (int32_t)(uint32_t)q0;
        }
    }
    __syncthreads();
    const uint32_t q0 = (uint32_t)bcast[1];

    /* 4. values into rows, then out */
    if (tid < z.nblk) {
        uint32_t q = q0 + pre;
        float *row = rows + tid * stride;
        if (FAST) {
#pragma unroll
            for (uint32_t j = 0; j < 32; j++) {
                q += d[j];
                if (j < n) row[j] = __fmul_rn(__int2float_rn((int32_t)q), a.eb);
            }
        } else {
            const uint32_t B = b >> 3, r = b & 7u, ns = (n + 7) >> 3;
            BitReader rs, rh, rl;
            rs.init(sw, o + 1);
            rh.init(sw, o + 1 + ns);
            rl.init(sw, o + 1 + ns + B * n);
            for (uint32_t j = 0; j < n; j++) {
                if (b) {
                    uint32_t v = B ? bswap32(rh.get(8 * B) << (32 - 8 * B)) << r : 0u;
                    if (r) v |= rl.get(r);
                    if (rs.get(1)) v = 0u - v;
                    q += v;
                }
                row[j] = __fmul_rn(__int2float_rn((int32_t)q), a.eb);
            }
        }
    }
    if (z.has_head && tid == 0) a.y[z.seg_start] = __fmul_rn(__int2float_rn(head), a.eb);
    __syncthreads();
    for (uint32_t k = warp; k < z.nblk; k += nw) {
        uint32_t nk = zg_block_len(z.seg_len, L, z.blk0 + k);
        float *dst = a.y + z.e_first + (uint64_t)k * L;
        for (uint32_t j = lane; j < nk; j += 32) dst[j] = rows[k * stride + j];
    }
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_decompress(const DecompressArgs &a, cudaStream_t st)
{
    const bool fast = a.g.L <= 32;
    const void *fn = fast ? (const void *)k_decompress<true> : (const void *)k_decompress<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.sm.total);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)a.g.ntiles), block(a.g.TB);
    if (fast)
        k_decompress<true><<<grid, block, a.sm.total, st>>>(a);
    else
        k_decompress<false><<<grid, block, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
