/*
 * zk_compress.cu -- fused single-pass compressor.
 *
 * Replaces ZCCL_float_openmp_threadblock_arg (ZCCL/src/ZCCL_float.c:501-807)
 * and produces the same bytes.  Persistent CTAs take tiles of TB blocks in
 * ticket order; one thread owns one block.  Per tile:
 *   1. its floats (and the element before them) arrived by a TMA bulk copy
 *      issued while the previous tile was being coded (double buffering);
 *      a warp-cooperative transpose puts every block in its own padded row,
 *      so the per-thread walk below has no bank conflicts, and finds the
 *      tile's largest magnitude, which decides whether the one-multiply
 *      quantization is exact for the whole tile;
 *   2. every thread quantizes its block (truncation, ZCCL_float.c:580),
 *      forms the running deltas (ZCCL_float.c:581-582; the element before the
 *      block supplies the first one), sign mask, largest magnitude, width
 *      (ZCCL_float.c:606) and encoded size;
 *   3. a block-wide scan gives each block its offset in the tile; the tile's
 *      size is published for the decoupled look-back at once, the blocks are
 *      packed into shared memory, and only then is the tile's place in the
 *      stream resolved (the reference's per-thread scan and second memcpy
 *      pass, ZCCL_float.c:774-791, disappear);
 *   4. the packed tile goes out with 16-byte vector stores realigned to its
 *      byte offset, and the tile records the side index: block widths, its
 *      byte offset, and the quantized value before it.
 * Full 32-element blocks with exact fast quantization take straight-line
 * code; short tail blocks, blocks above 32 elements and tiles that need the
 * slow exact quantization take an element-at-a-time path.
 */
#include "zkern.cuh"

namespace {

template <bool FAST>
__global__ void __launch_bounds__(128) k_compress(const CompressArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);
    uint64_t *bc = reinterpret_cast<uint64_t *>(smem + 160); /* [0] tile, [2] prefix */
    uint32_t *s_amax = reinterpret_cast<uint32_t *>(smem + 192);
    float *rows = reinterpret_cast<float *>(smem + a.sm.rows);
    uint8_t *buf = smem + a.sm.in0; /* the tile's floats, then its packed bytes */
    const uint32_t buf_sa = smem_u32(buf);

    const ZGeom &g = a.g;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nw = blockDim.x >> 5;
    const uint32_t L = g.L, stride = zg_row_stride(L);
    uint32_t bad = 0;

    if (tid == 0) mbar_init(bar, 1);

    for (uint32_t it = 0;; it++) {
        /* A tile is claimed only when this CTA is ready to work on it: a
         * claimed tile publishes its size soon after, so later tiles never
         * wait on a tile that sits idle behind another one. */
        if (tid == 0) {
            const uint64_t t = atomicAdd(a.w.ticket, 1u);
            bc[0] = t;
            *s_amax = 0;
            if (t < g.ntiles) {
                ZTile zt;
                zg_tile(&g, t, &zt);
                const uint32_t nel = (uint32_t)(zt.e_end - zt.e_first + 1);
                tma_load_superset(buf, reinterpret_cast<const uint8_t *>(a.x + (zt.e_first - 1)),
                                  nel * 4u, bar);
            }
        }
        __syncthreads();
        const uint64_t tile = bc[0];
        if (tile >= g.ntiles) break;
        ZTile z;
        zg_tile(&g, tile, &z);

        /* 1. wait for this tile's floats, transpose blocks into rows, find
         *    the largest magnitude */
        mbar_wait(bar, it & 1u, a.w.err);
        const float *xin =
            reinterpret_cast<const float *>(buf + ((uintptr_t)(a.x + (z.e_first - 1)) & 15u));
        const float xprev0 = xin[0]; /* the head, or the last element of the previous tile */
        uint32_t amax = abs_bits(xprev0);
        if (FAST && L == 32 && z.nblk == g.TB && z.e_end - z.e_first == 32ull * g.TB) {
            /* a full tile: every row is 32 floats; unrolled so that many
             * shared loads are in flight per warp */
            const uint32_t nrow = g.TB / nw; /* rows per warp */
#pragma unroll 8
            for (uint32_t r = 0; r < nrow; r++) {
                const uint32_t k = warp + r * nw;
                const float v = xin[1 + k * 32 + lane];
                amax = max(amax, abs_bits(v));
                rows[k * stride + lane] = v;
            }
        } else {
            for (uint32_t k = warp; k < z.nblk; k += nw) {
                const uint32_t n = zg_block_len(z.seg_len, L, z.blk0 + k);
                for (uint32_t j = lane; j < n; j += 32) {
                    const float v = xin[1 + k * L + j];
                    amax = max(amax, abs_bits(v));
                    rows[k * stride + j] = v;
                }
            }
        }
        amax = __reduce_max_sync(0xffffffffu, amax);
        if (lane == 0) atomicMax(s_amax, amax);
        __syncthreads();
        const bool fastq = tile_fast_ok(*s_amax, a.inv);

        /* 2. quantize, delta, width */
        const bool own = tid < z.nblk;
        const uint32_t n = own ? zg_block_len(z.seg_len, L, z.blk0 + tid) : 0u;
        const bool full = FAST && fastq && n == 32; /* straight-line path */
        const float *row = rows + tid * stride;
        const float xp = !own ? 0.0f : (tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1]);
        uint32_t b = 0, size = 0, smask = 0;
        uint32_t m[32];
        if (full) {
            int32_t qp = quantize_fast(xp, a.inv);
            uint32_t mx = 0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int32_t q = quantize_fast(row[j], a.inv);
                const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                qp = q;
                smask = (smask << 1) | ((uint32_t)d >> 31);
                m[j] = (uint32_t)abs(d); /* |INT_MIN| wraps to 2^31, as in the reference */
                mx = max(mx, m[j]);
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes(b, 32);
        } else if (own) {
            int32_t qp = fastq ? quantize_fast(xp, a.inv) : quantize(xp, a.inv, bad);
            uint32_t mx = 0;
            for (uint32_t j = 0; j < n; j++) {
                const int32_t q = fastq ? quantize_fast(row[j], a.inv) : quantize(row[j], a.inv, bad);
                mx = max(mx, (uint32_t)abs((int32_t)((uint32_t)q - (uint32_t)qp)));
                qp = q;
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes(b, n);
        }

        /* 3. offsets in the tile, publish the tile size, pack, then place */
        const uint32_t headb = z.has_head ? 4u : 0u;
        uint32_t total;
        const uint32_t off = cta_excl_scan(size, wsum, &total);
        total += headb;
        if (warp == 0) lb_publish(a.w.status, tile, total, tile == 0, 0);
        const int32_t qprev0 = fastq ? quantize_fast(xprev0, a.inv) : quantize(xprev0, a.inv, bad);
        smem_zero(buf, total + 8); /* the floats are all in rows now */
        __syncthreads();
        if (z.has_head && tid == 0) *reinterpret_cast<int32_t *>(buf) = qprev0;
        const uint32_t o = headb + off;
        if (full) {
            encode_full(buf_sa, o, b, smask, m);
        } else if (own) {
            int32_t qp = fastq ? quantize_fast(xp, a.inv) : quantize(xp, a.inv, bad);
            encode_any(buf_sa, o, b, n, [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                const int32_t q = fastq ? quantize_fast(row[j], a.inv) : quantize(row[j], a.inv, bad);
                const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                qp = q;
                neg = (uint32_t)d >> 31;
                mg = (uint32_t)abs(d);
            });
        }
        if (warp == 0) {
            const uint64_t prefix = lb_resolve(a.w.status, tile, total, tile == 0, 0, a.w.err);
            if (lane == 0) bc[2] = prefix;
        }
        __syncthreads();

        /* 4. write the tile and its index entries */
        const uint64_t base = 8ull * g.T + bc[2];
        const bool fits = base + total <= a.cap; /* uniform over the CTA */
        if (!fits) bad |= ZERR_CAPACITY;
        if (own) a.idx.widths[z.gblk0 + tid] = (uint8_t)b;
        if (tid == 0) {
            a.idx.tile_off[tile] = base;
            a.idx.tile_qprev[tile] = qprev0;
            if (fits && z.has_head && z.seg < g.T) {
                const uint64_t h = base - 8ull * g.T;
#pragma unroll
                for (int k = 0; k < 8; k++) a.out[8ull * z.seg + k] = (uint8_t)(h >> (8 * k));
            }
            if (tile == g.ntiles - 1) *a.idx.size = base + total;
        }
        if (fits) store_realign(a.out + base, buf, total);
        __syncthreads(); /* rows, buf and the broadcast slots are reused by the next tile */
    }
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_compress(const CompressArgs &a, cudaStream_t st)
{
    const bool fast = a.g.L <= 32;
    const void *fn = fast ? (const void *)k_compress<true> : (const void *)k_compress<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.sm.total);
    if (e != cudaSuccess) return e;
    unsigned grid = persistent_grid(fn, a.g.TB, a.sm.total, a.g.ntiles);
    if (fast)
        k_compress<true><<<grid, a.g.TB, a.sm.total, st>>>(a);
    else
        k_compress<false><<<grid, a.g.TB, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
