/*
 * zk_compress.cu -- fused single-pass compressor.
 *
 * Replaces ZCCL_float_openmp_threadblock_arg (ZCCL/src/ZCCL_float.c:501-807)
 * and produces the same bytes.  Persistent CTAs take tiles of TB blocks in
 * ticket order; one thread owns one block.  Per tile:
 *   1. its floats (and the element before them) arrive by one TMA bulk
 *      copy; a warp-cooperative transpose puts every block in its own padded
 *      row, so the per-thread walk below has no bank conflicts, and finds
 *      the tile's largest magnitude, which decides whether the one-multiply
 *      quantization is exact for the whole tile;
 *   2. every thread quantizes its block (truncation, ZCCL_float.c:580),
 *      forms the running deltas (ZCCL_float.c:581-582; the element before the
 *      block supplies the first one), sign mask, largest magnitude, width
 *      (ZCCL_float.c:606) and encoded size;
 *   3. a block-wide scan gives each block its offset in the tile, and the
 *      tile's size is published for the decoupled look-back at once;
 *   4. the CTA places the tile it packed one round before: a CTA-wide
 *      look-back gives its byte offset, its bytes go out with 16-byte vector
 *      stores realigned to that offset, and the side index (block widths,
 *      byte offset, quantized value before the tile) is written.  Placing a
 *      tile one round late gives its predecessors a whole tile's time to
 *      publish their sizes, so the look-back rarely waits, and the CTA never
 *      waits while it holds a claimed tile whose size is not yet published
 *      (the reference's per-thread scan and second memcpy pass,
 *      ZCCL_float.c:774-791, disappear);
 *   5. the next tile is claimed and its copy started, and this tile's
 *      blocks are packed into shared memory meanwhile.
 * Full 32-element blocks with exact fast quantization take straight-line
 * code; other blocks of up to 32 elements are handled element by element
 * into the same registers, and blocks above 32 elements are re-read from
 * their rows while packing.
 */
#include "zkern.cuh"

namespace {

/* Thread 0: claim the next tile in ticket order and start the TMA copy of
 * its floats (and the element before them) into `in`.  The claimed index
 * lands in *slot; the caller synchronises before reading it. */
__device__ __forceinline__ void claim_tile(const CompressArgs &a, uint8_t *in, uint64_t *bar,
                                           uint64_t *slot, uint32_t *s_amax)
{
    if (threadIdx.x != 0) return;
    const uint64_t t = atomicAdd(a.w.ticket, 1u);
    *slot = t;
    *s_amax = 0;
    if (t < a.g.ntiles) {
        ZTile zt;
        zg_tile(&a.g, t, &zt);
        const uint32_t nel = (uint32_t)(zt.e_end - zt.e_first + 1);
        tma_load_superset(in, reinterpret_cast<const uint8_t *>(a.x + (zt.e_first - 1)), nel * 4u, bar);
    }
}

/* Six CTAs per SM fit the shared memory (about 35 KB each); asking for
 * them caps the registers at 80, and the few values spilled around the
 * placement cost less than a seventh of the SM's warps. */
template <bool FAST>
__global__ void __launch_bounds__(128, 6) k_compress(const CompressArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);
    uint64_t *bc = reinterpret_cast<uint64_t *>(smem + 160); /* [0] claimed tile */
    uint32_t *s_amax = reinterpret_cast<uint32_t *>(smem + 192);
    uint64_t *rec = reinterpret_cast<uint64_t *>(smem + 256);
    float *rows = reinterpret_cast<float *>(smem + a.sm.rows); /* FAST: the same space as in */
    uint8_t *in = smem + a.sm.in0;
    uint8_t *outb = smem + a.sm.out;
    const uint32_t out_sa = smem_u32(outb);

    const ZGeom &g = a.g;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nw = blockDim.x >> 5;
    const uint32_t L = g.L, stride = zg_row_stride(L);
    uint32_t bad = 0;
    ZPending pd = {ZP_NONE, 0, 0, 0};

    if (tid == 0) mbar_init(bar, 1);
    claim_tile(a, in, bar, &bc[0], s_amax);
    __syncthreads();
    uint64_t tile = bc[0];

    for (uint32_t it = 0;; it++) {
        if (tile >= g.ntiles) break;
        ZTile z;
        zg_tile(&g, tile, &z);

        /* 1. wait for the floats, move every block into its own padded row
         *    (so the per-thread walk below has no bank conflicts), and find
         *    the tile's largest magnitude */
        mbar_wait(bar, it & 1u, a.w.err);
        const float *xin =
            reinterpret_cast<const float *>(in + ((uintptr_t)(a.x + (z.e_first - 1)) & 15u));
        const float xprev0 = xin[0]; /* the head, or the last element of the previous tile */
        uint32_t amax = abs_bits(xprev0);
        if (FAST) {
            /* warp w owns rows w, w + nw, ... (32 of them: TB = 128 when
             * L <= 32); all floats are read before any row overwrites them */
            float v[32];
            const bool full = L == 32 && z.nblk == g.TB && z.e_end - z.e_first == 32ull * g.TB;
            if (full) {
#pragma unroll
                for (int r = 0; r < 32; r++) v[r] = xin[1 + (warp + r * nw) * 32 + lane];
            } else {
#pragma unroll
                for (int r = 0; r < 32; r++) {
                    const uint32_t k = warp + r * nw;
                    v[r] = 0.0f;
                    if (k < z.nblk && lane < zg_block_len(z.seg_len, L, z.blk0 + k))
                        v[r] = xin[1 + k * L + lane];
                }
            }
#pragma unroll
            for (int r = 0; r < 32; r++) amax = max(amax, abs_bits(v[r]));
            __syncthreads();
            if (lane < L) { /* a row holds L floats */
#pragma unroll
                for (int r = 0; r < 32; r++) rows[(warp + r * nw) * stride + lane] = v[r];
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
        const float *row = rows + tid * stride;
        const float xp = !own ? 0.0f : (tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1]);
        uint32_t b = 0, size = 0, smask = 0;
        uint32_t m[32];
        if (FAST && fastq && n == 32) { /* the straight-line path */
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
        } else if (FAST && own) { /* a short block or the exact slow quantization */
            int32_t qp = fastq ? quantize_fast(xp, a.inv) : quantize(xp, a.inv, bad);
            uint32_t mx = 0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                m[j] = 0;
                if ((uint32_t)j < n) {
                    const int32_t q = fastq ? quantize_fast(row[j], a.inv) : quantize(row[j], a.inv, bad);
                    const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                    qp = q;
                    smask |= ((uint32_t)d >> 31) << (31 - j);
                    m[j] = (uint32_t)abs(d);
                    mx = max(mx, m[j]);
                }
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes(b, n);
        } else if (own) { /* blocks above 32 elements: the rows are read again when packing */
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

        /* 3. offsets in the tile and early publication of its size; the
         *    scan's barriers also end every read of the rows above when
         *    L <= 32 */
        const uint32_t headb = z.has_head ? 4u : 0u;
        uint32_t total;
        const uint32_t off = cta_excl_scan(size, wsum, &total);
        total += headb;
        if (warp == 0) lb_publish(a.w.status, tile, total, tile == 0, 0);
        const int32_t qprev0 = fastq ? quantize_fast(xprev0, a.inv) : quantize(xprev0, a.inv, bad);

        /* 4. place the tile packed one round ago: its size went out a whole
         *    tile's time ago, so its predecessors have had time to publish
         *    theirs.  This CTA holds no claimed tile without a published
         *    size while it waits here. */
        if (pd.tile != ZP_NONE)
            place_tile(g, pd, outb, a.out, a.cap, a.idx, true, a.w.status, a.w.err, rec, bad);
        __syncthreads(); /* out is free again */

        /* 5. claim the next tile, whose floats arrive while this one is
         *    packed (with L <= 32 the rows are no longer needed: the
         *    magnitudes are in registers) */
        if (FAST) claim_tile(a, in, bar, &bc[0], s_amax);
        smem_zero(outb, total + 8);
        __syncthreads();
        if (z.has_head && tid == 0) *reinterpret_cast<int32_t *>(outb) = qprev0;
        const uint32_t o = headb + off;
        if (FAST) {
            if (n == 32) {
                encode_full(out_sa, o, b, smask, m);
            } else if (own) {
                encode_any(out_sa, o, b, n, [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                    neg = (smask >> (31u - j)) & 1u;
                    mg = pick(m, j);
                });
            }
        } else {
            if (own) {
                int32_t qp = fastq ? quantize_fast(xp, a.inv) : quantize(xp, a.inv, bad);
                encode_any(out_sa, o, b, n, [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                    const int32_t q = fastq ? quantize_fast(row[j], a.inv) : quantize(row[j], a.inv, bad);
                    const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                    qp = q;
                    neg = (uint32_t)d >> 31;
                    mg = (uint32_t)abs(d);
                });
            }
            __syncthreads(); /* the rows have been read for the last time */
            claim_tile(a, in, bar, &bc[0], s_amax);
        }
        pd.tile = tile;
        pd.total = total;
        pd.b = b;
        pd.q = (uint32_t)qprev0;
        __syncthreads(); /* the claimed index is visible; the packed tile is complete */
        tile = bc[0];
    }
    /* the last packed tile */
    if (pd.tile != ZP_NONE)
        place_tile(g, pd, outb, a.out, a.cap, a.idx, true, a.w.status, a.w.err, rec, bad);
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
