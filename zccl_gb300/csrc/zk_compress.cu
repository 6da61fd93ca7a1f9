/*
 * zk_compress.cu -- fused single-pass compressor.
 *
 * Replaces ZCCL_float_openmp_threadblock_arg (ZCCL/src/ZCCL_float.c:501-807)
 * and produces the same bytes.  Persistent CTAs take tiles of TB blocks in
 * ticket order.  Each CTA runs TB compute threads, one per block, and one
 * placer warp.  Per tile, the compute warps
 *   1. receive its floats (and the element before them) by one TMA bulk
 *      copy; a warp-cooperative transpose puts every block in its own padded
 *      row, so the per-thread walk below has no bank conflicts, and finds
 *      the tile's largest magnitude, which decides whether the one-multiply
 *      quantization is exact for the whole tile;
 *   2. quantize every block (truncation, ZCCL_float.c:580) and form the
 *      running deltas (ZCCL_float.c:581-582; the element before the block
 *      supplies the first one), sign mask, largest magnitude, width
 *      (ZCCL_float.c:606) and encoded size;
 *   3. scan the block sizes for their offsets in the tile and publish the
 *      tile's size for the decoupled look-back at once;
 *   4. claim the next tile (starting its copy) and pack this one into
 *      shared memory, then hand it to the placer.
 * The packed tiles wait in a shared-memory ring that holds two typical
 * tiles.  The placer finds each one's byte offset with the look-back, writes
 * its bytes with 16-byte vector stores realigned to that offset, records
 * the offset and zeroes the ring bytes it has written out (the ring starts
 * zeroed, so packing needs no zeroing pass and the tile's scan one barrier),
 * all while the compute warps work on the next tiles, so the
 * look-back's latency never stalls them (the reference's per-thread scan and
 * second memcpy pass, ZCCL_float.c:774-791, disappear).
 * Full 32-element blocks with exact fast quantization take straight-line
 * code; other blocks of up to 32 elements are handled element by element
 * into the same registers, and blocks above 32 elements are re-read from
 * their rows while packing.
 */
#include <cstring>

#include "zkern.cuh"

namespace {

/* A full tile of L = 32 whose element before it starts a 128-byte row of
 * its job's input (the single job's, or a batch job with a tensor map of
 * its own) arrives by one TMA tensor load of 256 rows of 32
 * floats (the element before the tile first, 128-byte swizzle: 16-byte
 * chunk k of row r at chunk k ^ (r & 7)) and a 16-byte copy that starts at
 * its last element; every thread then reads its block straight from its
 * row with vector loads that meet no bank conflict. */
__device__ __forceinline__ bool box_tile(const CompressArgs &a, const CompressJob &J, const ZTile &z)
{
    const ZGeom &g = J.g;
    return a.rows_map && (!a.batch.jobs || J.boxed) && g.L == 32 && g.TB == 256 && z.nblk == 256 &&
           z.e_end - z.e_first == 8192 && ((z.e_first - 1) & 31) == 0;
}

/* Thread 0: ticket t (taken a little earlier, so that the atomic's latency
 * overlaps other work) becomes the claimed tile: its job is copied into
 * `slot` and the TMA copy of its floats (and the element before them) into
 * `in` (or, for a box tile, into `box`) starts.  The tile within its job
 * lands in *s_tile (ZP_NONE when all are taken), the job in *s_job; the
 * caller synchronises before reading them. */
__device__ __forceinline__ void claim_tile(const CompressArgs &a, uint64_t t, uint8_t *in, uint64_t *bar,
                                           uint64_t *s_tile, uint32_t *s_job, uint32_t *s_amax,
                                           CompressJob *slot, uint32_t *slot_job, uint8_t *box,
                                           const CUtensorMap *xmap)
{
    if (threadIdx.x != 0) return;
    *s_amax = 0;
    const uint64_t total = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    if (t >= total) {
        *s_tile = ZP_NONE;
        return;
    }
    uint64_t local;
    const uint32_t j = batch_job(a.batch, t, &local);
    if (*slot_job != j) { /* the slot keeps its job from tile to tile */
        copy16(slot, a.batch.jobs ? static_cast<const CompressJob *>(a.batch.jobs) + j : &a.job,
               sizeof(CompressJob));
        *slot_job = j;
    }
    *s_tile = local;
    *s_job = j;
    ZTile zt;
    zg_tile(&slot->g, local, &zt);
    if (box && box_tile(a, *slot, zt)) {
        fence_proxy_async_smem(); /* earlier generic accesses of the box before the async writes */
        mbar_expect_tx(bar, 32768u + 16u);
        const CUtensorMap *m = a.batch.jobs ? static_cast<const CUtensorMap *>(a.batch.maps) + j : xmap;
        tma_load_2d(smem_u32(box), m, 0, (int32_t)((zt.e_first - 1) >> 5), bar);
        bulk_g2s(box + 32768, slot->x + (zt.e_end - 1), 16u, bar); /* 16-byte aligned, like the row */
        return;
    }
    const uint32_t nel = (uint32_t)(zt.e_end - zt.e_first + 1);
    tma_load_superset(in, reinterpret_cast<const uint8_t *>(slot->x + (zt.e_first - 1)), nel * 4u, bar);
}

/* Block size TB + 32: warps 0 .. TB/32 - 1 compute (one thread per block of
 * the tile), the last warp places packed tiles in the stream. */
template <bool FAST>
__global__ void __launch_bounds__(288, 3) k_compress(const __grid_constant__ CompressArgs a,
                                                     const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar_tma = reinterpret_cast<uint64_t *>(smem);      /* the tile's floats arrived */
    uint32_t *wsum0 = reinterpret_cast<uint32_t *>(smem + 32);   /* [33] scan scratch, even rounds */
    uint32_t *wsum1 = reinterpret_cast<uint32_t *>(smem + 320);  /* [33] odd rounds */
    uint64_t *s_tile = reinterpret_cast<uint64_t *>(smem + 168); /* the claimed tile (within its job) */
    uint32_t *s_amax = reinterpret_cast<uint32_t *>(smem + 176);
    uint32_t *s_pos = reinterpret_cast<uint32_t *>(smem + 184);  /* ring position of this tile */
    uint32_t *s_job = reinterpret_cast<uint32_t *>(smem + 188);  /* the claimed tile's job */
    uint32_t *s_slot = reinterpret_cast<uint32_t *>(smem + 192); /* [2] the job each job slot holds */
    ZRing *ring = reinterpret_cast<ZRing *>(smem + 256);
    CompressJob *cj = reinterpret_cast<CompressJob *>(smem + a.sm.jobs); /* [2], by round */
    ZPlace *pj = reinterpret_cast<ZPlace *>(smem + a.sm.jobs + 2 * sizeof(CompressJob));
    float *rows = reinterpret_cast<float *>(smem + a.sm.rows); /* FAST: the same space as in */
    uint8_t *in = smem + a.sm.in0;
    uint8_t *outb = smem + a.sm.out; /* the ring of packed tiles */

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t NC = blockDim.x - 32, nw = NC >> 5; /* compute threads (TB), compute warps */
    const uint32_t L = a.job.g.L, stride = zg_row_stride(L); /* one L for the whole batch */
    uint32_t bad = 0;
    /* the box of a box tile: 32 KB + 16 bytes at the first 1024-byte
     * boundary of the input region, if it fits there */
    const uint32_t box_sa = (smem_u32(in) + 1023u) & ~1023u;
    uint8_t *box = FAST && a.rows_map && box_sa + 32768u + 16u <= smem_u32(smem) + a.sm.out
                       ? in + (box_sa - smem_u32(in))
                       : nullptr;

    if (tid == 0) {
        mbar_init(bar_tma, 1);
        ring->packed = 0;
        ring->placed = 0;
        s_slot[0] = s_slot[1] = 0xFFFFFFFFu;
    }
    /* the ring starts zeroed, and the placer zeroes what it has written out */
    for (uint32_t i = tid; i < (zg_ring_bytes(L, blockDim.x - 32) + 48u) / 16u; i += blockDim.x)
        reinterpret_cast<uint4 *>(outb)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();

    if (tid >= NC) { /* the placer warp */
        const uint64_t max_tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
        placer_loop(
            ring, outb, pj, a.w.err, max_tiles, bad, true, a.w.lb_spin,
            [&](uint64_t k) {
                if (lane == 0) ring_wait(&ring->packed, (uint32_t)k + 1, a.w.err);
            },
            [&](uint32_t j, ZPlace *p) {
            if (a.batch.jobs) {
                const CompressJob &J = static_cast<const CompressJob *>(a.batch.jobs)[j];
                p->g = J.g;
                p->out = J.out;
                p->cap = J.cap;
                p->idx = J.idx;
                p->status = J.status;
            } else {
                p->g = a.job.g;
                p->out = a.job.out;
                p->cap = a.job.cap;
                p->idx = a.job.idx;
                p->status = a.job.status;
            }
        });
        if (bad) atomicOr(a.w.err, bad);
        return;
    }

    /* the compute warps */
    const uint32_t R = zg_ring_bytes(L, NC);
    uint32_t pos_prev = 0, end_prev = 0; /* thread 0: the previous tile's place in the ring */
    if (tid == 0) claim_tile(a, atomicAdd(a.w.ticket, 1u), in, bar_tma, s_tile, s_job, s_amax, &cj[0], &s_slot[0], box, &xmap);
    named_sync(1, NC);
    uint64_t tile = *s_tile;
    uint32_t job = *s_job;

    for (uint32_t it = 0;; it++) {
        if (tile == ZP_NONE) {
            /* tell the placer there is nothing more (once it has read the slot) */
            if (tid == 0) {
                ring_wait(&ring->placed, it >= 1 ? it - 1 : 0u, a.w.err);
                ring_publish(ring, it, ZP_NONE, 0, 0, 0);
            }
            break;
        }
        const CompressJob &J = cj[it & 1u];
        const ZGeom &g = J.g;
        ZTile z;
        zg_tile(&g, tile, &z);

        /* 1. wait for the floats; unless they came as a box, move every
         *    block into its own padded row (so the per-thread walk below has
         *    no bank conflicts).  Blocks above 32 elements also find the
         *    tile's largest magnitude, which decides whether the
         *    one-multiply quantization is exact for the whole tile. */
        mbar_wait(bar_tma, it & 1u, a.w.err);
        const bool bx = FAST && box && box_tile(a, J, z);
        const float *xin =
            reinterpret_cast<const float *>(in + ((uintptr_t)(J.x + (z.e_first - 1)) & 15u));
        /* the head, or the last element of the previous tile */
        const float xprev0 = bx ? ld_shared_f32(box_sa) : xin[0];
        bool fastq = true;
        if (FAST && !bx) {
            /* TB rows (32 per compute warp) in four chunks, warp w owning
             * rows w, w + nw, ... of each.  The rows overlay the floats: row
             * k (stride above L) covers floats of rows k and later only, and
             * never a float of a lower chunk.  So chunks go highest first,
             * each read into registers before any of its rows is written. */
            const bool full = L == 32 && z.nblk == g.TB && z.e_end - z.e_first == 32ull * g.TB;
            for (int c = 3; c >= 0; c--) {
                float v[8];
                if (full) {
#pragma unroll
                    for (int r = 0; r < 8; r++) v[r] = xin[1 + (warp + (uint32_t)(8 * c + r) * nw) * 32 + lane];
                } else {
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        const uint32_t k = warp + (uint32_t)(8 * c + r) * nw;
                        v[r] = 0.0f;
                        if (k < z.nblk && lane < zg_block_len(z.seg_len, L, z.blk0 + k))
                            v[r] = xin[1 + k * L + lane];
                    }
                }
                named_sync(1, NC);
                if (lane < L) { /* a row holds L floats */
#pragma unroll
                    for (int r = 0; r < 8; r++) rows[(warp + (uint32_t)(8 * c + r) * nw) * stride + lane] = v[r];
                }
            }
            named_sync(1, NC);
        } else if (!FAST) {
            uint32_t amax = abs_bits(xprev0);
            for (uint32_t k = warp; k < z.nblk; k += nw) {
                const uint32_t n = zg_block_len(z.seg_len, L, z.blk0 + k);
                for (uint32_t j = lane; j < n; j += 32) {
                    const float v = xin[1 + k * L + j];
                    amax = max(amax, abs_bits(v));
                    rows[k * stride + j] = v;
                }
            }
            amax = __reduce_max_sync(0xffffffffu, amax);
            if (lane == 0) atomicMax(s_amax, amax);
            named_sync(1, NC);
            fastq = tile_fast_ok(*s_amax, J.inv);
        }

        /* 2. quantize, delta, width.  A full block of up to 32 elements
         *    takes the one-multiply quantization and checks on the way that
         *    every product stayed below 2^24 in magnitude (then it is exact,
         *    and a NaN fails the check); otherwise the block is done again
         *    with the exact quantization. */
        const bool own = tid < z.nblk;
        const uint32_t n = own ? zg_block_len(z.seg_len, L, z.blk0 + tid) : 0u;
        const float *row = rows + tid * stride;
        const uint32_t rb = box_sa + tid * 128u, x4 = (tid & 7u) << 4; /* a box tile: this row */
        uint32_t b = 0, size = 0, smask = 0;
        uint32_t m[32];
        bool done = false;
        if (FAST && own && n == 32) { /* the straight-line path */
            bool ok = true;
            uint32_t mx = 0;
            int32_t qp = 0;
            auto step = [&](float x, int j) {
                const float pz = __fmul_rz(x, J.inv);
                ok = ok && fabsf(pz) < 16777216.0f;
                const int32_t q = __float2int_rz(pz);
                const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                qp = q;
                smask = (smask << 1) | ((uint32_t)d >> 31);
                m[j] = (uint32_t)abs(d); /* |INT_MIN| wraps to 2^31, as in the reference */
                mx = max(mx, m[j]);
            };
            auto first = [&](float x) {
                const float pz = __fmul_rz(x, J.inv);
                ok = fabsf(pz) < 16777216.0f;
                qp = __float2int_rz(pz);
            };
            if (bx) { /* chunk 0 is the element before the block and its first three */
                float4 c = ld_shared_v4(rb | x4);
                /* the last float is the next row's first; row 256 is the 16 bytes after the box */
                float last = __shfl_down_sync(0xffffffffu, c.x, 1);
                if (lane == 31) last = ld_shared_f32(rb + 128u);
                first(c.x);
                step(c.y, 0);
                step(c.z, 1);
                step(c.w, 2);
#pragma unroll
                for (uint32_t k = 1; k < 8; k++) {
                    c = ld_shared_v4(rb | ((k << 4) ^ x4));
                    step(c.x, 4 * k - 1);
                    step(c.y, 4 * k);
                    step(c.z, 4 * k + 1);
                    step(c.w, 4 * k + 2);
                }
                step(last, 31);
            } else {
                first(tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1]);
#pragma unroll
                for (int j = 0; j < 32; j++) step(row[j], j);
            }
            if (ok) {
                b = width_of(mx, a.wt);
                size = g.fmt == ZG_FASTMODE1 ? block32_bytes(b) : zg_block_bytes_f(g.fmt, b, 32);
                done = true;
            }
        }
        if (FAST && own && !done) { /* a short block or the exact quantization */
            /* element j of a box row sits at box float 32 tid + 1 + j */
            auto elem = [&](uint32_t j) -> float {
                if (!bx) return row[j];
                const uint32_t q = 32u * tid + 1u + j, r = q >> 5;
                return ld_shared_f32(box_sa + r * 128u + ((((q >> 2) & 7u) ^ (r & 7u)) << 4) + (q & 3u) * 4u);
            };
            const float xp = bx ? ld_shared_f32(rb | x4) : (tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1]);
            int32_t qp = quantize(xp, J.inv, bad);
            uint32_t mx = 0;
            smask = 0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                m[j] = 0;
                if ((uint32_t)j < n) {
                    const int32_t q = quantize(elem(j), J.inv, bad);
                    const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                    qp = q;
                    smask |= ((uint32_t)d >> 31) << (31 - j);
                    m[j] = (uint32_t)abs(d);
                    mx = max(mx, m[j]);
                }
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes_f(g.fmt, b, n);
        } else if (!FAST && own) { /* blocks above 32 elements: the rows are read again when packing */
            const float xp = tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1];
            int32_t qp = fastq ? quantize_fast(xp, J.inv) : quantize(xp, J.inv, bad);
            uint32_t mx = 0;
            for (uint32_t j = 0; j < n; j++) {
                const int32_t q = fastq ? quantize_fast(row[j], J.inv) : quantize(row[j], J.inv, bad);
                mx = max(mx, (uint32_t)abs((int32_t)((uint32_t)q - (uint32_t)qp)));
                qp = q;
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes_f(g.fmt, b, n);
        }

        /* 3. offsets in the tile and early publication of its size (the
         *    scan's barriers also end every read of the rows above when
         *    L <= 32); the index entries that do not depend on the tile's
         *    place */
        const uint32_t headb = z.has_head ? 4u : 0u;
        uint32_t total;
        const uint32_t off = grp_excl_scan1(size, (it & 1u) ? wsum1 : wsum0, &total, NC, 1);
        total += headb;
        if (warp == 0) lb_publish(J.status, tile, total, tile == 0, 0);
        uint32_t ticket = 0; /* the next tile's, taken now and used after the ring reservation */
        if (tid == 0) ticket = atomicAdd(a.w.ticket, 1u);
        const int32_t qprev0 = quantize(xprev0, J.inv, bad);
        if (own) J.idx.widths[z.gblk0 + tid] = (uint8_t)b;
        if (tid == 0) J.idx.tile_qprev[tile] = qprev0;

        /* 4. take room for the packed tile in the ring (waiting, if need
         *    be, for the placer to write out an earlier one), claim the next
         *    tile (its floats arrive while this one is packed) and pack this
         *    one.  Claiming after any such wait means these warps never wait
         *    while holding a claimed tile whose size is not yet published. */
        if (tid == 0) {
            *s_pos = ring_reserve(ring, it, zg_ring_need(total), R, pos_prev, end_prev, a.w.err);
            if (FAST) claim_tile(a, ticket, in, bar_tma, s_tile, s_job, s_amax, &cj[(it + 1) & 1u], &s_slot[(it + 1) & 1u], box, &xmap);
        }
        named_sync(1, NC);
        const uint32_t pos = *s_pos;
        uint8_t *pk = outb + pos;
        const uint32_t pk_sa = smem_u32(pk); /* zeroed: at the start, then by the placer */
        if (z.has_head && tid == 0) *reinterpret_cast<int32_t *>(pk) = qprev0;
        const uint32_t o = headb + off;
        if (FAST) {
            if (n == 32) {
                if (g.fmt == ZG_FASTMODE1)
                    encode_block32(pk_sa, o, b, smask, m);
                else
                    encode_full(pk_sa, o, b, smask, m, g.fmt);
            } else if (own) {
                encode_any(
                    pk_sa, o, b, n,
                    [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                        neg = (smask >> (31u - j)) & 1u;
                        mg = pick(m, j);
                    },
                    g.fmt);
            }
        } else {
            if (own) {
                const float xp = tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1];
                int32_t qp = fastq ? quantize_fast(xp, J.inv) : quantize(xp, J.inv, bad);
                encode_any(
                    pk_sa, o, b, n,
                    [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                        const int32_t q = fastq ? quantize_fast(row[j], J.inv) : quantize(row[j], J.inv, bad);
                        const int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                        qp = q;
                        neg = (uint32_t)d >> 31;
                        mg = (uint32_t)abs(d);
                    },
                    g.fmt);
            }
            named_sync(1, NC); /* the rows have been read for the last time */
            if (tid == 0) claim_tile(a, ticket, in, bar_tma, s_tile, s_job, s_amax, &cj[(it + 1) & 1u], &s_slot[(it + 1) & 1u], box, &xmap);
        }
        named_sync(1, NC); /* the packed tile is complete; the claimed index is visible */
        if (tid == 0) ring_publish(ring, it, tile, job, total, pos);
        tile = *s_tile;
        job = *s_job;
    }
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_compress(const CompressArgs &a, cudaStream_t st)
{
    const bool fast = a.job.g.L <= 32;
    const void *fn = fast ? (const void *)k_compress<true> : (const void *)k_compress<false>;
    cudaError_t e = set_max_smem(fn, a.sm.total);
    if (e != cudaSuccess) return e;
    const unsigned threads = a.job.g.TB + 32; /* compute warps and the placer warp */
    const uint64_t tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    unsigned grid = persistent_grid(fn, threads, a.sm.total, tiles);
    if (a.grid && a.grid < grid) grid = a.grid;
    CompressArgs b = a;
    alignas(64) CUtensorMap map;
    memset(&map, 0, sizeof map);
    b.rows_map = fast && (a.batch.jobs ? a.batch.maps != nullptr : zk_rows_map(&map, a.job.x, a.job.g.n, 256));
    if (fast)
        k_compress<true><<<grid, threads, a.sm.total, st>>>(b, map);
    else
        k_compress<false><<<grid, threads, a.sm.total, st>>>(b, map);
    return cudaGetLastError();
}
