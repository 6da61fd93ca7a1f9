/*
 * zk_homadd.cu -- homomorphic add of P compressed streams in one pass.
 *
 * Replaces ZCCL_float_homomophic_add_openmp_threadblock
 * (ZCCL/src/ZCCLd_float.c:988-1679).  The reference result is the canonical
 * encoding of the summed int32 deltas with int32-added heads
 * (ZCCLd_float.c:1072, :1172-1219; a zero-width side is copied verbatim,
 * :1103-1153, which is the same bytes because every input block is itself
 * canonical).  Integer addition is associative modulo 2^32, so one pass over
 * P inputs equals the ring's pairwise fold in any order, bit for bit.
 *
 * Persistent CTAs take tiles in ticket order, one compute thread per block
 * plus one placer warp.  A tile's P inputs form a stream of TMA copies
 * through two buffers: while one input's tile bytes are unpacked and added
 * into per-thread registers, the next input's sizes are scanned from its
 * width index and its bytes are already in flight.  Zero-width input blocks
 * are skipped without touching their bytes.  After the last input the sum
 * is re-encoded like the compressor does (width, scan, early look-back
 * publish, packing), and the placer warp finds its place in the stream with
 * the look-back and writes it out while the compute warps add the next
 * tile.  The starting value per tile is the sum of the inputs' values.
 */
#include "zkern.cuh"

namespace {

struct BlockSlot {
    uint32_t b, n, off;
};

/* Thread 0: the TMA copy of `total` bytes of an input tile at byte `base`
 * (from the index, so checked against the readable bytes) into buf. */
__device__ __forceinline__ void issue_input(const HomInput &in, uint64_t base, uint32_t total, uint8_t *buf,
                                            uint64_t *bar, uint64_t *s_base, uint32_t &bad)
{
    uint32_t nload = total;
    /* overflow-safe: base comes from the index and is not trusted */
    if (base > in.avail || total > in.avail - base) {
        bad |= ZERR_BOUNDS;
        nload = base < in.avail ? (uint32_t)min((uint64_t)total, in.avail - base) : 0u;
        if (base > in.avail) base = 0;
    }
    *s_base = base;
    tma_load_superset(buf, in.bytes + base, nload, bar);
}

/* The compute threads: sizes of input p's blocks in tile t, their offsets,
 * and (thread 0) the TMA copy of those bytes into buf. */
__device__ __forceinline__ BlockSlot stage_input(const HomAddJob &J, uint64_t t, uint32_t p,
                                                 uint8_t *buf, uint64_t *bar, uint32_t *wsum,
                                                 uint64_t *s_base, uint32_t &bad)
{
    const HomInput &in = J.in[p];
    BlockSlot sl = {0, 0, 0};
    ZTile z;
    zg_tile(&J.g, t, &z);
    uint32_t size = 0;
    if (threadIdx.x < z.nblk) {
        sl.n = zg_block_len(z.seg_len, J.g.L, z.blk0 + threadIdx.x);
        sl.b = in.widths[z.gblk0 + threadIdx.x];
        if (sl.b > 32) {
            bad |= ZERR_CORRUPT;
            sl.b = 0;
        }
        size = zg_block_bytes(sl.b, sl.n);
    }
    uint64_t base0 = 0;
    if (threadIdx.x == 0) base0 = in.tile_off[t]; /* on its way during the scan */
    uint32_t total;
    sl.off = grp_excl_scan(size, wsum, &total, J.g.TB, 1);
    if (threadIdx.x == 0) issue_input(in, base0, total + (z.has_head ? 4u : 0u), buf, bar, s_base, bad);
    return sl;
}

/* One thread: a job into shared memory, with only the inputs it uses. */
__device__ __forceinline__ void copy_job(HomAddJob *dst, const HomAddJob *src)
{
    const uint32_t P = src->P < ZH_MAXP ? src->P : ZH_MAXP;
    copy16(dst, src, (uint32_t)offsetof(HomAddJob, in));
    copy16(&dst->in[0], &src->in[0], (uint32_t)((P * sizeof(HomInput) + 15u) & ~15u));
    copy16(&dst->P, &src->P, (uint32_t)(sizeof(HomAddJob) - offsetof(HomAddJob, P)));
}

/* Thread 0: ticket t (taken a little earlier, so that the atomic's latency
 * overlaps other work) becomes the claimed tile: its job is copied into
 * `slot`, the tile within its job lands in *s_tile (ZP_NONE when all are
 * taken), the job in *s_job.  The caller synchronises before reading them. */
__device__ __forceinline__ void take_ticket(const HomAddArgs &a, uint64_t t, uint64_t *s_tile, uint32_t *s_job,
                                            HomAddJob *slot)
{
    if (threadIdx.x != 0) return;
    const uint64_t total = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    if (t >= total) {
        *s_tile = ZP_NONE;
        return;
    }
    uint64_t local;
    const uint32_t j = batch_job(a.batch, t, &local);
    copy_job(slot, a.batch.jobs ? static_cast<const HomAddJob *>(a.batch.jobs) + j : &a.job);
    *s_tile = local;
    *s_job = j;
}

/* Block size TB + 32: warps 0 .. TB/32 - 1 add (one thread per block of the
 * tile), the last warp places packed sums in the stream. */
template <bool FAST>
__global__ void __launch_bounds__(288, 2) k_homadd(const __grid_constant__ HomAddArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);          /* [2] input copies */
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 32);    /* [33] */
    uint64_t *s_tile = reinterpret_cast<uint64_t *>(smem + 168); /* the claimed tile (within its job) */
    uint32_t *s_pos = reinterpret_cast<uint32_t *>(smem + 176);  /* ring position of this sum */
    uint32_t *s_job = reinterpret_cast<uint32_t *>(smem + 180);  /* the claimed tile's job */
    uint64_t *s_base = reinterpret_cast<uint64_t *>(smem + 192); /* [2] */
    ZRing *ring = reinterpret_cast<ZRing *>(smem + 256);
    HomAddJob *hj = reinterpret_cast<HomAddJob *>(smem + a.sm.jobs); /* [2], by round */
    ZPlace *pj = reinterpret_cast<ZPlace *>(smem + a.sm.jobs + 2 * sizeof(HomAddJob));
    uint32_t *acc_rows = reinterpret_cast<uint32_t *>(smem + a.sm.rows);
    uint8_t *outs = smem + a.sm.out; /* the ring of packed sums */

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t NC = blockDim.x - 32; /* compute threads (TB) */
    const uint32_t L = a.job.g.L, stride = zg_row_stride(L); /* one L for the whole batch */
    uint32_t bad = 0;
    /* see k_decompress: a failed index walk stops every CTA alike */
    if (*(volatile const uint32_t *)a.w.walk_err) return;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        ring->packed = 0;
        ring->placed = 0;
    }
    __syncthreads();

    if (tid >= NC) { /* the placer warp */
        const uint64_t max_tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
        placer_loop(ring, outs, pj, a.w.err, max_tiles, bad, [&](uint32_t j, ZPlace *p) {
            if (a.batch.jobs) {
                const HomAddJob &J = static_cast<const HomAddJob *>(a.batch.jobs)[j];
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

    /* the compute warps.  Tiles are claimed one at a time when these warps
     * are ready for them, and they never wait while holding a claimed tile
     * whose size is not yet published. */
    uint32_t *ws1 = reinterpret_cast<uint32_t *>(smem + 320); /* [33] second scan scratch */
    uint8_t *const buf0 = smem + a.sm.in0, *const buf1 = smem + a.sm.in1;
    uint32_t acc[32];
    uint32_t ld = 0; /* index of the current copy in the two-buffer stream */
    const uint32_t R = zg_ring_bytes(L, NC);
    uint32_t pos_prev = 0, end_prev = 0; /* thread 0: the previous sum's place in the ring */
    if (tid == 0) take_ticket(a, atomicAdd(a.w.ticket, 1u), s_tile, s_job, &hj[0]);
    named_sync(1, NC);
    uint64_t tile = *s_tile;
    uint32_t job = *s_job;
    BlockSlot cur = {0, 0, 0};
    if (tile != ZP_NONE) cur = stage_input(hj[0], tile, 0, smem + a.sm.in0, &bar[0], wsum, &s_base[0], bad);

    for (uint32_t it = 0;; it++) {
        if (tile == ZP_NONE) {
            /* tell the placer there is nothing more (once it has read the slot) */
            if (tid == 0) {
                ring_wait(&ring->placed, it >= 1 ? it - 1 : 0u, a.w.err);
                ring_publish(ring, it, ZP_NONE, 0, 0, 0);
            }
            break;
        }
        const HomAddJob &J = hj[it & 1u];
        const ZGeom &g = J.g;
        const uint32_t P = J.P;
        ZTile z;
        zg_tile(&g, tile, &z);
        const bool own = tid < z.nblk;
        const uint32_t n = cur.n;
        const bool full = FAST && own && n == 32;
        if (FAST) {
#pragma unroll
            for (int j = 0; j < 32; j++) acc[j] = 0;
        } else if (own) {
            for (uint32_t j = 0; j < n; j++) acc_rows[tid * stride + j] = 0;
        }
        uint32_t hsum = 0, qsum = 0, nzmask = 0;
        const uint32_t headb = z.has_head ? 4u : 0u;

        uint32_t ticket = 0; /* the next tile's, taken before the last input and used after it */
        for (uint32_t p = 0; p < P; p++, ld++) {
            const uint32_t cb = ld & 1u;
            if (p + 1 == P && tid == 0) ticket = atomicAdd(a.w.ticket, 1u);
            /* the next input's copy runs while this one is added */
            BlockSlot nxt = {0, 0, 0};
            if (p + 1 < P)
                nxt = stage_input(J, tile, p + 1, smem + (cb ? a.sm.in0 : a.sm.in1), &bar[cb ^ 1u],
                                  wsum, &s_base[cb ^ 1u], bad);
            if (J.qprev_valid && tid == 0) qsum += (uint32_t)J.in[p].tile_qprev[tile];
            mbar_wait(&bar[cb], (ld >> 1) & 1u, a.w.err);
            const uint8_t *buf = smem + (cb ? a.sm.in1 : a.sm.in0);
            const uint32_t *sw = reinterpret_cast<const uint32_t *>(buf);
            const uint32_t ph = (uint32_t)((uintptr_t)(J.in[p].bytes + s_base[cb]) & 15u);
            if (z.has_head && tid == 0) {
                uint32_t h = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) h |= (uint32_t)buf[ph + k] << (8 * k);
                hsum += h;
            }
            if (own) {
                const uint32_t b = cur.b, o = ph + headb + cur.off;
                if (buf[o] != b) bad |= ZERR_CORRUPT;
                if (b) {
                    nzmask |= 1u << (p & 31);
                    if (full) {
                        uint32_t v[32];
                        decode_full(sw, o, b, v);
#pragma unroll
                        for (int j = 0; j < 32; j++) acc[j] += v[j];
                    } else if (FAST) {
                        decode_any(sw, o, b, n, [&](uint32_t j, uint32_t v) { add_at(acc, j, v); });
                    } else {
                        decode_any(sw, o, b, n,
                                   [&](uint32_t j, uint32_t v) { acc_rows[tid * stride + j] += v; });
                    }
                }
            }
            cur = nxt;
            /* the buffer just read is refilled by the copy staged next round,
             * after that round's scan has synchronised every compute thread */
        }

        /* the claimed next tile: its first input's widths and offset load
         * while this sum's widths are found */
        HomAddJob &Jn = hj[(it + 1) & 1u];
        take_ticket(a, ticket, s_tile, s_job, &Jn);
        named_sync(1, NC);
        const uint64_t next = *s_tile;
        const uint32_t next_job = *s_job;
        ZTile zn;
        uint32_t wn = 0, nn = 0;
        uint64_t basen = 0;
        if (next != ZP_NONE) {
            zg_tile(&Jn.g, next, &zn);
            if (tid < zn.nblk) {
                nn = zg_block_len(zn.seg_len, Jn.g.L, zn.blk0 + tid);
                wn = Jn.in[0].widths[zn.gblk0 + tid];
            }
            if (tid == 0) basen = Jn.in[0].tile_off[next];
        }

        /* branch-case counters of the two-input add (ZCCLd_float.c:2175-2764) */
        if (a.cases && P == 2) {
            const uint32_t c0 = __popc(__ballot_sync(0xffffffffu, own && nzmask == 0u));
            const uint32_t c1 = __popc(__ballot_sync(0xffffffffu, own && nzmask == 2u));
            const uint32_t c2 = __popc(__ballot_sync(0xffffffffu, own && nzmask == 1u));
            const uint32_t c3 = __popc(__ballot_sync(0xffffffffu, own && nzmask == 3u));
            if (lane == 0) {
                atomicAdd(a.cases + 0, (unsigned long long)c0);
                atomicAdd(a.cases + 1, (unsigned long long)c1);
                atomicAdd(a.cases + 2, (unsigned long long)c2);
                atomicAdd(a.cases + 3, (unsigned long long)c3);
            }
        }
        /* width of the sum, offsets in the tile, early size publication */
        uint32_t b = 0, size = 0, smask = 0;
        if (full) {
            uint32_t mx = 0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                smask = (smask << 1) | (acc[j] >> 31);
                acc[j] = (uint32_t)abs((int32_t)acc[j]);
                mx = max(mx, acc[j]);
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes(b, 32);
        } else if (own) {
            uint32_t mx = 0;
            for (uint32_t j = 0; j < n; j++) {
                const uint32_t v = FAST ? pick(acc, j) : acc_rows[tid * stride + j];
                mx = max(mx, (uint32_t)abs((int32_t)v));
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes(b, n);
        }
        /* one scan for this sum's block offsets and the next tile's first input's */
        uint32_t sizen = 0;
        if (wn > 32) {
            bad |= ZERR_CORRUPT;
            wn = 0;
        }
        if (next != ZP_NONE && tid < zn.nblk) sizen = zg_block_bytes(wn, nn);
        uint32_t total, off, offn, totaln;
        grp_excl_scan2(size, sizen, wsum, ws1, off, offn, total, totaln, NC, 1);
        total += headb;
        if (next != ZP_NONE) { /* every input of this tile is decoded: the buffer is free */
            if (tid == 0)
                issue_input(Jn.in[0], basen, totaln + (zn.has_head ? 4u : 0u), ld & 1u ? buf1 : buf0,
                            &bar[ld & 1u], &s_base[ld & 1u], bad);
            cur.b = wn;
            cur.n = nn;
            cur.off = offn;
        }
        if (warp == 0) lb_publish(J.status, tile, total, tile == 0, 0);
        if (own) J.idx.widths[z.gblk0 + tid] = (uint8_t)b;
        if (tid == 0 && J.qprev_valid) J.idx.tile_qprev[tile] = (int32_t)qsum;

        /* take room for the packed sum in the ring (waiting, if need be, for
         * the placer to write out an earlier one) and pack this sum while
         * the next tile's first input arrives */
        if (tid == 0) *s_pos = ring_reserve(ring, it, zg_ring_need(total), R, pos_prev, end_prev, a.w.err);
        named_sync(1, NC);
        const uint32_t pos = *s_pos;
        uint8_t *pk = outs + pos;
        const uint32_t pk_sa = smem_u32(pk);
        smem_zero(pk, total + 8, tid, NC);
        named_sync(1, NC);
        if (z.has_head && tid == 0) *reinterpret_cast<uint32_t *>(pk) = hsum;
        const uint32_t o = headb + off;
        if (full) {
            encode_full(pk_sa, o, b, smask, acc);
        } else if (own) {
            encode_any(pk_sa, o, b, n, [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                const uint32_t v = FAST ? pick(acc, j) : acc_rows[tid * stride + j];
                neg = v >> 31;
                mg = (uint32_t)abs((int32_t)v);
            });
        }
        named_sync(1, NC); /* the packed sum is complete; acc_rows are free */
        if (tid == 0) ring_publish(ring, it, tile, job, total, pos);
        tile = next;
        job = next_job;
    }
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_homadd(const HomAddArgs &a, cudaStream_t st)
{
    const bool fast = a.job.g.L <= 32;
    const void *fn = fast ? (const void *)k_homadd<true> : (const void *)k_homadd<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.sm.total);
    if (e != cudaSuccess) return e;
    const unsigned threads = a.job.g.TB + 32; /* compute warps and the placer warp */
    const uint64_t tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    unsigned grid = persistent_grid(fn, threads, a.sm.total, tiles);
    if (a.grid && a.grid < grid) grid = a.grid;
    if (fast)
        k_homadd<true><<<grid, threads, a.sm.total, st>>>(a);
    else
        k_homadd<false><<<grid, threads, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
