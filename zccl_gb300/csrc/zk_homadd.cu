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
 * Persistent CTAs take tiles in ticket order with three kinds of warps.  A
 * loader warp turns every input of every claimed tile into one TMA copy
 * into one of two buffers, with a table of each block's offset and width
 * found from the input's width index.  The adding warps, one thread per
 * block, unpack their block of each input as it arrives and add it into
 * registers (zero-width blocks are skipped without touching their bytes),
 * handing each buffer back through an mbarrier.  After the last input the
 * sum is re-encoded like the compressor does (width, scan, early look-back
 * publish, packing into a shared-memory ring), and the placer warp finds its
 * place in the stream with the look-back and writes it out while the adding
 * warps go on.  The starting value per tile is the sum of the inputs'
 * values.
 */
#include "zkern.cuh"

namespace {

/* The job of batch ticket j (or the single job), read in place. */
__device__ __forceinline__ const HomAddJob &job_of(const HomAddArgs &a, uint32_t j)
{
    return a.batch.jobs ? static_cast<const HomAddJob *>(a.batch.jobs)[j] : a.job;
}

/* The loader warp.  It claims tiles in ticket order and, for every input of
 * every claimed tile, finds each block's width and offset from the input's
 * width index (eight blocks per lane and a warp scan), waits for a free
 * buffer, writes them into the buffer's block table (offset << 8 | width),
 * and starts one TMA copy of the tile's bytes; the copy's mbarrier tells the
 * adding warps.  After the last tile it hands over a stage marked ZP_NONE.
 *
 * For a single job the work is software-pipelined one copy ahead: the next
 * copy's tile is claimed and resolved (its geometry comes from the kernel's
 * parameters) and its offset and widths are requested before the current
 * copy is scanned, awaited and started, so their latency overlaps that work
 * instead of adding up once per copy (instrumented, the adding warps had
 * waited for inputs 28 % of their time without it).  A tile is claimed only
 * when it is about to be prepared: a ticket held longer lengthens the other
 * CTAs' look-backs.  A claimed tile is always processed, in order, and the
 * adding warps never wait on another CTA before they publish their tile's
 * size, so every look-back wait ends.  Batches use loader_loop_batch. */
template <bool FAST>
__device__ __forceinline__ void loader_loop(const HomAddArgs &a, uint8_t *buf0, uint8_t *buf1, HStage *stage,
                                            HTile *td, uint32_t *btab0, uint32_t *btab1, uint64_t *full,
                                            uint64_t *empty, uint32_t &bad)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t ntiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    const uint32_t L = a.job.g.L;

    /* the prepared copy: tile nt of job nj, input np of nP */
    uint64_t nt = 0, nbase = 0;
    uint32_t nj = 0, np = 0, nP = 0, nq = 0, nbw[8];
    ZTile nz;
    /* claim and resolve the next tile as the prepared copy's (input 0);
     * false when every tile is taken */
    auto open_next = [&]() -> bool {
        uint64_t tk = 0, t = 0;
        uint32_t j = 0;
        if (lane == 0) {
            tk = atomicAdd(a.w.ticket, 1u);
            if (tk < ntiles) j = batch_job(a.batch, tk, &t);
        }
        tk = __shfl_sync(0xffffffffu, tk, 0);
        if (tk >= ntiles) return false;
        nt = __shfl_sync(0xffffffffu, t, 0);
        nj = __shfl_sync(0xffffffffu, j, 0);
        np = 0;
        const HomAddJob &J = job_of(a, nj);
        zg_tile(&J.g, nt, &nz);
        nP = J.P;
        nq = J.qprev_valid && lane < nP ? (uint32_t)J.in[lane].tile_qprev[nt] : 0u;
        return true;
    };
    /* request the prepared copy's tile offset and block widths */
    auto request = [&]() {
        const HomInput &in = job_of(a, nj).in[np];
        if (lane == 0) nbase = in.tile_off[nt];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t i = 8u * lane + (uint32_t)k;
            nbw[k] = i < nz.nblk ? (uint32_t)in.widths[nz.gblk0 + i] : 0u;
        }
    };

    bool have = open_next();
    if (have) request();
    uint32_t seq = 0, ti = 0; /* copies handed over, tiles opened */
    while (have) {
        /* the current copy is the prepared one */
        const uint64_t t = nt;
        const uint32_t j = nj, p = np, P = nP, qv = nq;
        const ZTile z = nz;
        uint64_t base = nbase;
        uint32_t bw[8];
#pragma unroll
        for (int k = 0; k < 8; k++) bw[k] = nbw[k];

        /* prepare the next copy: the next input of this tile, or the next tile */
        const bool last = p + 1 >= P;
        bool next = true;
        if (!last) {
            np = p + 1;
            request();
        } else {
            next = open_next();
            if (next) request();
        }

        /* hand over the current copy */
        const HomAddJob &J = job_of(a, j);
        const HomInput &in = J.in[p];
        uint32_t off[8], sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t i = 8u * lane + (uint32_t)k;
            uint32_t size = 0;
            if (i < z.nblk) {
                if (bw[k] > 32) {
                    bad |= ZERR_CORRUPT;
                    bw[k] = 0;
                }
                size = zg_block_bytes(bw[k], zg_block_len(z.seg_len, L, z.blk0 + i));
            }
            off[k] = sum;
            sum += size;
        }
        const uint32_t incl = warp_incl_scan(sum);
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31) + (z.has_head ? 4u : 0u);
        const uint32_t qsum = p == 0 ? __reduce_add_sync(0xffffffffu, qv) : 0u;
        const uint32_t s = seq & 1u;
        if (seq >= 2) mbar_wait(&empty[s], ((seq >> 1) + 1u) & 1u, a.w.err); /* copy seq - 2 consumed */
        if (p == 0 && lane == 0) { /* the tile's record, before its first copy is handed over */
            HTile &d = td[ti % ZH_TILE_RECS];
            d.gblk0 = z.gblk0;
            d.widths = J.idx.widths;
            d.tile_qprev = J.qprev_valid ? J.idx.tile_qprev : nullptr;
            d.status = J.status;
            d.P = P;
            d.nblk = z.nblk;
            d.nlast = z.nblk ? zg_block_len(z.seg_len, L, z.blk0 + z.nblk - 1) : 0u;
            d.has_head = z.has_head;
            d.qsum = qsum;
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t i = 8u * lane + (uint32_t)k;
            if (i < z.nblk) (s ? btab1 : btab0)[i] = (incl - sum + off[k]) << 8 | bw[k];
        }
        __syncwarp();
        if (lane == 0) {
            uint32_t nload = total;
            /* overflow-safe: base comes from the index and is not trusted */
            if (base > in.avail || total > in.avail - base) {
                bad |= ZERR_BOUNDS;
                nload = base < in.avail ? (uint32_t)min((uint64_t)total, in.avail - base) : 0u;
                if (base > in.avail) base = 0;
            }
            stage[s].tile = t;
            stage[s].job = j;
            stage[s].p = p;
            stage[s].ph = (uint32_t)((uintptr_t)(in.bytes + base) & 15u);
            tma_load_superset(s ? buf1 : buf0, in.bytes + base, nload, &full[s]);
        }
        seq++;
        if (last) ti++;
        have = next;
    }
    /* no more tiles */
    const uint32_t s = seq & 1u;
    if (seq >= 2) mbar_wait(&empty[s], ((seq >> 1) + 1u) & 1u, a.w.err);
    if (lane == 0) {
        stage[s].tile = ZP_NONE;
        mbar_arrive(&full[s]);
    }
}

/* The loader for a batch: the same hand-over without the pipelining of
 * loader_loop.  Measured on the 2048-pair gradient-bucket batch, whose tiles
 * mostly belong to different small jobs, the pipelined form's job lookups
 * (dependent loads from the batch's job table) cost more than its overlap
 * gains: the sum batch ran 6.1-6.9 ms against 5.1 ms with this loop. */
__device__ __forceinline__ void loader_loop_batch(const HomAddArgs &a, uint8_t *buf0, uint8_t *buf1, HStage *stage,
                                            HTile *td, uint32_t *btab0, uint32_t *btab1, uint64_t *full,
                                            uint64_t *empty, uint32_t &bad)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t ntiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    uint32_t seq = 0; /* copies handed over so far */
    for (uint32_t ti = 0;; ti++) {
        uint64_t t = 0, tk = 0;
        uint32_t j = 0;
        if (lane == 0) {
            tk = atomicAdd(a.w.ticket, 1u);
            if (tk < ntiles) j = batch_job(a.batch, tk, &t);
        }
        tk = __shfl_sync(0xffffffffu, tk, 0);
        if (tk >= ntiles) {
            const uint32_t s = seq & 1u;
            if (seq >= 2) mbar_wait(&empty[s], ((seq >> 1) + 1u) & 1u, a.w.err);
            if (lane == 0) {
                stage[s].tile = ZP_NONE;
                mbar_arrive(&full[s]);
            }
            return;
        }
        t = __shfl_sync(0xffffffffu, t, 0);
        j = __shfl_sync(0xffffffffu, j, 0);
        const HomAddJob &J = job_of(a, j);
        ZTile z;
        zg_tile(&J.g, t, &z);
        const uint32_t P = J.P;
        for (uint32_t p = 0; p < P; p++, seq++) {
            const HomInput &in = J.in[p];
            uint64_t base = 0;
            if (lane == 0) base = in.tile_off[t];
            uint32_t bw[8], off[8], sum = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t i = 8u * lane + (uint32_t)k;
                uint32_t b = 0, size = 0;
                if (i < z.nblk) {
                    b = in.widths[z.gblk0 + i];
                    if (b > 32) {
                        bad |= ZERR_CORRUPT;
                        b = 0;
                    }
                    size = zg_block_bytes(b, zg_block_len(z.seg_len, J.g.L, z.blk0 + i));
                }
                bw[k] = b;
                off[k] = sum;
                sum += size;
            }
            const uint32_t incl = warp_incl_scan(sum);
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31) + (z.has_head ? 4u : 0u);
            const uint32_t s = seq & 1u;
            if (seq >= 2) mbar_wait(&empty[s], ((seq >> 1) + 1u) & 1u, a.w.err); /* copy seq - 2 consumed */
            if (p == 0 && lane == 0) { /* the tile's record, before its first copy is handed over */
                HTile &d = td[ti % ZH_TILE_RECS];
                uint32_t qsum = 0;
                if (J.qprev_valid)
                    for (uint32_t q = 0; q < P; q++) qsum += (uint32_t)J.in[q].tile_qprev[t];
                d.gblk0 = z.gblk0;
                d.widths = J.idx.widths;
                d.tile_qprev = J.qprev_valid ? J.idx.tile_qprev : nullptr;
                d.status = J.status;
                d.P = P;
                d.nblk = z.nblk;
                d.nlast = z.nblk ? zg_block_len(z.seg_len, J.g.L, z.blk0 + z.nblk - 1) : 0u;
                d.has_head = z.has_head;
                d.qsum = qsum;
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t i = 8u * lane + (uint32_t)k;
                if (i < z.nblk) (s ? btab1 : btab0)[i] = (incl - sum + off[k]) << 8 | bw[k];
            }
            __syncwarp();
            if (lane == 0) {
                uint32_t nload = total;
                /* overflow-safe: base comes from the index and is not trusted */
                if (base > in.avail || total > in.avail - base) {
                    bad |= ZERR_BOUNDS;
                    nload = base < in.avail ? (uint32_t)min((uint64_t)total, in.avail - base) : 0u;
                    if (base > in.avail) base = 0;
                }
                stage[s].tile = t;
                stage[s].job = j;
                stage[s].p = p;
                stage[s].ph = (uint32_t)((uintptr_t)(in.bytes + base) & 15u);
                tma_load_superset(s ? buf1 : buf0, in.bytes + base, nload, &full[s]);
            }
        }
    }
}

/* Block size TB + 64: warps 0 .. TB/32 - 1 add (one thread per block of the
 * tile), warp TB/32 places packed sums in the stream, warp TB/32 + 1 loads
 * the inputs.  The adding warps meet at one barrier per tile (the scan of
 * the sum's block sizes); inputs arrive and buffers are returned through
 * mbarriers, and packed sums go to the placer through a per-slot mbarrier
 * that every adding warp arrives on. */
template <bool FAST>
__global__ void __launch_bounds__(320, 2) k_homadd(const __grid_constant__ HomAddArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem);        /* [2] input copy arrived */
    uint64_t *empty = reinterpret_cast<uint64_t *>(smem + 16);  /* [2] input buffer consumed */
    uint32_t *wsum0 = reinterpret_cast<uint32_t *>(smem + 48);  /* [33] scan scratch, even tiles */
    uint32_t *wsum1 = reinterpret_cast<uint32_t *>(smem + 184); /* [33] odd tiles */
    static_assert(320 + sizeof(ZRing4) <= 1024, "the ring's control block fits below the rows");
    ZRing4 *ring = reinterpret_cast<ZRing4 *>(smem + 320);
    ZPlace *pj = reinterpret_cast<ZPlace *>(smem + a.sm.jobs);
    HStage *stage = reinterpret_cast<HStage *>(smem + a.sm.jobs + zg_a16(sizeof(ZPlace))); /* [2] */
    HTile *td = reinterpret_cast<HTile *>(stage + 2); /* [ZH_TILE_RECS] */
    uint32_t *const btab0 = reinterpret_cast<uint32_t *>(td + ZH_TILE_RECS), *const btab1 = btab0 + a.job.g.TB;
    uint32_t *acc_rows = reinterpret_cast<uint32_t *>(smem + a.sm.rows);
    uint8_t *outs = smem + a.sm.out; /* the ring of packed sums */
    uint8_t *const buf0 = smem + a.sm.in0, *const buf1 = smem + a.sm.in1;

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t NC = blockDim.x - 64, nwc = NC >> 5; /* adding threads (TB), adding warps */
    const uint32_t L = a.job.g.L, stride = zg_row_stride(L); /* one L for the whole batch */
    const uint32_t R = a.sm.jobs - a.sm.out - 48u; /* the ring: every byte up to the job region, less the slack */
    uint32_t bad = 0;
    /* see k_decompress: a failed index walk stops every CTA alike */
    if (*(volatile const uint32_t *)a.w.walk_err) return;
    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&empty[0], nwc);
        mbar_init(&empty[1], nwc);
        ring4_init(ring, nwc);
    }
    /* the ring starts zeroed, and the placer zeroes what it has written out */
    for (uint32_t i = tid; i < (R + 48u) / 16u; i += blockDim.x) reinterpret_cast<uint4 *>(outs)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();

    if (warp == nwc) { /* the placer warp */
        const uint64_t max_tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
        placer_loop4(ring, outs, pj, a.w.err, max_tiles, bad, a.w.lb_spin, [&](uint32_t j, ZPlace *p) {
                const HomAddJob &J = job_of(a, j);
                p->g = J.g;
                p->out = J.out;
                p->cap = J.cap;
                p->idx = J.idx;
                p->status = J.status;
            });
        if (bad) atomicOr(a.w.err, bad);
        return;
    }
    if (warp == nwc + 1) { /* the loader warp */
        if (a.batch.jobs)
            loader_loop_batch(a, buf0, buf1, stage, td, btab0, btab1, full, empty, bad);
        else
            loader_loop<FAST>(a, buf0, buf1, stage, td, btab0, btab1, full, empty, bad);
        if (bad) atomicOr(a.w.err, bad);
        return;
    }

    /* the adding warps */
    uint32_t acc[32];
    uint32_t seq = 0;                    /* input copies consumed */
    uint32_t H = 0, hp = 0; /* ring bytes taken and the ring's next position (the same in every thread) */
    const uint64_t max_tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    for (uint32_t it = 0; it <= max_tiles; it++) { /* bounded even if a wait gave up */
        uint32_t s = seq & 1u;
        mbar_wait(&full[s], (seq >> 1) & 1u, a.w.err);
        const uint64_t tile = stage[s].tile;
        if (tile == ZP_NONE) {
            if (tid == 0) ring4_sized(ring, it, ZP_NONE, 0, 0, a.w.err); /* nothing more */
            break;
        }
        const uint32_t job = stage[s].job;
        const HTile &D = td[it % ZH_TILE_RECS];
        const uint32_t P = D.P, nblk = D.nblk;
        const bool has_head = D.has_head != 0;
        const bool own = tid < nblk;
        const uint32_t n = !own ? 0u : tid + 1u < nblk ? L : D.nlast;
        const bool full32 = FAST && own && n == 32;
        if (FAST) {
#pragma unroll
            for (int j = 0; j < 32; j++) acc[j] = 0;
        } else if (own) {
            for (uint32_t j = 0; j < n; j++) acc_rows[tid * stride + j] = 0;
        }
        uint32_t hsum = 0, nzmask = 0;
        const uint32_t headb = has_head ? 4u : 0u;

        for (uint32_t p = 0; p < P; p++, seq++) {
            s = seq & 1u;
            if (p) mbar_wait(&full[s], (seq >> 1) & 1u, a.w.err);
            const uint8_t *buf = s ? buf1 : buf0;
            const uint32_t *sw = reinterpret_cast<const uint32_t *>(buf);
            const uint32_t ph = stage[s].ph;
            if (has_head && tid == 0) {
                uint32_t h = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) h |= (uint32_t)buf[ph + k] << (8 * k);
                hsum += h;
            }
            if (own) {
                const uint32_t e = (s ? btab1 : btab0)[tid], b = e & 0xFFu, o = ph + headb + (e >> 8);
                if (buf[o] != b) bad |= ZERR_CORRUPT;
                if (b) {
                    nzmask |= 1u << (p & 31);
                    if (full32) {
                        decode_add_full(sw, o, b, acc);
                    } else if (FAST) {
                        decode_any(sw, o, b, n, [&](uint32_t j, uint32_t v) { add_at(acc, j, v); });
                    } else {
                        decode_any(sw, o, b, n,
                                   [&](uint32_t j, uint32_t v) { acc_rows[tid * stride + j] += v; });
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]); /* this warp is done with the buffer */
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
        if (full32) {
            uint32_t mx = 0;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                smask = __funnelshift_l(acc[j], smask, 1); /* (smask << 1) | sign of element j */
                acc[j] = (uint32_t)abs((int32_t)acc[j]);
                mx = max(mx, acc[j]);
            }
            b = width_of(mx, a.wt);
            size = block32_bytes(b);
        } else if (own) {
            uint32_t mx = 0;
            for (uint32_t j = 0; j < n; j++) {
                const uint32_t v = FAST ? pick(acc, j) : acc_rows[tid * stride + j];
                mx = max(mx, (uint32_t)abs((int32_t)v));
            }
            b = width_of(mx, a.wt);
            size = zg_block_bytes(b, n);
        }
        uint32_t total;
        const uint32_t off = grp_excl_scan1(size, (it & 1u) ? wsum1 : wsum0, &total, NC, 1);
        total += headb;
        if (warp == 0) lb_publish(D.status, tile, total, tile == 0, 0);
        if (tid == 0) ring4_sized(ring, it, tile, job, total, a.w.err); /* the placer's look-back starts */
        if (own) D.widths[D.gblk0 + tid] = (uint8_t)b;
        if (tid == 0 && D.tile_qprev) D.tile_qprev[tile] = (int32_t)D.qsum;

        /* room for the packed sum in the ring: every thread finds the same
         * place and waits, if need be, for the placer to have written out
         * (and zeroed) what was there */
        uint32_t mend;
        const uint32_t pos = ring4_space(ring, zg_ring_need(total), R, H, hp, mend, a.w.err);
        uint8_t *pk = outs + pos;
        const uint32_t pk_sa = smem_u32(pk);
        if (has_head && tid == 0) *reinterpret_cast<uint32_t *>(pk) = hsum;
        const uint32_t o = headb + off;
        if (full32) {
            encode_block32(pk_sa, o, b, smask, acc);
        } else if (own) {
            encode_any(pk_sa, o, b, n, [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                const uint32_t v = FAST ? pick(acc, j) : acc_rows[tid * stride + j];
                neg = v >> 31;
                mg = (uint32_t)abs((int32_t)v);
            });
        }
        if (tid == 0) ring4_where(ring, it, pos, mend);
        __syncwarp();
        if (lane == 0) mbar_arrive(&ring->packed[it % ZR_SLOTS]); /* this warp's blocks are packed */
    }
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_homadd(const HomAddArgs &a, cudaStream_t st)
{
    const bool fast = a.job.g.L <= 32;
    const void *fn = fast ? (const void *)k_homadd<true> : (const void *)k_homadd<false>;
    cudaError_t e = set_max_smem(fn, a.sm.total);
    if (e != cudaSuccess) return e;
    const unsigned threads = a.job.g.TB + 64; /* adding warps, the placer warp, the loader warp */
    const uint64_t tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    unsigned grid = persistent_grid(fn, threads, a.sm.total, tiles);
    if (a.grid && a.grid < grid) grid = a.grid;
    if (fast)
        k_homadd<true><<<grid, threads, a.sm.total, st>>>(a);
    else
        k_homadd<false><<<grid, threads, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
