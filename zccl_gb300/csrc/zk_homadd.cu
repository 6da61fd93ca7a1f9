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
 * Persistent CTAs take tiles in ticket order, one thread per block.  A
 * tile's P inputs form a stream of TMA copies through two buffers: while one
 * input's tile bytes are unpacked and added into per-thread registers, the
 * next input's sizes are scanned from its width index and its bytes are
 * already in flight.  Zero-width input blocks are skipped without touching
 * their bytes.  After the last input the sum is re-encoded like the
 * compressor does (width, scan, early look-back publish); like the
 * compressor, the CTA then places the sum it packed one round before (one
 * tile after that sum published its size), claims its next tile and starts
 * that tile's first copy, and packs the new sum while the copy runs.  The
 * starting value per tile is the sum of the inputs' values.
 */
#include "zkern.cuh"

namespace {

struct BlockSlot {
    uint32_t b, n, off;
};

/* All threads: sizes of input p's blocks in tile t, their offsets, and
 * (thread 0) the TMA copy of those bytes into buf. */
__device__ __forceinline__ BlockSlot stage_input(const HomAddArgs &a, uint64_t t, uint32_t p,
                                                 uint8_t *buf, uint64_t *bar, uint32_t *wsum,
                                                 uint64_t *s_base, uint32_t &bad)
{
    const HomInput &in = a.in[p];
    BlockSlot sl = {0, 0, 0};
    ZTile z;
    zg_tile(&a.g, t, &z);
    uint32_t size = 0;
    if (threadIdx.x < z.nblk) {
        sl.n = zg_block_len(z.seg_len, a.g.L, z.blk0 + threadIdx.x);
        sl.b = in.widths[z.gblk0 + threadIdx.x];
        if (sl.b > 32) {
            bad |= ZERR_CORRUPT;
            sl.b = 0;
        }
        size = zg_block_bytes(sl.b, sl.n);
    }
    uint32_t total;
    sl.off = cta_excl_scan(size, wsum, &total);
    total += z.has_head ? 4u : 0u;
    if (threadIdx.x == 0) {
        uint64_t base = in.tile_off[t];
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
    return sl;
}

template <bool FAST>
__global__ void __launch_bounds__(128) k_homadd(const HomAddArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem); /* [2] */
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);
    uint64_t *bc = reinterpret_cast<uint64_t *>(smem + 160);     /* [0] tile */
    uint64_t *s_base = reinterpret_cast<uint64_t *>(smem + 192); /* [2] */
    uint64_t *rec = reinterpret_cast<uint64_t *>(smem + 256);
    uint32_t *acc_rows = reinterpret_cast<uint32_t *>(smem + a.sm.rows);
    uint8_t *outs = smem + a.sm.out;
    const uint32_t outs_sa = smem_u32(outs);

    const ZGeom &g = a.g;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t L = g.L, stride = zg_row_stride(L), P = a.P;
    uint32_t bad = 0;
    /* see k_decompress: a failed index walk stops every CTA alike */
    if (*(volatile const uint32_t *)a.w.walk_err) return;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    uint32_t acc[32];
    uint32_t ld = 0; /* index of the current copy in the two-buffer stream */
    ZPending pd = {ZP_NONE, 0, 0, 0};

    /* Tiles are claimed one at a time when the CTA is ready for them, and
     * the CTA never waits while it holds a claimed tile whose size is not
     * yet published, so later tiles never wait on a tile sitting idle. */
    if (tid == 0) bc[0] = atomicAdd(a.w.ticket, 1u);
    __syncthreads();
    uint64_t tile = bc[0];
    BlockSlot cur = {0, 0, 0};
    if (tile < g.ntiles)
        cur = stage_input(a, tile, 0, smem + a.sm.in0, &bar[0], wsum, &s_base[0], bad);

    for (;;) {
        if (tile >= g.ntiles) break;
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

        for (uint32_t p = 0; p < P; p++, ld++) {
            const uint32_t cb = ld & 1u;
            /* the next input's copy runs while this one is added */
            BlockSlot nxt = {0, 0, 0};
            if (p + 1 < P)
                nxt = stage_input(a, tile, p + 1, smem + (cb ? a.sm.in0 : a.sm.in1), &bar[cb ^ 1u],
                                  wsum, &s_base[cb ^ 1u], bad);
            if (a.qprev_valid && tid == 0) qsum += (uint32_t)a.in[p].tile_qprev[tile];
            mbar_wait(&bar[cb], (ld >> 1) & 1u, a.w.err);
            const uint8_t *buf = smem + (cb ? a.sm.in1 : a.sm.in0);
            const uint32_t *sw = reinterpret_cast<const uint32_t *>(buf);
            const uint32_t ph = (uint32_t)((uintptr_t)(a.in[p].bytes + s_base[cb]) & 15u);
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
             * after that round's scan has synchronised every thread */
        }

        /* branch-case counters of the two-input add (ZCCLd_float.c:2175-2764) */
        if (a.cases && P == 2) {
            const uint32_t c0 = __syncthreads_count(own && nzmask == 0u);
            const uint32_t c1 = __syncthreads_count(own && nzmask == 2u);
            const uint32_t c2 = __syncthreads_count(own && nzmask == 1u);
            const uint32_t c3 = __syncthreads_count(own && nzmask == 3u);
            if (tid == 0) {
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
        uint32_t total;
        const uint32_t off = cta_excl_scan(size, wsum, &total);
        total += headb;
        if (warp == 0) lb_publish(a.w.status, tile, total, tile == 0, 0);

        /* place the sum packed one round ago (its size went out a whole tile
         * earlier), then claim the next tile and start its first input's
         * copy, and pack this sum while it arrives */
        if (pd.tile != ZP_NONE)
            place_tile(g, pd, outs, a.out, a.cap, a.idx, a.qprev_valid != 0, a.w.status, a.w.err, rec,
                       bad);
        if (tid == 0) bc[0] = atomicAdd(a.w.ticket, 1u);
        __syncthreads();
        const uint64_t next = bc[0];
        if (next < g.ntiles)
            cur = stage_input(a, next, 0, smem + (ld & 1u ? a.sm.in1 : a.sm.in0), &bar[ld & 1u], wsum,
                              &s_base[ld & 1u], bad);
        smem_zero(outs, total + 8);
        __syncthreads();
        if (z.has_head && tid == 0) *reinterpret_cast<uint32_t *>(outs) = hsum;
        const uint32_t o = headb + off;
        if (full) {
            encode_full(outs_sa, o, b, smask, acc);
        } else if (own) {
            encode_any(outs_sa, o, b, n, [&](uint32_t j, uint32_t &neg, uint32_t &mg) {
                const uint32_t v = FAST ? pick(acc, j) : acc_rows[tid * stride + j];
                neg = v >> 31;
                mg = (uint32_t)abs((int32_t)v);
            });
        }
        pd.tile = tile;
        pd.total = total;
        pd.b = b;
        pd.q = qsum;
        tile = next;
        __syncthreads(); /* the packed sum is complete; acc_rows are free */
    }
    /* the last packed sum */
    if (pd.tile != ZP_NONE)
        place_tile(g, pd, outs, a.out, a.cap, a.idx, a.qprev_valid != 0, a.w.status, a.w.err, rec, bad);
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_homadd(const HomAddArgs &a, cudaStream_t st)
{
    const bool fast = a.g.L <= 32;
    const void *fn = fast ? (const void *)k_homadd<true> : (const void *)k_homadd<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.sm.total);
    if (e != cudaSuccess) return e;
    unsigned grid = persistent_grid(fn, a.g.TB, a.sm.total, a.g.ntiles);
    if (fast)
        k_homadd<true><<<grid, a.g.TB, a.sm.total, st>>>(a);
    else
        k_homadd<false><<<grid, a.g.TB, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
