/*
 * zk_decompress.cu -- decompressor.
 *
 * Replaces ZCCL_float_decompress_openmp_threadblock_arg
 * (ZCCL/src/ZCCLd_float.c:538-754) and produces the same floats.  Persistent
 * CTAs, one thread per block, mirroring the compressor.  With the index
 * holding every tile's starting value the tiles are independent: CTA c
 * takes tiles c, c + grid, ... and loads the index entries of the tile
 * after next while it works.  A stream that arrived as bytes gets those
 * values first: the same kernel in its SUMS form writes every tile's delta
 * sum into the index, and k_qprev_scan turns them, segment by segment, into
 * starting values from the segment's raw head.
 * Per tile:
 *   1. for the NEXT tile: block sizes from the width index, a block-wide
 *      scan for every block's offset, and one TMA bulk copy of its bytes,
 *      so the copy runs while the current tile is decoded (double buffer);
 *   2. every thread unpacks its block (sign bits, high bytes, low-bit
 *      stream, ZCCL/src/ZCCL_TypeManager.c:423-950) into int32 deltas;
 *   3. a block-wide scan of the per-block delta sums, started from the
 *      quantized value before the tile (from the index), restores the
 *      running values (ZCCLd_float.c:617-628);
 *   4. x = (float)q * eb (ZCCLd_float.c:624) into padded rows, written out
 *      row by row with coalesced stores.
 */
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "zkern.cuh"

namespace {

/* Per-thread view of its block in a staged tile. */
struct BlockSlot {
    uint32_t b, n, off;
};

/* The index entries one tile needs: this thread's block width, and on
 * thread 0 the tile's byte offset and the quantized value before it.  Loaded
 * a tile ahead of their use, so the loads' latency is hidden. */
struct TileIdx {
    uint32_t b;
    uint64_t base;
    uint32_t q0;
};

__device__ __forceinline__ TileIdx load_idx(const DecompressArgs &a, uint64_t t, const ZTile &z)
{
    TileIdx r = {0, 0, 0};
    if (t >= a.g.ntiles) return r;
    if (threadIdx.x < z.nblk) r.b = a.idx.widths[z.gblk0 + threadIdx.x];
    if (threadIdx.x == 0) {
        r.base = a.idx.tile_off[t];
        if (a.qprev_valid) r.q0 = (uint32_t)a.idx.tile_qprev[t];
    }
    return r;
}

/* Thread 0: the TMA copy of a tile's `total` bytes at the index's byte
 * offset (checked against the readable bytes) into buf; its offset and
 * starting value into *s_base and *s_q0. */
__device__ __forceinline__ void issue_tile(const DecompressArgs &a, const TileIdx &ix, uint32_t total, uint8_t *buf,
                                           uint64_t *bar, uint64_t *s_base, uint32_t *s_q0, uint32_t &bad)
{
    uint64_t base = ix.base;
    uint32_t nload = total;
    /* overflow-safe: base comes from the index and is not trusted */
    if (base > a.avail || total > a.avail - base) {
        bad |= ZERR_BOUNDS;
        nload = base < a.avail ? (uint32_t)min((uint64_t)total, a.avail - base) : 0u;
        if (base > a.avail) base = 0;
    }
    *s_base = base;
    *s_q0 = ix.q0;
    tma_load_superset(buf, a.in + base, nload, bar);
}

/* All threads: sizes of tile t's blocks (geometry z), their offsets, and
 * (thread 0) the TMA copy of the tile's bytes into buf.  Returns the slot of
 * this thread's block; the tile's byte offset lands in *s_base, its starting
 * value in *s_q0. */
__device__ __forceinline__ BlockSlot stage_tile(const DecompressArgs &a, const ZTile &z, const TileIdx &ix,
                                                uint8_t *buf, uint64_t *bar, uint32_t *wsum,
                                                uint64_t *s_base, uint32_t *s_q0, uint32_t &bad)
{
    BlockSlot sl = {0, 0, 0};
    uint32_t size = 0;
    if (threadIdx.x < z.nblk) {
        sl.n = zg_block_len(z.seg_len, a.g.L, z.blk0 + threadIdx.x);
        sl.b = ix.b;
        if (sl.b > 32) {
            bad |= ZERR_CORRUPT;
            sl.b = 0;
        }
        size = a.g.fmt == ZG_FASTMODE1 && sl.n == 32 ? block32_bytes(sl.b) : zg_block_bytes_f(a.g.fmt, sl.b, sl.n);
    }
    uint32_t total;
    sl.off = cta_excl_scan(size, wsum, &total);
    if (threadIdx.x == 0) issue_tile(a, ix, total + (z.has_head ? 4u : 0u), buf, bar, s_base, s_q0, bad);
    return sl;
}

/* CTA c takes tiles c, c + grid, c + 2 grid, ..., with the index entries of
 * the tile after next already loading.  SUMS: only each tile's wrapped sum of
 * deltas, into the index's tile_qprev (k_qprev_scan completes it). */
template <bool FAST, bool SUMS>
__global__ void __launch_bounds__(256, 3) k_decompress(const DecompressArgs a, const __grid_constant__ CUtensorMap ymap)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem); /* [2] */
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);
    uint64_t *s_base = reinterpret_cast<uint64_t *>(smem + 192); /* [2] */
    uint32_t *s_q0 = reinterpret_cast<uint32_t *>(smem + 208);   /* [2] */
    uint32_t *ws1 = reinterpret_cast<uint32_t *>(smem + 320); /* [33] second scan scratch */
    uint32_t *ws2 = reinterpret_cast<uint32_t *>(smem + 464); /* [33] the same pair, odd rounds */
    uint32_t *ws3 = reinterpret_cast<uint32_t *>(smem + 608); /* [33] */
    /* [4] geometry of the tiles in flight, each found once by thread 0 before
     * a scan's barrier: the tile's (it % 4), the next one's, the one after
     * (for its index entries); a slot is rewritten two rounds after its
     * tile's, when every thread is past that tile */
    ZTile *zs = reinterpret_cast<ZTile *>(smem + 752);
    static_assert(752 + 4 * sizeof(ZTile) <= 1024, "the tile records fit below the rows");
    float *rows = reinterpret_cast<float *>(smem + a.sm.rows);

    const ZGeom &g = a.g;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nw = blockDim.x >> 5;
    const uint32_t L = g.L, stride = zg_row_stride(L);
    uint32_t bad = 0;
    /* Full tiles of L = 32 whose first element minus one starts a 128-byte
     * row of y leave by TMA tensor stores, one per warp of 32 rows of 32
     * floats (the element before the tile first), from a 1024-byte-aligned
     * box with the 128-byte swizzle (16-byte chunk k of row r at chunk
     * k ^ (r & 7)), so that each thread's vector stores of its row meet no
     * bank conflict. */
    const uint32_t rows_sa = smem_u32(rows);
    const uint32_t box_sa = (rows_sa + 1023u) & ~1023u;
    const bool rows_ok = FAST && a.rows_map && L == 32 && g.TB == 256 && blockDim.x == 256 &&
                         box_sa + 32768u <= rows_sa + g.TB * stride * 4u;
    /* The index walk ran to completion before this launch, so every CTA sees
     * the same word: after a failed walk no CTA touches the stream and no
     * CTA waits on another. */
    if (*(volatile const uint32_t *)a.w.walk_err) return;

    uint64_t tile = blockIdx.x;
    uint64_t tnext = tile + gridDim.x; /* the static order's next tile */
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        if (tile < g.ntiles) zg_tile(&g, tile, &zs[0]);
        if (tnext < g.ntiles) zg_tile(&g, tnext, &zs[1]);
    }
    __syncthreads();
    TileIdx ix = load_idx(a, tile, zs[0]);
    BlockSlot cur = {0, 0, 0};
    if (tile < g.ntiles) cur = stage_tile(a, zs[0], ix, smem + a.sm.in0, &bar[0], wsum, &s_base[0], &s_q0[0], bad);
    ix = load_idx(a, tnext, zs[1]);

    /* One barrier a tile, the scan's (one more before the rows leave when a
     * tile has short or long blocks).  The input buffer the next copy
     * overwrites was last read before this tile's scan; the tile's byte
     * offset and starting value (thread 0, at the copy) are visible through
     * the copy's mbarrier; each warp writes and sends out only its own 32
     * rows, and its box rows are free again once its lane 0 has seen its
     * last store read them, before the scan. */
    for (uint32_t it = 0;; it++) {
        const uint32_t cb = it & 1u;
        if (tile >= g.ntiles) break;
        const ZTile &z = zs[it & 3u];

        BlockSlot nxt = {0, 0, 0}; /* the next tile's block, found in step 3 */
        uint32_t next_bytes = 0;  /* the next tile's bytes */
        bool issue_now = true;    /* its copy starts right after the scan */
        TileIdx ixn;              /* its index entries */

        /* 2. unpack this tile's deltas */
        mbar_wait(&bar[cb], (it >> 1) & 1u, a.w.err);
        const uint8_t *buf = smem + (cb ? a.sm.in1 : a.sm.in0);
        const uint32_t *sw = reinterpret_cast<const uint32_t *>(buf);
        const uint32_t ph = (uint32_t)((uintptr_t)(a.in + s_base[cb]) & 15u);
        int32_t head = 0;
        if (z.has_head) {
            uint32_t h = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) h |= (uint32_t)buf[ph + k] << (8 * k);
            head = (int32_t)h;
        }
        const uint32_t headb = z.has_head ? 4u : 0u;
        const uint32_t o = ph + headb + cur.off; /* this block, in buffer coordinates */
        const uint32_t b = cur.b, n = cur.n;
        const bool own = tid < z.nblk;
        const bool full = FAST && own && n == 32;
        uint32_t d[32];
        uint32_t bsum = 0;
        if (own && buf[o] != b) bad |= ZERR_CORRUPT;
        if (full) {
            bsum = g.fmt == ZG_FASTMODE1 ? decode_block32(sw, o, b, d) : decode_full(sw, o, b, d, g.fmt);
        } else if (own) { /* short or long block: sum now, decode again for the values */
            decode_any(sw, o, b, n, [&](uint32_t, uint32_t v) { bsum += v; }, g.fmt);
        }

        /* 3. starting value of every block.  In index order the next tile's
         *    block offsets come from the same scan (its widths arrived a tile
         *    ago), and its copy starts right after, into the other buffer. */
        uint32_t tsum, pre;
        {
            const ZTile &zn = zs[(it + 1u) & 3u];
            uint32_t sizen = 0;
            if (tid == 0 && tnext + gridDim.x < g.ntiles) zg_tile(&g, tnext + gridDim.x, &zs[(it + 2u) & 3u]);
            if (tnext < g.ntiles) {
                if (tid < zn.nblk) {
                    nxt.n = zg_block_len(zn.seg_len, L, zn.blk0 + tid);
                    nxt.b = ix.b;
                    if (nxt.b > 32) {
                        bad |= ZERR_CORRUPT;
                        nxt.b = 0;
                    }
                    sizen = g.fmt == ZG_FASTMODE1 && nxt.n == 32 ? block32_bytes(nxt.b)
                                                                  : zg_block_bytes_f(g.fmt, nxt.b, nxt.n);
                }
            }
            uint32_t totn;
            if (!SUMS && lane == 0) bulk_wait_read0(); /* the warp's last box store has left the rows */
            grp_excl_scan2_1(bsum, sizen, cb ? wsum : ws2, cb ? ws1 : ws3, pre, nxt.off, tsum, totn, blockDim.x, 0);
            /* with one input buffer, a tile with short or long blocks reads
             * it again for the values: its successor's copy waits for that */
            next_bytes = totn + (tnext < g.ntiles && zn.has_head ? 4u : 0u);
            issue_now = SUMS || a.sm.in0 != a.sm.in1 ||
                        (FAST && L == 32 && z.nblk == g.TB && z.e_end - z.e_first == 32ull * g.TB);
            if (tnext < g.ntiles && tid == 0 && issue_now)
                issue_tile(a, ix, next_bytes, smem + (cb ? a.sm.in0 : a.sm.in1), &bar[cb ^ 1u], &s_base[cb ^ 1u],
                           &s_q0[cb ^ 1u], bad);
            ixn = ix;
            ix = load_idx(a, tnext + gridDim.x, zs[(it + 2u) & 3u]);
        }
        if (SUMS) { /* the tile's delta sum; the values wait for the scan */
            if (tid == 0) a.idx.tile_qprev[tile] = (int32_t)tsum;
            cur = nxt;
            tile = tnext;
            tnext += gridDim.x;
            continue;
        }
        const uint32_t q0 = z.has_head ? (uint32_t)head : s_q0[cb];
        const bool box = rows_ok && z.nblk == 256 && z.e_end - z.e_first == 8192 && ((z.e_first - 1) & 31) == 0;

        /* 4. values into rows, then out */
        float *row = rows + tid * stride;
        if (box) { /* every block is full: element e_first + 32 tid + j is box float 1 + 32 tid + j */
            uint32_t q = q0 + pre;
            /* the float before this block, the previous block's last (or the
             * value before the tile: the head, or the previous tile's last
             * element, stored there too with the same bits) */
            const float prev = __fmul_rn(__int2float_rn((int32_t)q), a.eb);
            float v[32];
#pragma unroll
            for (int j = 0; j < 32; j++) {
                q += d[j];
                v[j] = __fmul_rn(__int2float_rn((int32_t)q), a.eb);
            }
            const uint32_t rb = box_sa + tid * 128u, x4 = (tid & 7u) << 4;
            st_shared_v4(rb | x4, prev, v[0], v[1], v[2]);
#pragma unroll
            for (uint32_t k = 1; k < 8; k++)
                st_shared_v4(rb | ((k << 4) ^ x4), v[4 * k - 1], v[4 * k], v[4 * k + 1], v[4 * k + 2]);
            if (tid == 255) a.y[z.e_end - 1] = v[31]; /* past the box; the others are the next rows' first */
            fence_proxy_async_smem();
            __syncwarp();
            /* the warp's 32 rows leave by one TMA store */
            if (lane == 0) tma_store_2d(&ymap, box_sa + warp * 4096u, 0, (int32_t)((z.e_first - 1) >> 5) + 32 * (int32_t)warp);
        } else if (full) {
            uint32_t q = q0 + pre;
#pragma unroll
            for (int j = 0; j < 32; j++) {
                q += d[j];
                row[j] = __fmul_rn(__int2float_rn((int32_t)q), a.eb);
            }
        } else if (own) {
            uint32_t q = q0 + pre;
            decode_any(
                sw, o, b, n,
                [&](uint32_t j, uint32_t v) {
                    q += v;
                    row[j] = __fmul_rn(__int2float_rn((int32_t)q), a.eb);
                },
                g.fmt);
        }
        if (z.has_head && tid == 0) a.y[z.seg_start] = __fmul_rn(__int2float_rn(head), a.eb);
        if (box) { /* each warp has sent its rows out above */
        } else if (FAST && L == 32 && z.nblk == g.TB && z.e_end - z.e_first == 32ull * g.TB && nw * 32u == g.TB) {
            /* a full tile: each warp stores its own 32 rows (no barrier),
             * unrolled so that many stores are in flight */
            __syncwarp();
            float *dst = a.y + z.e_first + lane;
#pragma unroll 8
            for (uint32_t r = 0; r < 32; r++) {
                const uint32_t k = warp * 32u + r;
                dst[k * 32u] = rows[k * stride + lane];
            }
        } else {
            __syncthreads();
            if (!issue_now && tnext < g.ntiles && tid == 0) /* every read of the one input buffer is done */
                issue_tile(a, ixn, next_bytes, smem + (cb ? a.sm.in0 : a.sm.in1), &bar[cb ^ 1u], &s_base[cb ^ 1u],
                           &s_q0[cb ^ 1u], bad);
            for (uint32_t k = warp; k < z.nblk; k += nw) {
                const uint32_t nk = zg_block_len(z.seg_len, L, z.blk0 + k);
                float *dst = a.y + z.e_first + (uint64_t)k * L;
                for (uint32_t j = lane; j < nk; j += 32) dst[j] = rows[k * stride + j];
            }
        }
        cur = nxt;
        tile = tnext;
        tnext += gridDim.x;
    }
    if (lane == 0) bulk_wait0();
    if (bad) atomicOr(a.w.err, bad);
}

/* One warp per segment: its tiles' delta sums (from k_decompress<_, true>)
 * become the quantized value before each tile, starting from the
 * segment's raw int32 head (the four bytes at its first tile's offset) and
 * wrapping like the reference's int32 running value (ZCCLd_float.c:582-628). */
__global__ void k_qprev_scan(const DecompressArgs a)
{
    const ZGeom &g = a.g;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t seg = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint64_t nseg = (uint64_t)g.T + (g.rem ? 1u : 0u);
    if (seg >= nseg || *(volatile const uint32_t *)a.w.walk_err) return;
    const uint64_t t0 = seg < g.T ? seg * g.nt_reg : (uint64_t)g.T * g.nt_reg;
    const uint64_t nt = seg < g.T ? g.nt_reg : g.nt_rm;
    const uint64_t off = a.idx.tile_off[t0];
    uint32_t run = 0;
    if (off <= a.avail && a.avail - off >= 4) {
#pragma unroll
        for (int k = 0; k < 4; k++) run |= (uint32_t)a.in[off + k] << (8 * k);
    } else if (lane == 0) {
        atomicOr(a.w.err, ZERR_BOUNDS);
    }
    for (uint64_t k0 = 0; k0 < nt; k0 += 32) {
        const uint64_t k = k0 + lane;
        const uint32_t v = k < nt ? (uint32_t)a.idx.tile_qprev[t0 + k] : 0u;
        const uint32_t inc = warp_incl_scan(v);
        if (k < nt) a.idx.tile_qprev[t0 + k] = (int32_t)(run + inc - v);
        run += __shfl_sync(0xffffffffu, inc, 31);
    }
}

/* cuTensorMapEncodeTiled from the driver, looked up once. */
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

} // namespace

bool zk_rows_map(CUtensorMap *map, const void *p, uint64_t n, uint32_t box_rows)
{
    const uint64_t nrows = n / 32u;
    if (((uintptr_t)p & 15u) || nrows < 256u || nrows > 0x7fffffffull) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dim[2] = {32u, nrows};
    const cuuint64_t stride[1] = {128u};
    const cuuint32_t box[2] = {32u, box_rows};
    const cuuint32_t estride[2] = {1u, 1u};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(p), dim, stride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_decompress(const DecompressArgs &a, cudaStream_t st)
{
    const bool fast = a.g.L <= 32;
    /* a stream without starting values: tile sums, then the scan per segment */
    if (!a.qprev_valid) {
        const void *fs = fast ? (const void *)k_decompress<true, true> : (const void *)k_decompress<false, true>;
        cudaError_t e = set_max_smem(fs, a.sm.total);
        if (e != cudaSuccess) return e;
        alignas(64) CUtensorMap none;
        memset(&none, 0, sizeof none);
        DecompressArgs b = a;
        b.rows_map = 0;
        void *args[] = {&b, &none};
        e = cudaLaunchKernel(fs, dim3(persistent_grid(fs, a.g.TB, a.sm.total, a.g.ntiles)), dim3(a.g.TB), args,
                             a.sm.total, st);
        if (e != cudaSuccess) return e;
        const unsigned nseg = a.g.T + (a.g.rem ? 1u : 0u);
        k_qprev_scan<<<(nseg + 3) / 4, 128, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const void *fn = fast ? (const void *)k_decompress<true, false> : (const void *)k_decompress<false, false>;
    cudaError_t e = set_max_smem(fn, a.sm.total);
    if (e != cudaSuccess) return e;
    unsigned grid = persistent_grid(fn, a.g.TB, a.sm.total, a.g.ntiles);
    DecompressArgs b = a;
    b.qprev_valid = 1;
    alignas(64) CUtensorMap map;
    memset(&map, 0, sizeof map);
    b.rows_map = fast && zk_rows_map(&map, a.y, a.g.n, 32);
    void *args[] = {&b, &map};
    return cudaLaunchKernel(fn, dim3(grid), dim3(a.g.TB), args, a.sm.total, st);
}
