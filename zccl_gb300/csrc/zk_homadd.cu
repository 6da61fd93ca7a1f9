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
 * One CTA per tile, one thread per block.  For each input in turn: block
 * sizes from its width index, one TMA bulk copy of its tile bytes, and each
 * thread adds the block's deltas into registers; zero-width input blocks
 * are skipped without touching their bytes.  The sum is then re-encoded
 * exactly like the compressor (width, scan, look-back, packed staging, TMA
 * bulk store) and the output's side index is written; the output's
 * quantized value before each tile is the sum of the inputs' values.
 */
#include "zkern.cuh"

namespace {

template <bool FAST>
__global__ void __launch_bounds__(128) k_homadd(const HomAddArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);
    uint64_t *bcast = reinterpret_cast<uint64_t *>(smem + 160);
    uint32_t *acc_rows = reinterpret_cast<uint32_t *>(smem + a.sm.rows);
    uint8_t *stage = smem + a.sm.stage;
    uint32_t *sw = reinterpret_cast<uint32_t *>(stage);

    const ZGeom &g = a.g;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t L = g.L, stride = zg_row_stride(L);
    uint32_t bad = 0;
    /* The index walk ran to completion before this launch, so every CTA sees
     * the same word: after a failed walk no CTA touches the stream and no
     * CTA waits on another. */
    if (*(volatile const uint32_t *)a.w.walk_err) return;

    if (tid == 0) {
        bcast[0] = atomicAdd(a.w.ticket, 1u);
        mbar_init(bar, 1);
    }
    __syncthreads();
    const uint64_t tile = bcast[0];
    ZTile z;
    zg_tile(&g, tile, &z);
    const bool own = tid < z.nblk;
    const uint32_t n = own ? zg_block_len(z.seg_len, L, z.blk0 + tid) : 0u;
    const uint32_t headb = z.has_head ? 4u : 0u;

    uint32_t acc[FAST ? 32 : 1];
    if (FAST) {
#pragma unroll
        for (uint32_t j = 0; j < 32; j++) acc[j] = 0;
    } else if (own) {
        for (uint32_t j = 0; j < n; j++) acc_rows[tid * stride + j] = 0;
    }
    uint32_t hsum = 0, qsum = 0, nzmask = 0;

    for (uint32_t p = 0; p < a.P; p++) {
        const HomInput in = a.in[p];
        uint32_t b = 0, size = 0;
        if (own) {
            b = in.widths[z.gblk0 + tid];
            if (b > 32) {
                bad |= ZERR_CORRUPT;
                b = 0;
            }
            size = zg_block_bytes(b, n);
            if (b) nzmask |= 1u << (p & 31);
        }
        uint32_t total;
        const uint32_t off = cta_excl_scan(size, wsum, &total);
        total += headb;
        const uint64_t base = in.tile_off[tile];
        uint32_t nload = total;
        /* overflow-safe: base comes from the index and is not trusted */
        if (base > in.avail || total > in.avail - base) {
            bad |= ZERR_BOUNDS;
            nload = base < in.avail ? (uint32_t)min((uint64_t)total, in.avail - base) : 0u;
        }
        const uint32_t ph = stage_in(stage, in.bytes + base, nload, bar);
        stage_in_wait(bar, p & 1u, a.w.err);
        if (z.has_head) {
            uint32_t h = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) h |= (uint32_t)stage[ph + k] << (8 * k);
            hsum += h;
        }
        if (a.qprev_valid) qsum += (uint32_t)in.tile_qprev[tile];
        if (own) {
            const uint32_t o = ph + headb + off;
            if (stage[o] != b) bad |= ZERR_CORRUPT;
            if (b) {
                const uint32_t B = b >> 3, r = b & 7u, ns = (n + 7) >> 3;
                if (FAST) {
                    /* -(hi << r | lo) == -(hi << r) - lo: each part is added
                     * with the element's sign as soon as it is read */
                    BitReader br;
                    br.init(sw, o + 1);
                    const uint32_t sg = br.get(8 * ns) << (32 - 8 * ns);
                    if (B) {
#pragma unroll
                        for (uint32_t j = 0; j < 32; j++)
                            if (j < n) {
                                uint32_t t = bswap32(br.get(8 * B) << (32 - 8 * B)) << r;
                                acc[j] += ((sg >> (31 - j)) & 1u) ? 0u - t : t;
                            }
                    }
                    if (r) {
#pragma unroll
                        for (uint32_t j = 0; j < 32; j++)
                            if (j < n) {
                                uint32_t t = br.get(r);
                                acc[j] += ((sg >> (31 - j)) & 1u) ? 0u - t : t;
                            }
                    }
                } else {
                    BitReader rs, rh, rl;
                    rs.init(sw, o + 1);
                    rh.init(sw, o + 1 + ns);
                    rl.init(sw, o + 1 + ns + B * n);
                    for (uint32_t j = 0; j < n; j++) {
                        uint32_t v = B ? bswap32(rh.get(8 * B) << (32 - 8 * B)) << r : 0u;
                        if (r) v |= rl.get(r);
                        if (rs.get(1)) v = 0u - v;
                        acc_rows[tid * stride + j] += v;
                    }
                }
            }
        }
        __syncthreads(); /* staging is reused by the next input */
    }

    /* branch-case counters of the two-input add (ZCCLd_float.c:2175-2764) */
    if (a.cases && a.P == 2) {
        uint32_t c0 = __syncthreads_count(own && nzmask == 0u);
        uint32_t c1 = __syncthreads_count(own && nzmask == 2u);
        uint32_t c2 = __syncthreads_count(own && nzmask == 1u);
        uint32_t c3 = __syncthreads_count(own && nzmask == 3u);
        if (tid == 0) {
            atomicAdd(a.cases + 0, (unsigned long long)c0);
            atomicAdd(a.cases + 1, (unsigned long long)c1);
            atomicAdd(a.cases + 2, (unsigned long long)c2);
            atomicAdd(a.cases + 3, (unsigned long long)c3);
        }
    }

    /* re-encode the sum */
    uint32_t b = 0, size = 0, smask = 0, mx = 0;
    if (own) {
        if (FAST) {
#pragma unroll
            for (uint32_t j = 0; j < 32; j++) {
                int32_t d = (int32_t)acc[j];
                uint32_t neg = d < 0 ? 1u : 0u;
                uint32_t mg = neg ? 0u - acc[j] : acc[j];
                smask |= neg << (31 - j);
                mx = mx > mg ? mx : mg;
                acc[j] = mg;
            }
        } else {
            for (uint32_t j = 0; j < n; j++) {
                uint32_t v = acc_rows[tid * stride + j];
                uint32_t mg = (int32_t)v < 0 ? 0u - v : v;
                mx = mx > mg ? mx : mg;
            }
        }
        b = width_of(mx, a.wt);
        size = zg_block_bytes(b, n);
    }
    uint32_t total;
    const uint32_t off = cta_excl_scan(size, wsum, &total);
    total += headb;
    if (warp == 0) {
        uint64_t prefix = lookback(a.w.status, tile, total, tile == 0, 0, a.w.err);
        if (lane == 0) bcast[1] = prefix;
    }
    __syncthreads();
    const uint64_t base = 8ull * g.T + bcast[1];
    const bool fits = base + total <= a.cap; /* uniform over the CTA */
    if (!fits) bad |= ZERR_CAPACITY;

    if (own) a.idx.widths[z.gblk0 + tid] = (uint8_t)b;
    if (tid == 0) {
        a.idx.tile_off[tile] = base;
        if (a.qprev_valid) a.idx.tile_qprev[tile] = (int32_t)qsum;
        if (fits && z.has_head && z.seg < g.T) {
            uint64_t h = base - 8ull * g.T;
#pragma unroll
            for (int k = 0; k < 8; k++) a.out[8ull * z.seg + k] = (uint8_t)(h >> (8 * k));
        }
        if (tile == g.ntiles - 1) *a.idx.size = base + total;
    }

    uint8_t *gout = a.out + base;
    const uint32_t sph = (uint32_t)((uintptr_t)gout & 15u);
    if (z.has_head && tid == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) stage[sph + k] = (uint8_t)(hsum >> (8 * k));
    }
    if (own) {
        const uint32_t o = sph + headb + off;
        const uint32_t B = b >> 3, r = b & 7u, ns = (n + 7) >> 3;
        if (FAST) {
            BitWriter bw;
            bw.init(sw, o, size);
            bw.put(b, 8);
            if (b) {
                bw.put(smask >> (32 - 8 * ns), 8 * ns);
                if (B) {
#pragma unroll
                    for (uint32_t j = 0; j < 32; j++)
                        if (j < n) bw.put(bswap32(acc[j] >> r) >> (32 - 8 * B), 8 * B);
                }
                if (r) {
                    const uint32_t mask = (1u << r) - 1u;
#pragma unroll
                    for (uint32_t j = 0; j < 32; j++)
                        if (j < n) bw.put(acc[j] & mask, r);
                }
            }
            bw.finish();
        } else {
            stage[o] = (uint8_t)b;
            if (b) {
                BitWriter ws, wh, wl;
                ws.init(sw, o + 1, ns);
                wh.init(sw, o + 1 + ns, B * n);
                wl.init(sw, o + 1 + ns + B * n, size - 1 - ns - B * n);
                const uint32_t mask = r ? (1u << r) - 1u : 0u;
                for (uint32_t j = 0; j < n; j++) {
                    uint32_t v = acc_rows[tid * stride + j];
                    uint32_t neg = (int32_t)v < 0 ? 1u : 0u;
                    uint32_t mg = neg ? 0u - v : v;
                    ws.put(neg, 1);
                    if (B) wh.put(bswap32(mg >> r) >> (32 - 8 * B), 8 * B);
                    if (r) wl.put(mg & mask, r);
                }
                ws.finish();
                if (B) wh.finish();
                if (r) wl.finish();
            }
        }
    }
    if (fits) stage_out(gout, stage, total);
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_homadd(const HomAddArgs &a, cudaStream_t st)
{
    const bool fast = a.g.L <= 32;
    const void *fn = fast ? (const void *)k_homadd<true> : (const void *)k_homadd<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.sm.total);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)a.g.ntiles), block(a.g.TB);
    if (fast)
        k_homadd<true><<<grid, block, a.sm.total, st>>>(a);
    else
        k_homadd<false><<<grid, block, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
