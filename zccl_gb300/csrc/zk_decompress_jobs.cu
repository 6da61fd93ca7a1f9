/*
 * zk_decompress_jobs.cu -- decompression of many indexed streams in one
 * launch, writing the floats or adding them into the destination.
 *
 * Two callers need it: the ring allreduces' steps, whose P decompressions
 * run as one batch (ZCCL/src/ZCCL_ring_ho.c:163-169 for the allgather,
 * ZCCL/src/ZCCL_ring.c:1074-1076 for the DOC reduce step), and the DOC
 * reduce step's decompress-then-add, which here is one pass: the decoded
 * value (float)q * eb (ZCCLd_float.c:624) is added to the destination float
 * with one rounding, the float sum MPI_Reduce_local computes.
 *
 * Every stream carries its side index with its tiles' starting values (the
 * outputs of compression and sum batches do).  Persistent CTAs take the
 * batch's tiles in a static order; per tile, thread 0 copies the tile's job
 * into shared memory when it changes, the block sizes come from the width
 * index and a CTA scan, one TMA bulk copy brings the tile's bytes, every
 * thread unpacks its block, a second scan restores the running values, and
 * the floats leave through padded rows with coalesced stores (or
 * read-add-write in accumulate mode).
 */
#include "zkern.cuh"

namespace {

__device__ __forceinline__ const DecompressJob &djob(const DecompressJobsArgs &a, uint32_t j)
{
    return a.batch.jobs ? static_cast<const DecompressJob *>(a.batch.jobs)[j] : a.job;
}

template <bool FAST>
__global__ void __launch_bounds__(256, 3) k_decompress_jobs(const __grid_constant__ DecompressJobsArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *wsum = reinterpret_cast<uint32_t *>(smem + 16);   /* [33] */
    uint32_t *wsum2 = reinterpret_cast<uint32_t *>(smem + 160); /* [33] */
    uint64_t *s_local = reinterpret_cast<uint64_t *>(smem + 304);
    uint64_t *s_base = reinterpret_cast<uint64_t *>(smem + 312);
    uint32_t *s_q0 = reinterpret_cast<uint32_t *>(smem + 320);
    uint32_t *s_slot = reinterpret_cast<uint32_t *>(smem + 324); /* the job in the slot */
    DecompressJob *sj = reinterpret_cast<DecompressJob *>(smem + a.sm.jobs);
    float *rows = reinterpret_cast<float *>(smem + a.sm.rows);
    uint8_t *buf = smem + a.sm.in0;

    const uint32_t tid = threadIdx.x;
    const uint32_t L = a.job.g.L, stride = zg_row_stride(L); /* one L for the whole batch */
    uint32_t bad = 0;
    if (*(volatile const uint32_t *)a.w.walk_err) return;
    if (tid == 0) {
        mbar_init(bar, 1);
        *s_slot = 0xFFFFFFFFu;
    }
    const uint64_t ntiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    uint32_t it = 0;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
        __syncthreads(); /* the previous tile's rows and bytes have been read */
        if (tid == 0) {
            uint64_t local;
            const uint32_t j = batch_job(a.batch, t, &local);
            if (*s_slot != j) {
                copy16(sj, &djob(a, j), sizeof(DecompressJob));
                *s_slot = j;
            }
            *s_local = local;
        }
        __syncthreads();
        const DecompressJob &J = *sj;
        const ZGeom &g = J.g;
        const uint64_t local = *s_local;
        ZTile z;
        zg_tile(&g, local, &z);
        const bool own = tid < z.nblk;
        uint32_t b = 0, n = 0, size = 0;
        if (own) {
            n = zg_block_len(z.seg_len, L, z.blk0 + tid);
            b = J.idx.widths[z.gblk0 + tid];
            if (b > 32) {
                bad |= ZERR_CORRUPT;
                b = 0;
            }
            size = zg_block_bytes_f(g.fmt, b, n);
        }
        uint32_t total;
        const uint32_t off = cta_excl_scan(size, wsum, &total);
        const uint32_t headb = z.has_head ? 4u : 0u;
        if (tid == 0) {
            uint64_t base = J.idx.tile_off[local];
            uint32_t nload = total + headb;
            /* overflow-safe: base comes from the index and is not trusted */
            if (base > J.avail || nload > J.avail - base) {
                bad |= ZERR_BOUNDS;
                nload = base < J.avail ? (uint32_t)min((uint64_t)nload, J.avail - base) : 0u;
                if (base > J.avail) base = 0;
            }
            *s_base = base;
            *s_q0 = (uint32_t)J.idx.tile_qprev[local];
            tma_load_superset(buf, J.in + base, nload, bar);
        }
        mbar_wait(bar, it & 1u, a.w.err);
        const uint32_t *sw = reinterpret_cast<const uint32_t *>(buf);
        const uint32_t ph = (uint32_t)((uintptr_t)(J.in + *s_base) & 15u);
        int32_t head = 0;
        if (z.has_head) {
            uint32_t h = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) h |= (uint32_t)buf[ph + k] << (8 * k);
            head = (int32_t)h;
        }
        const uint32_t o = ph + headb + off;
        const bool full = FAST && own && n == 32;
        uint32_t d[32];
        uint32_t bsum = 0;
        if (own && buf[o] != b) bad |= ZERR_CORRUPT;
        if (full) {
            bsum = g.fmt == ZG_FASTMODE1 ? decode_block32(sw, o, b, d) : decode_full(sw, o, b, d, g.fmt);
        } else if (own) {
            decode_any(sw, o, b, n, [&](uint32_t, uint32_t v) { bsum += v; }, g.fmt);
        }
        uint32_t tsum;
        const uint32_t pre = cta_excl_scan(bsum, wsum2, &tsum);
        const uint32_t q0 = z.has_head ? (uint32_t)head : *s_q0;
        float *row = rows + tid * stride;
        const float eb = J.eb;
        uint32_t q = q0 + pre;
        if (full) {
#pragma unroll
            for (int j = 0; j < 32; j++) {
                q += d[j];
                row[j] = __fmul_rn(__int2float_rn((int32_t)q), eb);
            }
        } else if (own) {
            decode_any(
                sw, o, b, n,
                [&](uint32_t j, uint32_t v) {
                    q += v;
                    row[j] = __fmul_rn(__int2float_rn((int32_t)q), eb);
                },
                g.fmt);
        }
        __syncthreads();
        const bool acc = J.accumulate != 0;
        if (z.has_head && tid == 0) {
            const float h = __fmul_rn(__int2float_rn(head), eb);
            J.y[z.seg_start] = acc ? __fadd_rn(J.y[z.seg_start], h) : h;
        }
        /* the tile's floats are contiguous after the head: element i is row
         * i / L, column i % L, and a warp's 32 consecutive i share one row
         * when L = 32 */
        const uint32_t cnt = (uint32_t)(z.e_end - z.e_first);
        float *dst = J.y + z.e_first;
        const uint32_t nt = blockDim.x;
        if (acc) {
            /* the destination's floats are read 16 per thread ahead of the
             * adds, so that the loads overlap instead of each waiting for
             * the one before */
            constexpr uint32_t U = 16;
            for (uint32_t i0 = 0; i0 < cnt; i0 += U * nt) {
                float v[U];
#pragma unroll
                for (uint32_t u = 0; u < U; u++) {
                    const uint32_t i = i0 + u * nt + tid;
                    v[u] = i < cnt ? dst[i] : 0.f;
                }
#pragma unroll
                for (uint32_t u = 0; u < U; u++) {
                    const uint32_t i = i0 + u * nt + tid;
                    if (i < cnt) dst[i] = __fadd_rn(v[u], rows[(i / L) * stride + i % L]);
                }
            }
        } else {
            for (uint32_t i = tid; i < cnt; i += nt) dst[i] = rows[(i / L) * stride + i % L];
        }
    }
    if (bad) atomicOr(a.w.err, bad);
}

} // namespace

cudaError_t launch_decompress_jobs(const DecompressJobsArgs &a, cudaStream_t st)
{
    const bool fast = a.job.g.L <= 32;
    const void *fn = fast ? (const void *)k_decompress_jobs<true> : (const void *)k_decompress_jobs<false>;
    cudaError_t e = set_max_smem(fn, a.sm.total);
    if (e != cudaSuccess) return e;
    const uint32_t TB = a.job.g.TB;
    const uint64_t tiles = a.batch.jobs ? a.batch.ntiles : a.job.g.ntiles;
    unsigned grid = persistent_grid(fn, TB, a.sm.total, tiles);
    if (a.grid && a.grid < grid) grid = a.grid;
    if (fast)
        k_decompress_jobs<true><<<grid, TB, a.sm.total, st>>>(a);
    else
        k_decompress_jobs<false><<<grid, TB, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
