/*
 * zk_compress.cu -- fused single-pass compressor.
 *
 * Replaces ZCCL_float_openmp_threadblock_arg (ZCCL/src/ZCCL_float.c:501-807)
 * and produces the same bytes.  One CTA per tile of TB blocks, one thread per
 * block:
 *   1. TMA bulk copy of the tile's floats (plus the element before it) into
 *      shared memory, then a warp-cooperative transpose into padded rows so
 *      each thread walks its own block without bank conflicts;
 *   2. every thread quantizes its block (truncation, ZCCL_float.c:580),
 *      forms the running deltas (ZCCL_float.c:581-582; the element before the
 *      block supplies the first one), its sign mask, maximum magnitude, width
 *      (ZCCL_float.c:606) and encoded size;
 *   3. block-wide exclusive scan of the sizes, then a decoupled look-back
 *      across tiles places the tile in the output in the same pass (the
 *      reference's per-thread scan and second memcpy pass,
 *      ZCCL_float.c:774-791, disappear);
 *   4. every thread packs its block into a shared staging copy of the output
 *      that keeps the global 16-byte phase, and one TMA bulk store writes it.
 * The tile also records the side index: block widths, the tile's byte
 * offset and the quantized value before it.
 */
#include "zkern.cuh"

namespace {

template <bool FAST>
__global__ void __launch_bounds__(128) k_compress(const CompressArgs a)
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

    if (tid == 0) {
        bcast[0] = atomicAdd(a.w.ticket, 1u);
        mbar_init(bar, 1);
    }
    __syncthreads();
    const uint64_t tile = bcast[0];
    ZTile z;
    zg_tile(&g, tile, &z);

    /* 1. stage x[e_first - 1, e_end) and transpose into rows */
    const uint32_t nel = (uint32_t)(z.e_end - z.e_first + 1);
    const uint32_t ph =
        stage_in(stage, reinterpret_cast<const uint8_t *>(a.x + (z.e_first - 1)), nel * 4u, bar);
    stage_in_wait(bar, 0, a.w.err);
    const float *xin = reinterpret_cast<const float *>(stage + ph);
    for (uint32_t k = warp; k < z.nblk; k += nw) {
        uint32_t n = zg_block_len(z.seg_len, L, z.blk0 + k);
        for (uint32_t j = lane; j < n; j += 32) rows[k * stride + j] = xin[1 + k * L + j];
    }
    const float xprev0 = xin[0]; /* head for tile 0 of a segment, else last element of the previous tile */
    __syncthreads();

    /* 2. per-block quantize / delta / width */
    uint32_t b = 0, size = 0, n = 0, smask = 0, mx = 0;
    uint32_t m[FAST ? 32 : 1];
    float xp = 0.0f;
    if (tid < z.nblk) {
        n = zg_block_len(z.seg_len, L, z.blk0 + tid);
        const float *row = rows + tid * stride;
        xp = tid == 0 ? xprev0 : rows[(tid - 1) * stride + L - 1];
        int32_t qp = quantize(xp, a.inv, bad);
        if (FAST) {
#pragma unroll
            for (uint32_t j = 0; j < 32; j++) {
                uint32_t mg = 0;
                if (j < n) {
                    int32_t q = quantize(row[j], a.inv, bad);
                    int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                    qp = q;
                    uint32_t neg = d < 0 ? 1u : 0u;
                    mg = neg ? 0u - (uint32_t)d : (uint32_t)d;
                    smask |= neg << (31 - j);
                    mx = mx > mg ? mx : mg;
                }
                m[j] = mg;
            }
        } else {
            for (uint32_t j = 0; j < n; j++) {
                int32_t q = quantize(row[j], a.inv, bad);
                int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                qp = q;
                uint32_t mg = d < 0 ? 0u - (uint32_t)d : (uint32_t)d;
                mx = mx > mg ? mx : mg;
            }
        }
        b = width_of(mx, a.wt);
        size = zg_block_bytes(b, n);
    }

    /* 3. place the tile: block scan + look-back */
    const uint32_t headb = z.has_head ? 4u : 0u;
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

    if (tid < z.nblk) a.idx.widths[z.gblk0 + tid] = (uint8_t)b;
    const int32_t qprev0 = quantize(xprev0, a.inv, bad);
    if (tid == 0) {
        a.idx.tile_off[tile] = base;
        a.idx.tile_qprev[tile] = qprev0;
        if (fits && z.has_head && z.seg < g.T) {
            uint64_t h = base - 8ull * g.T;
#pragma unroll
            for (int k = 0; k < 8; k++) a.out[8ull * z.seg + k] = (uint8_t)(h >> (8 * k));
        }
        if (tile == g.ntiles - 1) *a.idx.size = base + total;
    }

    /* 4. pack into staging (16-byte phase of the destination) and store */
    uint8_t *gout = a.out + base;
    const uint32_t sph = (uint32_t)((uintptr_t)gout & 15u);
    uint32_t *sw = reinterpret_cast<uint32_t *>(stage);
    if (z.has_head && tid == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) stage[sph + k] = (uint8_t)((uint32_t)qprev0 >> (8 * k));
    }
    if (tid < z.nblk) {
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
                        if (j < n) bw.put(bswap32(m[j] >> r) >> (32 - 8 * B), 8 * B);
                }
                if (r) {
                    const uint32_t mask = (1u << r) - 1u;
#pragma unroll
                    for (uint32_t j = 0; j < 32; j++)
                        if (j < n) bw.put(m[j] & mask, r);
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
                const float *row = rows + tid * stride;
                int32_t qp = quantize(xp, a.inv, bad);
                const uint32_t mask = r ? (1u << r) - 1u : 0u;
                for (uint32_t j = 0; j < n; j++) {
                    int32_t q = quantize(row[j], a.inv, bad);
                    int32_t d = (int32_t)((uint32_t)q - (uint32_t)qp);
                    qp = q;
                    uint32_t neg = d < 0 ? 1u : 0u;
                    uint32_t mg = neg ? 0u - (uint32_t)d : (uint32_t)d;
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

cudaError_t launch_compress(const CompressArgs &a, cudaStream_t st)
{
    const bool fast = a.g.L <= 32;
    const void *fn = fast ? (const void *)k_compress<true> : (const void *)k_compress<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, a.sm.total);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)a.g.ntiles), block(a.g.TB);
    if (fast)
        k_compress<true><<<grid, block, a.sm.total, st>>>(a);
    else
        k_compress<false><<<grid, block, a.sm.total, st>>>(a);
    return cudaGetLastError();
}
