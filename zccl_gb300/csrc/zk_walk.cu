/*
 * zk_walk.cu -- side-index builder for streams that arrive as bytes only
 * (written by the reference, or by any writer that did not keep the index).
 *
 * The wire format has no block index: inside a chunk, block k starts where
 * block k-1 ends, and only the 1-byte width header says how long a block is
 * (ZCCL/src/ZCCLd_float.c:598-614).  The chunk starts come from the T-entry
 * header.  This builder follows each chunk's headers from its start (one
 * thread per chunk), records every width, the byte offset of every tile and
 * the stream's total size, and checks the walk against the geometry: widths
 * must be <= 32, every chunk must end exactly where the next one starts, and
 * no block may pass the readable bytes.
 */
#include "zkern.cuh"

namespace {

/* Walk one segment starting at byte `pos` (its head); returns the byte just
 * past its last block, or UINT64_MAX after an error. */
__device__ uint64_t walk_segment(const WalkArgs &a, uint32_t seg, uint64_t pos)
{
    const ZGeom &g = a.g;
    uint64_t len, nb, gblk, tile0;
    if (seg < g.T) {
        len = g.tbs;
        nb = g.nb_reg;
        gblk = (uint64_t)seg * g.nb_reg;
        tile0 = (uint64_t)seg * g.nt_reg;
    } else {
        len = g.rem;
        nb = g.nb_rm;
        gblk = (uint64_t)g.T * g.nb_reg;
        tile0 = (uint64_t)g.T * g.nt_reg;
    }
    if (pos + 4 > a.avail) {
        atomicOr(a.err, ZERR_BOUNDS);
        return UINT64_MAX;
    }
    a.idx.tile_off[tile0] = pos;
    pos += 4;
    for (uint64_t j = 0; j < nb; j++) {
        if (j && j % g.TB == 0) a.idx.tile_off[tile0 + j / g.TB] = pos;
        if (pos >= a.avail) {
            atomicOr(a.err, ZERR_BOUNDS);
            return UINT64_MAX;
        }
        uint32_t b = a.in[pos];
        if (b > 32) {
            atomicOr(a.err, ZERR_CORRUPT);
            return UINT64_MAX;
        }
        a.idx.widths[gblk + j] = (uint8_t)b;
        pos += zg_block_bytes(b, zg_block_len(len, g.L, j));
    }
    if (pos > a.avail) {
        atomicOr(a.err, ZERR_BOUNDS);
        return UINT64_MAX;
    }
    return pos;
}

__device__ uint64_t load_u64(const uint8_t *p)
{
    uint64_t v = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) v |= (uint64_t)p[k] << (8 * k);
    return v;
}

__global__ void k_walk(const WalkArgs a)
{
    const ZGeom &g = a.g;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.T) return;
    const uint64_t hdr = 8ull * g.T;
    if (hdr > a.avail) {
        atomicOr(a.err, ZERR_BOUNDS);
        return;
    }
    const uint64_t rel = load_u64(a.in + 8ull * s);
    if (s == 0 && rel != 0) atomicOr(a.err, ZERR_CORRUPT); /* header[0] is always 0 */
    if (rel > a.avail - hdr) {
        atomicOr(a.err, ZERR_BOUNDS);
        return;
    }
    uint64_t pos = hdr + rel;
    uint64_t end = walk_segment(a, s, pos);
    if (end == UINT64_MAX) return;
    if (s + 1 < g.T) {
        if (end != hdr + load_u64(a.in + 8ull * (s + 1))) atomicOr(a.err, ZERR_CORRUPT);
    } else {
        if (g.rem) end = walk_segment(a, g.T, end);
        if (end != UINT64_MAX) *a.idx.size = end;
    }
}

} // namespace

cudaError_t launch_walk(const WalkArgs &a, cudaStream_t st)
{
    const unsigned threads = 64;
    k_walk<<<(a.g.T + threads - 1) / threads, threads, 0, st>>>(a);
    return cudaGetLastError();
}
