/*
 * zgeom.h -- geometry of a fastmode1 stream, shared by host and device code.
 *
 * A stream of N floats written by T OpenMP threads with block size L
 * (ZCCL/src/ZCCL_float.c:532-545, ZCCL/src/ZCCLd_float.c:558-566):
 *
 *   tbs = N / T, rem = N % T
 *   segment s < T : elements [s*tbs, (s+1)*tbs)       -> chunk s
 *   segment T     : elements [T*tbs, N) when rem > 0  -> appended to chunk T-1
 *   a segment of len elements = raw int32 head + ceil((len-1)/L) blocks; all
 *   blocks hold L elements except the last, which holds (len-1) % L when
 *   that is non-zero.
 *
 * On the device a segment is cut into tiles of up to TB consecutive blocks;
 * tile 0 of a segment also owns the segment's head.  Tiles are numbered in
 * stream order, so the byte offset of a tile is the exclusive prefix sum of
 * the byte sizes of all tiles before it.  One CUDA thread owns one block.
 */
#ifndef ZCCL_GB300_ZGEOM_H
#define ZCCL_GB300_ZGEOM_H

#include <stdint.h>

#ifdef __CUDACC__
#define ZG_HD __host__ __device__ __forceinline__
#else
#define ZG_HD static inline
#endif

#define ZG_MAX_L 256 /* largest block size the kernels accept */

typedef struct ZGeom {
    uint64_t n;       /* elements */
    uint64_t tbs;     /* elements per regular segment (n / T) */
    uint32_t T;       /* writer thread count = chunks in the header */
    uint32_t L;       /* block size */
    uint32_t rem;     /* n % T: length of the extra segment (0 = none) */
    uint32_t TB;      /* blocks per tile */
    uint64_t nb_reg;  /* blocks per regular segment */
    uint64_t nt_reg;  /* tiles per regular segment */
    uint64_t nb_rm;   /* blocks of the extra segment */
    uint64_t nt_rm;   /* tiles of the extra segment (0 when rem == 0) */
    uint64_t nblocks; /* all blocks */
    uint64_t ntiles;  /* all tiles */
    uint32_t fmt;     /* block magnitude layout: ZG_FASTMODE1 or ZG_FIXED_BYTES */
    uint32_t pad_;
} ZGeom;

/* Block magnitude layouts.  fastmode1: B = b/8 whole bytes per magnitude
 * (little-endian), then its r = b%8 low bits as an MSB-first stream
 * (ZCCL/src/ZCCL_TypeManager.c:12-91).  The fixed-rate appendix codec keeps
 * whole bytes only, B = b/8 + 1 of them (at most 4), r = 0
 * (ZCCL/src/ZCCL_appendix.c:18-39).  Everything else is shared. */
#define ZG_FASTMODE1 0u
#define ZG_FIXED_BYTES 1u

/* Per-tile view computed from a tile index. */
typedef struct ZTile {
    uint64_t seg_start; /* first element (the head) of the segment */
    uint64_t seg_len;   /* elements of the segment */
    uint64_t blk0;      /* first block of the tile, index within the segment */
    uint64_t gblk0;     /* first block of the tile, index within the stream */
    uint64_t e_first;   /* first element of the first block (head + 1 + blk0*L) */
    uint64_t e_end;     /* one past the last element of the tile's last block */
    uint32_t seg;       /* segment index (T for the extra segment) */
    uint32_t nblk;      /* blocks in the tile (0 for a segment of length 1) */
    uint32_t has_head;  /* tile 0 of its segment */
} ZTile;

ZG_HD uint64_t zg_div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

ZG_HD uint32_t zg_tile_blocks(uint32_t L)
{
    if (L <= 32) return 256;
    uint32_t k = 4096u / (32u * L);
    return 32u * (k ? k : 1u);
}

/* Bytes of a block of n elements encoded at width b
 * (ZCCL/src/ZCCL_TypeManager.c:24-29 plus header and sign bytes). */
ZG_HD uint32_t zg_block_bytes(uint32_t b, uint32_t n)
{
    if (b == 0) return 1;
    return 1 + (n + 7) / 8 + (b >> 3) * n + ((b & 7) * n + 7) / 8;
}

/* Whole bytes B and low bits r per magnitude of a width-b block in layout fmt. */
ZG_HD void zg_split(uint32_t fmt, uint32_t b, uint32_t *B, uint32_t *r)
{
    if (fmt == ZG_FIXED_BYTES) {
        *B = (b >> 3) + 1 < 4 ? (b >> 3) + 1 : 4;
        *r = 0;
    } else {
        *B = b >> 3;
        *r = b & 7;
    }
}

/* zg_block_bytes in layout fmt; both layouts take the same bytes at width 32. */
ZG_HD uint32_t zg_block_bytes_f(uint32_t fmt, uint32_t b, uint32_t n)
{
    if (b == 0) return 1;
    uint32_t B, r;
    zg_split(fmt, b, &B, &r);
    return 1 + (n + 7) / 8 + B * n + (r * n + 7) / 8;
}

/* Row stride (in 4-byte words) of the padded per-block shared-memory layout:
 * odd, so thread t reading word j of row t hits bank (t*stride + j) % 32,
 * distinct across a warp. */
ZG_HD uint32_t zg_row_stride(uint32_t L) { return (L & 1) ? L + 2 : L + 1; }

ZG_HD uint64_t zg_seg_blocks(uint64_t len, uint32_t L) { return len ? zg_div_up(len - 1, L) : 0; }

ZG_HD int zg_init(ZGeom *g, uint64_t n, uint32_t L, uint32_t T)
{
    if (T == 0 || L == 0 || L > ZG_MAX_L || n < T) return -1;
    g->n = n;
    g->T = T;
    g->L = L;
    g->fmt = ZG_FASTMODE1;
    g->pad_ = 0;
    g->tbs = n / T;
    g->rem = (uint32_t)(n % T);
    g->TB = zg_tile_blocks(L);
    g->nb_reg = zg_seg_blocks(g->tbs, L);
    g->nt_reg = g->nb_reg ? zg_div_up(g->nb_reg, g->TB) : 1;
    g->nb_rm = zg_seg_blocks(g->rem, L);
    g->nt_rm = g->rem ? (g->nb_rm ? zg_div_up(g->nb_rm, g->TB) : 1) : 0;
    g->nblocks = (uint64_t)T * g->nb_reg + g->nb_rm;
    g->ntiles = (uint64_t)T * g->nt_reg + g->nt_rm;
    if (g->ntiles >> 32) return -1; /* tile indices are 32-bit on the device */
    return 0;
}

ZG_HD void zg_tile(const ZGeom *g, uint64_t t, ZTile *z)
{
    uint64_t k, nb;
    if (t < (uint64_t)g->T * g->nt_reg) {
        uint64_t s = (uint32_t)t / (uint32_t)g->nt_reg; /* tiles and tiles per segment < 2^32 */
        k = t - s * g->nt_reg;
        z->seg = (uint32_t)s;
        z->seg_start = s * g->tbs;
        z->seg_len = g->tbs;
        nb = g->nb_reg;
        z->gblk0 = s * g->nb_reg + k * g->TB;
    } else {
        k = t - (uint64_t)g->T * g->nt_reg;
        z->seg = g->T;
        z->seg_start = (uint64_t)g->T * g->tbs;
        z->seg_len = g->rem;
        nb = g->nb_rm;
        z->gblk0 = (uint64_t)g->T * g->nb_reg + k * g->TB;
    }
    z->blk0 = k * g->TB;
    uint64_t left = nb > z->blk0 ? nb - z->blk0 : 0;
    z->nblk = (uint32_t)(left < g->TB ? left : g->TB);
    z->has_head = (k == 0);
    z->e_first = z->seg_start + 1 + z->blk0 * g->L;
    uint64_t last = (z->blk0 + z->nblk) * g->L; /* elements after the head, capped below */
    if (last > z->seg_len - 1) last = z->seg_len - 1;
    z->e_end = z->seg_start + 1 + last;
}

/* Elements of block j (index within the segment) of a segment of len. */
ZG_HD uint32_t zg_block_len(uint64_t len, uint32_t L, uint64_t j)
{
    uint64_t left = len - 1 - j * L;
    return (uint32_t)(left < L ? left : L);
}

/* Upper bound on the bytes of a whole stream (every block at width 32). */
ZG_HD uint64_t zg_seg_worst(uint64_t len, uint32_t L)
{
    if (!len) return 0;
    uint64_t nfull = (len - 1) / L, ntail = (len - 1) % L;
    uint64_t s = 4 + nfull * zg_block_bytes(32, L);
    if (ntail) s += zg_block_bytes(32, (uint32_t)ntail);
    return s;
}

ZG_HD uint64_t zg_stream_worst(const ZGeom *g)
{
    return 8ull * g->T + (uint64_t)g->T * zg_seg_worst(g->tbs, g->L) + zg_seg_worst(g->rem, g->L);
}

/* Shared-memory layout of the codec kernels (bytes), all regions 16-byte
 * aligned:
 *   [0, 256)   mbarriers, scan scratch, broadcast slots
 *   [256, 512) look-back records
 *   rows       per-block rows, TB x row_stride 4-byte words (floats or ints)
 *   in0, in1   double-buffered TMA input (raw floats or tile bytes)
 *   out        packed output tile (compressor, homomorphic add)
 *   jobs       copies of the jobs in progress (job_bytes) */
typedef struct ZSmem {
    uint32_t rows, in0, in1, out, jobs, total;
} ZSmem;

ZG_HD uint32_t zg_a16(uint32_t v) { return (v + 15u) & ~15u; }

/* Largest tile in bytes: head + TB blocks at width 32. */
ZG_HD uint32_t zg_tile_worst(uint32_t L, uint32_t TB) { return TB * zg_block_bytes(32, L) + 4u; }

/* Bytes a packed tile of `total` bytes takes in the output ring (its bytes,
 * the packer's zeroed tail, 16-byte granularity), and the ring's size: the
 * largest tile fits; readers may look 32 bytes past a tile, so the region
 * behind the ring has that slack. */
ZG_HD uint32_t zg_ring_need(uint32_t total) { return (total + 8u + 15u) & ~15u; }
ZG_HD uint32_t zg_ring_bytes(uint32_t L, uint32_t TB) { return zg_ring_need(zg_tile_worst(L, TB)); }

/* kind: 0 compressor, 1 decompressor, 2 homomorphic add.
 * The compressor stages one tile of floats at a time (in1 == in0) and keeps
 * a packed tile in out until the next tile has been quantized.  With
 * L <= 32 every warp holds its rows' floats in registers while they move
 * from the input into the rows, so the rows share the input's space
 * (rows == in0); longer blocks get separate regions.  The decompressor and
 * the homomorphic add double-buffer their input. */
ZG_HD ZSmem zg_smem_base(uint32_t kind, uint32_t L, uint32_t TB);

ZG_HD ZSmem zg_smem(uint32_t kind, uint32_t L, uint32_t TB, uint32_t job_bytes)
{
    ZSmem m = zg_smem_base(kind, L, TB);
    m.jobs = m.total;
    m.total = zg_a16(m.jobs + job_bytes);
    return m;
}

ZG_HD ZSmem zg_smem_base(uint32_t kind, uint32_t L, uint32_t TB)
{
    ZSmem m;
    const uint32_t rows_bytes = TB * zg_row_stride(L) * 4u;
    const uint32_t raw_in = (TB * L + 1u) * 4u + 32u;     /* floats, 16-byte superset */
    const uint32_t tile_in = zg_tile_worst(L, TB) + 48u;  /* bytes, superset + reader slack */
    const uint32_t tile_out = zg_ring_bytes(L, TB) + 48u; /* the ring; readers look 32 past */
    const int need_rows = kind != 2 || L > 32;
    m.rows = 1024u;
    if (kind == 0) {
        if (L <= 32) {
            m.in0 = m.rows;
            m.in1 = m.in0;
            m.out = zg_a16(m.rows + (rows_bytes > raw_in ? rows_bytes : raw_in));
            m.total = zg_a16(m.out + tile_out);
        } else {
            m.in0 = zg_a16(m.rows + rows_bytes);
            m.in1 = m.in0;
            m.out = zg_a16(m.in0 + raw_in);
            m.total = zg_a16(m.out + tile_out);
        }
        return m;
    }
    m.in0 = zg_a16(m.rows + (need_rows ? rows_bytes : 0u));
    if (kind == 1) { /* one input buffer: three CTAs per SM instead of two buffers' two */
        m.in1 = m.in0;
        m.out = zg_a16(m.in0 + tile_in);
        m.total = m.out;
        return m;
    }
    m.in1 = zg_a16(m.in0 + tile_in);
    m.out = zg_a16(m.in1 + tile_in);
    m.total = zg_a16(m.out + tile_out);
    return m;
}

#endif
