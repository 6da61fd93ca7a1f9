/*
 * zk_walk.cu -- side-index builder for streams that arrive as bytes only
 * (written by the reference, or by any writer that did not keep the index).
 *
 * The wire format has no block index: inside a chunk, block k starts where
 * block k-1 ends, and only its 1-byte width header says how long it is
 * (ZCCL/src/ZCCLd_float.c:598-614).  Walking the headers is a chain of
 * dependent loads as long as the chunk, so it is split into windows of WW
 * bytes and done in parallel, exactly:
 *
 *   W0  chunk starts from the T-entry header; per segment its block region
 *       and window count; heads' tile offsets.
 *   W1  for every window and every possible entry offset e in [0, M) (M = the
 *       largest block): the exit offset into the next window and the blocks
 *       passed.  The path from entry 0 is stitched from 32 speculative
 *       sub-window walks run in parallel (see below), and every other entry
 *       is walked only until it meets that path, so a window costs a few
 *       dozen dependent steps instead of a full walk.
 *   W2  compose the tables: per group of G windows (parallel), then per
 *       segment across groups, giving each group its true entry offset and
 *       first block number.
 *   W3  per window, the path from its true entry, stitched the same way,
 *       gives every block's width and every tile's offset, written by all
 *       lanes at once; each chunk must end where the next starts.
 *   W4  the extra segment of the last chunk (N % T elements) and the total
 *       size.
 * Widths above 32, chunk ends that disagree with the header, and blocks past
 * the readable bytes set ZERR_CORRUPT / ZERR_BOUNDS instead of faulting.
 */
#include "zkern.cuh"

namespace {

constexpr uint32_t WARPS_W1 = 8;
constexpr uint32_t WARPS_W3 = 16; /* warps per group in W3: two windows each */

__device__ __forceinline__ uint64_t load_u64(const uint8_t *p)
{
    uint64_t v = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) v |= (uint64_t)p[k] << (8 * k);
    return v;
}

/* Size of a full block whose header byte is b; bytes that cannot be a
 * header (b > 32) count as 1 so speculative walks stay bounded. */
__device__ __forceinline__ uint32_t full_size(uint32_t b, uint32_t L, uint32_t fmt)
{
    return b <= 32 ? zg_block_bytes_f(fmt, b, L) : 1u;
}

/* Segment of a window / group index: last s with base[s] <= i. */
__device__ __forceinline__ uint32_t find_seg(const uint32_t *base, uint32_t T, uint32_t i)
{
    uint32_t lo = 0, hi = T; /* base[lo] <= i < base[hi] */
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* ---- W0 -------------------------------------------------------------- */
__global__ void k_walk_setup(const WalkArgs a)
{
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint64_t hdr = 8ull * g.T;
    __shared__ uint32_t wsum[33];
    uint32_t carry_w = 0, carry_g = 0;
    for (uint32_t s0 = 0; s0 < g.T; s0 += blockDim.x) {
        const uint32_t s = s0 + threadIdx.x;
        uint32_t nwin = 0;
        if (s < g.T) {
            uint64_t P = 0, R = 0;
            bool ok = hdr <= a.avail;
            if (!ok) atomicOr(a.err, ZERR_BOUNDS);
            if (ok) {
                uint64_t rel = load_u64(a.in + 8ull * s);
                if (s == 0 && rel != 0) atomicOr(a.err, ZERR_CORRUPT);
                if (rel > a.avail - hdr || hdr + rel + 4 > a.avail) {
                    atomicOr(a.err, ZERR_BOUNDS);
                    ok = false;
                } else {
                    a.idx.tile_off[(uint64_t)s * g.nt_reg] = hdr + rel;
                    P = hdr + rel + 4;
                    if (s + 1 < g.T) {
                        uint64_t rn = load_u64(a.in + 8ull * (s + 1));
                        R = hdr + rn;
                        /* chunk starts increase and a stream never exceeds end_bound,
                         * which keeps the window count within the scratch */
                        if (rn > a.avail - hdr || R < P || R > a.end_bound) {
                            atomicOr(a.err, ZERR_CORRUPT);
                            ok = false;
                        }
                    } else {
                        /* the last chunk: no later start bounds it, but its
                         * blocks take at most a segment's worst size (a
                         * remainder segment follows them and is walked apart) */
                        R = a.avail < a.end_bound ? a.avail : a.end_bound;
                        const uint64_t worst = P - 4 + zg_seg_worst(g.tbs, g.L);
                        if (R > worst) R = worst;
                        if (R < P) R = P;
                    }
                }
            }
            if (ok && g.nb_reg > 0) nwin = (uint32_t)zg_div_up(R - P, WALK_WW);
            if (ok && g.nb_reg > 0 && nwin == 0) {
                atomicOr(a.err, ZERR_BOUNDS);
                ok = false;
            }
            w.seg_P[s] = P;
            w.seg_R[s] = R;
            w.seg_end[s] = (ok && g.nb_reg == 0) ? P : 0;
            w.seg_ok[s] = ok ? 1u : 0u;
            if (ok && g.nb_reg == 0 && s + 1 < g.T && P != R) atomicOr(a.err, ZERR_CORRUPT);
        }
        uint32_t tot_w, tot_g;
        uint32_t bw = cta_excl_scan(nwin, wsum, &tot_w);
        uint32_t bg = cta_excl_scan((nwin + WALK_G - 1) / WALK_G, wsum, &tot_g);
        if (s < g.T) {
            w.win_base[s] = carry_w + bw;
            w.grp_base[s] = carry_g + bg;
        }
        carry_w += tot_w;
        carry_g += tot_g;
    }
    if (threadIdx.x == 0) {
        w.win_base[g.T] = carry_w;
        w.grp_base[g.T] = carry_g;
    }
}

/* ---- shared by W1 and W3: the path of the headers through one window ---
 *
 * A window of WW = 32 x 128 bytes sits in shared memory.  Lane j walks the
 * headers speculatively from byte 128 j until it leaves its sub-window and
 * records the positions it visited (a 128-bit map).  A walk from a true
 * block start is the true path, and two walks that meet at a position go
 * on together, so the true path from a known entry is stitched across the
 * sub-windows: where it enters sub-window j at a position lane j visited,
 * it is lane j's walk from there on; otherwise it is walked until it meets
 * lane j's walk or leaves the sub-window (a few blocks).  Bytes that cannot
 * be headers (above 32) count as 1-byte blocks, so walks stay bounded. */
constexpr uint32_t SUB = WALK_WW / 32; /* bytes per sub-window */
static_assert(SUB == 128, "a sub-window map is four 32-bit words");

struct WinPath {
    uint32_t spec[32][4]; /* lane j's visited positions in sub-window j */
    uint32_t sx[32];      /* where lane j's walk left its sub-window */
    uint32_t tm[32][4];   /* the true path's positions, per sub-window */
    uint32_t pref[33];    /* true-path positions before sub-window j; [32] = all */
    uint32_t exit;        /* where the true path leaves the window */
};

__device__ __forceinline__ bool map_bit(const uint32_t *m, uint32_t i)
{
    return (m[i >> 5] >> (i & 31u)) & 1u;
}

/* All lanes: the speculative sub-window walks. */
__device__ __forceinline__ void spec_walks(const uint8_t *bytes, uint32_t L, uint32_t fmt, WinPath *wp)
{
    const uint32_t lane = threadIdx.x & 31u, lo = lane * SUB;
    uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0, pos = lo;
    while (pos < lo + SUB) {
        const uint32_t i = pos - lo, bit = 1u << (i & 31u), w = i >> 5;
        m0 |= w == 0 ? bit : 0u;
        m1 |= w == 1 ? bit : 0u;
        m2 |= w == 2 ? bit : 0u;
        m3 |= w == 3 ? bit : 0u;
        pos += full_size(bytes[pos], L, fmt);
    }
    wp->spec[lane][0] = m0;
    wp->spec[lane][1] = m1;
    wp->spec[lane][2] = m2;
    wp->spec[lane][3] = m3;
    wp->sx[lane] = pos;
}

/* One lane: the true path from window position `entry`, per sub-window,
 * with the prefix counts; returns where it leaves the window. */
__device__ __forceinline__ uint32_t stitch(const uint8_t *bytes, uint32_t L, uint32_t fmt, uint32_t entry, WinPath *wp)
{
    uint32_t p = entry, cnt = 0;
    for (uint32_t j = 0; j < 32; j++) {
        const uint32_t lo = j * SUB, hi = lo + SUB;
        uint32_t t[4] = {0, 0, 0, 0};
        wp->pref[j] = cnt;
        if (p < hi) {
            uint32_t q = p;
            for (;;) {
                const uint32_t i = q - lo;
                if (map_bit(wp->spec[j], i)) { /* joins lane j's walk: the rest of it */
#pragma unroll
                    for (uint32_t w = 0; w < 4; w++) {
                        const uint32_t sw = wp->spec[j][w];
                        t[w] |= w < (i >> 5) ? 0u : w > (i >> 5) ? sw : sw & ~((1u << (i & 31u)) - 1u);
                    }
                    q = wp->sx[j];
                    break;
                }
#pragma unroll
                for (uint32_t w = 0; w < 4; w++) t[w] |= w == (i >> 5) ? 1u << (i & 31u) : 0u;
                q += full_size(bytes[q], L, fmt);
                if (q >= hi) break;
            }
            p = q;
        }
#pragma unroll
        for (uint32_t w = 0; w < 4; w++) {
            wp->tm[j][w] = t[w];
            cnt += __popc(t[w]);
        }
    }
    wp->pref[32] = cnt;
    wp->exit = p;
    return p;
}

/* True-path positions before window position q (q < WW). */
__device__ __forceinline__ uint32_t path_rank(const WinPath *wp, uint32_t q)
{
    const uint32_t j = q / SUB, i = q % SUB;
    uint32_t r = wp->pref[j];
#pragma unroll
    for (uint32_t w = 0; w < 4; w++) {
        const uint32_t m = wp->tm[j][w];
        r += w < (i >> 5) ? __popc(m) : w == (i >> 5) ? __popc(m & ((1u << (i & 31u)) - 1u)) : 0u;
    }
    return r;
}

__device__ __forceinline__ void load_window(const WalkArgs &a, uint64_t start, uint8_t *bytes)
{
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t i = lane; i < WALK_WW + a.M; i += 32) {
        const uint64_t p = start + i;
        bytes[i] = p < a.avail ? a.in[p] : 0;
    }
}

/* ---- W1 -------------------------------------------------------------- */
__global__ void __launch_bounds__(32 * WARPS_W1) k_walk_tables(const WalkArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t M = a.M;
    const uint32_t wg = blockIdx.x * WARPS_W1 + warp;
    if (wg >= w.win_base[g.T]) return;
    const uint32_t s = find_seg(w.win_base, g.T, wg);
    const uint64_t start = w.seg_P[s] + (uint64_t)(wg - w.win_base[s]) * WALK_WW;

    /* per-warp shared area: bytes[WW + M + 16] | WinPath */
    uint8_t *bytes = smem + warp * a.w1_warp_bytes;
    WinPath *wp = reinterpret_cast<WinPath *>(bytes + ((WALK_WW + M + 16 + 15) & ~15u));
    load_window(a, start, bytes);
    __syncwarp();
    spec_walks(bytes, g.L, g.fmt, wp);
    __syncwarp();
    if (lane == 0) stitch(bytes, g.L, g.fmt, 0, wp);
    __syncwarp();
    /* entry e: walk until the path from entry 0 is met (then its exit and
     * the blocks left on it) or the window ends */
    const uint32_t x0 = wp->exit - WALK_WW, c0 = wp->pref[32];
    uint32_t *tab = a.ws.wtab + (uint64_t)wg * M;
    for (uint32_t e = lane; e < M; e += 32) {
        uint32_t q = e, k = 0;
        while (q < WALK_WW && !map_bit(wp->tm[q / SUB], q % SUB)) {
            q += full_size(bytes[q], g.L, g.fmt);
            k++;
        }
        const uint32_t ex = q < WALK_WW ? x0 : q - WALK_WW;
        const uint32_t cnt = q < WALK_WW ? k + c0 - path_rank(wp, q) : k;
        tab[e] = (ex << 16) | cnt;
    }
}

/* ---- W2a: compose the window tables of each group ---------------------- */
__global__ void k_walk_groups(const WalkArgs a)
{
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t gg = blockIdx.x;
    if (gg >= w.grp_base[g.T]) return;
    const uint32_t s = find_seg(w.grp_base, g.T, gg);
    const uint32_t nwin = w.win_base[s + 1] - w.win_base[s];
    const uint32_t w0 = (gg - w.grp_base[s]) * WALK_G;
    const uint32_t w1 = min(w0 + WALK_G, nwin);
    for (uint32_t e = threadIdx.x; e < a.M; e += blockDim.x) {
        uint32_t x = e;
        uint64_t c = 0;
        for (uint32_t k = w0; k < w1; k++) {
            uint32_t t = __ldg(w.wtab + (uint64_t)(w.win_base[s] + k) * a.M + x);
            c += t & 0xFFFFu;
            x = t >> 16;
        }
        w.gtab[(uint64_t)gg * a.M + e] = (c << 32) | x;
    }
}

/* ---- W2b: per segment, carry the entry offset across its groups -------- */
__global__ void k_walk_segments(const WalkArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *rows = reinterpret_cast<uint64_t *>(smem);
    __shared__ uint64_t s_base;
    __shared__ uint32_t s_x;
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t s = blockIdx.x;
    if (!w.seg_ok[s]) return;
    const uint32_t g0 = w.grp_base[s], g1 = w.grp_base[s + 1];
    uint32_t x = 0;
    uint64_t base = 0;
    for (uint32_t b0 = g0; b0 < g1; b0 += a.seg_batch) {
        const uint32_t nb = min(a.seg_batch, g1 - b0);
        if (base < g.nb_reg) /* groups past the last block need no table */
            for (uint32_t i = threadIdx.x; i < nb * a.M; i += blockDim.x)
                rows[i] = w.gtab[(uint64_t)b0 * a.M + i];
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t j = 0; j < nb; j++) {
                w.gentry[b0 + j] = x;
                w.gbase[b0 + j] = base;
                if (base < g.nb_reg) {
                    uint64_t t = rows[j * a.M + x];
                    base += t >> 32;
                    x = (uint32_t)t;
                }
            }
            s_base = base;
            s_x = x;
        }
        __syncthreads();
        base = s_base;
        x = s_x;
    }
}

/* ---- W3: the true walk of every window ------------------------------- */
__global__ void __launch_bounds__(32 * WARPS_W3) k_walk_final(const WalkArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t gg = blockIdx.x;
    if (gg >= w.grp_base[g.T]) return;
    const uint32_t s = find_seg(w.grp_base, g.T, gg);
    if (!w.seg_ok[s]) return;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t nwin = w.win_base[s + 1] - w.win_base[s];
    const uint32_t w0 = (gg - w.grp_base[s]) * WALK_G;
    const uint32_t w1 = min(w0 + WALK_G, nwin);
    uint32_t *entry = reinterpret_cast<uint32_t *>(smem);
    uint64_t *bbase = reinterpret_cast<uint64_t *>(smem + 4 * WALK_G);
    uint8_t *wbuf = smem + 12 * WALK_G;
    const uint32_t wstride = a.w1_warp_bytes;

    const uint64_t nb = g.nb_reg;
    const uint64_t nfull = (g.tbs - 1) / g.L;
    const uint32_t ntail = (uint32_t)((g.tbs - 1) % g.L);
    const uint64_t gblk0 = (uint64_t)s * g.nb_reg, tile0 = (uint64_t)s * g.nt_reg;

    if (threadIdx.x == 0) {
        uint32_t x = w.gentry[gg];
        uint64_t b = w.gbase[gg];
        for (uint32_t k = w0; k < w1; k++) {
            entry[k - w0] = x;
            bbase[k - w0] = b;
            if (b >= nb) continue;
            uint32_t t = w.wtab[(uint64_t)(w.win_base[s] + k) * a.M + x];
            b += t & 0xFFFFu;
            x = t >> 16;
        }
    }
    __syncthreads();
    for (uint32_t k = w0 + warp; k < w1; k += nw) {
        const uint64_t b0 = bbase[k - w0];
        if (b0 >= nb) continue;
        const uint64_t start = w.seg_P[s] + (uint64_t)k * WALK_WW;
        uint8_t *buf = wbuf + warp * wstride;
        WinPath *wp = reinterpret_cast<WinPath *>(buf + ((WALK_WW + a.M + 16 + 15) & ~15u));
        load_window(a, start, buf);
        __syncwarp();
        spec_walks(buf, g.L, g.fmt, wp);
        __syncwarp();
        if (lane == 0) stitch(buf, g.L, g.fmt, entry[k - w0], wp);
        __syncwarp();
        /* lane j records the true-path blocks of its sub-window */
        uint64_t blk = b0 + wp->pref[lane];
#pragma unroll
        for (uint32_t wd = 0; wd < 4; wd++) {
            uint32_t m = wp->tm[lane][wd];
            while (m && blk < nb) {
                const uint32_t pos = lane * SUB + wd * 32 + (uint32_t)(__ffs(m) - 1);
                m &= m - 1;
                const uint64_t gpos = start + pos;
                if (gpos >= a.avail) {
                    atomicOr(a.err, ZERR_BOUNDS);
                    m = 0;
                    break;
                }
                const uint32_t b = buf[pos];
                if (b > 32) {
                    atomicOr(a.err, ZERR_CORRUPT);
                    m = 0;
                    break;
                }
                if (blk % g.TB == 0 && blk) a.idx.tile_off[tile0 + blk / g.TB] = gpos;
                a.idx.widths[gblk0 + blk] = (uint8_t)b;
                const uint32_t n = blk < nfull ? g.L : ntail;
                blk++;
                if (blk == nb) {
                    const uint64_t end = gpos + zg_block_bytes_f(g.fmt, b, n);
                    if (end > a.avail) atomicOr(a.err, ZERR_BOUNDS);
                    w.seg_end[s] = end;
                    if (s + 1 < g.T && end != w.seg_R[s]) atomicOr(a.err, ZERR_CORRUPT);
                }
            }
        }
        __syncwarp();
    }
}

/* ---- W4: extra segment and total size -------------------------------- */
__global__ void k_walk_finish(const WalkArgs a)
{
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    if (threadIdx.x != 0) return;
    for (uint32_t s = 0; s < g.T; s++) {
        if (!w.seg_ok[s]) return; /* W0 already reported why */
        if (w.seg_end[s] == 0) {  /* the walk never reached this segment's last block */
            atomicOr(a.err, ZERR_CORRUPT);
            return;
        }
    }
    uint64_t pos = w.seg_end[g.T - 1];
    if (g.rem) {
        const uint64_t tile0 = (uint64_t)g.T * g.nt_reg, gblk0 = (uint64_t)g.T * g.nb_reg;
        if (pos + 4 > a.avail) {
            atomicOr(a.err, ZERR_BOUNDS);
            return;
        }
        a.idx.tile_off[tile0] = pos;
        pos += 4;
        for (uint64_t j = 0; j < g.nb_rm; j++) {
            if (j && j % g.TB == 0) a.idx.tile_off[tile0 + j / g.TB] = pos;
            if (pos >= a.avail) {
                atomicOr(a.err, ZERR_BOUNDS);
                return;
            }
            uint32_t b = a.in[pos];
            if (b > 32) {
                atomicOr(a.err, ZERR_CORRUPT);
                return;
            }
            a.idx.widths[gblk0 + j] = (uint8_t)b;
            pos += zg_block_bytes_f(g.fmt, b, zg_block_len(g.rem, g.L, j));
        }
        if (pos > a.avail) {
            atomicOr(a.err, ZERR_BOUNDS);
            return;
        }
    }
    *a.idx.size = pos;
}

} // namespace

size_t walk_w1_warp_bytes(uint32_t M)
{
    return ((WALK_WW + M + 16 + 15) & ~15u) + sizeof(WinPath);
}

cudaError_t launch_walk(const WalkArgs &a0, cudaStream_t st)
{
    WalkArgs a = a0;
    a.M = zg_block_bytes(32, a.g.L);
    a.w1_warp_bytes = (uint32_t)walk_w1_warp_bytes(a.M);
    cudaError_t e;
    k_walk_setup<<<1, 256, 0, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const uint32_t smem1 = WARPS_W1 * a.w1_warp_bytes;
    if ((e = cudaFuncSetAttribute(k_walk_tables, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem1)) != cudaSuccess)
        return e;
    k_walk_tables<<<(a.max_windows + WARPS_W1 - 1) / WARPS_W1, 32 * WARPS_W1, smem1, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_walk_groups<<<a.max_groups, 128, 0, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    a.seg_batch = (160u * 1024u) / (8u * a.M);
    if (a.seg_batch > WALK_G) a.seg_batch = WALK_G;
    if (a.seg_batch < 1) a.seg_batch = 1;
    const uint32_t smem2 = a.seg_batch * a.M * 8u;
    if ((e = cudaFuncSetAttribute(k_walk_segments, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem2)) != cudaSuccess)
        return e;
    k_walk_segments<<<a.g.T, 256, smem2, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const uint32_t wstride = (uint32_t)walk_w1_warp_bytes(a.M);
    const uint32_t smem3 = 12 * WALK_G + WARPS_W3 * wstride;
    if ((e = cudaFuncSetAttribute(k_walk_final, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem3)) != cudaSuccess)
        return e;
    k_walk_final<<<a.max_groups, 32 * WARPS_W3, smem3, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_walk_finish<<<1, 32, 0, st>>>(a);
    return cudaGetLastError();
}
