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
 *       passed.  Each lane makes one backward pass over its 128-byte
 *       sub-window, giving for every position where a walk from it leaves the
 *       sub-window and how many blocks it passes; a walk from any entry is
 *       then one hop per sub-window.
 *   W2  compose the tables: per group of G windows (parallel), then per
 *       segment across groups, giving each group its true entry offset and
 *       first block number.
 *   W3  per window, the path from its true entry, followed by one lane
 *       along 32 speculative sub-window walks run in parallel (see below),
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
constexpr uint32_t WARPS_W3 = 8; /* warps per CTA in W3, a window each at a time */

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

/* full_size on a walk's critical path: for 32-element fastmode1 blocks
 * (header, four sign bytes, 4 b bytes of magnitudes; a zero-width block is
 * its header alone) two operations instead of the general formula. */
struct Sizer {
    uint32_t L, fmt, fast;
    __device__ __forceinline__ Sizer(uint32_t L_, uint32_t fmt_)
        : L(L_), fmt(fmt_), fast(L_ == 32u && fmt_ == ZG_FASTMODE1) {}
    __device__ __forceinline__ uint32_t operator()(uint32_t b) const
    {
        if (fast) return b - 1u < 32u ? 4u * b + 5u : 1u;
        return full_size(b, L, fmt);
    }
};

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

/* ---- the exits of every position of a sub-window ----------------------
 *
 * A window of WW = 32 x 128 bytes sits in shared memory, copied into rows of
 * SUB + 4 bytes so that lane j reads sub-window j with no bank conflict.
 * Lane j makes one backward pass over its sub-window: for every position i,
 * where a walk of the headers from i leaves the sub-window (and, for W1, how
 * many blocks it passes), from the result at the position i steps to.  The
 * results are kept at i * 33 + j, again free of bank conflicts.  A walk from
 * any entry then takes one hop per sub-window.  Bytes that cannot be headers
 * (above 32) count as 1-byte blocks, so walks stay bounded. */
constexpr uint32_t SUB = WALK_WW / 32; /* bytes per sub-window */
static_assert(SUB == 128, "a sub-window map is four 32-bit words");
constexpr uint32_t W1_ROW = SUB + 4;  /* bytes per skewed row */
constexpr uint32_t W1_RES = SUB * 33; /* results */

/* All lanes: the window's bytes into the skewed rows (row k: sub-window k). */
__device__ __forceinline__ void copy_rows(const uint8_t *bytes, uint8_t *rows)
{
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll 4
    for (uint32_t k = 0; k < 32; k++) { /* row k: lane copies bytes 4 lane .. 4 lane + 3 */
        const uint8_t *src = bytes + SUB * k + 4u * lane;
        const uint32_t v = (uint32_t)src[0] | (uint32_t)src[1] << 8 | (uint32_t)src[2] << 16 | (uint32_t)src[3] << 24;
        *reinterpret_cast<uint32_t *>(rows + W1_ROW * k + 4u * lane) = v;
    }
}

/* Lane j's backward pass over its row: res[i * 33 + j] = (exit - SUB) << 8 |
 * blocks passed. */
template <class R>
__device__ __forceinline__ void backward_pass(const uint8_t *row, R *res, const Sizer &size)
{
    const uint32_t lane = threadIdx.x & 31u;
    for (int i = (int)SUB - 1; i >= 0; i--) {
        const uint32_t nxt = (uint32_t)i + size(row[i]);
        res[i * 33 + lane] = (R)(nxt >= SUB ? (nxt - SUB) << 8 | 1u : (uint32_t)res[nxt * 33 + lane] + 1u);
    }
}

/* Bytes of a warp's window area: the window with its alignment slack,
 * then the WinPath. */
__host__ __device__ inline uint32_t win_area(uint32_t M) { return (WALK_WW + M + 32u + 15u) & ~15u; }

/* The window [start, start + WW + M) of the stream into the 16-byte-aligned
 * area buf (bytes past avail read as 0), by aligned 16-byte loads that the
 * warp issues together; returns where the window's first byte landed. */
__device__ __forceinline__ const uint8_t *load_window(const WalkArgs &a, uint64_t start, uint8_t *buf)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uintptr_t base = reinterpret_cast<uintptr_t>(a.in), end = base + a.avail;
    const uintptr_t lo = (base + start) & ~(uintptr_t)15;
    const uint32_t ph = (uint32_t)(base + start - lo), nl = (ph + WALK_WW + a.M + 15u) / 16u;
    uint4 *d = reinterpret_cast<uint4 *>(buf);
#pragma unroll 8
    for (uint32_t i = lane; i < nl; i += 32) {
        const uintptr_t p = lo + 16u * i;
        if (p >= base && p + 16u <= end) {
            d[i] = *reinterpret_cast<const uint4 *>(p);
        } else { /* a line across either end of the readable bytes */
            uint32_t v[4] = {0, 0, 0, 0};
            for (uint32_t k = 0; k < 16; k++) {
                const uintptr_t q = p + k;
                if (q >= base && q < end) v[k >> 2] |= (uint32_t)*reinterpret_cast<const uint8_t *>(q) << (8 * (k & 3));
            }
            d[i] = make_uint4(v[0], v[1], v[2], v[3]);
        }
    }
    return buf + ph;
}

/* ---- W1 --------------------------------------------------------------
 * Per window, the backward passes give every position's exit from its
 * sub-window and the blocks passed.  The exits go out to the workspace
 * (one byte per position, for W3), and the window's table is made: for
 * every entry offset e < M, the exit offset into the next window and the
 * blocks passed, a walk of one hop per sub-window.  A result is (exit - end
 * of the sub-window) << 8 | blocks passed (<= SUB), 16 bits while blocks are
 * shorter than 256 bytes (block sizes up to 48), else 32.  Per warp: the
 * results (the plain window copy lands there first), then the skewed rows. */

__host__ __device__ inline uint32_t w1_warp_bytes(uint32_t M)
{
    const uint32_t res = W1_RES * (M < 256 ? 2u : 4u), win = win_area(M);
    return (res > win ? res : win) + 32u * W1_ROW;
}

template <class R>
__global__ void __launch_bounds__(32 * WARPS_W1) k_walk_tables(const WalkArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t M = a.M;
    const Sizer size(g.L, g.fmt);
    /* persistent: the warps stride over the windows the header gives */
    for (uint32_t wg = blockIdx.x * WARPS_W1 + warp; wg < w.win_base[g.T]; wg += gridDim.x * WARPS_W1) {
        const uint32_t s = find_seg(w.win_base, g.T, wg);
        const uint64_t start = w.seg_P[s] + (uint64_t)(wg - w.win_base[s]) * WALK_WW;

        uint8_t *area = smem + warp * a.w1_warp_bytes;
        R *res = reinterpret_cast<R *>(area);
        uint8_t *rows = area + (a.w1_warp_bytes - 32u * W1_ROW);
        const uint8_t *bytes = load_window(a, start, area);
        __syncwarp();
        copy_rows(bytes, rows);
        __syncwarp();
        backward_pass(rows + W1_ROW * lane, res, size);
        __syncwarp();
        /* the exits, element p = 128 j + i of the window's row of WW (bytes
         * while blocks are shorter than 256 bytes, else 16 bits), as whole
         * words: lane l writes words l, l + 32, ... */
        constexpr uint32_t EB = sizeof(R) / 2; /* bytes per exit */
        uint32_t *ex = reinterpret_cast<uint32_t *>(a.ws.wexit + (uint64_t)wg * WALK_WW * EB);
#pragma unroll 4
        for (uint32_t q = lane; q < WALK_WW * EB / 4u; q += 32) {
            const uint32_t p0 = q * (4u / EB), j = p0 / SUB, i = p0 % SUB;
            uint32_t v = 0;
#pragma unroll
            for (uint32_t t = 0; t < 4u / EB; t++) v |= ((uint32_t)res[(i + t) * 33 + j] >> 8) << (8 * EB * t);
            ex[q] = v;
        }
        uint32_t *tab = a.ws.wtab + (uint64_t)wg * M;
        /* the table: the walks from the M entries leave sub-window 0 at
         * few distinct places (walks that meet go on together), so only
         * the walks from those places are followed to the window's end,
         * one lane each, and every entry adds its first hop; the rows'
         * space (free after the backward passes) holds the places' flags
         * and results */
        auto walk = [&](uint32_t pos, uint32_t cnt) -> uint32_t {
            while (pos < WALK_WW) {
                const uint32_t j = pos / SUB, r = res[(pos % SUB) * 33 + j];
                cnt += r & 0xFFu;
                pos = (j + 1) * SUB + (r >> 8);
            }
            return (pos - WALK_WW) << 16 | cnt;
        };
        /* where the walk from entry e leaves sub-window 0 (SUB + offset)
         * and the blocks it passed there */
        auto first = [&](uint32_t e, uint32_t &c0) -> uint32_t {
            if (e >= SUB) {
                c0 = 0;
                return e;
            }
            const uint32_t r = res[e * 33];
            c0 = r & 0xFFu;
            return SUB + (r >> 8);
        };
        if (5u * M <= 32u * W1_ROW) {
            uint8_t *need = rows;                                        /* [M] */
            uint32_t *fin = reinterpret_cast<uint32_t *>(rows + ((M + 15u) & ~15u)); /* [M] */
            for (uint32_t x = lane; x < M; x += 32) need[x] = 0;
            __syncwarp();
            for (uint32_t e = lane; e < M; e += 32) {
                uint32_t c0;
                need[first(e, c0) - SUB] = 1;
            }
            __syncwarp();
            for (uint32_t x = lane; x < M; x += 32)
                if (need[x]) fin[x] = walk(SUB + x, 0);
            __syncwarp();
            for (uint32_t e = lane; e < M; e += 32) {
                uint32_t c0;
                const uint32_t f = fin[first(e, c0) - SUB];
                tab[e] = f + c0; /* the count in the low 16 bits stays below 2^16 */
            }
        } else {
            for (uint32_t e = lane; e < M; e += 32) tab[e] = walk(e, 0);
        }
        __syncwarp(); /* the area is reused for the next window */
    }
}

/* ---- W2a: compose the window tables of each group ----------------------
 * For every entry offset into the group, the walk through its windows'
 * tables; each step's entry offset and the blocks passed before it are kept
 * (gwin), so that once the group's true entry is known every window's is a
 * single load. */
__global__ void k_walk_groups(const WalkArgs a)
{
    extern __shared__ __align__(16) uint32_t tabs[]; /* the group's window tables */
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t gg = blockIdx.x;
    if (gg >= w.grp_base[g.T]) return;
    const uint32_t s = find_seg(w.grp_base, g.T, gg);
    const uint32_t nwin = w.win_base[s + 1] - w.win_base[s];
    const uint32_t w0 = (gg - w.grp_base[s]) * WALK_G;
    const uint32_t w1 = min(w0 + WALK_G, nwin);
    /* one coalesced copy, so that the walks' dependent steps read shared memory */
    const uint32_t *gt = w.wtab + (uint64_t)(w.win_base[s] + w0) * a.M;
    for (uint32_t i = threadIdx.x; i < (w1 - w0) * a.M; i += blockDim.x) tabs[i] = __ldg(gt + i);
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < a.M; e += blockDim.x) {
        uint32_t x = e;
        uint64_t c = 0;
        uint32_t *gw = w.gwin + ((uint64_t)gg * a.M + e) * WALK_G;
        for (uint32_t k = 0; k < w1 - w0; k++) {
            gw[k] = (uint32_t)c << 12 | x; /* c < 32 windows x 4096 blocks; x < M < 4096 */
            const uint32_t t = tabs[k * a.M + x];
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

/* ---- W3: the true walk of every window -------------------------------
 * One warp per window: its true entry and first block are one load (gwin at
 * its group's true entry); lane 0 hops once per sub-window from the entry,
 * on the exits W1 left for every position, and notes where the true path
 * enters each one; then every lane walks its sub-window from there, and all
 * lanes write the widths and tile offsets of their blocks at once.  Shared
 * bytes per warp: the window, its exits, the path. */
constexpr uint32_t NOT_ENTERED = 0xFFFFFFFFu;

struct WinPath {
    uint32_t tm[32][4]; /* the true path's positions, per sub-window */
    uint32_t ent[32];   /* where the true path enters sub-window j, or NOT_ENTERED */
    uint32_t pref[33];  /* true-path positions before sub-window j; [32] = all */
};

__host__ __device__ inline uint32_t w3_exit_bytes(uint32_t M) { return WALK_WW * (M < 256 ? 1u : 2u); }
__host__ __device__ inline uint32_t w3_warp_bytes(uint32_t M)
{
    return (win_area(M) + w3_exit_bytes(M) + (uint32_t)sizeof(WinPath) + 15u) & ~15u;
}

/* All lanes: the window's exits (W1's row of WW elements) into ex, by
 * aligned 16-byte loads. */
__device__ __forceinline__ void load_exits(const uint8_t *src, uint8_t *ex, uint32_t bytes)
{
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll 4
    for (uint32_t i = lane; i < bytes / 16u; i += 32)
        reinterpret_cast<uint4 *>(ex)[i] = reinterpret_cast<const uint4 *>(src)[i];
}

/* All lanes: the true path of the window from `entry` into wp (maps, prefix
 * counts), from the window's bytes and exits. */
template <class E>
__device__ __forceinline__ void true_path(const uint8_t *bytes, const E *ex, uint32_t entry, const Sizer &size,
                                          WinPath *wp)
{
    const uint32_t lane = threadIdx.x & 31u;
    wp->ent[lane] = NOT_ENTERED;
    __syncwarp();
    if (lane == 0) { /* one hop per sub-window (a long block may step over one) */
        uint32_t pos = entry;
        while (pos < WALK_WW) {
            const uint32_t j = pos / SUB;
            wp->ent[j] = pos % SUB;
            pos = (j + 1) * SUB + (uint32_t)ex[pos];
        }
    }
    __syncwarp();
    uint32_t t[4] = {0, 0, 0, 0};
    const uint8_t *sub = bytes + lane * SUB;
    for (uint32_t q = wp->ent[lane]; q < SUB; q += size(sub[q])) /* NOT_ENTERED: no step */
#pragma unroll
        for (uint32_t w = 0; w < 4; w++) t[w] |= w == (q >> 5) ? 1u << (q & 31u) : 0u;
#pragma unroll
    for (uint32_t w = 0; w < 4; w++) wp->tm[lane][w] = t[w];
    const uint32_t cnt = __popc(t[0]) + __popc(t[1]) + __popc(t[2]) + __popc(t[3]);
    const uint32_t incl = warp_incl_scan(cnt);
    wp->pref[lane] = incl - cnt;
    if (lane == 31) wp->pref[32] = incl;
}

template <class E>
__global__ void __launch_bounds__(32 * WARPS_W3, 3) k_walk_final(const WalkArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const ZGeom &g = a.g;
    const WalkScratch &w = a.ws;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t xb = w3_exit_bytes(a.M);
    const Sizer size(g.L, g.fmt);
    const uint64_t nb = g.nb_reg;
    const uint64_t nfull = (g.tbs - 1) / g.L;
    const uint32_t ntail = (uint32_t)((g.tbs - 1) % g.L);
    uint8_t *area = smem + warp * w3_warp_bytes(a.M);
    E *ex = reinterpret_cast<E *>(area + win_area(a.M));
    WinPath *wp = reinterpret_cast<WinPath *>(area + win_area(a.M) + xb);
    /* persistent: the warps stride over the windows the header gives */
    for (uint32_t wi = blockIdx.x * nw + warp; wi < w.win_base[g.T]; wi += gridDim.x * nw) {
        const uint32_t s = find_seg(w.win_base, g.T, wi);
        if (!w.seg_ok[s]) continue; /* uniform over the warp */
        const uint32_t k = wi - w.win_base[s]; /* the window within its segment */
        const uint32_t gg = w.grp_base[s] + k / WALK_G;
        const uint32_t v = w.gwin[((uint64_t)gg * a.M + w.gentry[gg]) * WALK_G + k % WALK_G];
        const uint64_t b0 = w.gbase[gg] + (v >> 12);
        if (b0 >= nb) continue;
        const uint64_t gblk0 = (uint64_t)s * g.nb_reg, tile0 = (uint64_t)s * g.nt_reg;
        const uint64_t start = w.seg_P[s] + (uint64_t)k * WALK_WW;
        load_exits(w.wexit + (uint64_t)wi * xb, reinterpret_cast<uint8_t *>(ex), xb);
        const uint8_t *bytes = load_window(a, start, area);
        __syncwarp();
        true_path(bytes, ex, v & 0xFFFu, size, wp);
        __syncwarp();
        /* lane j records the true-path blocks of its sub-window; the
         * next tile boundary at or after its first block is found once */
        uint64_t blk = b0 + wp->pref[lane];
        const uint64_t tq = blk / g.TB;
        uint64_t tnext = tq * g.TB, tidx = tq;
        if (tnext < blk) {
            tnext += g.TB;
            tidx++;
        }
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
                const uint32_t b = bytes[pos];
                if (b > 32) {
                    atomicOr(a.err, ZERR_CORRUPT);
                    m = 0;
                    break;
                }
                if (blk == tnext) {
                    if (blk) a.idx.tile_off[tile0 + tidx] = gpos;
                    tnext += g.TB;
                    tidx++;
                }
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

size_t walk_w1_warp_bytes(uint32_t M) { return w1_warp_bytes(M); }

/* Persistent grid: the CTAs that fit at once, at most `most`. */
static unsigned walk_grid(const void *fn, unsigned threads, size_t smem, unsigned most)
{
    const unsigned g = (unsigned)sm_count() * (unsigned)blocks_per_sm(fn, (int)threads, smem);
    return most < g ? (most ? most : 1) : g;
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
    const void *f1 = a.M < 256 ? (const void *)k_walk_tables<uint16_t> : (const void *)k_walk_tables<uint32_t>;
    if ((e = set_max_smem(f1, smem1)) != cudaSuccess) return e;
    const unsigned grid1 = walk_grid(f1, 32 * WARPS_W1, smem1, (a.max_windows + WARPS_W1 - 1) / WARPS_W1);
    if (a.M < 256)
        k_walk_tables<uint16_t><<<grid1, 32 * WARPS_W1, smem1, st>>>(a);
    else
        k_walk_tables<uint32_t><<<grid1, 32 * WARPS_W1, smem1, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const unsigned threads2 = std::min(1024u, (a.M + 31u) / 32u * 32u); /* one thread per entry offset */
    const uint32_t smem2a = 4u * WALK_G * a.M;
    if ((e = set_max_smem((const void *)k_walk_groups, smem2a)) != cudaSuccess) return e;
    k_walk_groups<<<a.max_groups, threads2, smem2a, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    a.seg_batch = (160u * 1024u) / (8u * a.M);
    if (a.seg_batch > WALK_G) a.seg_batch = WALK_G;
    if (a.seg_batch < 1) a.seg_batch = 1;
    const uint32_t smem2 = a.seg_batch * a.M * 8u;
    if ((e = set_max_smem((const void *)k_walk_segments, smem2)) != cudaSuccess)
        return e;
    k_walk_segments<<<a.g.T, 256, smem2, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const uint32_t wstride = w3_warp_bytes(a.M);
    /* as many warps as fit (fewer for the largest blocks) */
    int dev = 0, smax = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess)
        return e;
    uint32_t warps3 = WARPS_W3;
    while (warps3 > 1 && warps3 * wstride > (uint32_t)smax) warps3--;
    const uint32_t smem3 = warps3 * wstride;
    const void *f3 = a.M < 256 ? (const void *)k_walk_final<uint8_t> : (const void *)k_walk_final<uint16_t>;
    if ((e = set_max_smem(f3, smem3)) != cudaSuccess) return e;
    const unsigned grid3 = walk_grid(f3, 32 * warps3, smem3, (a.max_windows + warps3 - 1) / warps3);
    if (a.M < 256)
        k_walk_final<uint8_t><<<grid3, 32 * warps3, smem3, st>>>(a);
    else
        k_walk_final<uint16_t><<<grid3, 32 * warps3, smem3, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_walk_finish<<<1, 32, 0, st>>>(a);
    return cudaGetLastError();
}
