/*
 * zkern.cuh -- kernel argument blocks and launchers (internal interface
 * between the C-ABI layer and the kernels).
 */
#ifndef ZCCL_GB300_ZKERN_CUH
#define ZCCL_GB300_ZKERN_CUH

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "zdev.cuh"
#include "zgeom.h"

#define ZH_MAXP 32 /* most inputs one homomorphic-add launch accepts */

/* Per-call scratch in device memory, zeroed before every call:
 * err | walk_err | ticket | pad | status[ntiles]. */
struct ZWork {
    uint32_t *err;      /* ZERR_* bits of the codec kernels */
    uint32_t *walk_err; /* ZERR_* bits of the index walk that ran before, if any */
    uint32_t *ticket;   /* next tile to hand out */
    uint64_t *status;   /* decoupled look-back state, one word per tile */
    uint32_t lb_spin;   /* polls before a look-back wait gives up */
};

/* Side index of a resident stream: enough to find every block without
 * walking the 1-byte headers, and the quantized value before every tile so
 * decompression needs no scan. */
struct ZIndex {
    uint8_t *widths;     /* [nblocks] width byte of every block, stream order */
    uint64_t *tile_off;  /* [ntiles]  byte offset (from stream start) of each tile's first unit */
    int32_t *tile_qprev; /* [ntiles]  quantized value of the element before the tile's first block */
    uint64_t *size;      /* [1]       total stream bytes */
};

/* One buffer to compress: the kernels take a single job from their
 * arguments, or a batch of jobs from device memory, whose tiles then form
 * one ticket sequence (tile_job gives every batch tile its job, job_tile0
 * every job its first batch tile). */
struct alignas(16) CompressJob {
    ZGeom g;
    const float *x;
    uint8_t *out;
    uint64_t cap; /* writable bytes at `out` */
    ZIndex idx;
    uint64_t *status; /* this buffer's look-back words, one per tile */
    float inv;        /* 1.0f / eb, computed on the host in float */
    uint32_t boxed;   /* batch job: batch.maps[job] views x as rows of 32 floats */
};

struct ZBatch {
    const void *jobs;          /* CompressJob[] or HomAddJob[]; null: the single job */
    const uint16_t *tile_job;  /* [ntiles] */
    const uint64_t *job_tile0; /* [njobs] */
    uint32_t njobs;
    uint64_t ntiles;  /* tiles of all jobs */
    const void *maps; /* compress: CUtensorMap[njobs] in device memory (used where a job is boxed), or null */
};

struct CompressArgs {
    CompressJob job; /* the single job (batch.jobs == null) */
    ZBatch batch;
    ZWork w; /* err and ticket; status is per job */
    ZWidthTable wt;
    ZSmem sm;
    uint32_t grid; /* CTAs to launch, 0 = as many as fit */
    int rows_map;  /* set by the launcher: its tensor map views job.x as rows of 32 floats */
};

struct DecompressArgs {
    const uint8_t *in;
    uint64_t avail; /* readable bytes at `in` */
    float *y;
    ZGeom g;
    float eb;
    ZIndex idx;      /* widths and tile_off must be valid */
    int qprev_valid; /* tile_qprev valid; else recovered by look-back and written */
    ZWork w;
    ZSmem sm;
    int rows_map;    /* set by the launcher: its tensor map views y as rows of 32 floats */
};

struct HomInput {
    const uint8_t *bytes;
    uint64_t avail;
    const uint8_t *widths;
    const uint64_t *tile_off;
    const int32_t *tile_qprev;
};

/* One homomorphic sum of P streams. */
struct alignas(16) HomAddJob {
    ZGeom g;
    HomInput in[ZH_MAXP];
    uint32_t P;
    int qprev_valid;  /* every input's tile_qprev is valid */
    uint8_t *out;
    uint64_t cap;     /* writable bytes at `out` */
    ZIndex idx;       /* index of the output stream */
    uint64_t *status; /* look-back words of the output, one per tile */
};

/* One indexed stream to decompress (with its tiles' starting values): the
 * floats go to y, or are added to y with accumulate. */
struct alignas(16) DecompressJob {
    ZGeom g;
    const uint8_t *in;
    uint64_t avail; /* readable bytes at `in` */
    float *y;
    ZIndex idx;
    float eb;
    int accumulate;
};

struct DecompressJobsArgs {
    DecompressJob job; /* the single job (batch.jobs == null) */
    ZBatch batch;
    ZWork w; /* err, walk_err */
    ZSmem sm;
    uint32_t grid; /* CTAs to launch, 0 = as many as fit */
};

/* One staged input tile of the homomorphic add: which tile and input it
 * is, and where its bytes start within the buffer (the TMA copy keeps the
 * source's 16-byte phase). */
struct HStage {
    uint64_t tile; /* within its job; ZP_NONE: no more tiles */
    uint32_t job;
    uint32_t p;    /* the input */
    uint32_t ph;   /* the tile's first byte in the buffer */
    uint32_t pad[3];
};

/* What the adding warps need of a claimed tile, written by the loader with
 * the tile's first input so that the adders read shared memory instead of
 * the job in device or parameter memory.  ZH_TILE_RECS records, by tile
 * count: the loader runs at most two input copies ahead of the adders, so a
 * record is reused only after its tile is packed. */
struct HTile {
    uint64_t gblk0;      /* first block of the tile in its stream */
    uint8_t *widths;     /* the sum's width index */
    int32_t *tile_qprev; /* the sum's tile starting values, or null */
    uint64_t *status;    /* the sum's look-back words */
    uint32_t P, nblk;
    uint32_t nlast;      /* elements of the tile's last block */
    uint32_t has_head;   /* tile 0 of its segment */
    uint32_t qsum;       /* the inputs' starting values of the tile, summed */
    uint32_t pad[3];
};
#define ZH_TILE_RECS 4u

struct HomAddArgs {
    HomAddJob job; /* the single job (batch.jobs == null) */
    ZBatch batch;
    unsigned long long *cases; /* optional [4]: both zero, first zero, second zero, both non-zero (P == 2) */
    ZWork w;
    ZWidthTable wt;
    ZSmem sm;
    uint32_t grid; /* CTAs to launch, 0 = as many as fit */
};

#define WALK_WW 4096u /* bytes per window of the parallel header walk */
#define WALK_G 32u     /* windows per group */

/* Device scratch of the header walk (part of the workspace). */
struct WalkScratch {
    uint64_t *seg_P;    /* [T]   first block byte of each regular segment */
    uint64_t *seg_R;    /* [T]   end of its byte region (next chunk start, or a bound) */
    uint64_t *seg_end;  /* [T]   byte after its last block, found by the walk */
    uint32_t *seg_ok;   /* [T]   header entries usable */
    uint32_t *win_base; /* [T+1] first window of each segment (prefix sum) */
    uint32_t *grp_base; /* [T+1] first window group of each segment */
    uint32_t *wtab;     /* [max_windows * M] exit offset << 16 | blocks, per entry offset */
    uint64_t *gtab;     /* [max_groups * M]  blocks << 32 | exit offset, per group */
    uint32_t *gentry;   /* [max_groups] true entry offset of each group */
    uint64_t *gbase;    /* [max_groups] first block (in its segment) of each group */
    uint8_t *wexit;     /* [max_windows * WW] per position: exit - end of its sub-window */
    uint32_t *gwin;     /* [max_groups * M * WALK_G] per group, entry offset and window k of it:
                           blocks before k << 12 | entry offset of k */
};

struct WalkArgs {
    const uint8_t *in;
    uint64_t avail;     /* readable bytes at `in` */
    uint64_t end_bound; /* no stream of this geometry is longer */
    ZGeom g;
    ZIndex idx;
    uint32_t *err;
    WalkScratch ws;
    uint32_t max_windows, max_groups;
    uint32_t M;             /* largest full block in bytes (filled by launch_walk) */
    uint32_t w1_warp_bytes; /* filled by launch_walk */
    uint32_t seg_batch;     /* group tables staged per step of W2b (filled by launch_walk) */
};

/* Shared bytes per warp of the window-table kernel. */
size_t walk_w1_warp_bytes(uint32_t M);

/* Grid of a persistent kernel: every CTA that fits on the device at once,
 * but no more CTAs than tiles. */
#define ZP_NONE (~0ull) /* no more tiles */

/* ------------------------------------------------------------------
 * Hand-off of packed tiles from the compute warps to the placer warp.
 *
 * The packed tiles wait in a ring of R bytes of shared memory (R holds
 * the largest tile; two typical tiles fit at once), so the compute warps
 * can pack tile k + 1 while the placer still writes out tile k.  Two
 * counters order the hand-off: `packed` (tiles packed, written by compute
 * thread 0) and `placed` (tiles written out, written by placer lane 0).
 * Tile k's size, ring position and index sit in slot k % 2.  All waits are
 * bounded: on time-out ZERR_TIMEOUT is set and the caller goes on.
 * ------------------------------------------------------------------ */
struct ZRing {
    uint32_t packed, placed;
    uint32_t pos[2], total[2];
    uint64_t tile[2]; /* the tile within its job */
    uint32_t job[2];  /* its job in the batch (0 for a single job) */
};

__device__ __forceinline__ void ring_set(uint32_t *p, uint32_t v)
{
    asm volatile("st.release.cta.shared.u32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t ring_get(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.cta.shared.u32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}

/* One thread: wait until *p >= v. */
__device__ __forceinline__ void ring_wait(const uint32_t *p, uint32_t v, uint32_t *err)
{
    for (uint32_t i = 0; i < (1u << 24); i++) {
        if ((int32_t)(ring_get(p) - v) >= 0) return;
        __nanosleep(64);
    }
    atomicOr(err, ZERR_TIMEOUT);
}

/* Compute thread 0, before packing tile k (0-based) of `need` bytes: its
 * ring position, after waiting until the placer has released the space.
 * end_prev / pos_prev describe tile k - 1 (updated here). */
__device__ __forceinline__ uint32_t ring_reserve(ZRing *ring, uint32_t k, uint32_t need, uint32_t R,
                                                 uint32_t &pos_prev, uint32_t &end_prev, uint32_t *err)
{
    const uint32_t pos = end_prev + need <= R ? end_prev : 0u;
    /* tile k - 2 is always out of the way (its slot is reused); tile k - 1
     * too when this tile wraps onto it */
    uint32_t req = k >= 1 ? k - 1 : 0u;
    if (k >= 1 && pos < end_prev && pos + need > pos_prev) req = k;
    ring_wait(&ring->placed, req, err);
    pos_prev = pos;
    end_prev = pos + need;
    return pos;
}

/* Compute thread 0, after every compute thread has finished packing tile k
 * (pass ZP_NONE as `tile` once there are no more tiles). */
__device__ __forceinline__ void ring_publish(ZRing *ring, uint32_t k, uint64_t tile, uint32_t job,
                                             uint32_t total, uint32_t pos)
{
    ring->tile[k & 1u] = tile;
    ring->job[k & 1u] = job;
    ring->total[k & 1u] = total;
    ring->pos[k & 1u] = pos;
    ring_set(&ring->packed, k + 1);
}

/* ------------------------------------------------------------------
 * The same hand-off with early sizes and ZR_SLOTS slots.  A tile's identity and
 * size go to the placer (mbarrier `sized`, one arrival by thread 0) right
 * after the scan has found them, so the placer's look-back runs while the
 * tile is still being packed; `packed` (one arrival per packing warp) then
 * hands over its bytes.  Ring space is counted in running bytes: a tile
 * takes the next `need` bytes (skipping to the ring's start when it would
 * not fit before the end) and may be written once the placer's running
 * count of released bytes, `tail`, shows that the space is free.  Up to
 * ZR_SLOTS tiles are between sizing and write-out at once (the ring's bytes
 * hold one worst-case tile, far more typical ones), so the packing warps do
 * not wait for a placer delayed by a slow look-back; 16 measured 3.7 %
 * faster than 4 on the two-way add.  Its control block sits below the
 * rows at offset 1024 of shared memory.
 * ------------------------------------------------------------------ */
#define ZR_SLOTS 16u

struct ZRing4 {
    uint32_t placed; /* tiles written out (placer lane 0, release) */
    uint32_t tail;   /* running count of released ring bytes (release) */
    uint32_t total[ZR_SLOTS], pos[ZR_SLOTS], mend[ZR_SLOTS], job[ZR_SLOTS];
    uint64_t tile[ZR_SLOTS];
    uint64_t sized[ZR_SLOTS], packed[ZR_SLOTS]; /* mbarriers */
};

/* Thread 0, before the CTA's first barrier. */
__device__ __forceinline__ void ring4_init(ZRing4 *r, uint32_t packers)
{
    r->placed = 0;
    r->tail = 0;
    for (uint32_t i = 0; i < ZR_SLOTS; i++) {
        mbar_init(&r->sized[i], 1);
        mbar_init(&r->packed[i], packers);
    }
}

/* Thread 0: tile k's identity and size for the placer, once the placer is
 * done with tile k - ZR_SLOTS, the previous user of the slot.  ZP_NONE as
 * `tile` ends the placer. */
__device__ __forceinline__ void ring4_sized(ZRing4 *r, uint32_t k, uint64_t tile, uint32_t job, uint32_t total,
                                            uint32_t *err)
{
    if (k >= ZR_SLOTS) ring_wait(&r->placed, k - ZR_SLOTS + 1, err);
    const uint32_t s = k % ZR_SLOTS;
    r->tile[s] = tile;
    r->job[s] = job;
    r->total[s] = total;
    mbar_arrive(&r->sized[s]);
}

/* Every packing thread (the same result in each): the ring position of the
 * next tile of `need` bytes, after waiting until its bytes are free.  H is
 * the running count of ring bytes taken (compared with wrap-around) and hp
 * the ring position after the last tile; *mend receives the tile's running
 * end. */
__device__ __forceinline__ uint32_t ring4_space(ZRing4 *r, uint32_t need, uint32_t R, uint32_t &H, uint32_t &hp,
                                                uint32_t &mend, uint32_t *err)
{
    const uint32_t H0 = H;
    uint32_t M = H, pos = hp;
    if (pos + need > R) { /* skip the ring's end */
        M += R - pos;
        pos = 0;
    }
    H = M + need;
    hp = pos + need;
    mend = H;
    /* the bytes' previous contents end at running byte M + need - R, but
     * nothing past H0 was ever written: after a skip the requirement is at
     * most that every earlier tile is out */
    uint32_t req = M + need - R;
    if ((int32_t)(req - H0) > 0) req = H0;
    ring_wait(&r->tail, req, err);
    return pos;
}

/* Thread 0, before its warp's `packed` arrival: where tile k lies. */
__device__ __forceinline__ void ring4_where(ZRing4 *r, uint32_t k, uint32_t pos, uint32_t mend)
{
    r->pos[k % ZR_SLOTS] = pos;
    r->mend[k % ZR_SLOTS] = mend;
}

/* What the placer needs of a job. */
struct ZPlace {
    ZGeom g;
    uint8_t *out;
    uint64_t cap;
    ZIndex idx;
    uint64_t *status;
};

/* Shared bytes of the homomorphic add's job region: the placer's job, two
 * stage records, the tile records and two block tables (offset << 8 |
 * width per block). */
static inline uint32_t homadd_job_bytes(uint32_t TB)
{
    return zg_a16((uint32_t)sizeof(ZPlace)) + 2u * (uint32_t)sizeof(HStage) + ZH_TILE_RECS * (uint32_t)sizeof(HTile) +
           2u * TB * 4u;
}


/* The placer warp: for every packed tile, in order, the decoupled look-back
 * gives its byte offset in its stream; its bytes go out with 16-byte vector
 * stores realigned to that offset, with its offset in the side index, the
 * stream size after the stream's last tile and, for a segment's first tile,
 * the chunk offset in the header.  wait_packed(k) (all lanes) returns once
 * tile k is packed; fetch(job, ZPlace *) (lane 0) copies a job's placement
 * data into shared memory.  With `zero`, the ring bytes of a tile are set
 * back to zero once written out, so the packers find zeroed space. */
template <class Wait, class Fetch>
__device__ __forceinline__ void placer_loop(ZRing *ring, uint8_t *ringb, ZPlace *pj, uint32_t *err,
                                            uint64_t max_tiles, uint32_t &bad, bool zero, uint32_t spin,
                                            Wait wait_packed, Fetch fetch)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t cur_job = 0xFFFFFFFFu;
    for (uint64_t k = 0; k <= max_tiles; k++) {
        wait_packed(k);
        __syncwarp();
        const uint32_t slot = (uint32_t)k & 1u;
        const uint64_t t = ring->tile[slot];
        const uint32_t job = ring->job[slot];
        const uint32_t total = ring->total[slot], pos = ring->pos[slot];
        if (t == ZP_NONE) break;
        if (job != cur_job) {
            if (lane == 0) fetch(job, pj);
            __syncwarp();
            cur_job = job;
        }
        const ZGeom &g = pj->g;
        const uint64_t base = 8ull * g.T + lb_resolve(pj->status, t, total, t == 0, 0, err, spin);
        const bool fits = base + total <= pj->cap;
        if (!fits) bad |= ZERR_CAPACITY;
        if (lane == 0) {
            ZTile z;
            zg_tile(&g, t, &z);
            pj->idx.tile_off[t] = base;
            if (fits && z.has_head && z.seg < g.T) {
                const uint64_t h = base - 8ull * g.T;
#pragma unroll
                for (int k8 = 0; k8 < 8; k8++) pj->out[8ull * z.seg + k8] = (uint8_t)(h >> (8 * k8));
            }
            if (t == g.ntiles - 1) *pj->idx.size = base + total;
        }
        if (fits) store_realign(pj->out + base, ringb + pos, total, lane, 32);
        if (zero) {
            __syncwarp(); /* every lane has read the tile */
            uint4 *zr = reinterpret_cast<uint4 *>(ringb + pos);
            for (uint32_t i = lane; i < zg_ring_need(total) / 16u; i += 32) zr[i] = make_uint4(0, 0, 0, 0);
        }
        __syncwarp();
        if (lane == 0) ring_set(&ring->placed, (uint32_t)k + 1);
    }
}

/* The placer warp on a ZRing4: for tile k, the look-back starts as soon
 * as its size is known; the side-index entries follow, and once the tile is
 * packed its bytes go out and its ring bytes are zeroed and released. */
template <class Fetch>
__device__ __forceinline__ void placer_loop4(ZRing4 *r, uint8_t *ringb, ZPlace *pj, uint32_t *err,
                                             uint64_t max_tiles, uint32_t &bad, uint32_t spin, Fetch fetch)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t cur_job = 0xFFFFFFFFu;
    for (uint64_t k = 0; k <= max_tiles; k++) {
        const uint32_t s = (uint32_t)(k % ZR_SLOTS), par = (uint32_t)(k / ZR_SLOTS) & 1u;
        mbar_wait(&r->sized[s], par, err);
        const uint64_t t = r->tile[s];
        const uint32_t job = r->job[s], total = r->total[s];
        if (t == ZP_NONE) break;
        if (job != cur_job) {
            if (lane == 0) fetch(job, pj);
            __syncwarp();
            cur_job = job;
        }
        const ZGeom &g = pj->g;
        const uint64_t base = 8ull * g.T + lb_resolve(pj->status, t, total, t == 0, 0, err, spin);
        const bool fits = base + total <= pj->cap;
        if (!fits) bad |= ZERR_CAPACITY;
        if (lane == 0) {
            ZTile z;
            zg_tile(&g, t, &z);
            pj->idx.tile_off[t] = base;
            if (fits && z.has_head && z.seg < g.T) {
                const uint64_t h = base - 8ull * g.T;
#pragma unroll
                for (int k8 = 0; k8 < 8; k8++) pj->out[8ull * z.seg + k8] = (uint8_t)(h >> (8 * k8));
            }
            if (t == g.ntiles - 1) *pj->idx.size = base + total;
        }
        mbar_wait(&r->packed[s], par, err);
        const uint32_t pos = r->pos[s], mend = r->mend[s];
        if (fits) store_realign(pj->out + base, ringb + pos, total, lane, 32);
        __syncwarp(); /* every lane has read the tile */
        uint4 *zr = reinterpret_cast<uint4 *>(ringb + pos);
        for (uint32_t i = lane; i < zg_ring_need(total) / 16u; i += 32) zr[i] = make_uint4(0, 0, 0, 0);
        __syncwarp();
        if (lane == 0) {
            ring_set(&r->tail, mend);
            ring_set(&r->placed, (uint32_t)k + 1);
        }
    }
}

/* One thread: copy n bytes (a multiple of 16, both 16-byte aligned) one
 * vector at a time, so a job copy holds few registers. */
__device__ __forceinline__ void copy16(void *dst, const void *src, uint32_t n)
{
    uint4 *d = static_cast<uint4 *>(dst);
    const uint4 *s = static_cast<const uint4 *>(src);
#pragma unroll 1
    for (uint32_t i = 0; i < n / 16u; i++) d[i] = s[i];
}

/* Thread 0: the job and local tile of batch ticket t. */
__device__ __forceinline__ uint32_t batch_job(const ZBatch &b, uint64_t t, uint64_t *local)
{
    if (!b.jobs) {
        *local = t;
        return 0;
    }
    const uint32_t j = b.tile_job[t];
    *local = t - b.job_tile0[j];
    return j;
}

/* Launch-shape queries, remembered per device and kernel: the occupancy
 * calculator and the shared-memory attribute cost host time on every
 * launch, and a pipelined host-buffer call launches a hundred kernels. */
struct LaunchCache {
    struct Occ {
        const void *fn;
        int dev, threads, per;
        size_t smem;
    };
    struct Attr {
        const void *fn;
        int dev;
        size_t smem;
    };
    std::mutex mu;
    Occ occ[96];
    Attr attr[64];
    int nocc = 0, nattr = 0;
    int nsm[64] = {0};
};

static inline LaunchCache &launch_cache()
{
    static LaunchCache c;
    return c;
}

/* Blocks of fn per SM at this block size and shared memory (at least 1). */
static inline int blocks_per_sm(const void *fn, int threads, size_t smem)
{
    LaunchCache &c = launch_cache();
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(c.mu);
        for (int i = 0; i < c.nocc; i++)
            if (c.occ[i].fn == fn && c.occ[i].dev == dev && c.occ[i].threads == threads && c.occ[i].smem == smem)
                return c.occ[i].per;
    }
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        per = 0;
    }
    if (per < 1) per = 1;
    std::lock_guard<std::mutex> lk(c.mu);
    if (c.nocc < 96) c.occ[c.nocc++] = {fn, dev, threads, per, smem};
    return per;
}

/* SMs of the current device. */
static inline int sm_count()
{
    LaunchCache &c = launch_cache();
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && c.nsm[dev] > 0) return c.nsm[dev];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
        cudaGetLastError();
        return 1;
    }
    if (dev >= 0 && dev < 64) c.nsm[dev] = n;
    return n;
}

/* cudaFuncSetAttribute(fn, MaxDynamicSharedMemorySize, smem), skipped when
 * an equal or larger value is already set for fn on this device. */
static inline cudaError_t set_max_smem(const void *fn, size_t smem)
{
    LaunchCache &c = launch_cache();
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(c.mu);
        for (int i = 0; i < c.nattr; i++)
            if (c.attr[i].fn == fn && c.attr[i].dev == dev && c.attr[i].smem >= smem) return cudaSuccess;
    }
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(c.mu);
    for (int i = 0; i < c.nattr; i++)
        if (c.attr[i].fn == fn && c.attr[i].dev == dev) {
            c.attr[i].smem = smem;
            return cudaSuccess;
        }
    if (c.nattr < 64) c.attr[c.nattr++] = {fn, dev, smem};
    return cudaSuccess;
}

static inline unsigned persistent_grid(const void *fn, int threads, size_t smem, uint64_t ntiles)
{
    const uint64_t g = (uint64_t)sm_count() * (uint64_t)blocks_per_sm(fn, threads, smem);
    return (unsigned)(g < ntiles ? g : ntiles);
}

/* Launchers; each returns the cudaError_t of the launch. */
cudaError_t launch_compress(const CompressArgs &a, cudaStream_t st);
cudaError_t launch_decompress(const DecompressArgs &a, cudaStream_t st);

/* The SZp 3-D codec (zk_szp3d.cu): scratch bytes (err words, block sizes and
 * offsets, and for compress the quantized volume), the largest stream, and
 * the two passes, enqueued on st.  *d_size (device) receives the stream size. */
size_t sz3_workspace_bytes(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t bs, bool compress);
size_t sz3_max_stream_bytes(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t bs);
cudaError_t sz3_compress(uint8_t *out, uint64_t cap, const float *x, uint64_t d1, uint64_t d2, uint64_t d3,
                         uint32_t bs, double eb, void *ws, uint64_t *d_size, cudaStream_t st);
cudaError_t sz3_decompress(float *y, const uint8_t *in, uint64_t avail, uint64_t d1, uint64_t d2, uint64_t d3,
                           uint32_t bs, double eb, void *ws, cudaStream_t st);

/* The OpenMP form of the SZp 3-D codec (zk_szp3d_split.cu): the thread
 * grid of T threads over a d1 x d2 x d3 volume, its sizes, and the two
 * passes (sub-volume after sub-volume through the serial-form kernels).
 * sz3_split_plan fails when T is out of range or an axis has fewer planes
 * than parts.  Decompression takes the T header offsets on the host. */
struct Sz3Split3 {
    uint32_t T;
    uint32_t parts[3]; /* thread grid, parts[0] >= parts[1] >= parts[2] */
    uint64_t dim[3];
};
bool sz3_split_plan(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t T, Sz3Split3 *sp);
void sz3_split_origin(const Sz3Split3 &sp, uint32_t r, uint64_t o[3], uint64_t s[3]);
void sz3_split_extent(const Sz3Split3 &sp, uint32_t r, uint64_t s[3]);
size_t sz3_split_max_stream_bytes(const Sz3Split3 &sp, uint32_t bs);
size_t sz3_split_workspace_bytes(const Sz3Split3 &sp, uint32_t bs, bool compress);
cudaError_t sz3_split_compress(uint8_t *out, uint64_t cap, const float *x, const Sz3Split3 &sp, uint32_t bs, double eb,
                               void *ws, uint64_t *d_size, cudaStream_t st);
cudaError_t sz3_split_decompress(float *y, const uint8_t *in, uint64_t avail, const uint64_t *offs, const Sz3Split3 &sp,
                                 uint32_t bs, double eb, void *ws, cudaStream_t st);

/* Host: a 2-D TMA map of the floats p[0, n) as rows of 32, boxes of
 * box_rows rows (256: a whole tile; 32: one warp's rows), 128-byte swizzle
 * (16-byte chunk k of row r lands at chunk k ^ (r & 7) of a 1024-byte-aligned
 * box).  False when p is not 16-byte aligned, holds fewer than one tile's
 * 256 rows, or the driver's encoder is unavailable. */
bool zk_rows_map(CUtensorMap *map, const void *p, uint64_t n, uint32_t box_rows);
cudaError_t launch_homadd(const HomAddArgs &a, cudaStream_t st);
cudaError_t launch_decompress_jobs(const DecompressJobsArgs &a, cudaStream_t st);
cudaError_t launch_walk(const WalkArgs &a, cudaStream_t st);

#endif
