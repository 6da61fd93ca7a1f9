/*
 * zccl_capi.cu -- the C ABI declared in include/zccl_gpu.h.
 *
 * Device API: argument checks, index / workspace layout, kernel launches.
 * Drop-in layer: the reference's six codec entry points on top of it, with
 * host pointers staged through cached device buffers and device pointers
 * used in place.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/zccl_gpu.h"
#include "zkern.cuh"

namespace {

/* ------------------------------------------------------------------ */
/* width thresholds from this host's libm                              */
/* ------------------------------------------------------------------ */

ZWidthTable g_wt;
std::once_flag g_wt_once;

/* The reference's width: (int)(log2f(max)) + 1 with max an unsigned int
 * (ZCCL/src/ZCCL_float.c:606). */
__host__ int host_width(uint32_t m)
{
    volatile float f = (float)m;
    return (int)(log2f(f)) + 1;
}

void init_width_table()
{
    g_wt.thr[0] = 0xFFFFFFFFu;
    for (uint32_t w = 1; w <= 32; w++) {
        uint64_t lo = 1ull << (w - 1), m = (1ull << w) - 1;
        uint32_t first = 0xFFFFFFFFu;
        while (m >= lo && host_width((uint32_t)m) == (int)w + 1) {
            first = (uint32_t)m;
            m--;
        }
        g_wt.thr[w] = first;
    }
}

const ZWidthTable &width_table()
{
    std::call_once(g_wt_once, init_width_table);
    return g_wt;
}

/* ------------------------------------------------------------------ */
/* layouts                                                             */
/* ------------------------------------------------------------------ */

size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

int make_geom(size_t n, int L, int T, ZGeom *g)
{
    if (L < 1 || T < 1) return ZCCL_GPU_EINVAL;
    if (zg_init(g, (uint64_t)n, (uint32_t)L, (uint32_t)T) != 0) return ZCCL_GPU_EINVAL;
    return ZCCL_GPU_OK;
}

/* Side index: size | tile_off[ntiles] | tile_qprev[ntiles] | widths[nblocks] */
struct IndexLayout {
    size_t tile_off, qprev, widths, total;
};

IndexLayout index_layout(const ZGeom &g)
{
    IndexLayout l;
    l.tile_off = 16;
    l.qprev = align16(l.tile_off + 8 * g.ntiles);
    l.widths = align16(l.qprev + 4 * g.ntiles);
    l.total = align16(l.widths + g.nblocks) + 16;
    return l;
}

ZIndex bind_index(void *mem, const ZGeom &g)
{
    IndexLayout l = index_layout(g);
    uint8_t *p = (uint8_t *)mem;
    ZIndex z;
    z.size = (uint64_t *)p;
    z.tile_off = (uint64_t *)(p + l.tile_off);
    z.tile_qprev = (int32_t *)(p + l.qprev);
    z.widths = p + l.widths;
    return z;
}

/* Workspace: err u32 | walk_err u32 | ticket u32 | pad | status[ntiles] |
 * header-walk scratch.  Only the first part is cleared per call. */
struct WalkLayout {
    uint32_t M, max_windows, max_groups;
    size_t seg_P, seg_R, seg_end, seg_ok, win_base, grp_base, wtab, gtab, gentry, gbase, wexit, gwin, total;
};

size_t ws_clear_bytes(const ZGeom &g) { return 16 + 8 * g.ntiles; }

/* Zero what a call needs zeroed at launch: the tile ticket and the
 * look-back words.  The two status words in front of them are left alone,
 * so errors of earlier calls on the workspace stay visible until
 * zccl_gpu_check() reads and clears them. */
cudaError_t ws_clear(void *ws, const ZGeom &g, cudaStream_t st)
{
    return cudaMemsetAsync((uint8_t *)ws + 8, 0, ws_clear_bytes(g) - 8, st);
}

WalkLayout walk_layout(const ZGeom &g)
{
    WalkLayout l;
    l.M = zg_block_bytes(32, g.L);
    l.max_windows = (uint32_t)(zg_stream_worst(&g) / WALK_WW + g.T + 2);
    l.max_groups = (l.max_windows + WALK_G - 1) / WALK_G + g.T + 1;
    size_t o = align16(ws_clear_bytes(g));
    l.seg_P = o; o = align16(o + 8ull * g.T);
    l.seg_R = o; o = align16(o + 8ull * g.T);
    l.seg_end = o; o = align16(o + 8ull * g.T);
    l.seg_ok = o; o = align16(o + 4ull * g.T);
    l.win_base = o; o = align16(o + 4ull * (g.T + 1));
    l.grp_base = o; o = align16(o + 4ull * (g.T + 1));
    l.wtab = o; o = align16(o + 4ull * l.max_windows * l.M);
    l.gtab = o; o = align16(o + 8ull * l.max_groups * l.M);
    l.gentry = o; o = align16(o + 4ull * l.max_groups);
    l.gbase = o; o = align16(o + 8ull * l.max_groups);
    l.wexit = o; o = align16(o + (size_t)WALK_WW * l.max_windows * (l.M < 256 ? 1u : 2u));
    l.gwin = o; o = align16(o + 4ull * l.max_groups * l.M * WALK_G);
    l.total = o + 16;
    return l;
}

size_t ws_bytes(const ZGeom &g) { return walk_layout(g).total; }

ZWork bind_ws(void *ws)
{
    uint8_t *p = (uint8_t *)ws;
    ZWork w;
    w.err = (uint32_t *)p;
    w.walk_err = (uint32_t *)(p + 4);
    w.ticket = (uint32_t *)(p + 8);
    w.status = (uint64_t *)(p + 16);
    w.lb_spin = LB_SPIN_LIMIT;
    return w;
}

/* Test hook: with ZCCL_GPU_TEST_STALL_TILE0=1 in the environment a
 * compression hands out tiles from 1 on, so tile 0 never publishes its size
 * and its successor's look-back must give up, after 4096 polls instead of
 * the usual limit.  The call then reports ZCCL_GPU_ETIMEOUT; nothing waits
 * without bound on the way. */
bool test_stall_tile0()
{
    const char *v = getenv("ZCCL_GPU_TEST_STALL_TILE0");
    return v && v[0] == '1' && v[1] == 0;
}

int status_of_bits(uint32_t bits)
{
    if (bits & ZERR_TIMEOUT) return ZCCL_GPU_ETIMEOUT;
    /* running out of bytes makes later checks fail too: report it first */
    if (bits & ZERR_BOUNDS) return ZCCL_GPU_EBOUNDS;
    if (bits & ZERR_CORRUPT) return ZCCL_GPU_ECORRUPT;
    if (bits & ZERR_CAPACITY) return ZCCL_GPU_ECAPACITY;
    if (bits & ZERR_RANGE) return ZCCL_GPU_ERANGE;
    return ZCCL_GPU_OK;
}

int cuda_status(cudaError_t e) { return e == cudaSuccess ? ZCCL_GPU_OK : ZCCL_GPU_ECUDA; }

/* Enqueue the index walk of a byte-only stream (no workspace reset). */
int walk_stream(zccl_gpu_stream *s, const ZGeom &g, void *ws, cudaStream_t st)
{
    const WalkLayout l = walk_layout(g);
    uint8_t *p = (uint8_t *)ws;
    WalkArgs a;
    memset(&a, 0, sizeof(a));
    a.in = s->bytes;
    a.avail = s->capacity;
    a.end_bound = zg_stream_worst(&g);
    a.g = g;
    a.idx = bind_index(s->index, g);
    a.err = bind_ws(ws).walk_err;
    a.ws.seg_P = (uint64_t *)(p + l.seg_P);
    a.ws.seg_R = (uint64_t *)(p + l.seg_R);
    a.ws.seg_end = (uint64_t *)(p + l.seg_end);
    a.ws.seg_ok = (uint32_t *)(p + l.seg_ok);
    a.ws.win_base = (uint32_t *)(p + l.win_base);
    a.ws.grp_base = (uint32_t *)(p + l.grp_base);
    a.ws.wtab = (uint32_t *)(p + l.wtab);
    a.ws.gtab = (uint64_t *)(p + l.gtab);
    a.ws.gentry = (uint32_t *)(p + l.gentry);
    a.ws.gbase = (uint64_t *)(p + l.gbase);
    a.ws.wexit = p + l.wexit;
    a.ws.gwin = (uint32_t *)(p + l.gwin);
    a.max_windows = l.max_windows;
    a.max_groups = l.max_groups;
    int rc = cuda_status(launch_walk(a, st));
    if (rc == ZCCL_GPU_OK) {
        s->indexed = 1;
        s->qprev_valid = 0;
    }
    return rc;
}

bool valid_stream(const zccl_gpu_stream *s) { return s && s->bytes && s->index; }

/* Shared-memory layouts, with room for the kernels' copies of their jobs:
 * two compute slots (the tile in progress and the one just claimed) and the
 * placer's. */
ZSmem compress_smem(const ZGeom &g)
{
    return zg_smem(0, g.L, g.TB, (uint32_t)(2 * sizeof(CompressJob) + sizeof(ZPlace)));
}

/* The add's layout.  Two CTAs share an SM (registers allow no more), so
 * the shared memory they leave unused goes to the ring of packed sums: the
 * longer the ring, the longer a tile may wait there for its look-back before
 * the adding warps run out of room. */
ZSmem homadd_smem(const ZGeom &g)
{
    ZSmem m = zg_smem(2, g.L, g.TB, homadd_job_bytes(g.TB));
    static int per_cta = -1;
    if (per_cta < 0) {
        int dev = 0, sm = 0, rsv = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess) {
            cudaGetLastError();
            sm = 0;
        }
        per_cta = sm > 0 ? sm / 2 - rsv - 1024 : 0; /* a kilobyte of margin */
    }
    if (per_cta > (int)m.total) {
        const uint32_t extra = ((uint32_t)per_cta - m.total) & ~15u;
        m.jobs += extra;
        m.total += extra;
    }
    return m;
}

/* The decompressor's layout (padded rows, one input buffer) with room for
 * the copy of the job in progress. */
ZSmem decompress_jobs_smem(const ZGeom &g) { return zg_smem(1, g.L, g.TB, (uint32_t)sizeof(DecompressJob)); }

} // namespace

/* ==================================================================== */
/* device API                                                           */
/* ==================================================================== */

extern "C" size_t zccl_gpu_max_stream_bytes(size_t n, int L, int T)
{
    ZGeom g;
    if (make_geom(n, L, T, &g)) return 0;
    return (size_t)zg_stream_worst(&g);
}

extern "C" size_t zccl_gpu_index_bytes(size_t n, int L, int T)
{
    ZGeom g;
    if (make_geom(n, L, T, &g)) return 0;
    return index_layout(g).total;
}

extern "C" size_t zccl_gpu_workspace_bytes(size_t n, int L, int T)
{
    ZGeom g;
    if (make_geom(n, L, T, &g)) return 0;
    return ws_bytes(g);
}

extern "C" void zccl_gpu_width_table(uint32_t thr[33])
{
    const ZWidthTable &wt = width_table();
    memcpy(thr, wt.thr, sizeof(wt.thr));
}

/* Compress in block layout fmt (ZG_FASTMODE1 or ZG_FIXED_BYTES). */
static int compress_fmt(zccl_gpu_stream *out, const float *d_in, size_t n, float eb, int L, int T, void *d_ws,
                        void *cuda_stream, uint32_t fmt)
{
    ZGeom g;
    if (make_geom(n, L, T, &g) || !valid_stream(out) || !d_in || !d_ws) return ZCCL_GPU_EINVAL;
    g.fmt = fmt;
    if (!(eb > 0.0f) || !isfinite(eb)) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    CompressArgs a;
    memset(&a, 0, sizeof(a));
    a.job.g = g;
    a.job.x = d_in;
    a.job.out = out->bytes;
    a.job.cap = out->capacity;
    a.job.inv = 1.0f / eb; /* float division, as ZCCL/src/ZCCL_float.c:540 */
    a.job.idx = bind_index(out->index, g);
    a.w = bind_ws(d_ws);
    a.job.status = a.w.status;
    a.wt = width_table();
    a.sm = compress_smem(g);
    if (ws_clear(d_ws, g, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (test_stall_tile0()) {
        static const uint32_t one = 1;
        if (cudaMemcpyAsync(a.w.ticket, &one, 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
        a.w.lb_spin = 4096;
    }
    int rc = cuda_status(launch_compress(a, st));
    if (rc == ZCCL_GPU_OK) {
        out->indexed = 1;
        out->qprev_valid = 1;
    }
    return rc;
}

extern "C" int zccl_gpu_compress(zccl_gpu_stream *out, const float *d_in, size_t n, float eb, int L,
                                 int T, void *d_ws, void *cuda_stream)
{
    return compress_fmt(out, d_in, n, eb, L, T, d_ws, cuda_stream, ZG_FASTMODE1);
}

extern "C" int zccl_gpu_compress_fixed(zccl_gpu_stream *out, const float *d_in, size_t n, float eb, int L,
                                       int T, void *d_ws, void *cuda_stream)
{
    return compress_fmt(out, d_in, n, eb, L, T, d_ws, cuda_stream, ZG_FIXED_BYTES);
}

extern "C" int zccl_gpu_build_index(zccl_gpu_stream *s, size_t n, int L, int T, void *d_ws,
                                    void *cuda_stream)
{
    ZGeom g;
    if (make_geom(n, L, T, &g) || !valid_stream(s) || !d_ws) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    if (ws_clear(d_ws, g, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    return walk_stream(s, g, d_ws, st);
}

/* Decompress a stream in block layout fmt. */
static int decompress_fmt(float *d_out, zccl_gpu_stream *in, size_t n, float eb, int L, int T, void *d_ws,
                          void *cuda_stream, uint32_t fmt)
{
    ZGeom g;
    if (make_geom(n, L, T, &g) || !valid_stream(in) || !d_out || !d_ws) return ZCCL_GPU_EINVAL;
    g.fmt = fmt;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    if (ws_clear(d_ws, g, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    ZWork w = bind_ws(d_ws);
    if (!in->indexed) {
        int rc = walk_stream(in, g, d_ws, st);
        if (rc) return rc;
    }
    DecompressArgs a;
    a.in = in->bytes;
    a.avail = in->capacity;
    a.y = d_out;
    a.g = g;
    a.eb = eb;
    a.idx = bind_index(in->index, g);
    a.qprev_valid = in->qprev_valid;
    a.w = w;
    a.sm = zg_smem(1, g.L, g.TB, 0);
    int rc = cuda_status(launch_decompress(a, st));
    if (rc == ZCCL_GPU_OK) in->qprev_valid = 1;
    return rc;
}

extern "C" int zccl_gpu_decompress(float *d_out, zccl_gpu_stream *in, size_t n, float eb, int L,
                                   int T, void *d_ws, void *cuda_stream)
{
    return decompress_fmt(d_out, in, n, eb, L, T, d_ws, cuda_stream, ZG_FASTMODE1);
}

extern "C" int zccl_gpu_decompress_fixed(float *d_out, zccl_gpu_stream *in, size_t n, float eb, int L,
                                         int T, void *d_ws, void *cuda_stream)
{
    return decompress_fmt(d_out, in, n, eb, L, T, d_ws, cuda_stream, ZG_FIXED_BYTES);
}

extern "C" int zccl_gpu_decompress_accumulate(float *d_acc, const zccl_gpu_stream *in, size_t n, float eb, int L,
                                              int T, void *d_ws, void *cuda_stream)
{
    ZGeom g;
    if (make_geom(n, L, T, &g) || !valid_stream(in) || !in->indexed || !in->qprev_valid || !d_acc || !d_ws ||
        !(eb > 0.0f) || !isfinite(eb))
        return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    if (ws_clear(d_ws, g, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    DecompressJobsArgs a;
    memset(&a, 0, sizeof(a));
    a.job.g = g;
    a.job.in = in->bytes;
    a.job.avail = in->capacity;
    a.job.y = d_acc;
    a.job.idx = bind_index(in->index, g);
    a.job.eb = eb;
    a.job.accumulate = 1;
    a.w = bind_ws(d_ws);
    a.sm = decompress_jobs_smem(g);
    return cuda_status(launch_decompress_jobs(a, st));
}

/* The add of P inputs given by their bytes and index arrays (which need
 * not sit in one stream's index layout), on a cleared workspace. */
static int homadd_inputs(zccl_gpu_stream *out, const HomInput *in, int P, int qv, const ZGeom &g, void *d_ws,
                         unsigned long long *d_cases, cudaStream_t st)
{
    if (ws_clear(d_ws, g, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    ZWork w = bind_ws(d_ws);
    HomAddArgs a;
    memset(&a, 0, sizeof(a));
    for (int p = 0; p < P; p++) a.job.in[p] = in[p];
    a.job.P = (uint32_t)P;
    a.job.qprev_valid = qv;
    a.job.out = out->bytes;
    a.job.cap = out->capacity;
    a.job.idx = bind_index(out->index, g);
    a.job.g = g;
    a.job.status = w.status;
    a.cases = d_cases;
    a.w = w;
    a.wt = width_table();
    a.sm = homadd_smem(g);
    int rc = cuda_status(launch_homadd(a, st));
    if (rc == ZCCL_GPU_OK) {
        out->indexed = 1;
        out->qprev_valid = qv;
    }
    return rc;
}

extern "C" int zccl_gpu_homadd_cases(zccl_gpu_stream *out, zccl_gpu_stream *ins, int P, size_t n,
                                     int L, int T, void *d_ws, unsigned long long *d_cases,
                                     void *cuda_stream)
{
    ZGeom g;
    if (make_geom(n, L, T, &g) || !valid_stream(out) || !ins || P < 1 || P > ZH_MAXP || !d_ws)
        return ZCCL_GPU_EINVAL;
    for (int p = 0; p < P; p++)
        if (!valid_stream(&ins[p]) || ins[p].bytes == out->bytes) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    if (ws_clear(d_ws, g, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    HomInput in[ZH_MAXP];
    int qv = 1;
    for (int p = 0; p < P; p++) {
        if (!ins[p].indexed) {
            int rc = walk_stream(&ins[p], g, d_ws, st);
            if (rc) return rc;
        }
        ZIndex ix = bind_index(ins[p].index, g);
        in[p].bytes = ins[p].bytes;
        in[p].avail = ins[p].capacity;
        in[p].widths = ix.widths;
        in[p].tile_off = ix.tile_off;
        in[p].tile_qprev = ix.tile_qprev;
        qv &= ins[p].qprev_valid ? 1 : 0;
    }
    return homadd_inputs(out, in, P, qv, g, d_ws, d_cases, st);
}

extern "C" int zccl_gpu_homadd(zccl_gpu_stream *out, zccl_gpu_stream *ins, int P, size_t n, int L,
                               int T, void *d_ws, void *cuda_stream)
{
    return zccl_gpu_homadd_cases(out, ins, P, n, L, T, d_ws, nullptr, cuda_stream);
}

extern "C" int zccl_gpu_stream_size(const zccl_gpu_stream *s, size_t n, int L, int T, size_t *size,
                                    void *cuda_stream)
{
    ZGeom g;
    if (make_geom(n, L, T, &g) || !valid_stream(s) || !size) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    uint64_t v = 0;
    if (cudaMemcpyAsync(&v, s->index, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    *size = (size_t)v;
    return ZCCL_GPU_OK;
}

extern "C" int zccl_gpu_frame_size(const zccl_gpu_stream *s, void *d_frame, void *cuda_stream)
{
    if (!valid_stream(s) || !d_frame) return ZCCL_GPU_EINVAL;
    /* the index starts with the stream's total size, a little-endian uint64 */
    return cudaMemcpyAsync(d_frame, s->index, 8, cudaMemcpyDeviceToDevice, (cudaStream_t)cuda_stream) == cudaSuccess
               ? ZCCL_GPU_OK
               : ZCCL_GPU_ECUDA;
}

extern "C" int zccl_gpu_check(void *d_ws, void *cuda_stream)
{
    if (!d_ws) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    uint32_t bits[2] = {0, 0};
    if (cudaMemcpyAsync(bits, d_ws, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    /* read once: the next call starts with clean status words */
    if (cudaMemsetAsync(d_ws, 0, 8, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    /* a failed walk leaves nothing for the codec kernels to report */
    return status_of_bits(bits[1] ? bits[1] : bits[0]);
}

extern "C" const char *zccl_gpu_strerror(int status)
{
    switch (status) {
    case ZCCL_GPU_OK: return "ok";
    case ZCCL_GPU_EINVAL: return "invalid argument";
    case ZCCL_GPU_ECUDA: return "CUDA runtime error";
    case ZCCL_GPU_ERANGE: return "input not finite or |x/eb| >= 2^31";
    case ZCCL_GPU_ECORRUPT: return "stream inconsistent with its geometry";
    case ZCCL_GPU_EBOUNDS: return "stream runs past its readable bytes";
    case ZCCL_GPU_ETIMEOUT: return "device wait timed out";
    case ZCCL_GPU_ENOMEM: return "out of memory";
    case ZCCL_GPU_ECAPACITY: return "destination buffer too small";
    case ZCCL_GPU_ESCRATCH: return "input needs more than the fixed scratch array";
    default: return "unknown status";
    }
}

/* ==================================================================== */
/* batches                                                              */
/* ==================================================================== */

namespace {

size_t batch_job_size(int kind)
{
    return kind == ZCCL_GPU_BATCH_COMPRESS ? sizeof(CompressJob)
           : kind == ZCCL_GPU_BATCH_HOMADD ? sizeof(HomAddJob)
                                           : sizeof(DecompressJob);
}


/* d_mem: err | walk_err | ticket | pad | status[ntiles] | jobs | tile_job[ntiles] | job_tile0[njobs]
 * and, for compress batches, room for a 64-byte-aligned CUtensorMap per job
 * (rows: where that room starts; the maps start at its first 64-byte
 * boundary in memory). */
struct BatchLayout {
    size_t clear, jobs, map, tile0, rows, total;
};

BatchLayout batch_layout(int kind, size_t njobs, size_t ntiles)
{
    BatchLayout l;
    l.clear = 16 + 8 * ntiles;
    l.jobs = align16(l.clear);
    l.map = align16(l.jobs + njobs * batch_job_size(kind));
    l.tile0 = align16(l.map + 2 * ntiles);
    l.rows = l.tile0 + 8 * njobs;
    l.total = kind == ZCCL_GPU_BATCH_COMPRESS ? l.rows + 64 + sizeof(CUtensorMap) * njobs : l.rows;
    return l;
}

/* Geometry of every job, checked; returns the total tile count or 0. */
size_t batch_geoms(int kind, const zccl_gpu_batch_job *jobs, size_t njobs, int L, std::vector<ZGeom> &gs)
{
    if ((kind != ZCCL_GPU_BATCH_COMPRESS && kind != ZCCL_GPU_BATCH_HOMADD && kind != ZCCL_GPU_BATCH_DECOMPRESS) ||
        !jobs || njobs < 1 || njobs > 65535)
        return 0;
    gs.resize(njobs);
    size_t ntiles = 0;
    for (size_t j = 0; j < njobs; j++) {
        const zccl_gpu_batch_job &J = jobs[j];
        if (make_geom(J.n, L, J.T, &gs[j])) return 0;
        if (kind == ZCCL_GPU_BATCH_DECOMPRESS) {
            /* one input stream, indexed with its starting values */
            if (!J.ins || J.P != 1 || !valid_stream(J.ins) || !J.ins->indexed || !J.ins->qprev_valid ||
                !J.d_out || !(J.eb > 0.0f) || !isfinite(J.eb))
                return 0;
            ntiles += gs[j].ntiles;
            continue;
        }
        if (!valid_stream(J.out)) return 0;
        if (kind == ZCCL_GPU_BATCH_COMPRESS) {
            if (!J.d_in || !(J.eb > 0.0f) || !isfinite(J.eb)) return 0;
        } else {
            if (!J.ins || J.P < 1 || J.P > ZH_MAXP) return 0;
            for (int p = 0; p < J.P; p++)
                if (!valid_stream(&J.ins[p]) || !J.ins[p].indexed || J.ins[p].bytes == J.out->bytes) return 0;
        }
        ntiles += gs[j].ntiles;
    }
    return ntiles;
}

} // namespace

extern "C" size_t zccl_gpu_batch_bytes(int kind, const zccl_gpu_batch_job *jobs, size_t njobs, int L)
{
    std::vector<ZGeom> gs;
    const size_t ntiles = batch_geoms(kind, jobs, njobs, L, gs);
    return ntiles ? batch_layout(kind, njobs, ntiles).total : 0;
}

extern "C" int zccl_gpu_batch_plan(zccl_gpu_batch *b, int kind, const zccl_gpu_batch_job *jobs,
                                   size_t njobs, int L, void *d_mem, size_t bytes, void *cuda_stream)
{
    std::vector<ZGeom> gs;
    const size_t ntiles = b && d_mem ? batch_geoms(kind, jobs, njobs, L, gs) : 0;
    if (!ntiles || ntiles > 0xFFFFFFFFull) return ZCCL_GPU_EINVAL;
    const BatchLayout lay = batch_layout(kind, njobs, ntiles);
    if (bytes < lay.total) return ZCCL_GPU_ECAPACITY;
    uint8_t *base = static_cast<uint8_t *>(d_mem);
    uint64_t *status = reinterpret_cast<uint64_t *>(base + 16);
    std::vector<uint16_t> map(ntiles);
    std::vector<uint64_t> tile0(njobs);
    std::vector<CompressJob> cj(kind == ZCCL_GPU_BATCH_COMPRESS ? njobs : 0);
    /* compress: a rows-of-32-floats tensor map per job whose full tiles can
     * arrive as TMA boxes (L = 32, 256-block tiles, 16-byte-aligned input) */
    struct alignas(64) RowsMap { CUtensorMap m; };
    std::vector<RowsMap> rmaps(kind == ZCCL_GPU_BATCH_COMPRESS ? njobs : 0);
    const size_t rows_off = kind == ZCCL_GPU_BATCH_COMPRESS
                                ? (size_t)(((uintptr_t)(base + lay.rows) + 63u) & ~(uintptr_t)63u) - (uintptr_t)base
                                : 0;
    bool any_boxed = false;
    std::vector<HomAddJob> hj(kind == ZCCL_GPU_BATCH_HOMADD ? njobs : 0);
    std::vector<DecompressJob> dj(kind == ZCCL_GPU_BATCH_DECOMPRESS ? njobs : 0);
    int qv = 1;
    size_t t0 = 0;
    for (size_t j = 0; j < njobs; j++) {
        const zccl_gpu_batch_job &J = jobs[j];
        const ZGeom &g = gs[j];
        tile0[j] = t0;
        for (uint64_t t = 0; t < g.ntiles; t++) map[t0 + t] = (uint16_t)j;
        if (kind == ZCCL_GPU_BATCH_COMPRESS) {
            CompressJob &c = cj[j];
            memset(&c, 0, sizeof(c));
            c.g = g;
            c.x = J.d_in;
            c.out = J.out->bytes;
            c.cap = J.out->capacity;
            c.idx = bind_index(J.out->index, g);
            c.status = status + t0;
            c.inv = 1.0f / J.eb; /* float division, as ZCCL/src/ZCCL_float.c:540 */
            memset(&rmaps[j], 0, sizeof(RowsMap));
            c.boxed = L == 32 && g.TB == 256 && zk_rows_map(&rmaps[j].m, J.d_in, g.n, 256) ? 1u : 0u;
            any_boxed |= c.boxed != 0;
        } else if (kind == ZCCL_GPU_BATCH_DECOMPRESS) {
            DecompressJob &d = dj[j];
            memset(&d, 0, sizeof(d));
            d.g = g;
            d.in = J.ins->bytes;
            d.avail = J.ins->capacity;
            d.y = J.d_out;
            d.idx = bind_index(J.ins->index, g);
            d.eb = J.eb;
            d.accumulate = J.accumulate ? 1 : 0;
        } else {
            HomAddJob &h = hj[j];
            memset(&h, 0, sizeof(h));
            h.g = g;
            int jq = 1;
            for (int p = 0; p < J.P; p++) {
                const ZIndex ix = bind_index(J.ins[p].index, g);
                h.in[p].bytes = J.ins[p].bytes;
                h.in[p].avail = J.ins[p].capacity;
                h.in[p].widths = ix.widths;
                h.in[p].tile_off = ix.tile_off;
                h.in[p].tile_qprev = ix.tile_qprev;
                jq &= J.ins[p].qprev_valid ? 1 : 0;
            }
            h.P = (uint32_t)J.P;
            h.qprev_valid = jq;
            h.out = J.out->bytes;
            h.cap = J.out->capacity;
            h.idx = bind_index(J.out->index, g);
            h.status = status + t0;
            qv &= jq;
        }
        t0 += g.ntiles;
    }
    cudaStream_t st = (cudaStream_t)cuda_stream;
    const void *jsrc = kind == ZCCL_GPU_BATCH_COMPRESS ? (const void *)cj.data()
                       : kind == ZCCL_GPU_BATCH_HOMADD ? (const void *)hj.data()
                                                       : (const void *)dj.data();
    const size_t jbytes = njobs * batch_job_size(kind);
    if (cudaMemsetAsync(base, 0, 8, st) != cudaSuccess || /* clean status words */
        cudaMemcpyAsync(base + lay.jobs, jsrc, jbytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(base + lay.map, map.data(), 2 * ntiles, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(base + lay.tile0, tile0.data(), 8 * njobs, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (any_boxed &&
         cudaMemcpyAsync(base + rows_off, rmaps.data(), sizeof(RowsMap) * njobs, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    memset(b, 0, sizeof(*b));
    b->kind = kind;
    b->L = L;
    b->njobs = njobs;
    b->ntiles = ntiles;
    b->d_mem = d_mem;
    b->clear_bytes = lay.clear;
    b->jobs_off = lay.jobs;
    b->map_off = lay.map;
    b->tile0_off = lay.tile0;
    b->rows_off = any_boxed ? rows_off : 0;
    b->tb = gs[0].TB;
    const ZSmem sm = kind == ZCCL_GPU_BATCH_COMPRESS ? compress_smem(gs[0])
                     : kind == ZCCL_GPU_BATCH_HOMADD ? homadd_smem(gs[0])
                                                     : decompress_jobs_smem(gs[0]);
    static_assert(sizeof(sm) == sizeof(b->smem), "layout fields");
    memcpy(b->smem, &sm, sizeof(sm));
    b->qprev_valid = kind == ZCCL_GPU_BATCH_HOMADD ? qv : 1;
    if (kind != ZCCL_GPU_BATCH_DECOMPRESS)
        for (size_t j = 0; j < njobs; j++) {
            jobs[j].out->indexed = 1;
            jobs[j].out->qprev_valid = b->qprev_valid;
        }
    return ZCCL_GPU_OK;
}

extern "C" int zccl_gpu_batch_run(const zccl_gpu_batch *b, void *cuda_stream)
{
    if (!b || !b->d_mem || !b->ntiles) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    uint8_t *base = static_cast<uint8_t *>(b->d_mem);
    /* the status words stay until zccl_gpu_batch_check() reads them */
    if (cudaMemsetAsync(base + 8, 0, b->clear_bytes - 8, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    ZBatch bt;
    bt.jobs = base + b->jobs_off;
    bt.tile_job = reinterpret_cast<const uint16_t *>(base + b->map_off);
    bt.job_tile0 = reinterpret_cast<const uint64_t *>(base + b->tile0_off);
    bt.njobs = (uint32_t)b->njobs;
    bt.ntiles = b->ntiles;
    bt.maps = b->kind == ZCCL_GPU_BATCH_COMPRESS && b->rows_off ? base + b->rows_off : nullptr;
    ZSmem sm;
    memcpy(&sm, b->smem, sizeof(sm));
    if (b->kind == ZCCL_GPU_BATCH_COMPRESS) {
        CompressArgs a;
        memset(&a, 0, sizeof(a));
        a.job.g.L = (uint32_t)b->L; /* the batch's shared L and tile size */
        a.job.g.TB = b->tb;
        a.batch = bt;
        a.w = bind_ws(base);
        a.wt = width_table();
        a.sm = sm;
        a.grid = b->grid;
        return cuda_status(launch_compress(a, st));
    }
    if (b->kind == ZCCL_GPU_BATCH_DECOMPRESS) {
        DecompressJobsArgs a;
        memset(&a, 0, sizeof(a));
        a.job.g.L = (uint32_t)b->L;
        a.job.g.TB = b->tb;
        a.batch = bt;
        a.w = bind_ws(base);
        a.sm = sm;
        a.grid = b->grid;
        return cuda_status(launch_decompress_jobs(a, st));
    }
    HomAddArgs a;
    memset(&a, 0, sizeof(a));
    a.job.g.L = (uint32_t)b->L;
    a.job.g.TB = b->tb;
    a.batch = bt;
    a.w = bind_ws(base);
    a.wt = width_table();
    a.sm = sm;
    a.grid = b->grid;
    return cuda_status(launch_homadd(a, st));
}

extern "C" int zccl_gpu_batch_check(const zccl_gpu_batch *b, void *cuda_stream)
{
    return b ? zccl_gpu_check(b->d_mem, cuda_stream) : ZCCL_GPU_EINVAL;
}

extern "C" int zccl_gpu_batch_tune(zccl_gpu_batch *b, void *cuda_stream)
{
    if (!b || !b->d_mem) return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return ZCCL_GPU_ECUDA;
    }
    /* CTAs per SM from one to what fits (0), each timed over three runs after one warm-up */
    const unsigned per_sm[] = {1, 2, 3, 4, 6, 0};
    unsigned best = 0;
    float best_ms = 1e30f;
    int rc = ZCCL_GPU_OK;
    for (unsigned k : per_sm) {
        b->grid = k * (unsigned)nsm;
        rc = zccl_gpu_batch_run(b, st);
        for (int r = 0; r < 3 && rc == ZCCL_GPU_OK; r++) {
            if (r == 0) cudaEventRecord(e0, st);
            rc = zccl_gpu_batch_run(b, st);
        }
        if (rc) break;
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = ZCCL_GPU_ECUDA;
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            best = b->grid;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->grid = best;
    if (rc == ZCCL_GPU_OK) rc = zccl_gpu_check(b->d_mem, st);
    return rc;
}

/* ==================================================================== */
/* drop-in layer                                                        */
/* ==================================================================== */

namespace {

thread_local int t_last_status = ZCCL_GPU_OK;

/* Elements in the blocks of non-zero width of a stream, from its width
 * index: the one quantity besides n and the stream size that the
 * reference's memory-access counts depend on. */
__global__ void k_nonzero_elements(const uint8_t *widths, ZGeom g, unsigned long long *out)
{
    unsigned long long acc = 0;
    const uint64_t reg = (uint64_t)g.T * g.nb_reg;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < g.nblocks;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (!widths[i]) continue;
        acc += i < reg ? zg_block_len(g.tbs, g.L, i % g.nb_reg) : zg_block_len(g.rem, g.L, i - reg);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0 && acc) atomicAdd(out, acc);
}

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    int ensure(size_t bytes)
    {
        if (bytes <= n) return ZCCL_GPU_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t want = bytes + bytes / 8 + 256;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return ZCCL_GPU_ENOMEM;
        }
        /* a workspace starts with clean status words */
        if (cudaMemset(p, 0, 16) != cudaSuccess) {
            cudaFree(p);
            p = nullptr;
            return ZCCL_GPU_ECUDA;
        }
        n = want;
        return ZCCL_GPU_OK;
    }
};

/* Pinned host memory for small device-to-host reads that must be
 * asynchronous (sizes and stream headers of the pipelined drop-ins). */
struct PinBuf {
    void *p = nullptr;
    size_t n = 0;
    int ensure(size_t bytes)
    {
        if (bytes <= n) return ZCCL_GPU_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return ZCCL_GPU_ENOMEM;
        }
        n = bytes;
        return ZCCL_GPU_OK;
    }
};

/* Most chunk groups a pipelined drop-in splits a stream into, and the
 * compute streams ("lanes") their kernels are spread over: a group's index
 * walk launches few CTAs, so neighbouring groups' kernels run side by side. */
constexpr uint32_t kMaxGroups = 8;
constexpr uint32_t kLanes = 4;
constexpr uint32_t kWalkLanes = 2 * kLanes; /* workspaces: the add's second walk of lane l uses l + kLanes */
/* groups per call: compression has no walk, so finer groups overlap more;
 * decompression and the add walk each group's headers, whose kernels carry
 * a fixed cost per launch */
constexpr uint32_t kGroupsCompress = 8, kGroupsDecompress = 8, kGroupsHomadd = 8;

/* Cached device buffers of the drop-in layer, one set per device. */
struct DropCtx {
    std::mutex mu;
    cudaStream_t st = nullptr;
    cudaStream_t st2 = nullptr; /* a second input's copy, beside the first one's walk */
    cudaStream_t st_in = nullptr; /* the pipelined drop-ins' input copies */
    cudaEvent_t ev = nullptr;
    cudaEvent_t ev_in[kMaxGroups] = {}, ev_k[kMaxGroups] = {}, ev_w[kMaxGroups] = {};
    cudaStream_t lane[kLanes] = {};
    DevBuf lws[kWalkLanes], lix[kLanes][3]; /* per lane: two workspaces and three indexes */
    DevBuf fin, fout, s[3], ix[3], ws;
    DevBuf aux; /* counters read back by the _record entry points */
    PinBuf pin;
    PinBuf stat; /* the lanes' workspace status words, read back together */
};

DropCtx *drop_ctx()
{
    static std::mutex gmu;
    static DropCtx *ctxs[64] = {nullptr};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(gmu);
    if (!ctxs[dev]) {
        DropCtx *c = new DropCtx();
        /* The device feeds streams through a fixed number of hardware queues
         * (eight unless CUDA_DEVICE_MAX_CONNECTIONS says otherwise), and two
         * streams that share one run one after the other.  The pipelined
         * drop-ins therefore send their outputs out on the lanes that made
         * them (a separate copy stream was seen to wait behind another
         * lane's kernels) and keep to st_in and four lanes. */
        bool ok = cudaStreamCreateWithFlags(&c->st_in, cudaStreamNonBlocking) == cudaSuccess;
        for (uint32_t i = 0; ok && i < kLanes; i++)
            ok = cudaStreamCreateWithFlags(&c->lane[i], cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) == cudaSuccess &&
             cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&c->ev, cudaEventDisableTiming) == cudaSuccess;
        for (uint32_t i = 0; ok && i < kMaxGroups; i++)
            ok = cudaEventCreateWithFlags(&c->ev_in[i], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&c->ev_k[i], cudaEventDisableTiming) == cudaSuccess;
        for (uint32_t i = 0; ok && i < kMaxGroups; i++)
            ok = cudaEventCreateWithFlags(&c->ev_w[i], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            delete c;
            return nullptr;
        }
        ctxs[dev] = c;
    }
    return ctxs[dev];
}

/* Page-locked host memory (cudaHostAlloc, cudaHostRegister): copies from it
 * are asynchronous; from pageable memory the host waits for each one. */
bool is_pinned_ptr(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

bool is_device_ptr(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

/* Bytes from p to the end of its device allocation.  The driver call is
 * reached through the runtime's entry-point table so the library does not
 * link libcuda (it loads on hosts without a GPU driver). */
typedef CUresult (*PFN_range)(CUdeviceptr *, size_t *, CUdeviceptr);

size_t device_room(const void *p)
{
    static PFN_range fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_range)f;
        else
            cudaGetLastError();
    });
    CUdeviceptr base = 0;
    size_t size = 0;
    if (!fn || fn(&base, &size, (CUdeviceptr)p) != CUDA_SUCCESS) return 0;
    return (size_t)(base + size - (CUdeviceptr)p);
}

int finish(DropCtx *c, void *ws)
{
    int rc = zccl_gpu_check(ws, c->st);
    return rc;
}

/* Elements in the non-zero-width blocks of the indexed stream whose index
 * is at `index` (synchronous). */
int nonzero_elements(DropCtx *c, void *index, const ZGeom &g, uint64_t *nz)
{
    if (int rc = c->aux.ensure(64)) return rc;
    unsigned long long *d = static_cast<unsigned long long *>(c->aux.p);
    if (cudaMemsetAsync(d, 0, 8, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    const uint64_t want = (g.nblocks + 255) / 256;
    const unsigned grid = (unsigned)std::min<uint64_t>(want ? want : 1, 4096);
    k_nonzero_elements<<<grid, 256, 0, c->st>>>(bind_index(index, g).widths, g, d);
    unsigned long long v = 0;
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&v, d, 8, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
        cudaStreamSynchronize(c->st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    *nz = v;
    return ZCCL_GPU_OK;
}

void report(const char *fn, int rc)
{
    t_last_status = rc;
    if (rc != ZCCL_GPU_OK) fprintf(stderr, "zccl_gpu: %s: %s\n", fn, zccl_gpu_strerror(rc));
}

/* Make a stream view of cmp: in place for device memory, else copied.
 * *capped reports whether a host copy stopped short of the largest size the
 * stream could have. */
int stage_stream(DropCtx *c, int slot, const unsigned char *cmp, const ZGeom &g,
                 zccl_gpu_stream *s, bool full, bool *capped, cudaStream_t cst = nullptr)
{
    *capped = false;
    size_t ixb = index_layout(g).total;
    if (int rc = c->ix[slot].ensure(ixb)) return rc;
    s->index = c->ix[slot].p;
    s->indexed = 0;
    s->qprev_valid = 0;
    if (is_device_ptr(cmp)) {
        s->bytes = (unsigned char *)cmp;
        s->capacity = device_room(cmp);
        return s->capacity ? ZCCL_GPU_OK : ZCCL_GPU_EINVAL;
    }
    /* Host stream: the header gives the first T-1 chunk lengths; the last
     * chunk is read up to its largest possible size (first at most twice the
     * others' average), but not past the 4*nbEle bytes every reference
     * caller allocates for a stream. */
    const size_t hdr = 8ull * g.T;
    uint64_t last;
    memcpy(&last, cmp + 8ull * (g.T - 1), 8);
    size_t known = hdr + (size_t)last;
    size_t want = known + (size_t)(zg_seg_worst(g.tbs, g.L) + zg_seg_worst(g.rem, g.L));
    size_t room = 4 * (size_t)g.n > known + 4 ? 4 * (size_t)g.n : known + 4;
    size_t bytes = (full || want < room) ? want : room;
    /* a first read: the last chunk at twice the others' average length (a
     * chunk at its worst size is six times a typical one); a walk that runs
     * past it reports EBOUNDS and the caller reads again in full */
    if (!full && g.T > 1) {
        const size_t guess = known + 2 * ((size_t)last / (g.T - 1)) + 65536;
        if (guess < bytes) bytes = guess;
    }
    *capped = bytes < want;
    if (int rc = c->s[slot].ensure(bytes)) return rc;
    if (cudaMemcpyAsync(c->s[slot].p, cmp, bytes, cudaMemcpyHostToDevice, cst ? cst : c->st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    s->bytes = (unsigned char *)c->s[slot].p;
    s->capacity = bytes;
    return ZCCL_GPU_OK;
}

/* ---- pipelined host-buffer drop-ins --------------------------------
 * A stream's T chunks are independent (chunk t holds segment t, the last
 * also the remainder segment), and chunks s0 .. s1 - 1 with their offsets
 * rebased are themselves a valid stream of (s1 - s0) tbs (+ rem) elements
 * written by s1 - s0 threads: the same segments, the same bytes.  For host
 * buffers the drop-ins cut a call into such groups of chunks and run, group
 * by group, the host-to-device copy on one stream, the kernels on a second
 * and the device-to-host copy on a third, so that the two directions of the
 * CPU-GPU link and the kernels of neighbouring groups overlap instead of
 * following one another.  The output bytes are those of the whole-stream
 * path. */

struct Group {
    uint32_t s0, s1; /* chunks */
    uint64_t n, e0;  /* elements, first element */
    ZGeom g;         /* geometry of the group's stream */
};

size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

/* Whether host ranges [a, a + na) and [b, b + nb) share a byte. */
bool overlaps(const void *a, size_t na, const void *b, size_t nb)
{
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    return x < y + nb && y < x + na;
}

/* The chunk groups of a call on geometry g, or none when the call is not
 * worth cutting (one chunk, or fewer than 2^22 elements).  The last group
 * holds more chunks than the remainder segment has elements, so its stream
 * splits exactly like the whole one's tail. */
std::vector<Group> chunk_groups(const ZGeom &g, uint32_t most)
{
    std::vector<Group> out;
    const uint32_t T = g.T;
    if (T < 2 || g.n < (1ull << 22)) return out;
    const uint32_t G = std::min<uint32_t>(T, std::min<uint32_t>(most, kMaxGroups));
    std::vector<uint32_t> cut;
    for (uint32_t k = 0; k <= G; k++) cut.push_back((uint32_t)((uint64_t)T * k / G));
    while (cut.size() > 2 && T - cut[cut.size() - 2] <= g.rem) cut.erase(cut.end() - 2);
    if (cut.size() < 3) return out;
    for (size_t k = 0; k + 1 < cut.size(); k++) {
        Group q;
        q.s0 = cut[k];
        q.s1 = cut[k + 1];
        const bool last = q.s1 == T;
        q.n = (uint64_t)(q.s1 - q.s0) * g.tbs + (last ? g.rem : 0u);
        q.e0 = (uint64_t)q.s0 * g.tbs;
        if (make_geom((size_t)q.n, (int)g.L, (int)(q.s1 - q.s0), &q.g) || q.g.tbs != g.tbs ||
            q.g.rem != (last ? g.rem : 0u)) {
            out.clear();
            return out;
        }
        q.g.fmt = g.fmt;
        out.push_back(q);
    }
    return out;
}

size_t max_ws_bytes(const std::vector<Group> &gr)
{
    size_t m = 0;
    for (const Group &q : gr) m = std::max(m, ws_bytes(q.g));
    return m;
}

size_t max_index_bytes(const std::vector<Group> &gr)
{
    size_t m = 0;
    for (const Group &q : gr) m = std::max(m, index_layout(q.g).total);
    return m;
}

/* Waits for every copy and kernel of a pipelined call, then reads (and
 * clears) the lanes' workspace status words, as zccl_gpu_check() does, with
 * one wait for all of them. */
int pipe_finish(DropCtx *c, int rc, uint32_t lanes, bool walk_lanes = false)
{
    bool sync_ok = cudaStreamSynchronize(c->st_in) == cudaSuccess;
    for (uint32_t l = 0; l < lanes; l++) /* after an early stop, work may remain on any lane */
        sync_ok = cudaStreamSynchronize(c->lane[l]) == cudaSuccess && sync_ok;
    if (!sync_ok) return ZCCL_GPU_ECUDA;
    if (int e = c->stat.ensure(8 * kWalkLanes)) return rc ? rc : e;
    uint32_t *bits = (uint32_t *)c->stat.p;
    uint32_t idx[kWalkLanes], n = 0;
    cudaStream_t st = c->lane[0];
    for (uint32_t l = 0; l < lanes; l++)
        for (uint32_t h = 0; h < (walk_lanes ? 2u : 1u); h++) {
            const uint32_t i = l + h * kLanes;
            if (!c->lws[i].p) continue;
            if (cudaMemcpyAsync(bits + 2 * n, c->lws[i].p, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
                return ZCCL_GPU_ECUDA;
            idx[n++] = i;
        }
    if (cudaStreamSynchronize(st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    int rc2 = ZCCL_GPU_OK;
    bool cleared = false;
    for (uint32_t j = 0; j < n; j++) {
        if (!(bits[2 * j] | bits[2 * j + 1])) continue;
        /* a failed walk leaves nothing for the codec kernels to report */
        if (!rc2) rc2 = status_of_bits(bits[2 * j + 1] ? bits[2 * j + 1] : bits[2 * j]);
        if (cudaMemsetAsync(c->lws[idx[j]].p, 0, 8, st) != cudaSuccess) return ZCCL_GPU_ECUDA;
        cleared = true;
    }
    if (cleared && cudaStreamSynchronize(st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    return rc ? rc : rc2;
}

uint32_t lanes_for(size_t groups) { return (uint32_t)std::min<size_t>(groups, kLanes); }

/* The caller's output stream from the groups' device streams, group by
 * group in order: group k's size and header (in pinned memory once its
 * event has fired) give its chunk offsets, rebased into the caller's header,
 * and its chunk bytes are copied out on the stream given: the group's own
 * lane, before anything else is queued there.  (A separate copy stream can
 * share a hardware queue with a busy lane and wait behind its kernels.)
 * dev[k] is group k's device stream, cap[k] its capacity, pin + poff[k] its
 * size and header; with after_inputs every copy waits for c->ev (recorded
 * once every input copy is issued), for an output written over an input. */
struct Placer {
    DropCtx *c;
    const std::vector<Group> &gr;
    uint8_t *const *dev;
    const size_t *cap, *poff;
    unsigned char *out;
    uint32_t T;
    bool after_inputs;
    uint64_t run = 0; /* chunk bytes placed */
    size_t next = 0;  /* the next group to place */

    int place(cudaStream_t st)
    {
        const size_t k = next++;
        const Group &q = gr[k];
        const uint8_t *pin = (const uint8_t *)c->pin.p;
        if (cudaEventSynchronize(c->ev_k[k]) != cudaSuccess) return ZCCL_GPU_ECUDA;
        uint64_t size;
        memcpy(&size, pin + poff[k], 8);
        const uint64_t hdr = 8ull * (q.s1 - q.s0);
        if (size < hdr || size > cap[k]) return ZCCL_GPU_ECORRUPT; /* the status words tell why */
        for (uint32_t i = 0; i < q.s1 - q.s0; i++) {
            uint64_t e;
            memcpy(&e, pin + poff[k] + 8 + 8ull * i, 8);
            e += run;
            memcpy(out + 8ull * (q.s0 + i), &e, 8);
        }
        if ((after_inputs && cudaStreamWaitEvent(st, c->ev, 0) != cudaSuccess) ||
            cudaMemcpyAsync(out + 8ull * T + run, dev[k] + hdr, size - hdr, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess)
            return ZCCL_GPU_ECUDA;
        run += size - hdr;
        return ZCCL_GPU_OK;
    }
};

/* Compression of host floats into a host stream, group by group. */
int pipe_compress(DropCtx *c, unsigned char *out, const float *x, size_t *outSize, float eb, const ZGeom &g,
                  const std::vector<Group> &gr)
{
    const size_t G = gr.size();
    size_t soff[kMaxGroups + 1] = {0}, poff[kMaxGroups + 1] = {0}, cap[kMaxGroups];
    for (size_t k = 0; k < G; k++) {
        cap[k] = (size_t)zg_stream_worst(&gr[k].g);
        soff[k + 1] = soff[k] + a256(cap[k]);
        poff[k + 1] = poff[k] + 8 + 8ull * (gr[k].s1 - gr[k].s0);
    }
    const uint32_t NL = lanes_for(G);
    if (int rc = c->fin.ensure(4 * g.n)) return rc;
    if (int rc = c->s[0].ensure(soff[G])) return rc;
    for (uint32_t l = 0; l < NL; l++) {
        if (int rc = c->lix[l][0].ensure(max_index_bytes(gr))) return rc;
        if (int rc = c->lws[l].ensure(max_ws_bytes(gr))) return rc;
    }
    if (int rc = c->pin.ensure(poff[G])) return rc;
    float *fin = (float *)c->fin.p;
    uint8_t *dev[kMaxGroups];
    int rc = ZCCL_GPU_OK;
    /* from pinned memory every group's floats are queued for the link first,
     * so that the host waiting to place an earlier group never leaves the
     * link idle; from pageable memory (each copy holds the host) group by
     * group, each just before its kernels */
    auto copy_in = [&](size_t k) {
        return cudaMemcpyAsync(fin + gr[k].e0, x + gr[k].e0, 4 * gr[k].n, cudaMemcpyHostToDevice, c->st_in) ==
                       cudaSuccess &&
                       cudaEventRecord(c->ev_in[k], c->st_in) == cudaSuccess
                   ? ZCCL_GPU_OK
                   : ZCCL_GPU_ECUDA;
    };
    const bool upfront = is_pinned_ptr(x);
    for (size_t k = 0; upfront && k < G && !rc; k++) rc = copy_in(k);
    for (size_t k = 0; k < G; k++) dev[k] = (uint8_t *)c->s[0].p + soff[k];
    Placer pl{c, gr, dev, cap, poff, out, g.T, false};
    for (size_t k = 0; k < G && !rc; k++) {
        const Group &q = gr[k];
        const uint32_t l = (uint32_t)(k % NL);
        cudaStream_t st = c->lane[l];
        if (!upfront && (rc = copy_in(k))) break;
        if (k >= NL && (rc = pl.place(st))) break; /* group k - NL, which ran on this lane */
        if (cudaStreamWaitEvent(st, c->ev_in[k], 0) != cudaSuccess) {
            rc = ZCCL_GPU_ECUDA;
            break;
        }
        zccl_gpu_stream sub;
        sub.bytes = dev[k];
        sub.capacity = cap[k];
        sub.index = c->lix[l][0].p;
        sub.indexed = 0;
        sub.qprev_valid = 0;
        if ((rc = compress_fmt(&sub, fin + q.e0, (size_t)q.n, eb, (int)g.L, (int)(q.s1 - q.s0), c->lws[l].p, st,
                               g.fmt)))
            break;
        uint8_t *pin = (uint8_t *)c->pin.p + poff[k];
        if (cudaMemcpyAsync(pin, sub.index, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(pin + 8, dev[k], 8ull * (q.s1 - q.s0), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaEventRecord(c->ev_k[k], st) != cudaSuccess)
            rc = ZCCL_GPU_ECUDA;
    }
    while (!rc && pl.next < G) rc = pl.place(c->lane[pl.next % NL]);
    rc = pipe_finish(c, rc, NL);
    if (rc) return rc;
    *outSize = (size_t)(8ull * g.T + pl.run);
    return ZCCL_GPU_OK;
}

/* Chunk offsets of a host stream's header (T entries). */
std::vector<uint64_t> host_header(const unsigned char *cmp, uint32_t T)
{
    std::vector<uint64_t> e(T);
    memcpy(e.data(), cmp, 8ull * T);
    return e;
}

/* Bytes of host stream cmp that group q's chunks take: exact for all but
 * the group holding the last chunk, whose end is not in the header; that
 * one is read as the whole-stream path reads it (twice the others' average
 * chunk first, or up to the largest possible size when `full`). */
bool group_bytes(const ZGeom &g, const std::vector<uint64_t> &e, const Group &q, bool full, uint64_t *len,
                 bool *capped)
{
    *capped = false;
    const uint32_t T = g.T;
    if (q.s1 < T) {
        if (e[q.s1] < e[q.s0]) return false;
        *len = e[q.s1] - e[q.s0];
        return true;
    }
    const uint64_t last = e[T - 1];
    if (last < e[q.s0]) return false;
    const uint64_t known = last - e[q.s0]; /* bytes of the group's chunks before the last */
    const uint64_t worst = zg_seg_worst(g.tbs, g.L) + zg_seg_worst(g.rem, g.L);
    uint64_t want = known + worst;
    if (!full) {
        const uint64_t guess = known + 2 * (last / (T - 1)) + 65536;
        if (guess < want) {
            want = guess;
            *capped = true;
        }
    }
    *len = want;
    return true;
}

/* Decompression of a host stream into host floats, group by group.  *capped
 * reports whether the last group was read short (an EBOUNDS then calls for
 * the full read). */
int pipe_decompress(DropCtx *c, float *y, const unsigned char *cmp, float eb, const ZGeom &g,
                    const std::vector<Group> &gr, bool full, bool *capped)
{
    const size_t G = gr.size();
    const std::vector<uint64_t> e = host_header(cmp, g.T);
    uint64_t len[kMaxGroups];
    size_t soff[kMaxGroups + 1] = {0}, poff[kMaxGroups + 1] = {0};
    *capped = false;
    for (size_t k = 0; k < G; k++) {
        bool cp = false;
        if (!group_bytes(g, e, gr[k], full, &len[k], &cp)) return ZCCL_GPU_ECORRUPT;
        *capped |= cp;
        soff[k + 1] = soff[k] + a256(8ull * (gr[k].s1 - gr[k].s0) + len[k] + 64);
        poff[k + 1] = poff[k] + 8ull * (gr[k].s1 - gr[k].s0);
    }
    const uint32_t NL = lanes_for(G);
    if (int rc = c->fout.ensure(4 * g.n)) return rc;
    if (int rc = c->s[0].ensure(soff[G])) return rc;
    for (uint32_t l = 0; l < NL; l++) {
        if (int rc = c->lix[l][0].ensure(max_index_bytes(gr))) return rc;
        if (int rc = c->lws[l].ensure(max_ws_bytes(gr))) return rc;
    }
    if (int rc = c->pin.ensure(poff[G])) return rc;
    float *fout = (float *)c->fout.p;
    uint8_t *pin = (uint8_t *)c->pin.p;
    const unsigned char *body = cmp + 8ull * g.T;
    int rc = ZCCL_GPU_OK;
    for (size_t k = 0; k < G && !rc; k++) {
        const Group &q = gr[k];
        const uint32_t Ts = q.s1 - q.s0;
        const uint32_t l = (uint32_t)(k % NL);
        cudaStream_t st = c->lane[l];
        uint8_t *dev = (uint8_t *)c->s[0].p + soff[k];
        for (uint32_t i = 0; i < Ts; i++) { /* the group's own header, its offsets rebased */
            const uint64_t v = e[q.s0 + i] - e[q.s0];
            memcpy(pin + poff[k] + 8ull * i, &v, 8);
        }
        if (cudaMemcpyAsync(dev, pin + poff[k], 8ull * Ts, cudaMemcpyHostToDevice, c->st_in) != cudaSuccess ||
            cudaMemcpyAsync(dev + 8ull * Ts, body + e[q.s0], len[k], cudaMemcpyHostToDevice, c->st_in) !=
                cudaSuccess ||
            cudaEventRecord(c->ev_in[k], c->st_in) != cudaSuccess ||
            cudaStreamWaitEvent(st, c->ev_in[k], 0) != cudaSuccess) {
            rc = ZCCL_GPU_ECUDA;
            break;
        }
        zccl_gpu_stream sub;
        sub.bytes = dev;
        sub.capacity = 8ull * Ts + len[k];
        sub.index = c->lix[l][0].p;
        sub.indexed = 0;
        sub.qprev_valid = 0;
        if ((rc = decompress_fmt(fout + q.e0, &sub, (size_t)q.n, eb, (int)g.L, (int)Ts, c->lws[l].p, st, g.fmt)))
            break;
        /* the floats leave on the group's lane: a separate copy stream may
         * share a hardware queue with a busy lane (see drop_ctx) */
        if (cudaMemcpyAsync(y + q.e0, fout + q.e0, 4 * q.n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = ZCCL_GPU_ECUDA;
    }
    return pipe_finish(c, rc, NL);
}

/* Two-way homomorphic add of host streams into a host stream, group by
 * group: both inputs' chunks copied in, walked and added, the sum's chunks
 * copied out as each group's size arrives. */
int pipe_homadd(DropCtx *c, unsigned char *out, size_t *out_size, const unsigned char *cmp1,
                const unsigned char *cmp2, const ZGeom &g, const std::vector<Group> &gr, bool full, bool *capped)
{
    const size_t G = gr.size();
    const unsigned char *cmp[2] = {cmp1, cmp2};
    const std::vector<uint64_t> e[2] = {host_header(cmp1, g.T), host_header(cmp2, g.T)};
    uint64_t len[2][kMaxGroups];
    size_t ioff[kMaxGroups + 1] = {0}, soff[kMaxGroups + 1] = {0}, poff[kMaxGroups + 1] = {0}, cap[kMaxGroups];
    *capped = false;
    for (size_t k = 0; k < G; k++) {
        const uint64_t Ts = gr[k].s1 - gr[k].s0;
        for (int i = 0; i < 2; i++) {
            bool cp = false;
            if (!group_bytes(g, e[i], gr[k], full, &len[i][k], &cp)) return ZCCL_GPU_ECORRUPT;
            *capped |= cp;
        }
        ioff[k + 1] = ioff[k] + a256(8 * Ts + len[0][k] + 64) + a256(8 * Ts + len[1][k] + 64);
        cap[k] = (size_t)zg_stream_worst(&gr[k].g);
        soff[k + 1] = soff[k] + a256(cap[k]);
        /* pinned: the sum's size and header, then both inputs' rebased headers */
        poff[k + 1] = poff[k] + 8 + 8 * Ts + 2 * 8 * Ts;
    }
    const uint32_t NL = lanes_for(G);
    /* every group but the last (whose final chunk has no known end) walks
     * both inputs as one stream of 2 Ts chunks, the first input's chunks and
     * then the second's: one walk instead of two, each input's index a half
     * of the pair's */
    ZGeom gc[kMaxGroups];
    bool comb[kMaxGroups];
    size_t ixb = max_index_bytes(gr), wsb = max_ws_bytes(gr);
    for (size_t k = 0; k < G; k++) {
        const uint32_t Ts = gr[k].s1 - gr[k].s0;
        comb[k] = gr[k].s1 < g.T && !make_geom((size_t)(2 * gr[k].n), (int)g.L, (int)(2 * Ts), &gc[k]) &&
                  gc[k].tbs == g.tbs && gc[k].rem == 0;
        if (comb[k]) {
            gc[k].fmt = g.fmt;
            ixb = std::max(ixb, index_layout(gc[k]).total);
            wsb = std::max(wsb, ws_bytes(gc[k]));
        }
    }
    if (int rc = c->s[1].ensure(ioff[G])) return rc;
    if (int rc = c->s[2].ensure(soff[G])) return rc;
    for (uint32_t l = 0; l < NL; l++) {
        for (int i = 0; i < 3; i++)
            if (int rc = c->lix[l][i].ensure(ixb)) return rc;
        if (int rc = c->lws[l].ensure(wsb)) return rc;
        if (int rc = c->lws[kLanes + l].ensure(max_ws_bytes(gr))) return rc; /* second walks: one input's group */
    }
    if (int rc = c->pin.ensure(poff[G])) return rc;
    uint8_t *pin = (uint8_t *)c->pin.p;
    uint8_t *dev[kMaxGroups];
    int rc = ZCCL_GPU_OK;
    /* from pinned memory every group's input bytes are queued for the link
     * first, so that the host waiting to place an earlier group never leaves
     * the link idle; from pageable memory (each copy holds the host) group
     * by group, each just before its kernels */
    auto copy_in = [&](size_t k) -> int {
        int rc = ZCCL_GPU_OK;
        const Group &q = gr[k];
        const uint32_t Ts = q.s1 - q.s0;
        uint8_t *ib = (uint8_t *)c->s[1].p + ioff[k];
        if (comb[k]) {
            uint8_t *h = pin + poff[k] + 8 + 8ull * Ts; /* the 2 Ts combined chunk offsets */
            for (uint32_t j = 0; j < 2 * Ts; j++) {
                const int i = j < Ts ? 0 : 1;
                const uint64_t v = (i ? len[0][k] : 0) + e[i][q.s0 + j - i * Ts] - e[i][q.s0];
                memcpy(h + 8ull * j, &v, 8);
            }
            const size_t hb = 16ull * Ts;
            if (cudaMemcpyAsync(ib, h, hb, cudaMemcpyHostToDevice, c->st_in) != cudaSuccess ||
                cudaMemcpyAsync(ib + hb, cmp[0] + 8ull * g.T + e[0][q.s0], len[0][k], cudaMemcpyHostToDevice,
                                c->st_in) != cudaSuccess ||
                cudaMemcpyAsync(ib + hb + len[0][k], cmp[1] + 8ull * g.T + e[1][q.s0], len[1][k],
                                cudaMemcpyHostToDevice, c->st_in) != cudaSuccess)
                rc = ZCCL_GPU_ECUDA;
        } else {
            for (int i = 0; i < 2 && !rc; i++) {
                uint8_t *h = pin + poff[k] + 8 + 8ull * Ts + 8ull * Ts * i;
                for (uint32_t j = 0; j < Ts; j++) {
                    const uint64_t v = e[i][q.s0 + j] - e[i][q.s0];
                    memcpy(h + 8ull * j, &v, 8);
                }
                if (cudaMemcpyAsync(ib, h, 8ull * Ts, cudaMemcpyHostToDevice, c->st_in) != cudaSuccess ||
                    cudaMemcpyAsync(ib + 8ull * Ts, cmp[i] + 8ull * g.T + e[i][q.s0], len[i][k],
                                    cudaMemcpyHostToDevice, c->st_in) != cudaSuccess)
                    rc = ZCCL_GPU_ECUDA;
                ib += a256(8ull * Ts + len[i][k] + 64);
            }
        }
        if (!rc && cudaEventRecord(c->ev_in[k], c->st_in) != cudaSuccess) rc = ZCCL_GPU_ECUDA;
        return rc;
    };
    const bool upfront = is_pinned_ptr(cmp1) && is_pinned_ptr(cmp2);
    for (size_t k = 0; upfront && k < G && !rc; k++) rc = copy_in(k);
    /* the sum written over an input (the ring adds into its receive
     * buffer): no byte goes out before every input byte is in */
    const size_t out_span = (size_t)zg_stream_worst(&g);
    const size_t in_span0 = 8ull * g.T + (size_t)(e[0][gr[G - 1].s0] + len[0][G - 1]);
    const size_t in_span1 = 8ull * g.T + (size_t)(e[1][gr[G - 1].s0] + len[1][G - 1]);
    const bool after_inputs = overlaps(out, out_span, cmp1, in_span0) || overlaps(out, out_span, cmp2, in_span1);
    if (!upfront && after_inputs) /* an output over pageable inputs: every input in first */
        for (size_t k = 0; k < G && !rc; k++) rc = copy_in(k);
    if (!rc && after_inputs && cudaEventRecord(c->ev, c->st_in) != cudaSuccess) rc = ZCCL_GPU_ECUDA;
    const bool per_group = !upfront && !after_inputs;
    for (size_t k = 0; k < G; k++) dev[k] = (uint8_t *)c->s[2].p + soff[k];
    Placer pl{c, gr, dev, cap, poff, out, g.T, after_inputs};
    for (size_t k = 0; k < G && !rc; k++) {
        const Group &q = gr[k];
        const uint32_t Ts = q.s1 - q.s0;
        const uint32_t l = (uint32_t)(k % NL);
        /* a second input's walk runs on the next lane, beside the first's */
        cudaStream_t st = c->lane[l], st2 = c->lane[(l + 1) % NL];
        void *ws = c->lws[l].p, *ws2 = c->lws[kLanes + l].p;
        if (per_group && (rc = copy_in(k))) break;
        if (k >= NL && (rc = pl.place(st))) break; /* group k - NL, which ran on this lane */
        zccl_gpu_stream in[2], sum;
        uint8_t *ib = (uint8_t *)c->s[1].p + ioff[k];
        sum.bytes = dev[k];
        sum.capacity = cap[k];
        sum.index = c->lix[l][2].p;
        sum.indexed = 0;
        sum.qprev_valid = 0;
        if (comb[k]) {
            zccl_gpu_stream both;
            both.bytes = ib;
            both.capacity = 16ull * Ts + len[0][k] + len[1][k];
            both.index = c->lix[l][0].p;
            both.indexed = 0;
            both.qprev_valid = 0;
            if (cudaStreamWaitEvent(st, c->ev_in[k], 0) != cudaSuccess || ws_clear(ws, gc[k], st) != cudaSuccess) {
                rc = ZCCL_GPU_ECUDA;
                break;
            }
            if ((rc = walk_stream(&both, gc[k], ws, st))) break;
            const ZIndex ix = bind_index(both.index, gc[k]);
            HomInput hi[2];
            for (int i = 0; i < 2; i++) {
                hi[i].bytes = ib;
                hi[i].avail = both.capacity;
                hi[i].widths = ix.widths + (size_t)i * q.g.nblocks;
                hi[i].tile_off = ix.tile_off + (size_t)i * q.g.ntiles;
                hi[i].tile_qprev = ix.tile_qprev + (size_t)i * q.g.ntiles;
            }
            if ((rc = homadd_inputs(&sum, hi, 2, 0, q.g, ws, nullptr, st))) break;
        } else {
            for (int i = 0; i < 2; i++) {
                in[i].bytes = ib;
                in[i].capacity = 8ull * Ts + len[i][k];
                in[i].index = c->lix[l][i].p;
                in[i].indexed = 0;
                in[i].qprev_valid = 0;
                ib += a256(8ull * Ts + len[i][k] + 64);
            }
            /* the next lane's last group leaves before the second walk is
             * queued there; that walk's index is this lane's, free once the
             * add of this lane's previous group is done */
            if (st2 != st && pl.next + NL == k + 1 && (rc = pl.place(st2))) break;
            if (cudaStreamWaitEvent(st, c->ev_in[k], 0) != cudaSuccess ||
                cudaStreamWaitEvent(st2, c->ev_in[k], 0) != cudaSuccess ||
                (k >= NL && cudaStreamWaitEvent(st2, c->ev_k[k - NL], 0) != cudaSuccess) ||
                ws_clear(ws, q.g, st) != cudaSuccess || ws_clear(ws2, q.g, st2) != cudaSuccess) {
                rc = ZCCL_GPU_ECUDA;
                break;
            }
            /* a failed walk of the second input is reported by its lane's
             * status words; the add never trusts an index for its bounds */
            if ((rc = walk_stream(&in[0], q.g, ws, st)) || (rc = walk_stream(&in[1], q.g, ws2, st2))) break;
            if (cudaEventRecord(c->ev_w[k], st2) != cudaSuccess ||
                cudaStreamWaitEvent(st, c->ev_w[k], 0) != cudaSuccess) {
                rc = ZCCL_GPU_ECUDA;
                break;
            }
            if ((rc = zccl_gpu_homadd_cases(&sum, in, 2, (size_t)q.n, (int)g.L, (int)Ts, ws, nullptr, st))) break;
        }
        uint8_t *pk = pin + poff[k];
        if (cudaMemcpyAsync(pk, sum.index, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(pk + 8, dev[k], 8ull * Ts, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaEventRecord(c->ev_k[k], st) != cudaSuccess)
            rc = ZCCL_GPU_ECUDA;
    }
    while (!rc && pl.next < G) rc = pl.place(c->lane[pl.next % NL]);
    const uint64_t placed = pl.run;
    rc = pipe_finish(c, rc, NL, true);
    if (rc) return rc;
    *out_size += (size_t)(8ull * g.T + placed);
    return ZCCL_GPU_OK;
}

int dropin_compress(unsigned char *outputBytes, const float *oriData, size_t *outSize, float eb,
                    size_t n, int L, int T, uint32_t fmt = ZG_FASTMODE1, uint64_t *nz_out = nullptr)
{
    ZGeom g;
    if (!outputBytes || !oriData || !outSize || make_geom(n, L, T, &g)) return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    const float *d_in = oriData;
    if (!nz_out && !is_device_ptr(oriData) && !is_device_ptr(outputBytes) &&
        !overlaps(outputBytes, (size_t)zg_stream_worst(&g), oriData, 4 * n)) {
        g.fmt = fmt;
        const std::vector<Group> gr = chunk_groups(g, kGroupsCompress);
        if (!gr.empty()) return pipe_compress(c, outputBytes, oriData, outSize, eb, g, gr);
    }
    if (!is_device_ptr(oriData)) {
        if (int rc = c->fin.ensure(4 * n)) return rc;
        if (cudaMemcpyAsync(c->fin.p, oriData, 4 * n, cudaMemcpyHostToDevice, c->st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
        d_in = (const float *)c->fin.p;
    }
    const size_t worst = (size_t)zg_stream_worst(&g);
    const bool dout = is_device_ptr(outputBytes);
    const size_t room = dout ? device_room(outputBytes) : 0;
    zccl_gpu_stream s;
    if (int rc = c->ix[0].ensure(index_layout(g).total)) return rc;
    if (int rc = c->ws.ensure(ws_bytes(g))) return rc;
    s.index = c->ix[0].p;
    if (dout && room >= worst) {
        s.bytes = outputBytes;
        s.capacity = room;
    } else {
        if (int rc = c->s[0].ensure(worst)) return rc;
        s.bytes = (unsigned char *)c->s[0].p;
        s.capacity = worst;
    }
    if (int rc = compress_fmt(&s, d_in, n, eb, L, T, c->ws.p, c->st, fmt)) return rc;
    if (int rc = finish(c, c->ws.p)) return rc;
    size_t size = 0;
    if (int rc = zccl_gpu_stream_size(&s, n, L, T, &size, c->st)) return rc;
    if (nz_out)
        if (int rc = nonzero_elements(c, s.index, g, nz_out)) return rc;
    if (s.bytes != outputBytes) {
        if (dout && size > room) return ZCCL_GPU_ECAPACITY;
        cudaMemcpyKind k = dout ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (cudaMemcpyAsync(outputBytes, s.bytes, size, k, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
        if (cudaStreamSynchronize(c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    }
    *outSize = size;
    return ZCCL_GPU_OK;
}

int dropin_decompress(float *newData, size_t n, float eb, int L, const unsigned char *cmp, int T,
                      uint32_t fmt = ZG_FASTMODE1, uint64_t *nz_out = nullptr, uint64_t *size_out = nullptr)
{
    ZGeom g;
    if (!newData || !cmp || make_geom(n, L, T, &g)) return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    const bool dout = is_device_ptr(newData);
    if (!dout && !nz_out && !size_out && !is_device_ptr(cmp) &&
        !overlaps(newData, 4 * n, cmp, (size_t)zg_stream_worst(&g))) {
        g.fmt = fmt;
        const std::vector<Group> gr = chunk_groups(g, kGroupsDecompress);
        if (!gr.empty()) {
            bool capped = false;
            int rc = pipe_decompress(c, newData, cmp, eb, g, gr, false, &capped);
            if (rc == ZCCL_GPU_EBOUNDS && capped) rc = pipe_decompress(c, newData, cmp, eb, g, gr, true, &capped);
            return rc;
        }
    }
    if (int rc = c->ws.ensure(ws_bytes(g))) return rc;
    float *d_out = newData;
    if (!dout) {
        if (int rc = c->fout.ensure(4 * n)) return rc;
        d_out = (float *)c->fout.p;
    }
    /* A host stream is first read up to 4*nbEle bytes; only a stream that
     * really runs past that (tiny arrays, near-32-bit widths) is read again
     * up to its largest possible size. */
    for (int pass = 0;; pass++) {
        zccl_gpu_stream s;
        bool capped;
        if (int rc = stage_stream(c, 0, cmp, g, &s, pass > 0, &capped)) return rc;
        if (int rc = decompress_fmt(d_out, &s, n, eb, L, T, c->ws.p, c->st, fmt)) return rc;
        int rc = finish(c, c->ws.p);
        if (rc == ZCCL_GPU_EBOUNDS && capped && pass == 0) continue;
        if (rc) return rc;
        if (nz_out)
            if ((rc = nonzero_elements(c, s.index, g, nz_out))) return rc;
        if (size_out)
            if ((rc = zccl_gpu_stream_size(&s, n, L, T, (size_t *)size_out, c->st))) return rc;
        break;
    }
    if (!dout) {
        if (cudaMemcpyAsync(newData, d_out, 4 * n, cudaMemcpyDeviceToHost, c->st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
        if (cudaStreamSynchronize(c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    }
    return ZCCL_GPU_OK;
}

int dropin_homadd(unsigned char *final_cmp, size_t *final_size, size_t n, float eb, int L,
                  const unsigned char *cmp1, const unsigned char *cmp2, int T,
                  unsigned long long *cases_out = nullptr)
{
    (void)eb;
    ZGeom g;
    if (!final_cmp || !final_size || !cmp1 || !cmp2 || make_geom(n, L, T, &g)) return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!cases_out && !is_device_ptr(final_cmp) && !is_device_ptr(cmp1) && !is_device_ptr(cmp2)) {
        const std::vector<Group> gr = chunk_groups(g, kGroupsHomadd);
        if (!gr.empty()) {
            bool capped = false;
            int rc = pipe_homadd(c, final_cmp, final_size, cmp1, cmp2, g, gr, false, &capped);
            if (rc == ZCCL_GPU_EBOUNDS && capped) rc = pipe_homadd(c, final_cmp, final_size, cmp1, cmp2, g, gr, true, &capped);
            return rc;
        }
    }
    if (int rc = c->ws.ensure(ws_bytes(g))) return rc;
    zccl_gpu_stream in[2], out;
    const size_t worst = (size_t)zg_stream_worst(&g);
    if (int rc = c->s[2].ensure(worst)) return rc;
    if (int rc = c->ix[2].ensure(index_layout(g).total)) return rc;
    out.bytes = (unsigned char *)c->s[2].p;
    out.capacity = worst;
    out.index = c->ix[2].p;
    for (int pass = 0;; pass++) { /* second pass: see dropin_decompress */
        bool cap1, cap2;
        /* the first input's index walk runs while the second input is
         * copied on the other stream; then the second's walk, a check of
         * both, and the add of the indexed inputs */
        if (ws_clear(c->ws.p, g, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
        if (int rc = stage_stream(c, 0, cmp1, g, &in[0], pass > 0, &cap1)) return rc;
        if (int rc = walk_stream(&in[0], g, c->ws.p, c->st)) return rc;
        if (int rc = stage_stream(c, 1, cmp2, g, &in[1], pass > 0, &cap2, c->st2)) return rc;
        if (cudaEventRecord(c->ev, c->st2) != cudaSuccess || cudaStreamWaitEvent(c->st, c->ev, 0) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
        if (int rc = walk_stream(&in[1], g, c->ws.p, c->st)) return rc;
        int rc = finish(c, c->ws.p);
        unsigned long long *d_cases = nullptr;
        if (rc == ZCCL_GPU_OK && cases_out) {
            if ((rc = c->aux.ensure(64))) return rc;
            d_cases = static_cast<unsigned long long *>(c->aux.p) + 1;
            if (cudaMemsetAsync(d_cases, 0, 32, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
        }
        if (rc == ZCCL_GPU_OK) {
            if ((rc = zccl_gpu_homadd_cases(&out, in, 2, n, L, T, c->ws.p, d_cases, c->st))) return rc;
            rc = finish(c, c->ws.p);
        }
        if (rc == ZCCL_GPU_OK && d_cases &&
            (cudaMemcpyAsync(cases_out, d_cases, 32, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
             cudaStreamSynchronize(c->st) != cudaSuccess))
            return ZCCL_GPU_ECUDA;
        if (rc == ZCCL_GPU_EBOUNDS && (cap1 || cap2) && pass == 0) continue;
        if (rc) return rc;
        break;
    }
    size_t size = 0;
    if (int rc = zccl_gpu_stream_size(&out, n, L, T, &size, c->st)) return rc;
    const bool dout = is_device_ptr(final_cmp);
    if (dout && size > device_room(final_cmp)) return ZCCL_GPU_ECAPACITY;
    cudaMemcpyKind k = dout ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (cudaMemcpyAsync(final_cmp, out.bytes, size, k, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (cudaStreamSynchronize(c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    *final_size += size;
    return ZCCL_GPU_OK;
}

int omp_threads() { return omp_get_max_threads(); }

/* ---- SZp 3-D drop-ins ---------------------------------------------- */

bool sz3_args_ok(size_t d1, size_t d2, size_t d3, int bs, double eb)
{
    return d1 && d2 && d3 && bs >= 1 && bs <= 32 && eb > 0 && std::isfinite(eb);
}

/* Stream bytes from its rate table (host memory). */
size_t sz3_host_stream_bytes(const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs)
{
    const size_t nb1 = (d1 - 1) / bs + 1, nb2 = (d2 - 1) / bs + 1, nb3 = (d3 - 1) / bs + 1;
    size_t total = nb1 * nb2 * nb3, b = 0;
    for (size_t x = 0; x < nb1; x++)
        for (size_t y = 0; y < nb2; y++)
            for (size_t z = 0; z < nb3; z++, b++) {
                const size_t n = std::min<size_t>(bs, d1 - x * bs) * std::min<size_t>(bs, d2 - y * bs) *
                                 std::min<size_t>(bs, d3 - z * bs);
                const size_t r = cmp[b] > 32 ? 0 : cmp[b];
                if (r) total += (n + 7) / 8 + (r / 8) * n + ((r % 8) * n + 7) / 8;
            }
    return total;
}

int dropin_szp3d_compress(const float *x, unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs,
                          double eb, size_t *cmpSize)
{
    if (!x || !cmp || !cmpSize || !sz3_args_ok(d1, d2, d3, bs, eb)) return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    const size_t n = d1 * d2 * d3, cap = sz3_max_stream_bytes(d1, d2, d3, (uint32_t)bs);
    if (int rc = c->ws.ensure(sz3_workspace_bytes(d1, d2, d3, (uint32_t)bs, true) + 16)) return rc;
    const bool din = is_device_ptr(x), dout = is_device_ptr(cmp);
    const float *d_x = x;
    if (!din) {
        if (int rc = c->fin.ensure(4 * n)) return rc;
        if (cudaMemcpyAsync(c->fin.p, x, 4 * n, cudaMemcpyHostToDevice, c->st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
        d_x = (const float *)c->fin.p;
    }
    unsigned char *d_out = cmp;
    size_t room = dout ? device_room(cmp) : cap; /* callers allocate the stream; device: its allocation */
    if (!dout) {
        if (int rc = c->s[0].ensure(cap)) return rc;
        d_out = (unsigned char *)c->s[0].p;
    }
    uint64_t *d_size = (uint64_t *)((uint8_t *)c->ws.p + sz3_workspace_bytes(d1, d2, d3, (uint32_t)bs, true));
    if (cudaError_t e = sz3_compress(d_out, room, d_x, d1, d2, d3, (uint32_t)bs, eb, c->ws.p, d_size, c->st))
        return e == cudaErrorInvalidValue ? ZCCL_GPU_ECAPACITY : ZCCL_GPU_ECUDA;
    uint64_t size = 0;
    if (cudaMemcpyAsync(&size, d_size, 8, cudaMemcpyDeviceToHost, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (int rc = finish(c, c->ws.p)) return rc;
    if (!dout) {
        if (cudaMemcpyAsync(cmp, d_out, size, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
            cudaStreamSynchronize(c->st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
    }
    *cmpSize = (size_t)size;
    return ZCCL_GPU_OK;
}

int dropin_szp3d_decompress(float *y, const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs, double eb)
{
    if (!y || !cmp || !sz3_args_ok(d1, d2, d3, bs, eb)) return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    const size_t n = d1 * d2 * d3;
    if (int rc = c->ws.ensure(sz3_workspace_bytes(d1, d2, d3, (uint32_t)bs, false))) return rc;
    const bool din = is_device_ptr(cmp), dout = is_device_ptr(y);
    const unsigned char *d_in = cmp;
    size_t avail;
    if (din) {
        avail = device_room(cmp);
        if (!avail) return ZCCL_GPU_EINVAL;
    } else {
        avail = sz3_host_stream_bytes(cmp, d1, d2, d3, bs);
        if (int rc = c->s[0].ensure(avail)) return rc;
        if (cudaMemcpyAsync(c->s[0].p, cmp, avail, cudaMemcpyHostToDevice, c->st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
        d_in = (const unsigned char *)c->s[0].p;
    }
    float *d_y = y;
    if (!dout) {
        if (int rc = c->fout.ensure(4 * n)) return rc;
        d_y = (float *)c->fout.p;
    }
    if (sz3_decompress(d_y, d_in, avail, d1, d2, d3, (uint32_t)bs, eb, c->ws.p, c->st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    if (int rc = finish(c, c->ws.p)) return rc;
    if (!dout) {
        if (cudaMemcpyAsync(y, d_y, 4 * n, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
            cudaStreamSynchronize(c->st) != cudaSuccess)
            return ZCCL_GPU_ECUDA;
    }
    return ZCCL_GPU_OK;
}

/* The OpenMP form: T = omp_get_max_threads() sub-volumes. */
int dropin_szp3d_compress_split(const float *x, unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs, double eb,
                                size_t *cmpSize, int T)
{
    Sz3Split3 sp;
    if (!x || !cmp || !cmpSize || !sz3_args_ok(d1, d2, d3, bs, eb) || !sz3_split_plan(d1, d2, d3, (uint32_t)T, &sp))
        return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    const size_t n = d1 * d2 * d3, cap = sz3_split_max_stream_bytes(sp, (uint32_t)bs);
    const size_t wsb = sz3_split_workspace_bytes(sp, (uint32_t)bs, true);
    if (int rc = c->ws.ensure(wsb + 16)) return rc;
    const bool din = is_device_ptr(x), dout = is_device_ptr(cmp);
    const float *d_x = x;
    if (!din) {
        if (int rc = c->fin.ensure(4 * n)) return rc;
        if (cudaMemcpyAsync(c->fin.p, x, 4 * n, cudaMemcpyHostToDevice, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
        d_x = (const float *)c->fin.p;
    }
    unsigned char *d_out = cmp;
    const size_t room = dout ? device_room(cmp) : cap;
    if (!dout) {
        if (int rc = c->s[0].ensure(cap)) return rc;
        d_out = (unsigned char *)c->s[0].p;
    }
    uint64_t *d_size = (uint64_t *)((uint8_t *)c->ws.p + wsb);
    if (cudaError_t e = sz3_split_compress(d_out, room, d_x, sp, (uint32_t)bs, eb, c->ws.p, d_size, c->st))
        return e == cudaErrorInvalidValue ? ZCCL_GPU_ECAPACITY : ZCCL_GPU_ECUDA;
    uint64_t size = 0;
    if (cudaMemcpyAsync(&size, d_size, 8, cudaMemcpyDeviceToHost, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (int rc = finish(c, c->ws.p)) return rc;
    if (!dout && (cudaMemcpyAsync(cmp, d_out, size, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
                  cudaStreamSynchronize(c->st) != cudaSuccess))
        return ZCCL_GPU_ECUDA;
    *cmpSize = (size_t)size;
    return ZCCL_GPU_OK;
}

int dropin_szp3d_decompress_split(float *y, const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs,
                                  double eb, int T)
{
    Sz3Split3 sp;
    if (!y || !cmp || !sz3_args_ok(d1, d2, d3, bs, eb) || !sz3_split_plan(d1, d2, d3, (uint32_t)T, &sp))
        return ZCCL_GPU_EINVAL;
    DropCtx *c = drop_ctx();
    if (!c) return ZCCL_GPU_ECUDA;
    std::lock_guard<std::mutex> lk(c->mu);
    const size_t n = d1 * d2 * d3, hdr = 8ull * (size_t)T;
    if (int rc = c->ws.ensure(sz3_split_workspace_bytes(sp, (uint32_t)bs, false))) return rc;
    const bool din = is_device_ptr(cmp), dout = is_device_ptr(y);
    std::vector<uint64_t> offs(T);
    const unsigned char *d_in = cmp;
    size_t avail;
    if (din) {
        avail = device_room(cmp);
        if (avail < hdr || cudaMemcpy(offs.data(), cmp, hdr, cudaMemcpyDeviceToHost) != cudaSuccess)
            return ZCCL_GPU_EINVAL;
    } else {
        /* the stream's length: the last sub-stream's offset and its size
         * from its rate table */
        memcpy(offs.data(), cmp, hdr);
        uint64_t s[3];
        sz3_split_extent(sp, (uint32_t)T - 1, s);
        avail = hdr + (size_t)offs[T - 1] + sz3_host_stream_bytes(cmp + hdr + offs[T - 1], s[0], s[1], s[2], bs);
        if (int rc = c->s[0].ensure(avail)) return rc;
        if (cudaMemcpyAsync(c->s[0].p, cmp, avail, cudaMemcpyHostToDevice, c->st) != cudaSuccess) return ZCCL_GPU_ECUDA;
        d_in = (const unsigned char *)c->s[0].p;
    }
    float *d_y = y;
    if (!dout) {
        if (int rc = c->fout.ensure(4 * n)) return rc;
        d_y = (float *)c->fout.p;
    }
    if (cudaError_t e = sz3_split_decompress(d_y, d_in, avail, offs.data(), sp, (uint32_t)bs, eb, c->ws.p, c->st))
        return e == cudaErrorInvalidValue ? ZCCL_GPU_EBOUNDS : ZCCL_GPU_ECUDA;
    if (int rc = finish(c, c->ws.p)) return rc;
    if (!dout && (cudaMemcpyAsync(y, d_y, 4 * n, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
                  cudaStreamSynchronize(c->st) != cudaSuccess))
        return ZCCL_GPU_ECUDA;
    return ZCCL_GPU_OK;
}

} // namespace

extern "C" int zccl_gpu_last_status(void) { return t_last_status; }

extern "C" void ZCCL_float_openmp_threadblock_arg(unsigned char *outputBytes, float *oriData,
                                                  size_t *outSize, float absErrBound, size_t nbEle,
                                                  int blockSize)
{
    report(__func__, dropin_compress(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize,
                                     omp_threads()));
}

extern "C" void ZCCL_float_single_thread_arg(unsigned char *outputBytes, float *oriData,
                                             size_t *outSize, float absErrBound, size_t nbEle,
                                             int blockSize)
{
    report(__func__, dropin_compress(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize, 1));
}

extern "C" void ZCCL_float_decompress_openmp_threadblock_arg(float *newData, size_t nbEle,
                                                             float absErrBound, int blockSize,
                                                             unsigned char *cmpBytes)
{
    report(__func__,
           dropin_decompress(newData, nbEle, absErrBound, blockSize, cmpBytes, omp_threads()));
}

extern "C" void ZCCL_float_decompress_single_thread_arg(float *newData, size_t nbEle,
                                                        float absErrBound, int blockSize,
                                                        unsigned char *cmpBytes)
{
    report(__func__, dropin_decompress(newData, nbEle, absErrBound, blockSize, cmpBytes, 1));
}

extern "C" void ZCCL_float_homomophic_add_openmp_threadblock(unsigned char *final_cmpBytes,
                                                             size_t *final_cmpSize, size_t nbEle,
                                                             float absErrBound, int blockSize,
                                                             unsigned char *cmpBytes,
                                                             unsigned char *cmpBytes2)
{
    report(__func__, dropin_homadd(final_cmpBytes, final_cmpSize, nbEle, absErrBound, blockSize,
                                   cmpBytes, cmpBytes2, omp_threads()));
}

extern "C" void ZCCL_float_homomophic_add_single_thread(unsigned char *final_cmpBytes,
                                                        size_t *final_cmpSize, size_t nbEle,
                                                        float absErrBound, int blockSize,
                                                        unsigned char *cmpBytes,
                                                        unsigned char *cmpBytes2)
{
    report(__func__, dropin_homadd(final_cmpBytes, final_cmpSize, nbEle, absErrBound, blockSize,
                                   cmpBytes, cmpBytes2, 1));
}

/* ---- the allocating and the _record variants ----------------------------- */

extern "C" unsigned char *ZCCL_float_openmp_threadblock(float *oriData, size_t *outSize, float absErrBound,
                                                        size_t nbEle, int blockSize)
{
    /* The reference mallocs 4*nbEle bytes (ZCCL_float.c:204); the buffer
     * here holds the largest stream the geometry allows, which is never
     * less.  The caller frees it with free(). */
    const int T = omp_threads();
    ZGeom g;
    unsigned char *out = nullptr;
    int rc = ZCCL_GPU_EINVAL;
    if (outSize && make_geom(nbEle, blockSize, T, &g) == ZCCL_GPU_OK) {
        out = static_cast<unsigned char *>(malloc(std::max<size_t>(4 * nbEle, (size_t)zg_stream_worst(&g))));
        rc = out ? dropin_compress(out, oriData, outSize, absErrBound, nbEle, blockSize, T) : ZCCL_GPU_ENOMEM;
        if (rc != ZCCL_GPU_OK) {
            free(out);
            out = nullptr;
        }
    }
    report(__func__, rc);
    return out;
}

extern "C" void ZCCL_float_decompress_openmp_threadblock(float **newData, size_t nbEle, float absErrBound,
                                                        int blockSize, unsigned char *cmpBytes)
{
    /* *newData = malloc(4*nbEle) as in the reference (ZCCLd_float.c:29),
     * kept for the caller to free even when the call fails */
    if (!newData) {
        report(__func__, ZCCL_GPU_EINVAL);
        return;
    }
    *newData = static_cast<float *>(malloc(sizeof(float) * (nbEle ? nbEle : 1)));
    if (!*newData) {
        report(__func__, ZCCL_GPU_ENOMEM);
        return;
    }
    report(__func__, dropin_decompress(*newData, nbEle, absErrBound, blockSize, cmpBytes, omp_threads()));
}

extern "C" size_t ZCCL_float_single_thread_arg_record(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                                      float absErrBound, size_t nbEle, int blockSize)
{
    uint64_t nz = 0;
    const int rc = dropin_compress(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize, 1, ZG_FASTMODE1,
                                   &nz);
    report(__func__, rc);
    if (rc != ZCCL_GPU_OK) return 0;
    /* The reference's own count of the bytes its scalar code touches
     * (ZCCL_float.c:997-1208): 20 around the head, 12 per element of every
     * block, each block's bytes plus 8 per element of a non-zero-width one,
     * 56 for the offset table, and the chunk copied out (read and written).
     * It depends on the stream only, so it is computed from it. */
    const size_t C = *outSize, blocks = C - 12;
    return 20 + 12 * (nbEle - 1) + blocks + 8 * (size_t)nz + 56 + 2 * (C - 8);
}

extern "C" size_t ZCCL_float_decompress_single_thread_arg_record(float *newData, size_t nbEle, float absErrBound,
                                                                 int blockSize, unsigned char *cmpBytes)
{
    uint64_t nz = 0, C = 0;
    const int rc = dropin_decompress(newData, nbEle, absErrBound, blockSize, cmpBytes, 1, ZG_FASTMODE1, &nz, &C);
    report(__func__, rc);
    if (rc != ZCCL_GPU_OK) return 0;
    /* The reference's count (ZCCLd_float.c:383-533): 24 around the head,
     * each block's bytes, 8 per element of a zero-width block and 20 per
     * element of any other. */
    return 24 + (size_t)(C - 12) + 8 * (nbEle - 1) + 12 * (size_t)nz;
}

extern "C" void ZCCL_float_single_thread_arg_split_record(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                                          float absErrBound, size_t nbEle, int blockSize,
                                                          unsigned char *chunk_arr, size_t chunk_iter)
{
    /* The T = 1 stream, and its size also stored as size_t number
     * chunk_iter of chunk_arr (ZCCL_float.c:1691-1692), the frame table of
     * the split allreduce (ZCCL_ring.c:1496-1518).  chunk_arr may be host or
     * device memory. */
    int rc = dropin_compress(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize, 1);
    if (rc == ZCCL_GPU_OK && chunk_arr) {
        const size_t v = *outSize;
        unsigned char *dst = chunk_arr + chunk_iter * sizeof(size_t);
        if (is_device_ptr(chunk_arr))
            rc = cudaMemcpy(dst, &v, sizeof v, cudaMemcpyHostToDevice) == cudaSuccess ? ZCCL_GPU_OK : ZCCL_GPU_ECUDA;
        else
            memcpy(dst, &v, sizeof v);
    }
    report(__func__, rc);
}

extern "C" void ZCCL_float_homomophic_add_openmp_threadblock_record(unsigned char *final_cmpBytes,
                                                                    size_t *final_cmpSize, size_t nbEle,
                                                                    float absErrBound, int blockSize,
                                                                    unsigned char *cmpBytes, unsigned char *cmpBytes2,
                                                                    int *total_counter_1, int *total_counter_2,
                                                                    int *total_counter_3, int *total_counter_4)
{
    /* The add, and the reference's four branch counters over every block
     * pair (ZCCLd_float.c:2184-2246 and the tail and remainder copies):
     * both widths 0, first 0, second 0, neither; ADDED to the four ints
     * (ZCCLd_float.c:2759-2765), from device counters of the same add. */
    unsigned long long cases[4] = {0, 0, 0, 0};
    const int rc = dropin_homadd(final_cmpBytes, final_cmpSize, nbEle, absErrBound, blockSize, cmpBytes, cmpBytes2,
                                 omp_threads(), cases);
    if (rc == ZCCL_GPU_OK) {
        int *const dst[4] = {total_counter_1, total_counter_2, total_counter_3, total_counter_4};
        for (int k = 0; k < 4; k++)
            if (dst[k]) *dst[k] += (int)cases[k];
    }
    report(__func__, rc);
}

/* ---- SZp 3-D codec ---------------------------------------------------- */

extern "C" size_t zccl_gpu_szp3d_max_bytes(size_t d1, size_t d2, size_t d3, int bs)
{
    return sz3_args_ok(d1, d2, d3, bs, 1.0) ? sz3_max_stream_bytes(d1, d2, d3, (uint32_t)bs) : 0;
}

extern "C" size_t zccl_gpu_szp3d_workspace_bytes(size_t d1, size_t d2, size_t d3, int bs)
{
    return sz3_args_ok(d1, d2, d3, bs, 1.0) ? sz3_workspace_bytes(d1, d2, d3, (uint32_t)bs, true) : 0;
}

extern "C" int zccl_gpu_szp3d_compress(unsigned char *d_out, size_t capacity, const float *d_in, size_t d1,
                                       size_t d2, size_t d3, int bs, double eb, void *d_ws, size_t *d_size,
                                       void *cuda_stream)
{
    if (!d_out || !d_in || !d_ws || !sz3_args_ok(d1, d2, d3, bs, eb)) return ZCCL_GPU_EINVAL;
    const cudaError_t e = sz3_compress(d_out, capacity, d_in, d1, d2, d3, (uint32_t)bs, eb, d_ws,
                                       reinterpret_cast<uint64_t *>(d_size), (cudaStream_t)cuda_stream);
    return e == cudaSuccess ? ZCCL_GPU_OK : e == cudaErrorInvalidValue ? ZCCL_GPU_ECAPACITY : ZCCL_GPU_ECUDA;
}

extern "C" int zccl_gpu_szp3d_decompress(float *d_out, const unsigned char *d_in, size_t avail, size_t d1,
                                         size_t d2, size_t d3, int bs, double eb, void *d_ws, void *cuda_stream)
{
    if (!d_out || !d_in || !d_ws || !sz3_args_ok(d1, d2, d3, bs, eb)) return ZCCL_GPU_EINVAL;
    return cuda_status(sz3_decompress(d_out, d_in, avail, d1, d2, d3, (uint32_t)bs, eb, d_ws,
                                      (cudaStream_t)cuda_stream));
}

extern "C" void SZp_compress3D_fast(const float *oriData, unsigned char *cmpData, size_t dim1, size_t dim2,
                                    size_t dim3, int blockSideLength, double errorBound, size_t *cmpSize)
{
    report(__func__, dropin_szp3d_compress(oriData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound,
                                           cmpSize));
}

extern "C" void SZp_compress3D(const float *oriData, unsigned char *cmpData, size_t dim1, size_t dim2,
                               size_t dim3, int blockSideLength, double errorBound, size_t *cmpSize)
{
    report(__func__, dropin_szp3d_compress(oriData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound,
                                           cmpSize));
}

extern "C" void SZp_decompress3D(float *decData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                                 int blockSideLength, double errorBound)
{
    report(__func__, dropin_szp3d_decompress(decData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound));
}

extern "C" void SZp_decompress3D_fast(float *decData, unsigned char *cmpData, size_t dim1, size_t dim2,
                                      size_t dim3, int blockSideLength, double errorBound)
{
    report(__func__, dropin_szp3d_decompress(decData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound));
}

extern "C" void SZp_compress3D_fast_openmp(const float *oriData, unsigned char *cmpData, size_t dim1, size_t dim2,
                                           size_t dim3, int blockSideLength, double errorBound, size_t *cmpSize)
{
    report(__func__, dropin_szp3d_compress_split(oriData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound,
                                                 cmpSize, omp_threads()));
}

extern "C" void SZp_decompress3D_fast_openmp(float *decData, unsigned char *cmpData, size_t dim1, size_t dim2,
                                             size_t dim3, int blockSideLength, double errorBound)
{
    report(__func__, dropin_szp3d_decompress_split(decData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound,
                                                   omp_threads()));
}

extern "C" size_t zccl_gpu_szp3d_split_max_bytes(size_t d1, size_t d2, size_t d3, int bs, int T)
{
    Sz3Split3 sp;
    if (!sz3_args_ok(d1, d2, d3, bs, 1.0) || T < 1 || !sz3_split_plan(d1, d2, d3, (uint32_t)T, &sp)) return 0;
    return sz3_split_max_stream_bytes(sp, (uint32_t)bs);
}

extern "C" size_t zccl_gpu_szp3d_split_workspace_bytes(size_t d1, size_t d2, size_t d3, int bs, int T)
{
    Sz3Split3 sp;
    if (!sz3_args_ok(d1, d2, d3, bs, 1.0) || T < 1 || !sz3_split_plan(d1, d2, d3, (uint32_t)T, &sp)) return 0;
    return std::max(sz3_split_workspace_bytes(sp, (uint32_t)bs, true), sz3_split_workspace_bytes(sp, (uint32_t)bs, false));
}

extern "C" int zccl_gpu_szp3d_compress_split(unsigned char *d_out, size_t capacity, const float *d_in, size_t d1,
                                             size_t d2, size_t d3, int bs, double eb, int T, void *d_ws, size_t *d_size,
                                             void *cuda_stream)
{
    Sz3Split3 sp;
    if (!d_out || !d_in || !d_ws || !sz3_args_ok(d1, d2, d3, bs, eb) || T < 1 ||
        !sz3_split_plan(d1, d2, d3, (uint32_t)T, &sp))
        return ZCCL_GPU_EINVAL;
    const cudaError_t e = sz3_split_compress(d_out, capacity, d_in, sp, (uint32_t)bs, eb, d_ws,
                                             reinterpret_cast<uint64_t *>(d_size), (cudaStream_t)cuda_stream);
    return e == cudaSuccess ? ZCCL_GPU_OK : e == cudaErrorInvalidValue ? ZCCL_GPU_ECAPACITY : ZCCL_GPU_ECUDA;
}

extern "C" int zccl_gpu_szp3d_decompress_split(float *d_out, const unsigned char *d_in, size_t avail, size_t d1,
                                               size_t d2, size_t d3, int bs, double eb, int T, void *d_ws,
                                               void *cuda_stream)
{
    Sz3Split3 sp;
    if (!d_out || !d_in || !d_ws || !sz3_args_ok(d1, d2, d3, bs, eb) || T < 1 ||
        !sz3_split_plan(d1, d2, d3, (uint32_t)T, &sp) || avail < 8ull * (size_t)T)
        return ZCCL_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    std::vector<uint64_t> offs((size_t)T);
    if (cudaMemcpyAsync(offs.data(), d_in, 8ull * (size_t)T, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ZCCL_GPU_ECUDA;
    const cudaError_t e = sz3_split_decompress(d_out, d_in, avail, offs.data(), sp, (uint32_t)bs, eb, d_ws, st);
    return e == cudaSuccess ? ZCCL_GPU_OK : e == cudaErrorInvalidValue ? ZCCL_GPU_EBOUNDS : ZCCL_GPU_ECUDA;
}

/* ---- the fixed-rate appendix codec ------------------------------------ */

extern "C" void ZCCL_float_openmp_threadblock_arg_2(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                                    float absErrBound, size_t nbEle, int blockSize)
{
    report(__func__, dropin_compress(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize, omp_threads(),
                                     ZG_FIXED_BYTES));
}

extern "C" void ZCCL_float_decompress_openmp_threadblock_arg_2(float *newData, size_t nbEle, float absErrBound,
                                                               int blockSize, unsigned char *cmpBytes)
{
    report(__func__,
           dropin_decompress(newData, nbEle, absErrBound, blockSize, cmpBytes, omp_threads(), ZG_FIXED_BYTES));
}
