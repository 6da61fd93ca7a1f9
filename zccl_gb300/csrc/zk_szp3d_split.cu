/*
 * zk_szp3d_split.cu -- the SZp 3-D codec in its OpenMP form.
 *
 * SZp_compress3D_fast_openmp (ZCCL/src/ZCCL_float.c:1862-2048) and
 * SZp_decompress3D_fast_openmp (ZCCL/src/ZCCLd_float.c:2873-3034) split the
 * volume among T OpenMP threads: My_Dims_create (ZCCL/src/ZCCL_multidim.c:
 * 100-140) factors T into a tdims[0] x tdims[1] x tdims[2] grid of
 * sub-volumes (each axis cut into near-equal parts, the first `rem` parts
 * one plane longer), thread r takes sub-volume r in x-major order and
 * encodes it exactly as the serial codec encodes a volume of that shape
 * (Lorenzo state starts at zero at the sub-volume's faces), and the stream
 * is T little-endian size_t offsets, relative to their end, followed by the
 * T serial-form streams in thread order.
 *
 * Here the sub-volumes run one after another through the serial-form
 * kernels (zk_szp3d.cu) on the caller's stream: compression gathers a
 * sub-volume into contiguous scratch, encodes it, and appends the stream at
 * the running offset, which a one-CTA kernel reads from the sizes in device
 * memory (no host synchronization); decompression reads the offsets once,
 * decodes each sub-stream into scratch and scatters it into the volume.
 */
#include "zkern.cuh"

namespace {

/* dst[i][j][k] = src[o0 + i][o1 + j][o2 + k] (gather, a sub-volume out of a
 * d2 x d3-plane volume) or the reverse (scatter); one row of the sub-volume
 * per blockIdx.x step, threads along k, coalesced on both sides. */
template <bool GATHER>
__global__ void k_sub_copy(float *vol, float *sub, uint64_t d2, uint64_t d3, uint64_t o0, uint64_t o1, uint64_t o2,
                           uint64_t s0, uint64_t s1, uint64_t s2)
{
    for (uint64_t row = blockIdx.x; row < s0 * s1; row += gridDim.x) {
        const uint64_t i = row / s1, j = row - i * s1;
        float *v = vol + ((o0 + i) * d2 + o1 + j) * d3 + o2;
        float *s = sub + row * s2;
        for (uint64_t k = threadIdx.x; k < s2; k += blockDim.x) {
            if (GATHER)
                s[k] = v[k];
            else
                v[k] = s[k];
        }
    }
}

/* Sub-stream r of T, `sizes[r]` bytes in scratch `src`, goes to its place
 * in the stream: its offset (the sum of the sizes before it) into header
 * entry r, its bytes after the header at that offset.  After the last one,
 * *total = the stream's size.  A stream that would not fit `cap` sets
 * ZERR_CAPACITY and is not written. */
__global__ void k_append(uint8_t *out, uint64_t cap, const uint8_t *src, const uint64_t *sizes, uint32_t r,
                         uint32_t T, uint64_t *total, uint32_t *err)
{
    uint64_t off = 0;
    for (uint32_t u = 0; u < r; u++) off += sizes[u];
    const uint64_t n = sizes[r], base = 8ull * T + off;
    if (base + n > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ZERR_CAPACITY);
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x < 8) out[8ull * r + threadIdx.x] = (uint8_t)(off >> (8 * threadIdx.x));
    if (blockIdx.x == 0 && threadIdx.x == 0 && r + 1 == T && total) *total = base + n;
    /* slices of 64 KiB per CTA, each stored with 16-byte vector stores
     * realigned to the destination (src is 256-byte aligned with slack) */
    const uint64_t slice = 65536;
    for (uint64_t s0 = (uint64_t)blockIdx.x * slice; s0 < n; s0 += (uint64_t)gridDim.x * slice) {
        const uint32_t len = (uint32_t)(n - s0 < slice ? n - s0 : slice);
        store_realign(out + base + s0, src + s0, len, threadIdx.x, blockDim.x);
    }
}

unsigned sms()
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return nsm > 0 ? (unsigned)nsm : 1u;
}

unsigned rows_grid(uint64_t rows)
{
    const uint64_t cap = 8ull * sms();
    return (unsigned)(rows < 1 ? 1 : (rows > cap ? cap : rows));
}

size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

/* Workspace: the serial codec's scratch for the largest sub-volume (its
 * first 16 bytes are the status words) | sizes[T] | one sub-volume of
 * floats | (compression) one sub-stream. */
struct SplitWs {
    void *serial;
    uint64_t *sizes;
    float *sub;
    uint8_t *stream;
    size_t stream_cap, total;
};

SplitWs split_ws(void *ws, const Sz3Split3 &sp, uint32_t bs, bool compress)
{
    uint64_t s[3];
    sz3_split_extent(sp, 0, s); /* sub-volume 0 is the largest on every axis */
    SplitWs w;
    uint8_t *p = static_cast<uint8_t *>(ws);
    size_t o = a256(sz3_workspace_bytes(s[0], s[1], s[2], bs, compress));
    w.serial = p;
    w.sizes = reinterpret_cast<uint64_t *>(p + o);
    o = a256(o + 8ull * sp.T);
    w.sub = reinterpret_cast<float *>(p + o);
    o = a256(o + 4ull * s[0] * s[1] * s[2]);
    w.stream = p + o;
    w.stream_cap = compress ? sz3_max_stream_bytes(s[0], s[1], s[2], bs) : 0;
    o = a256(o + w.stream_cap + 64);
    w.total = o;
    return w;
}

} // namespace

/* My_Dims_create(T, 3, {0, 0, 0}) (ZCCL/src/ZCCL_multidim.c:100-140): the
 * prime factors of T, largest first, each multiplied into the currently
 * smallest axis (the first of equals), the three counts then sorted
 * descending. */
bool sz3_split_plan(uint64_t d1, uint64_t d2, uint64_t d3, uint32_t T, Sz3Split3 *sp)
{
    if (T < 1 || T > 65536) return false;
    uint32_t f[64], nf = 0, d[3] = {1, 1, 1};
    for (uint32_t i = 2, rem = T; i <= rem; i++)
        while (rem % i == 0) {
            f[nf++] = i;
            rem /= i;
        }
    for (uint32_t a = 0; a < nf; a++) /* descending */
        for (uint32_t b = a + 1; b < nf; b++)
            if (f[b] > f[a]) {
                const uint32_t t = f[a];
                f[a] = f[b];
                f[b] = t;
            }
    for (uint32_t i = 0; i < nf; i++) {
        uint32_t m = 0;
        for (uint32_t j = 1; j < 3; j++)
            if (d[j] < d[m]) m = j;
        d[m] *= f[i];
    }
    for (uint32_t a = 0; a < 3; a++)
        for (uint32_t b = a + 1; b < 3; b++)
            if (d[b] > d[a]) {
                const uint32_t t = d[a];
                d[a] = d[b];
                d[b] = t;
            }
    const uint64_t dim[3] = {d1, d2, d3};
    sp->T = T;
    for (int a = 0; a < 3; a++) {
        sp->parts[a] = d[a];
        sp->dim[a] = dim[a];
        /* the reference needs every sub-volume non-empty */
        if (dim[a] < d[a]) return false;
    }
    return true;
}

/* Origin and extent of sub-volume r (x-major thread order,
 * ZCCL_float.c:1904-1933). */
void sz3_split_origin(const Sz3Split3 &sp, uint32_t r, uint64_t o[3], uint64_t s[3])
{
    uint32_t c[3];
    c[0] = r / (sp.parts[1] * sp.parts[2]);
    c[1] = (r / sp.parts[2]) % sp.parts[1];
    c[2] = r % sp.parts[2];
    for (int a = 0; a < 3; a++) {
        const uint64_t base = sp.dim[a] / sp.parts[a], rem = sp.dim[a] % sp.parts[a];
        o[a] = c[a] * base + (c[a] < rem ? c[a] : rem);
        s[a] = base + (c[a] < rem ? 1u : 0u);
    }
}

void sz3_split_extent(const Sz3Split3 &sp, uint32_t r, uint64_t s[3])
{
    uint64_t o[3];
    sz3_split_origin(sp, r, o, s);
}

size_t sz3_split_max_stream_bytes(const Sz3Split3 &sp, uint32_t bs)
{
    size_t total = 8ull * sp.T;
    for (uint32_t r = 0; r < sp.T; r++) {
        uint64_t s[3];
        sz3_split_extent(sp, r, s);
        total += sz3_max_stream_bytes(s[0], s[1], s[2], bs);
    }
    return total;
}

size_t sz3_split_workspace_bytes(const Sz3Split3 &sp, uint32_t bs, bool compress)
{
    return split_ws(nullptr, sp, bs, compress).total;
}

cudaError_t sz3_split_compress(uint8_t *out, uint64_t cap, const float *x, const Sz3Split3 &sp, uint32_t bs, double eb,
                               void *ws, uint64_t *d_size, cudaStream_t st)
{
    const SplitWs w = split_ws(ws, sp, bs, true);
    if (cap < 8ull * sp.T) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(w.sizes, 0, 8ull * sp.T, st);
    if (e != cudaSuccess) return e;
    uint32_t *err = static_cast<uint32_t *>(w.serial); /* the serial codec's status words */
    for (uint32_t r = 0; r < sp.T; r++) {
        uint64_t o[3], s[3];
        sz3_split_origin(sp, r, o, s);
        k_sub_copy<true><<<rows_grid(s[0] * s[1]), 256, 0, st>>>(const_cast<float *>(x), w.sub, sp.dim[1], sp.dim[2],
                                                                 o[0], o[1], o[2], s[0], s[1], s[2]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = sz3_compress(w.stream, w.stream_cap, w.sub, s[0], s[1], s[2], bs, eb, w.serial, w.sizes + r, st)) !=
            cudaSuccess)
            return e;
        const uint64_t slices = (w.stream_cap + 65535) / 65536;
        k_append<<<(unsigned)(slices < 4ull * sms() ? (slices ? slices : 1) : 4ull * sms()), 256, 0, st>>>(
            out, cap, w.stream, w.sizes, r, sp.T, d_size, err);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t sz3_split_decompress(float *y, const uint8_t *in, uint64_t avail, const uint64_t *offs, const Sz3Split3 &sp,
                                 uint32_t bs, double eb, void *ws, cudaStream_t st)
{
    const SplitWs w = split_ws(ws, sp, bs, false);
    const uint64_t hdr = 8ull * sp.T;
    for (uint32_t r = 0; r < sp.T; r++) {
        uint64_t o[3], s[3];
        sz3_split_origin(sp, r, o, s);
        const uint64_t off = offs[r];
        if (off > avail - hdr) return cudaErrorInvalidValue; /* avail >= hdr is checked by the caller */
        cudaError_t e = sz3_decompress(w.sub, in + hdr + off, avail - hdr - off, s[0], s[1], s[2], bs, eb, w.serial, st);
        if (e != cudaSuccess) return e;
        k_sub_copy<false><<<rows_grid(s[0] * s[1]), 256, 0, st>>>(y, w.sub, sp.dim[1], sp.dim[2], o[0], o[1], o[2], s[0],
                                                                  s[1], s[2]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}
