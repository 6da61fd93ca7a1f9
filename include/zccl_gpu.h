/*
 * zccl_gpu.h -- C ABI of the GB300 implementation of ZCCL's fastmode1
 * compression hot path (compress, decompress, homomorphic add).
 *
 * Two layers:
 *
 * 1. Drop-in replacements.  Same names, signatures, argument meaning and
 *    byte layout as the reference's OpenMP codec, so a caller relinks
 *    against libzccl_gpu.so instead of libZCCL.  Pointers may be host memory
 *    (copied through the GPU) or device memory (used in place).  Calls are
 *    synchronous and return void like the reference; the outcome of the last
 *    call on the calling thread is available from zccl_gpu_last_status().
 *    The writer thread count T that fixes the stream layout is taken the way
 *    the reference takes it: omp_get_max_threads() for the *_openmp_*
 *    functions, 1 for the *_single_thread* ones.
 *
 * 2. The device API (zccl_gpu_*).  Explicit T, device pointers, a CUDA
 *    stream, status codes, and a side index kept next to every resident
 *    stream so decompression and homomorphic add never have to walk the
 *    1-byte block headers.  Calls are asynchronous on the given stream.
 */
#ifndef ZCCL_GPU_H
#define ZCCL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ===================================================================
 * 1. Drop-in replacements of the reference entry points
 * =================================================================== */

/* Replaces ZCCL_float_openmp_threadblock_arg, declared at
 * ZCCL/include/ZCCL_float.h:31 and defined at ZCCL/src/ZCCL_float.c:501.
 * Compresses nbEle floats into outputBytes and ASSIGNS *outSize.  As with
 * the reference, outputBytes must hold the whole stream; every reference
 * caller allocates 4*nbEle bytes. */
void ZCCL_float_openmp_threadblock_arg(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                       float absErrBound, size_t nbEle, int blockSize);

/* Replaces ZCCL_float_single_thread_arg (ZCCL/include/ZCCL_float.h:34,
 * ZCCL/src/ZCCL_float.c:809): the same stream with T = 1. */
void ZCCL_float_single_thread_arg(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                  float absErrBound, size_t nbEle, int blockSize);

/* Replaces ZCCL_float_decompress_openmp_threadblock_arg
 * (ZCCL/include/ZCCLd_float.h:21, ZCCL/src/ZCCLd_float.c:538).  The stream
 * carries no length; with a host pointer, cmpBytes must be readable for
 * min(4*nbEle, largest possible stream) bytes, the capacity every reference
 * caller gives its stream buffers (a stream longer than 4*nbEle -- tiny
 * arrays, or blocks near 32 bits wide -- must be readable up to its largest
 * possible size, zccl_gpu_max_stream_bytes()); with a device pointer, up to
 * the end of its allocation. */
void ZCCL_float_decompress_openmp_threadblock_arg(float *newData, size_t nbEle, float absErrBound,
                                                  int blockSize, unsigned char *cmpBytes);

/* Replaces ZCCL_float_decompress_single_thread_arg
 * (ZCCL/include/ZCCLd_float.h:23, ZCCL/src/ZCCLd_float.c:247), T = 1. */
void ZCCL_float_decompress_single_thread_arg(float *newData, size_t nbEle, float absErrBound,
                                             int blockSize, unsigned char *cmpBytes);

/* Replaces ZCCL_float_homomophic_add_openmp_threadblock (the reference's
 * spelling), ZCCL/include/ZCCLd_float.h:29, ZCCL/src/ZCCLd_float.c:988.
 * final_cmpBytes may alias cmpBytes2 (the ring allreduce adds in place,
 * ZCCL/src/ZCCL_ring_ho.c:281-287).  *final_cmpSize is INCREMENTED by the
 * result size, like the reference (ZCCLd_float.c:1027,1655); callers zero
 * it first. */
void ZCCL_float_homomophic_add_openmp_threadblock(unsigned char *final_cmpBytes,
                                                  size_t *final_cmpSize, size_t nbEle,
                                                  float absErrBound, int blockSize,
                                                  unsigned char *cmpBytes,
                                                  unsigned char *cmpBytes2);

/* Replaces ZCCL_float_homomophic_add_single_thread
 * (ZCCL/include/ZCCLd_float.h:33, ZCCL/src/ZCCLd_float.c:1681), T = 1. */
void ZCCL_float_homomophic_add_single_thread(unsigned char *final_cmpBytes, size_t *final_cmpSize,
                                             size_t nbEle, float absErrBound, int blockSize,
                                             unsigned char *cmpBytes, unsigned char *cmpBytes2);

/* Replaces ZCCL_float_openmp_threadblock (ZCCL/include/ZCCL_float.h:27-29,
 * ZCCL/src/ZCCL_float.c:192-499): compresses into a buffer it mallocs,
 * which the caller frees with free(); ASSIGNS *outSize; NULL on failure.
 * The stream is ZCCL_float_openmp_threadblock_arg's.  Where N % T != 0 the
 * reference packs the remainder segment's tail block with the regular
 * segments' tail count (ZCCL_float.c:452,456) -- a stream its decompressor
 * cannot read back whenever the two counts differ; here that block has its
 * own count, so both variants write the same bytes. */
unsigned char *ZCCL_float_openmp_threadblock(float *oriData, size_t *outSize, float absErrBound, size_t nbEle,
                                             int blockSize);

/* Replaces ZCCL_float_decompress_openmp_threadblock
 * (ZCCL/include/ZCCLd_float.h:19, ZCCL/src/ZCCLd_float.c:22-245):
 * *newData = malloc(4 * nbEle) (the caller frees it, also after a failed
 * call), then decompressed like the _arg variant. */
void ZCCL_float_decompress_openmp_threadblock(float **newData, size_t nbEle, float absErrBound, int blockSize,
                                              unsigned char *cmpBytes);

/* Replaces ZCCL_float_single_thread_arg_record
 * (ZCCL/include/ZCCL_float.h:36-37, ZCCL/src/ZCCL_float.c:990-1209): the
 * T = 1 stream, and the value the reference returns -- its own count of the
 * bytes its scalar code reads and writes while producing that stream (12
 * per element, each block's bytes plus 8 per element of a non-zero-width
 * block, the chunk copied out twice, 76 of bookkeeping).  The count is a
 * function of the stream, computed from it here; it does not measure the
 * GPU's memory traffic.  0 on failure. */
size_t ZCCL_float_single_thread_arg_record(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                           float absErrBound, size_t nbEle, int blockSize);

/* Replaces ZCCL_float_decompress_single_thread_arg_record
 * (ZCCL/include/ZCCLd_float.h:25, ZCCL/src/ZCCLd_float.c:376-536): T = 1
 * decompression, returning the reference's count for it (each block's
 * bytes, 8 per element of a zero-width block, 20 per element of any other,
 * 24 of bookkeeping), computed from the stream.  0 on failure. */
size_t ZCCL_float_decompress_single_thread_arg_record(float *newData, size_t nbEle, float absErrBound,
                                                      int blockSize, unsigned char *cmpBytes);

/* Replaces ZCCL_float_single_thread_arg_split_record
 * (ZCCL/include/ZCCL_float.h:45-52, ZCCL/src/ZCCL_float.c:1530-1705), which
 * the split allreduce calls once per chunk (ZCCL/src/ZCCL_ring.c:1496,1510):
 * the T = 1 stream into outputBytes, *outSize assigned, and the same size
 * stored as the size_t at index chunk_iter of chunk_arr (host or device
 * memory, any alignment). */
void ZCCL_float_single_thread_arg_split_record(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                               float absErrBound, size_t nbEle, int blockSize,
                                               unsigned char *chunk_arr, size_t chunk_iter);

/* Replaces ZCCL_float_homomophic_add_openmp_threadblock_record
 * (ZCCL/include/ZCCLd_float.h:31, ZCCL/src/ZCCLd_float.c:2067-2800): the
 * homomorphic add, and the reference's four branch counters over every
 * block pair ADDED to the ints: counter_1 both widths 0, counter_2 only the
 * first 0, counter_3 only the second 0, counter_4 neither (the device
 * counters of zccl_gpu_homadd_cases). */
void ZCCL_float_homomophic_add_openmp_threadblock_record(unsigned char *final_cmpBytes, size_t *final_cmpSize,
                                                         size_t nbEle, float absErrBound, int blockSize,
                                                         unsigned char *cmpBytes, unsigned char *cmpBytes2,
                                                         int *total_counter_1, int *total_counter_2,
                                                         int *total_counter_3, int *total_counter_4);

/* ===================================================================
 * 2. Device API
 * =================================================================== */

#define ZCCL_GPU_OK 0
#define ZCCL_GPU_EINVAL (-1)    /* bad arguments: n < T, L outside 1..256, null pointers */
#define ZCCL_GPU_ECUDA (-2)     /* a CUDA runtime call failed */
#define ZCCL_GPU_ERANGE (-3)    /* input not finite, or |x / eb| >= 2^31 */
#define ZCCL_GPU_ECORRUPT (-4)  /* stream bytes disagree with its geometry or index */
#define ZCCL_GPU_EBOUNDS (-5)   /* stream runs past its readable bytes */
#define ZCCL_GPU_ETIMEOUT (-6)  /* a bounded device wait gave up */
#define ZCCL_GPU_ENOMEM (-7)    /* device or host allocation failed */
#define ZCCL_GPU_ECAPACITY (-8) /* destination buffer too small */
#define ZCCL_GPU_ESCRATCH (-9)  /* input needs more than the fixed scratch array holds */

/* A compressed stream resident in device memory. */
typedef struct zccl_gpu_stream {
    unsigned char *bytes; /* device: wire bytes in the reference layout */
    size_t capacity;      /* bytes readable (and writable) at `bytes` */
    void *index;          /* device: side index, zccl_gpu_index_bytes() bytes */
    int indexed;          /* index holds block widths and tile offsets */
    int qprev_valid;      /* index holds the quantized value before each tile */
} zccl_gpu_stream;

/* Largest stream of n floats (every block at width 32). */
size_t zccl_gpu_max_stream_bytes(size_t n, int L, int T);
/* Bytes of the side index of one stream (about n/L + 12 per 8192 floats). */
size_t zccl_gpu_index_bytes(size_t n, int L, int T);
/* Bytes of device scratch one call needs (look-back state, error word, and
 * for streams that arrive without an index the header walk's tables, about
 * one byte per byte of the largest stream of this geometry).
 * Its first 8 bytes are two status words: zero them once when the
 * workspace is allocated.  Every call leaves them alone (it zeroes only its
 * own look-back state) and ORs the errors it detects into them, so the
 * errors of every call on a workspace since the last zccl_gpu_check() are
 * reported by that check, which then clears them. */
size_t zccl_gpu_workspace_bytes(size_t n, int L, int T);

/* Compress n device floats into out->bytes and fill out's index.
 * Enqueued on cuda_stream; the size is read with zccl_gpu_stream_size(). */
int zccl_gpu_compress(zccl_gpu_stream *out, const float *d_in, size_t n, float eb, int L, int T,
                      void *d_ws, void *cuda_stream);

/* Decompress into n device floats.  Builds the index first when
 * in->indexed is 0; recovers and stores the tile starting values when
 * in->qprev_valid is 0. */
int zccl_gpu_decompress(float *d_out, zccl_gpu_stream *in, size_t n, float eb, int L, int T,
                        void *d_ws, void *cuda_stream);

/* Homomorphic sum of P streams (same n, L, T, eb) into out, in one pass.
 * out->bytes must not alias any input.  Inputs without an index get one. */
int zccl_gpu_homadd(zccl_gpu_stream *out, zccl_gpu_stream *ins, int P, size_t n, int L, int T,
                    void *d_ws, void *cuda_stream);

/* Same, also accumulating the reference's four branch counters of a
 * two-input add (both zero, first zero, second zero, both non-zero,
 * ZCCL/src/ZCCLd_float.c:2175-2764) into d_cases[4] (device uint64). */
int zccl_gpu_homadd_cases(zccl_gpu_stream *out, zccl_gpu_stream *ins, int P, size_t n, int L,
                          int T, void *d_ws, unsigned long long *d_cases, void *cuda_stream);

/* Bytes of the fixed device scratch array zccl_gpu_compress_noalloc uses. */
#define ZCCL_GPU_NOALLOC_SCRATCH_BYTES (1u << 20)

/* zccl_gpu_compress without a workspace argument and without allocating any
 * memory; it has no counterpart in the reference.  It is for callers that
 * cannot allocate device memory while they compress: a collective's step
 * loop, where cudaMalloc or cudaFree can synchronize the whole device and
 * stall kernels that other ranks are waiting on, or a process whose device
 * memory is already held by a caching pool, where a fresh allocation fails.
 *
 * The scratch is a 1 MiB array (ZCCL_GPU_NOALLOC_SCRATCH_BYTES) inside this
 * library's device code, one per device.  A call needs 16 + 8 * tiles bytes
 * of it, a tile being up to 256 blocks of one segment (8192 floats at
 * L = 32), so n may reach about 1.07e9 floats at L = 32 and T = 1; fewer
 * with smaller L or many segments.  Larger inputs return ZCCL_GPU_ESCRATCH and
 * launch nothing.  Those bytes must be zero when the kernel starts; the
 * call clears them itself on cuda_stream.
 *
 * The first call with a device current looks up the array's address on that
 * device, a one-time setup; make it before any stream capture begins.  All
 * calls on a device share the one array: two calls whose work overlaps in
 * time (different streams or host threads) race on it, so order them, for
 * example by issuing them on one stream.  The output, status and size are
 * those of zccl_gpu_compress.  When d_scratch is not NULL and the call
 * returns ZCCL_GPU_OK it receives the array's address (else NULL), which
 * zccl_gpu_check() takes to read the device status of the calls made since
 * the last check.  The address is looked up once per device and kept, so
 * the library does not support cudaDeviceReset() between calls. */
int zccl_gpu_compress_noalloc(zccl_gpu_stream *out, const float *d_in, size_t n, float eb, int L,
                              int T, void *cuda_stream, void **d_scratch);

/* Decompress and add: d_acc[i] = d_acc[i] + x'[i] for the n floats x' of
 * the stream, each sum rounded once -- the float sum MPI_Reduce_local forms
 * in the decompress-add-recompress allreduce's reduce step
 * (ZCCL/src/ZCCL_ring.c:1074-1076), in one pass without a buffer of
 * decompressed floats.  The stream must be indexed with its tile starting
 * values (in->indexed and in->qprev_valid, as compression and sums leave
 * it); no counterpart function in the reference. */
int zccl_gpu_decompress_accumulate(float *d_acc, const zccl_gpu_stream *in, size_t n, float eb, int L, int T,
                                   void *d_ws, void *cuda_stream);

/* Build the side index of a stream that arrived as bytes only. */
int zccl_gpu_build_index(zccl_gpu_stream *s, size_t n, int L, int T, void *d_ws, void *cuda_stream);

/* Synchronize cuda_stream and return the total stream bytes of s. */
int zccl_gpu_stream_size(const zccl_gpu_stream *s, size_t n, int L, int T, size_t *size,
                         void *cuda_stream);

/* ---- the fixed-rate appendix codec --------------------------------------
 * ZCCL/src/ZCCL_appendix.c:65-590: fastmode1's stream with every block's
 * magnitudes stored as b/8 + 1 (at most 4) whole little-endian bytes and no
 * low-bit stream.  Same arguments, pointers and threading as the fastmode1
 * drop-ins above (declared with the same signatures at
 * ZCCL/include/ZCCL_appendix.h:12-24).  The reference's compressor gives the remainder segment's tail
 * block the regular segments' tail count (ZCCL_appendix.c:318-330), which
 * its own decompressor does not read back when the two counts differ; here
 * that block has its own count, the layout the decompressor reads. */
void ZCCL_float_openmp_threadblock_arg_2(unsigned char *outputBytes, float *oriData, size_t *outSize,
                                         float absErrBound, size_t nbEle, int blockSize);
void ZCCL_float_decompress_openmp_threadblock_arg_2(float *newData, size_t nbEle, float absErrBound,
                                                    int blockSize, unsigned char *cmpBytes);
/* Device API for streams in that layout (arguments as zccl_gpu_compress /
 * zccl_gpu_decompress; the descriptor does not record the layout, so a
 * stream is always read with the call of its writer's layout). */
int zccl_gpu_compress_fixed(zccl_gpu_stream *out, const float *d_in, size_t n, float eb, int L, int T,
                            void *d_ws, void *cuda_stream);
int zccl_gpu_decompress_fixed(float *d_out, zccl_gpu_stream *in, size_t n, float eb, int L, int T,
                              void *d_ws, void *cuda_stream);

/* ---- SZp 3-D codec, serial stream form --------------------------------
 * Drop-ins for the reference's serial 3-D Lorenzo codec: a dim1 x dim2 x
 * dim3 float volume (dim3 fastest) in blocks of blockSideLength^3 (1..32)
 * with absolute error bound errorBound; the stream is one rate byte per
 * block followed by the blocks' sign and fixed-length bits.  Host or device
 * pointers, synchronous, status in zccl_gpu_last_status().
 *   SZp_compress3D_fast   ZCCL/include/ZCCL_float.h:83-86  (ZCCL/src/ZCCL_float.c:1706)
 *   SZp_compress3D        ZCCL/include/ZCCL_float.h:88-91  (ZCCL/src/ZCCL_float.c:1791), same stream
 *   SZp_decompress3D      ZCCL/include/ZCCLd_float.h:40-43 (ZCCL/src/ZCCLd_float.c:2801)
 *   SZp_decompress3D_fast ZCCL/include/ZCCLd_float.h:35-38 (declared there, defined nowhere in the
 *                         reference; here the inverse of SZp_compress3D_fast, i.e. SZp_decompress3D) */
void SZp_compress3D_fast(const float *oriData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                         int blockSideLength, double errorBound, size_t *cmpSize);
void SZp_compress3D(const float *oriData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                    int blockSideLength, double errorBound, size_t *cmpSize);
void SZp_decompress3D(float *decData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                      int blockSideLength, double errorBound);
void SZp_decompress3D_fast(float *decData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                           int blockSideLength, double errorBound);

/* ---- SZp 3-D codec, OpenMP stream form --------------------------------
 * Drop-ins for SZp_compress3D_fast_openmp (ZCCL/include/ZCCL_float.h:98-101,
 * ZCCL/src/ZCCL_float.c:1862) and SZp_decompress3D_fast_openmp
 * (ZCCL/include/ZCCLd_float.h:45-48, ZCCL/src/ZCCLd_float.c:2873), which the
 * 3-D allgatherv calls (ZCCL/src/ZCCL_ring.c:2084,2174).  With T =
 * omp_get_max_threads() the volume is split into a grid of T sub-volumes
 * (My_Dims_create's factorisation of T, ZCCL/src/ZCCL_multidim.c:100-140);
 * the stream is T size_t offsets followed by each sub-volume's serial-form
 * stream.  Every axis must have at least as many planes as it has parts
 * (the reference needs the same), else ZCCL_GPU_EINVAL. */
void SZp_compress3D_fast_openmp(const float *oriData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                                int blockSideLength, double errorBound, size_t *cmpSize);
void SZp_decompress3D_fast_openmp(float *decData, unsigned char *cmpData, size_t dim1, size_t dim2, size_t dim3,
                                  int blockSideLength, double errorBound);

/* Device API of the OpenMP form with T explicit: largest stream, scratch
 * (its first 16 bytes are the status words zccl_gpu_check() reads), and the
 * two passes on cuda_stream.  compress writes the stream size to the device
 * size_t at d_size when it is not null; decompress reads the T offsets
 * (one synchronization) and needs `avail` readable bytes at d_in. */
size_t zccl_gpu_szp3d_split_max_bytes(size_t d1, size_t d2, size_t d3, int bs, int T);
size_t zccl_gpu_szp3d_split_workspace_bytes(size_t d1, size_t d2, size_t d3, int bs, int T);
int zccl_gpu_szp3d_compress_split(unsigned char *d_out, size_t capacity, const float *d_in, size_t d1, size_t d2,
                                  size_t d3, int bs, double eb, int T, void *d_ws, size_t *d_size, void *cuda_stream);
int zccl_gpu_szp3d_decompress_split(float *d_out, const unsigned char *d_in, size_t avail, size_t d1, size_t d2,
                                    size_t d3, int bs, double eb, int T, void *d_ws, void *cuda_stream);

/* Device API of the same codec: the largest stream, device scratch (the
 * first 16 bytes hold the status words zccl_gpu_check() reads), and the two
 * passes enqueued on cuda_stream.  compress writes the stream size to the
 * device size_t at d_size when it is not null; capacity too small for the
 * rate table gives ZCCL_GPU_ECAPACITY, too small for the payload a device
 * status of the same code. */
size_t zccl_gpu_szp3d_max_bytes(size_t d1, size_t d2, size_t d3, int bs);
size_t zccl_gpu_szp3d_workspace_bytes(size_t d1, size_t d2, size_t d3, int bs);
int zccl_gpu_szp3d_compress(unsigned char *d_out, size_t capacity, const float *d_in, size_t d1, size_t d2,
                            size_t d3, int bs, double eb, void *d_ws, size_t *d_size, void *cuda_stream);
int zccl_gpu_szp3d_decompress(float *d_out, const unsigned char *d_in, size_t avail, size_t d1, size_t d2,
                              size_t d3, int bs, double eb, void *d_ws, void *cuda_stream);

/* Segment framing of the segmented ring allgatherv
 * (MPIR_Allgatherv_intra_ring_RI2_mt_oa_record_seg, ZCCL/src/ZCCL_ring.c:1599-1774):
 * a compressed segment travels as its size (size_t, little-endian) followed by
 * its stream bytes (ZCCL_ring.c:1672-1673).  Enqueues on cuda_stream a device
 * copy of s's total size, once s has been produced on that stream, into the
 * 8 bytes at d_frame; no synchronization. */
int zccl_gpu_frame_size(const zccl_gpu_stream *s, void *d_frame, void *cuda_stream);

/* Synchronize cuda_stream and turn the workspace's device error bits into a
 * status code (ZCCL_GPU_OK when none), then clear them.  The bits are those
 * of every call on the workspace since the previous check; a failed header
 * walk also makes later calls on the workspace stop early until checked. */
int zccl_gpu_check(void *d_ws, void *cuda_stream);

/* -------------------------------------------------------------------
 * Batches: thousands of streams in one persistent launch.  No counterpart
 * in the reference, whose callers compress one buffer per call.
 *
 * A batch is planned once (tables built on the host and copied into the
 * caller's device memory, synchronously) and then run any number of times
 * with one memset and one kernel launch on the given stream -- no host
 * copies, so a run can be recorded into a CUDA graph.  All jobs of a batch
 * share L; n, T and (for compression) eb are per job.  Every stream keeps
 * the reference's byte layout and gets its side index as with the calls
 * above.  Sums take P indexed input streams of one geometry (for example
 * the outputs of a compression batch that ran before).
 * ------------------------------------------------------------------- */
#define ZCCL_GPU_BATCH_COMPRESS 0
#define ZCCL_GPU_BATCH_HOMADD 1
#define ZCCL_GPU_BATCH_DECOMPRESS 2

typedef struct zccl_gpu_batch_job {
    const float *d_in;    /* compression: n device floats */
    zccl_gpu_stream *ins; /* sum: P indexed input streams; decompression: the stream (P = 1),
                             indexed with its tile starting values (qprev_valid) */
    int P;                /* sum: number of inputs (1..32) */
    size_t n;             /* floats of the buffer */
    float eb;             /* compression, decompression: absolute error bound */
    int T;                /* writer thread count of the stream layout */
    zccl_gpu_stream *out; /* compression, sum: output stream (capacity >= zccl_gpu_max_stream_bytes) */
    float *d_out;         /* decompression: n device floats */
    int accumulate;       /* decompression: add the floats to d_out[] instead of storing them */
} zccl_gpu_batch_job;

typedef struct zccl_gpu_batch {
    int kind;         /* ZCCL_GPU_BATCH_COMPRESS, _HOMADD or _DECOMPRESS */
    int L;            /* block size of every job */
    unsigned grid;    /* CTAs per launch, 0 = as many as fit; set by zccl_gpu_batch_tune() */
    size_t njobs;     /* jobs in the batch */
    size_t ntiles;    /* tiles of all jobs */
    void *d_mem;      /* the caller's device memory, zccl_gpu_batch_bytes() bytes */
    size_t clear_bytes; /* leading bytes of d_mem zeroed before every run */
    size_t jobs_off, map_off, tile0_off; /* tables inside d_mem */
    unsigned tb;      /* blocks per tile */
    unsigned smem[6]; /* shared-memory layout of the launch */
    int qprev_valid;  /* sums: every input carries its tile starting values */
    size_t rows_off;  /* compress: the jobs' tensor maps inside d_mem, 0 = none */
} zccl_gpu_batch;

/* Device bytes a batch of these jobs needs (0 if a job is invalid). */
size_t zccl_gpu_batch_bytes(int kind, const zccl_gpu_batch_job *jobs, size_t njobs, int L);

/* Plan a batch into d_mem (bytes from zccl_gpu_batch_bytes); synchronous.
 * The output streams are marked indexed. */
int zccl_gpu_batch_plan(zccl_gpu_batch *b, int kind, const zccl_gpu_batch_job *jobs, size_t njobs,
                        int L, void *d_mem, size_t bytes, void *cuda_stream);

/* Run a planned batch on cuda_stream (asynchronous). */
int zccl_gpu_batch_run(const zccl_gpu_batch *b, void *cuda_stream);

/* The autotuner: time a few launch shapes of this batch on cuda_stream
 * (running it several times) and keep the fastest in b->grid. */
int zccl_gpu_batch_tune(zccl_gpu_batch *b, void *cuda_stream);

/* Synchronize cuda_stream and return the batch's device status (the errors
 * of every run since the plan or the previous check), then clear it. */
int zccl_gpu_batch_check(const zccl_gpu_batch *b, void *cuda_stream);

/* Status of the last drop-in call made by this thread. */
int zccl_gpu_last_status(void);

/* Text for a status code. */
const char *zccl_gpu_strerror(int status);

/* The width threshold table in use: thr[w] (w = 0..32) is the smallest
 * integer of bit length w whose (int)log2f((float)m) + 1 is w + 1 with this
 * host's libm, or 0xFFFFFFFF.  Fills 33 entries. */
void zccl_gpu_width_table(uint32_t thr[33]);

#ifdef __cplusplus
}
#endif
#endif
