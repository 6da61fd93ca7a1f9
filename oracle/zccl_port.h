/*
 * zccl_port.h -- CPU restatement of ZCCL's fastmode1 float32 codec.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: tests/ use it as the
 * checker and bench.py times it as the CPU baseline.  The GPU product never
 * links, loads or calls it.
 *
 * The thread count T is explicit here (the reference takes it implicitly from
 * the OpenMP runtime); T fixes the stream layout, see zccl_port.c.
 */
#ifndef ZCCL_PORT_H
#define ZCCL_PORT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Compress nbEle floats into out (8*T-byte chunk-offset header followed by T
 * chunks); *outSize is assigned.  Follows ZCCL/src/ZCCL_float.c:501-807. */
void port_compress(unsigned char *out, const float *in, size_t *outSize, float absErrBound,
                   size_t nbEle, int blockSize, int T);

/* Decompress a stream written with the same T.  ZCCL/src/ZCCLd_float.c:538-754. */
void port_decompress(float *out, size_t nbEle, float absErrBound, int blockSize,
                     const unsigned char *cmp, int T);

/* The same two with the block magnitude layout `fmt`: 0 is fastmode1, 1
 * the fixed-rate appendix codec (ZCCL_float_openmp_threadblock_arg_2 and
 * ZCCL_float_decompress_openmp_threadblock_arg_2, ZCCL/src/ZCCL_appendix.c:65-590),
 * whose blocks keep b/8 + 1 (at most 4) whole little-endian bytes per
 * magnitude and no low-bit stream; everything else is fastmode1's. */
void port_compress_f(unsigned char *out, const float *in, size_t *outSize, float absErrBound,
                     size_t nbEle, int blockSize, int T, int fmt);
void port_decompress_f(float *out, size_t nbEle, float absErrBound, int blockSize,
                       const unsigned char *cmp, int T, int fmt);

/* Homomorphic add of two streams (same nbEle, eb, L, T).  *outSize is
 * INCREMENTED, like the reference (ZCCL/src/ZCCLd_float.c:1027,1655).
 * out may alias cmp2.  ZCCL/src/ZCCLd_float.c:988-1679. */
void port_homadd(unsigned char *out, size_t *outSize, size_t nbEle, float absErrBound,
                 int blockSize, const unsigned char *cmp1, const unsigned char *cmp2, int T);

/* Width of a block whose largest delta magnitude is m, with the host libm:
 * 0 when m == 0, else (int)log2f((float)m) + 1 (ZCCL/src/ZCCL_float.c:606). */
int port_width(uint32_t m);

/* SZp 3-D codec, serial form: compress a dim1 x dim2 x dim3 volume (dim3
 * fastest) in blocks of bs^3 with absolute error bound eb; *cmpSize is
 * assigned.  ZCCL/src/ZCCL_float.c:1706-1860 (SZp_compress3D_fast and
 * SZp_compress3D write the same stream). */
void port_szp3d_compress(const float *x, unsigned char *out, size_t d1, size_t d2, size_t d3, int bs,
                         double eb, size_t *cmpSize);

/* Its inverse, ZCCL/src/ZCCLd_float.c:2801-2871 (SZp_decompress3D). */
void port_szp3d_decompress(float *y, const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs,
                           double eb);

/* The same codec in its OpenMP form (SZp_compress3D_fast_openmp,
 * ZCCL/src/ZCCL_float.c:1862-2048, and SZp_decompress3D_fast_openmp,
 * ZCCL/src/ZCCLd_float.c:2873-3034) for T threads: T size_t offsets, then
 * the serial-form stream of each thread's sub-volume; port_dims3 is the
 * thread grid, My_Dims_create(T, 3, {0,0,0}) (ZCCL/src/ZCCL_multidim.c:100). */
void port_dims3(int n, int d[3]);
void port_szp3d_compress_split(const float *x, unsigned char *out, size_t d1, size_t d2, size_t d3, int bs,
                               double eb, int T, size_t *cmpSize);
void port_szp3d_decompress_split(float *y, const unsigned char *cmp, size_t d1, size_t d2, size_t d3, int bs,
                                 double eb, int T);

/* The counts of the reference's _record variants, from a stream.  For a
 * T = 1 stream of nbEle floats: the memory-access counts returned by
 * ZCCL_float_single_thread_arg_record (ZCCL/src/ZCCL_float.c:990-1209)
 * when it wrote the stream, and by
 * ZCCL_float_decompress_single_thread_arg_record
 * (ZCCL/src/ZCCLd_float.c:376-536) when it reads it. */
void port_record_counts(const unsigned char *cmp, size_t nbEle, int blockSize, size_t *compress_count,
                        size_t *decompress_count);

/* The four branch counters that
 * ZCCL_float_homomophic_add_openmp_threadblock_record
 * (ZCCL/src/ZCCLd_float.c:2067-2800) adds up for two streams written with T
 * threads: both widths 0, first 0, second 0, neither. */
void port_homadd_cases(const unsigned char *cmp1, const unsigned char *cmp2, size_t nbEle, int blockSize, int T,
                       unsigned long long counts[4]);

#ifdef __cplusplus
}
#endif
#endif
