/*
 * zkern.cuh -- kernel argument blocks and launchers (internal interface
 * between the C-ABI layer and the kernels).
 */
#ifndef ZCCL_GB300_ZKERN_CUH
#define ZCCL_GB300_ZKERN_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "zdev.cuh"
#include "zgeom.h"

#define ZH_MAXP 32 /* most inputs one homomorphic-add launch accepts */

/* Per-call scratch in device memory, zeroed before every launch:
 * err | ticket | pad | status[ntiles]. */
struct ZWork {
    uint32_t *err;    /* ZERR_* bits */
    uint32_t *ticket; /* next tile to hand out */
    uint64_t *status; /* decoupled look-back state, one word per tile */
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

struct CompressArgs {
    const float *x;
    uint8_t *out;
    uint64_t cap; /* writable bytes at `out` */
    ZGeom g;
    float inv; /* 1.0f / eb, computed on the host in float */
    ZIndex idx;
    ZWork w;
    ZWidthTable wt;
    ZSmem sm;
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
};

struct HomInput {
    const uint8_t *bytes;
    uint64_t avail;
    const uint8_t *widths;
    const uint64_t *tile_off;
    const int32_t *tile_qprev;
};

struct HomAddArgs {
    HomInput in[ZH_MAXP];
    uint32_t P;
    int qprev_valid;       /* every input's tile_qprev is valid */
    uint8_t *out;
    uint64_t cap;          /* writable bytes at `out` */
    ZIndex idx;            /* index of the output stream */
    unsigned long long *cases; /* optional [4]: both zero, first zero, second zero, both non-zero (P == 2) */
    ZGeom g;
    ZWork w;
    ZWidthTable wt;
    ZSmem sm;
};

struct WalkArgs {
    const uint8_t *in;
    uint64_t avail;
    ZGeom g;
    ZIndex idx;
    uint32_t *err;
};

/* Launchers; each returns the cudaError_t of the launch. */
cudaError_t launch_compress(const CompressArgs &a, cudaStream_t st);
cudaError_t launch_decompress(const DecompressArgs &a, cudaStream_t st);
cudaError_t launch_homadd(const HomAddArgs &a, cudaStream_t st);
cudaError_t launch_walk(const WalkArgs &a, cudaStream_t st);

#endif
