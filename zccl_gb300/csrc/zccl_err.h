/*
 * zccl_err.h -- device error bits and host status codes.
 *
 * Kernels never trap: they OR one of the ZERR_* bits into an error word in
 * the workspace and keep going with bounded work; the host reads the word
 * after the launch and turns it into a status code.
 */
#ifndef ZCCL_GB300_ZERR_H
#define ZCCL_GB300_ZERR_H

#define ZERR_RANGE 0x1u   /* input not finite or |x/eb| >= 2^31 (undefined in the reference) */
#define ZERR_TIMEOUT 0x2u /* a bounded wait gave up */
#define ZERR_CORRUPT 0x4u /* stream bytes disagree with its geometry or index */
#define ZERR_BOUNDS 0x8u  /* a read would pass the end of the stream buffer */
#define ZERR_CAPACITY 0x10u /* the output stream does not fit its buffer */

#endif
