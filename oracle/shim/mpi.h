/* Types-only stand-in for <mpi.h>, used solely to compile the reference codec
 * sources into the oracle library.  The codec files include the MPI header
 * through ZCCL.h but call no MPI function on the compress / decompress /
 * homomorphic-add path; the MPI functions that the appendix file's allgather
 * variants call are link-time stubs (ref_stubs.c). */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H
typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef int MPI_Request;
typedef int MPI_Win;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_WIN_NULL 0
#define MPI_COMM_NULL 0
/* constants the appendix codec file (ZCCL/src/ZCCL_appendix.c) names in its
 * allgather functions, which the oracle never calls */
#define MPI_SUCCESS 0
#define MPI_INT 1
#define MPI_BYTE 2
/* and those the 3-D decomposition file (ZCCL/src/ZCCL_multidim.c) names in
 * its scatter helpers; the oracle only calls its My_Dims_create */
#define MPI_FLOAT 3
#define MPI_ORDER_C 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#endif
