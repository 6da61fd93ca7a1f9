/* Link-time stubs for the MPI calls that the reference codec files make
 * outside the codec: the allgather variants of the appendix file
 * (ZCCL/src/ZCCL_appendix.c:591-941) and the scatter helpers of the 3-D
 * decomposition file (ZCCL/src/ZCCL_multidim.c:13-95), whose My_Dims_create
 * the OpenMP SZp 3-D codec calls.  The oracle never calls any of them; they
 * abort if it ever did. */
#include <stdlib.h>

#define ORACLE_NO_MPI(name) \
    int name() { abort(); }
ORACLE_NO_MPI(MPI_Allgather)
ORACLE_NO_MPI(MPI_Comm_rank)
ORACLE_NO_MPI(MPI_Comm_size)
ORACLE_NO_MPI(MPI_Irecv)
ORACLE_NO_MPI(MPI_Isend)
ORACLE_NO_MPI(MPI_Recv)
ORACLE_NO_MPI(MPI_Send)
ORACLE_NO_MPI(MPI_Sendrecv)
ORACLE_NO_MPI(MPI_Test)
ORACLE_NO_MPI(MPI_Wait)
ORACLE_NO_MPI(MPI_Waitall)
ORACLE_NO_MPI(MPI_Cart_coords)
ORACLE_NO_MPI(MPI_Type_create_subarray)
ORACLE_NO_MPI(MPI_Type_commit)
ORACLE_NO_MPI(MPI_Type_free)
