/* Link-time stubs for the symbols the reference codec files reference from
 * the MPI side: My_Dims_create (ZCCL/src/ZCCL_multidim.c:100), called only by
 * the OpenMP 3-D SZp codec, and the MPI calls of the appendix file's
 * allgather variants (ZCCL/src/ZCCL_appendix.c:591-941).  The oracle never
 * calls any of them; the MPI stubs abort if it ever did. */
#include <stdlib.h>
void My_Dims_create(int nnodes, int ndims, int dims[])
{
    int i;
    for (i = 0; i < ndims; i++) dims[i] = 1;
    if (ndims > 0) dims[0] = nnodes;
}

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
