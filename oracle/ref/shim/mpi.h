/*
 * Single-rank stand-in for the subset of MPI that the reference solver calls.
 *
 * TEST INFRASTRUCTURE ONLY: this header exists so that the reference's own,
 * unmodified C sources can be compiled into the CPU oracle library
 * (oracle/_ref/). It is never linked into the GPU product.
 *
 * Semantics are those of an MPI job with exactly one rank:
 *   - Comm_size = 1, Comm_rank = 0;
 *   - reductions with MPI_IN_PLACE leave the buffer unchanged;
 *   - Sendrecv to oneself copies the send buffer into the receive buffer
 *     (this is the periodic y-halo exchange, src/parallel/halo.c:7-31);
 *   - Alltoallw with one peer packs the send buffer with the send datatype and
 *     unpacks it with the receive datatype (the x<->y pencil transpose,
 *     src/parallel/transpose.c:6-96);
 *   - MPI-IO maps onto stdio at explicit byte offsets (src/fileio.c:186-281).
 */
#if !defined(EIF_SHIM_MPI_H)
#define EIF_SHIM_MPI_H

#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef ptrdiff_t MPI_Aint;
typedef long long MPI_Offset;
typedef struct eif_mpi_status_ { int source, tag, error; } MPI_Status;
typedef struct eif_mpi_file_ *MPI_File;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_SUCCESS 0
#define MPI_ERR_FILE 27
#define MPI_MAX_ERROR_STRING 256

/* predefined datatypes: handle values index the shim's datatype table */
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)2)
#define MPI_DOUBLE ((MPI_Datatype)3)

#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)

#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_APPEND 128

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buffer, int count, MPI_Datatype datatype, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status);
int MPI_Type_create_hvector(int count, int blocklength, MPI_Aint stride, MPI_Datatype oldtype, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *datatype);
int MPI_Type_free(MPI_Datatype *datatype);
int MPI_Alltoallw(const void *sendbuf, const int sendcounts[], const int sdispls[], const MPI_Datatype sendtypes[],
                  void *recvbuf, const int recvcounts[], const int rdispls[], const MPI_Datatype recvtypes[],
                  MPI_Comm comm);
int MPI_Error_string(int errorcode, char *string, int *resultlen);
int MPI_File_open(MPI_Comm comm, const char *filename, int amode, MPI_Info info, MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void *buf, int count, MPI_Datatype datatype, MPI_Status *status);
int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void *buf, int count, MPI_Datatype datatype, MPI_Status *status);

#endif
