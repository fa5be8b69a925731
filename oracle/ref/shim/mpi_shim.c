/*
 * Single-rank MPI stand-in (see mpi.h for the contract). TEST INFRASTRUCTURE ONLY.
 *
 * Derived datatypes are kept in a small table. A datatype describes a list of
 * byte runs (offset, length) relative to the buffer start; packing walks the
 * runs in order, which is the MPI type-map order.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "mpi.h"

#define EIF_MAX_TYPES 4096

typedef struct {
  int in_use;
  int basic_size;          /* > 0 for predefined types */
  int count, blocklength;  /* hvector parameters */
  MPI_Aint stride;
  MPI_Datatype oldtype;
} eif_type_t;

static eif_type_t eif_types[EIF_MAX_TYPES] = {
  [MPI_BYTE] = {1, 1, 0, 0, 0, 0},
  [MPI_INT] = {1, (int)sizeof(int), 0, 0, 0, 0},
  [MPI_DOUBLE] = {1, (int)sizeof(double), 0, 0, 0, 0},
};

static const eif_type_t *type_of(MPI_Datatype t){
  if(t <= 0 || t >= EIF_MAX_TYPES || !eif_types[t].in_use){
    fprintf(stderr, "mpi shim: invalid datatype %d\n", t);
    abort();
  }
  return &eif_types[t];
}

/* number of payload bytes one element of the type carries */
static size_t type_size(MPI_Datatype t){
  const eif_type_t *d = type_of(t);
  if(d->basic_size > 0) return (size_t)d->basic_size;
  return (size_t)d->count*(size_t)d->blocklength*type_size(d->oldtype);
}

/* distance between consecutive elements in a contiguous block (lb = 0 for all types used here) */
static MPI_Aint type_extent(MPI_Datatype t){
  const eif_type_t *d = type_of(t);
  if(d->basic_size > 0) return d->basic_size;
  if(d->count == 0) return 0;
  return (MPI_Aint)(d->count-1)*d->stride+(MPI_Aint)d->blocklength*type_extent(d->oldtype);
}

/* copy one element of type t between a typed buffer and a packed stream */
static void walk(MPI_Datatype t, char *typed, char **packed, int to_packed){
  const eif_type_t *d = type_of(t);
  if(d->basic_size > 0){
    if(to_packed) memcpy(*packed, typed, (size_t)d->basic_size);
    else memcpy(typed, *packed, (size_t)d->basic_size);
    *packed += d->basic_size;
    return;
  }
  const MPI_Aint ext = type_extent(d->oldtype);
  for(int k = 0; k < d->count; k++){
    for(int b = 0; b < d->blocklength; b++){
      walk(d->oldtype, typed+k*d->stride+b*ext, packed, to_packed);
    }
  }
}

int MPI_Init(int *argc, char ***argv){ (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void){ return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm comm, int errorcode){ (void)comm; fprintf(stderr, "MPI_Abort(%d)\n", errorcode); exit(1); }
int MPI_Comm_size(MPI_Comm comm, int *size){ (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank){ (void)comm; *rank = 0; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm comm){ (void)comm; return MPI_SUCCESS; }

double MPI_Wtime(void){
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec+1.e-9*(double)ts.tv_nsec;
}

int MPI_Bcast(void *buffer, int count, MPI_Datatype datatype, int root, MPI_Comm comm){
  (void)buffer; (void)count; (void)datatype; (void)root; (void)comm;
  return MPI_SUCCESS;
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype datatype, MPI_Op op, MPI_Comm comm){
  (void)op; (void)comm;
  if(sendbuf != MPI_IN_PLACE){
    memmove(recvbuf, sendbuf, (size_t)count*type_size(datatype));
  }
  return MPI_SUCCESS;
}

int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status){
  (void)dest; (void)sendtag; (void)source; (void)recvtag; (void)comm; (void)status;
  size_t ns = (size_t)sendcount*type_size(sendtype);
  size_t nr = (size_t)recvcount*type_size(recvtype);
  memmove(recvbuf, sendbuf, ns < nr ? ns : nr);
  return MPI_SUCCESS;
}

int MPI_Type_create_hvector(int count, int blocklength, MPI_Aint stride, MPI_Datatype oldtype, MPI_Datatype *newtype){
  for(int t = MPI_DOUBLE+1; t < EIF_MAX_TYPES; t++){
    if(!eif_types[t].in_use){
      eif_types[t] = (eif_type_t){1, 0, count, blocklength, stride, oldtype};
      *newtype = t;
      return MPI_SUCCESS;
    }
  }
  fprintf(stderr, "mpi shim: datatype table full\n");
  abort();
}

int MPI_Type_commit(MPI_Datatype *datatype){ (void)type_of(*datatype); return MPI_SUCCESS; }

int MPI_Type_free(MPI_Datatype *datatype){
  if(*datatype > MPI_DOUBLE && *datatype < EIF_MAX_TYPES) eif_types[*datatype].in_use = 0;
  *datatype = 0;
  return MPI_SUCCESS;
}

int MPI_Alltoallw(const void *sendbuf, const int sendcounts[], const int sdispls[], const MPI_Datatype sendtypes[],
                  void *recvbuf, const int recvcounts[], const int rdispls[], const MPI_Datatype recvtypes[],
                  MPI_Comm comm){
  (void)comm;
  /* one peer (ourselves): pack with the send type, unpack with the receive type */
  size_t nbytes = (size_t)sendcounts[0]*type_size(sendtypes[0]);
  size_t rbytes = (size_t)recvcounts[0]*type_size(recvtypes[0]);
  if(nbytes != rbytes){
    fprintf(stderr, "mpi shim: Alltoallw size mismatch %zu vs %zu\n", nbytes, rbytes);
    abort();
  }
  char *stream = malloc(nbytes > 0 ? nbytes : 1);
  char *cur = stream;
  for(int e = 0; e < sendcounts[0]; e++){
    walk(sendtypes[0], (char *)sendbuf+sdispls[0]+e*type_extent(sendtypes[0]), &cur, 1);
  }
  cur = stream;
  for(int e = 0; e < recvcounts[0]; e++){
    walk(recvtypes[0], (char *)recvbuf+rdispls[0]+e*type_extent(recvtypes[0]), &cur, 0);
  }
  free(stream);
  return MPI_SUCCESS;
}

int MPI_Error_string(int errorcode, char *string, int *resultlen){
  *resultlen = snprintf(string, MPI_MAX_ERROR_STRING, "mpi shim error %d", errorcode);
  return MPI_SUCCESS;
}

struct eif_mpi_file_ { FILE *fp; };

int MPI_File_open(MPI_Comm comm, const char *filename, int amode, MPI_Info info, MPI_File *fh){
  (void)comm; (void)info;
  FILE *fp = fopen(filename, (amode & MPI_MODE_RDONLY) ? "rb" : "r+b");
  if(fp == NULL) return MPI_ERR_FILE;
  *fh = malloc(sizeof(struct eif_mpi_file_));
  (*fh)->fp = fp;
  return MPI_SUCCESS;
}

int MPI_File_close(MPI_File *fh){
  if(*fh){ fclose((*fh)->fp); free(*fh); *fh = NULL; }
  return MPI_SUCCESS;
}

int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void *buf, int count, MPI_Datatype datatype, MPI_Status *status){
  (void)status;
  fseek(fh->fp, (long)offset, SEEK_SET);
  size_t n = (size_t)count*type_size(datatype);
  return fread(buf, 1, n, fh->fp) == n ? MPI_SUCCESS : MPI_ERR_FILE;
}

int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void *buf, int count, MPI_Datatype datatype, MPI_Status *status){
  (void)status;
  fseek(fh->fp, (long)offset, SEEK_SET);
  size_t n = (size_t)count*type_size(datatype);
  return fwrite(buf, 1, n, fh->fp) == n ? MPI_SUCCESS : MPI_ERR_FILE;
}
