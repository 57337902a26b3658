/* mpi.h -- single-rank stand-in for the MPI calls made by the reference's
 * src_cpp_kokkos_host/{mpi_config,boundary}.cpp.  Test infrastructure for the oracle build only.
 * With ntiles = {1,1,1} the reference never sends or receives; the two MINLOC/MAXLOC
 * allreduces are identities on one rank.  Any point-to-point call aborts. */
#ifndef ORACLE_REFSHIM_MPI_H_
#define ORACLE_REFSHIM_MPI_H_

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_COMM_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_DOUBLE_INT 3
#define MPI_MINLOC 1
#define MPI_MAXLOC 2
#define MPI_SUM 3

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm *out) { *out = 2; return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, const int *, const int *, int, MPI_Comm *out) {
  *out = 3;
  return 0;
}
static inline int MPI_Cart_shift(MPI_Comm, int, int, int *lo, int *hi) {
  *lo = MPI_PROC_NULL;
  *hi = MPI_PROC_NULL;
  return 0;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int n, int *c) {
  for (int i = 0; i < n; i++) c[i] = 0;
  return 0;
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime(void) { return 0.0; }
static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  size_t sz = (t == MPI_DOUBLE_INT) ? 16 : (t == MPI_DOUBLE ? sizeof(double) : sizeof(int));
  memcpy(out, in, sz * (size_t)count);
  return 0;
}
static inline int MPI_Irecv(void *, size_t, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  fprintf(stderr, "refshim: MPI_Irecv is not available on one rank\n");
  abort();
}
static inline int MPI_Isend(const void *, size_t, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  fprintf(stderr, "refshim: MPI_Isend is not available on one rank\n");
  abort();
}
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }

/* MPI-IO as src_cpp_kokkos_host/output.cpp uses it, for one rank: every subarray view covers the
 * whole file (sizes == subsizes, starts == 0, checked), so a collective write is a plain write at
 * the view's displacement.  MPI_File_open does not truncate, as MPI does not. */
typedef long long MPI_Offset;
typedef int MPI_Info;
typedef FILE *MPI_File;
#define MPI_INFO_NULL 0
#define MPI_DATATYPE_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_ORDER_C 56
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4

static inline int MPI_Type_create_subarray(int ndims, const int *sizes, const int *subsizes, const int *starts, int,
                                           MPI_Datatype, MPI_Datatype *newtype) {
  for (int d = 0; d < ndims; d++)
    if (sizes[d] != subsizes[d] || starts[d] != 0) {
      fprintf(stderr, "refshim: a one-rank subarray must cover the whole array\n");
      abort();
    }
  *newtype = 100 + ndims;
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
static inline int MPI_File_open(MPI_Comm, const char *name, int, MPI_Info, MPI_File *fh) {
  *fh = fopen(name, "r+b");
  if (!*fh) *fh = fopen(name, "w+b");
  return *fh ? 0 : 1;
}
static inline int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype, MPI_Datatype, const char *, MPI_Info) {
  return fh && fseek(fh, (long)disp, SEEK_SET) == 0 ? 0 : 1;
}
static inline int MPI_File_write_all(MPI_File fh, const void *buf, MPI_Offset count, MPI_Datatype t, MPI_Status *) {
  const size_t sz = t == MPI_DOUBLE ? sizeof(double) : sizeof(int);
  return fh && fwrite(buf, sz, (size_t)count, fh) == (size_t)count ? 0 : 1;
}
static inline int MPI_File_close(MPI_File *fh) {
  if (*fh) fclose(*fh);
  *fh = 0;
  return 0;
}

#endif
