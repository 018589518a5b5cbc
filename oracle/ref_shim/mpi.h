/*
  Single-rank stand-in for <mpi.h>, used only to compile the reference
  TMR octree core (TMROctant.cpp, TMROctForest.cpp, TMRBase.cpp,
  TMR_STLTools.cpp) as a CPU checker.  It is test infrastructure: nothing in the tmr_gb300 product
  links it.

  Semantics: the communicator has exactly one rank (rank 0, size 1).
  Collectives copy the send buffer to the receive buffer.  The reference
  never posts a point-to-point message to its own rank (TMROctForest.cpp
  sendOctants: sends/recvs are skipped for i == mpi_rank), so Isend/Recv
  are never reached with a single rank and report an error if they are.

  A datatype is represented by its extent in bytes.
*/
#ifndef TMRG_REF_SHIM_MPI_H
#define TMRG_REF_SHIM_MPI_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef long MPI_Datatype;
typedef long MPI_Aint;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;
typedef int MPI_Op;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_COMM_SELF ((MPI_Comm)0)
#define MPI_SUCCESS 0
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT32_T ((MPI_Datatype)4)
#define MPI_INT16_T ((MPI_Datatype)2)
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_SUM ((MPI_Op)0)
#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)
#define MPI_IN_PLACE ((void *)1)

static inline int MPI_Comm_rank(MPI_Comm, int *r) {
  *r = 0;
  return 0;
}
static inline int MPI_Comm_size(MPI_Comm, int *s) {
  *s = 1;
  return 0;
}
static inline int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r,
                                int, MPI_Datatype, MPI_Comm) {
  if (s != MPI_IN_PLACE) memmove(r, s, (size_t)n * (size_t)t);
  return 0;
}
static inline int MPI_Alltoall(const void *s, int n, MPI_Datatype t, void *r,
                               int, MPI_Datatype, MPI_Comm) {
  memmove(r, s, (size_t)n * (size_t)t);
  return 0;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t,
                                MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) memmove(r, s, (size_t)n * (size_t)t);
  return 0;
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int,
                            MPI_Comm, MPI_Request *) {
  fprintf(stderr, "mpi shim: Isend on a single rank\n");
  abort();
}
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm,
                           MPI_Status *) {
  fprintf(stderr, "mpi shim: Recv on a single rank\n");
  abort();
}
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Type_create_struct(int n, const int *counts,
                                         const MPI_Aint *offsets,
                                         const MPI_Datatype *types,
                                         MPI_Datatype *out) {
  long ext = 0;
  for (int i = 0; i < n; i++) {
    long e = (long)offsets[i] + (long)counts[i] * (long)types[i];
    if (e > ext) ext = e;
  }
  *out = (MPI_Datatype)ext;
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
static inline int MPI_Type_free(MPI_Datatype *) { return 0; }
static inline double MPI_Wtime() { return 0.0; }
static inline int MPI_Gatherv(const void *s, int n, MPI_Datatype t, void *r, const int *,
                              const int *displs, MPI_Datatype, int, MPI_Comm) {
  memmove((char *)r + (size_t)displs[0] * (size_t)t, s, (size_t)n * (size_t)t);
  return 0;
}

/* MPI-IO on one rank: a stdio file; a view's displacement is where the
   next collective write lands. */
typedef struct {
  FILE *fp;
  long disp;
  MPI_Datatype etype;
} TMRG_MPI_File;
typedef TMRG_MPI_File *MPI_File;
typedef int MPI_Info;
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
static inline int MPI_File_open(MPI_Comm, const char *name, int, MPI_Info, MPI_File *f) {
  FILE *fp = fopen(name, "wb");
  if (!fp) {
    *f = 0;
    return 1;
  }
  *f = (MPI_File)calloc(1, sizeof(TMRG_MPI_File));
  (*f)->fp = fp;
  return 0;
}
static inline int MPI_File_write(MPI_File f, const void *b, int n, MPI_Datatype t,
                                 MPI_Status *) {
  fwrite(b, (size_t)t, (size_t)n, f->fp);
  return 0;
}
static inline int MPI_File_set_view(MPI_File f, long disp, MPI_Datatype etype, MPI_Datatype,
                                    const char *, MPI_Info) {
  f->disp = disp;
  f->etype = etype;
  return 0;
}
static inline int MPI_File_write_at_all(MPI_File f, long off, const void *b, int n,
                                        MPI_Datatype t, MPI_Status *) {
  fseek(f->fp, f->disp + off * (long)f->etype, SEEK_SET);
  fwrite(b, (size_t)t, (size_t)n, f->fp);
  return 0;
}
static inline int MPI_File_close(MPI_File *f) {
  fclose((*f)->fp);
  free(*f);
  *f = 0;
  return 0;
}

#endif
