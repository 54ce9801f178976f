/*
 * Single-rank MPI stand-in used only to compile the reference's own sources
 * into the CPU oracle (test infrastructure; never linked into the product).
 *
 * With one rank every point-to-point exchange list the reference builds is
 * empty, so Isend/Irecv/Wait* are never reached with work to do; Allreduce
 * of one rank is the identity (a copy).  Datatypes are encoded as their
 * element size in bytes so the copy length is count * datatype.  MPI-IO
 * maps to stdio at the view's byte displacement.
 */
#ifndef BCM_ORACLE_MPI_STUB_H
#define BCM_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <string.h>
#include <sys/types.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef FILE *MPI_File;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_INFO_NULL 0
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_MODE_RDWR 8
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t,
                                MPI_Op, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * (size_t)t);
  return 0;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm,
                            MPI_Request *q) { *q = 0; return 0; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm,
                            MPI_Request *q) { *q = 0; return 0; }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitany(int, MPI_Request *, int *i, MPI_Status *) {
  *i = 0; return 0;
}
static inline int MPI_Type_vector(int, int, int, MPI_Datatype o, MPI_Datatype *n) {
  *n = o; return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
/* MPI-IO of one rank: a FILE* positioned by set_view's displacement, so the
 * reference's writers (BCM_Output.cpp) produce their real files. */
static inline int MPI_File_open(MPI_Comm, const char *path, int amode, MPI_Info, MPI_File *f) {
  *f = fopen(path, (amode & (MPI_MODE_WRONLY | MPI_MODE_RDWR)) ? "r+b" : "rb");
  if (!*f && (amode & MPI_MODE_CREATE)) *f = fopen(path, "w+b");
  return *f ? 0 : 1;
}
static inline int MPI_File_close(MPI_File *f) {
  if (*f) fclose(*f);
  *f = 0;
  return 0;
}
static inline int MPI_File_set_view(MPI_File f, MPI_Offset disp, MPI_Datatype, MPI_Datatype,
                                    const char *, MPI_Info) {
  return f ? fseeko(f, (off_t)disp, SEEK_SET) : 1;
}
static inline int MPI_File_read(MPI_File f, void *buf, int n, MPI_Datatype t, MPI_Status *) {
  return f && fread(buf, (size_t)t, (size_t)n, f) == (size_t)n ? 0 : 1;
}
static inline int MPI_File_write(MPI_File f, const void *buf, int n, MPI_Datatype t,
                                 MPI_Status *) {
  return f && fwrite(buf, (size_t)t, (size_t)n, f) == (size_t)n ? 0 : 1;
}

#endif
