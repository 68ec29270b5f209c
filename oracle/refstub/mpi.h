/* Single-rank MPI stand-in used only to compile the reference solver's own
 * hot-path sources into the CPU oracle harness (oracle/_ref). Every
 * collective is a copy of the send buffer into the receive buffer, every
 * point-to-point call is a no-op: with one rank there is never a peer.
 * This file is test infrastructure, not part of the GPU product. */
#ifndef ORACLE_SINGLE_RANK_MPI_H
#define ORACLE_SINGLE_RANK_MPI_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_File;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_SIZE 3
#define MPI_SUCCESS 0
#define MPI_MODE_WRONLY 1
#define MPI_MODE_RDONLY 2
#define MPI_MODE_CREATE 4
#define MPI_IN_PLACE ((void*)1)

/* The datatype value is its size in bytes, which is all a copy needs. */
#define MPI_CXX_BOOL ((MPI_Datatype)sizeof(bool))
#define MPI_LOGICAL ((MPI_Datatype)sizeof(bool))
#define MPI_INTEGER ((MPI_Datatype)sizeof(int))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_DOUBLE_PRECISION ((MPI_Datatype)sizeof(double))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_CHARACTER ((MPI_Datatype)sizeof(char))
#define MPI_CHAR ((MPI_Datatype)sizeof(char))

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int ostub_copy_(const void* s, void* r, int n, MPI_Datatype t) {
  if (s != MPI_IN_PLACE && s != r && n > 0) memcpy(r, s, (size_t)n * (size_t)t);
  return 0;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { return ostub_copy_(s, r, n, t); }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) { return ostub_copy_(s, r, n, t); }
static inline int MPI_Scan(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { return ostub_copy_(s, r, n, t); }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) { return ostub_copy_(s, r, n, t); }
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) { return ostub_copy_(s, r, n, t); }
static inline int MPI_Allgatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int* d, MPI_Datatype, MPI_Comm) {
  return ostub_copy_(s, (char*)r + (size_t)d[0] * (size_t)t, n, t);
}
static inline int MPI_Gatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int* d, MPI_Datatype, int, MPI_Comm) {
  return ostub_copy_(s, (char*)r + (size_t)d[0] * (size_t)t, n, t);
}
static inline int MPI_Scatterv(const void* s, const int* c, const int* d, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
  return ostub_copy_((const char*)s + (size_t)d[0] * (size_t)t, r, c[0], t);
}
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return 0; }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return 0; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_File_open(MPI_Comm, const char*, int, MPI_Info, MPI_File*) { return 1; }
static inline int MPI_File_close(MPI_File*) { return 0; }
static inline int MPI_File_set_view(MPI_File, MPI_Offset, MPI_Datatype, MPI_Datatype, const char*, MPI_Info) { return 0; }
static inline int MPI_File_write(MPI_File, const void*, int, MPI_Datatype, MPI_Status*) { return 0; }
static inline int MPI_File_read(MPI_File, void*, int, MPI_Datatype, MPI_Status*) { return 0; }

#endif
