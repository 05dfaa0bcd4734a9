/*
 * Single-rank MPI stand-in used only to compile the upstream Branson headers
 * into the CPU reference harness (oracle/ref_harness.cc).  Test
 * infrastructure: never linked into the product library.
 *
 * Semantics are those of an MPI job with exactly one rank: every reduction is
 * the identity (in place: nothing to do; otherwise a copy of count elements),
 * broadcasts and barriers do nothing, and point-to-point calls are never
 * reached because a single replicated rank has no neighbours.
 */
#ifndef BGS_ORACLE_MPI_STUB_H
#define BGS_ORACLE_MPI_STUB_H

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cstdio>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_Win;
typedef long MPI_Aint;
struct MPI_Status { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; int count; };

#define MPI_COMM_WORLD 0
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_ANY_SOURCE (-1)
#define MPI_MODE_NOCHECK 1024
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_SUCCESS 0
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

/* builtin datatypes: handle = index into the size table below */
#define MPI_INT 1
#define MPI_UNSIGNED 2
#define MPI_UNSIGNED_LONG 3
#define MPI_DOUBLE 4
#define MPI_UNSIGNED_CHAR 5
#define MPI_CHAR 6
#define MPI_LONG 7
#define MPI_UNSIGNED_LONG_LONG 8
#define MPI_FLOAT 9

namespace bgs_mpi_stub {
inline int *type_sizes() {
  static int sizes[256] = {0,
                           (int)sizeof(int),
                           (int)sizeof(unsigned),
                           (int)sizeof(unsigned long),
                           (int)sizeof(double),
                           (int)sizeof(unsigned char),
                           (int)sizeof(char),
                           (int)sizeof(long),
                           (int)sizeof(unsigned long long),
                           (int)sizeof(float)};
  return sizes;
}
inline int &next_type() {
  static int next = 10;
  return next;
}
inline int size_of(MPI_Datatype t) {
  if (t < 0 || t >= 256) {
    std::fprintf(stderr, "mpi stub: bad datatype %d\n", t);
    std::abort();
  }
  return type_sizes()[t];
}
inline void copy(const void *send, void *recv, int count, MPI_Datatype t) {
  if (send == MPI_IN_PLACE || send == recv || count <= 0)
    return;
  std::memcpy(recv, send, (size_t)count * (size_t)size_of(t));
}
[[noreturn]] inline void unreachable(const char *what) {
  std::fprintf(stderr, "mpi stub: %s is not reachable with one rank\n", what);
  std::abort();
}
} // namespace bgs_mpi_stub

inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return MPI_SUCCESS; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *o) { *o = c; return MPI_SUCCESS; }
inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm *o) {
  *o = c;
  return MPI_SUCCESS;
}
inline int MPI_Get_processor_name(char *name, int *len) {
  std::strcpy(name, "oracle");
  *len = 6;
  return MPI_SUCCESS;
}
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  bgs_mpi_stub::copy(s, r, n, t);
  return MPI_SUCCESS;
}
inline int MPI_Iallreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm,
                          MPI_Request *q) {
  bgs_mpi_stub::copy(s, r, n, t);
  *q = 0;
  return MPI_SUCCESS;
}
inline int MPI_Type_create_struct(int count, const int *len, const MPI_Aint *disp,
                                  const MPI_Datatype *types, MPI_Datatype *out) {
  long extent = 0;
  for (int i = 0; i < count; ++i) {
    long end = disp[i] + (long)len[i] * bgs_mpi_stub::size_of(types[i]);
    if (end > extent)
      extent = end;
  }
  int id = bgs_mpi_stub::next_type()++;
  bgs_mpi_stub::type_sizes()[id] = (int)extent;
  *out = id;
  return MPI_SUCCESS;
}
inline int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
inline int MPI_Type_free(MPI_Datatype *) { return MPI_SUCCESS; }
inline int MPI_Type_dup(MPI_Datatype t, MPI_Datatype *o) { *o = t; return MPI_SUCCESS; }
inline int MPI_Type_size(MPI_Datatype t, int *s) { *s = bgs_mpi_stub::size_of(t); return MPI_SUCCESS; }
inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
inline int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
inline int MPI_Test(MPI_Request *, int *flag, MPI_Status *) { *flag = 1; return MPI_SUCCESS; }
inline int MPI_Get_count(const MPI_Status *, MPI_Datatype, int *c) { *c = 0; return MPI_SUCCESS; }
inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  bgs_mpi_stub::unreachable("MPI_Isend");
}
inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  bgs_mpi_stub::unreachable("MPI_Irecv");
}
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  bgs_mpi_stub::unreachable("MPI_Send");
}
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  bgs_mpi_stub::unreachable("MPI_Recv");
}
inline int MPI_Info_create(MPI_Info *i) { *i = 0; return MPI_SUCCESS; }
inline int MPI_Info_set(MPI_Info, const char *, const char *) { return MPI_SUCCESS; }
inline int MPI_Win_allocate(MPI_Aint, int, MPI_Info, MPI_Comm, void *, MPI_Win *) {
  bgs_mpi_stub::unreachable("MPI_Win_allocate");
}
inline int MPI_Win_free(MPI_Win *) { return MPI_SUCCESS; }
inline int MPI_Win_lock_all(int, MPI_Win) { return MPI_SUCCESS; }
inline int MPI_Win_unlock_all(MPI_Win) { return MPI_SUCCESS; }
inline int MPI_Win_sync(MPI_Win) { return MPI_SUCCESS; }
inline int MPI_Win_flush_all(MPI_Win) { return MPI_SUCCESS; }
inline int MPI_Put(const void *, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win) {
  bgs_mpi_stub::unreachable("MPI_Put");
}
inline int MPI_Rget(void *, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win,
                    MPI_Request *) {
  bgs_mpi_stub::unreachable("MPI_Rget");
}
inline int MPI_Raccumulate(const void *, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype,
                           MPI_Op, MPI_Win, MPI_Request *) {
  bgs_mpi_stub::unreachable("MPI_Raccumulate");
}

#endif
