/*
 * Single-rank stand-in for the MPI-3 subset that the reference's
 * ThreadSharedMemory / ChimeraSystemPtr translation units call, so that its
 * shared-window ("Ptr") code path compiles and runs as one process.
 * Project-written for the oracle build only (oracle/build_oracle.py); MPICH
 * is not installed here.
 *
 * Semantics with one rank: rank 0 of size 1; collectives copy or do nothing;
 * windows are plain host memory (allocate_shared = calloc, create = wrap the
 * caller's buffer); Put/Get are memcpy into/out of the target window.
 */
#ifndef SPC_ORACLE_MPI_STUB_H
#define SPC_ORACLE_MPI_STUB_H

#include <cstddef>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef std::ptrdiff_t MPI_Aint;
struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; };

struct spc_mpi_window {
  char *base;
  MPI_Aint size;
  int disp_unit;
  bool owns;
};
typedef spc_mpi_window *MPI_Win;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

static inline std::size_t spc_mpi_type_size(MPI_Datatype t) { return (std::size_t)t; }

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm *out) {
  *out = c + 1;
  return 0;
}
static inline int MPI_Comm_free(MPI_Comm *) { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Gather(const void *sb, int sc, MPI_Datatype st, void *rb, int, MPI_Datatype,
                             int, MPI_Comm) {
  if (sb != MPI_IN_PLACE && sb != rb) std::memmove(rb, sb, (std::size_t)sc * spc_mpi_type_size(st));
  return 0;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (sb != MPI_IN_PLACE && sb != rb) std::memmove(rb, sb, (std::size_t)n * spc_mpi_type_size(t));
  return 0;
}
/* Point-to-point traffic only happens between distinct ranks; with one rank
 * the reference never posts any, so these are inert. */
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *r) {
  *r = 0;
  return 0;
}
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *r) {
  *r = 0;
  return 0;
}
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }

static inline int MPI_Win_create(void *base, MPI_Aint size, int disp_unit, MPI_Info, MPI_Comm,
                                 MPI_Win *win) {
  *win = new spc_mpi_window{(char *)base, size, disp_unit, false};
  return 0;
}
static inline int MPI_Win_allocate_shared(MPI_Aint size, int disp_unit, MPI_Info, MPI_Comm,
                                          void *baseptr, MPI_Win *win) {
  char *mem = (char *)std::calloc(size > 0 ? (std::size_t)size : 1, 1);
  *win = new spc_mpi_window{mem, size, disp_unit, true};
  *(void **)baseptr = mem;
  return 0;
}
static inline int MPI_Win_shared_query(MPI_Win win, int, MPI_Aint *size, int *disp_unit,
                                       void *baseptr) {
  *size = win->size;
  *disp_unit = win->disp_unit;
  *(void **)baseptr = win->base;
  return 0;
}
static inline int MPI_Win_free(MPI_Win *win) {
  if (*win) {
    if ((*win)->owns) std::free((*win)->base);
    delete *win;
    *win = nullptr;
  }
  return 0;
}
static inline int MPI_Win_fence(int, MPI_Win) { return 0; }
static inline int MPI_Win_lock_all(int, MPI_Win) { return 0; }
static inline int MPI_Win_unlock_all(MPI_Win) { return 0; }
static inline int MPI_Win_sync(MPI_Win) { return 0; }
static inline int MPI_Put(const void *o, int oc, MPI_Datatype ot, int, MPI_Aint disp, int,
                          MPI_Datatype, MPI_Win win) {
  std::memmove(win->base + disp * win->disp_unit, o, (std::size_t)oc * spc_mpi_type_size(ot));
  return 0;
}
static inline int MPI_Get(void *o, int oc, MPI_Datatype ot, int, MPI_Aint disp, int,
                          MPI_Datatype, MPI_Win win) {
  std::memmove(o, win->base + disp * win->disp_unit, (std::size_t)oc * spc_mpi_type_size(ot));
  return 0;
}

#endif
