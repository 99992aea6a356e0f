/*
 * Single-rank stand-in for <mpi.h>.  TEST INFRASTRUCTURE ONLY.
 *
 * It exists so that the reference's own embedding kernels
 * (cpp/algo/algo.hpp, cpp/core/common.cpp) compile unmodified for a
 * one-process run, which is the configuration the GPU path replaces.
 * At one rank the reference never moves data between processes: every
 * exchange is guarded by `col_world_size > 1` (cpp/algo/algo.hpp:110,139,176)
 * or finds no remote ids (cpp/core/sparse_mat.hpp: `rank != procs[r]`).
 * The data-moving collectives below therefore abort if they are ever asked
 * to move data, so a silent wrong answer is impossible.
 */
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef intptr_t MPI_Aint;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_REQUEST_NULL 0
#define MPI_SUCCESS 0
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUM 1

#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_LONG_LONG_INT 3
#define MPI_FLOAT 4
#define MPI_DOUBLE 5
#define MPI_UINT64_T 6

/* Accepts both pointers and MPI_Aint values, as the real macro does. */
#define MPI_Aint_diff(a, b) ((MPI_Aint)((const char *)(a) - (const char *)(b)))

[[noreturn]] inline void shim_mpi_refuse(const char *what) {
  std::fprintf(stderr, "single-rank mpi shim: %s would move data between ranks\n", what);
  std::abort();
}

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Finalized(int *flag) { *flag = 0; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm *out) { *out = MPI_COMM_WORLD; return 0; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *out) { *out = c; return 0; }
inline int MPI_Comm_free(MPI_Comm *) { return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Type_create_struct(int, const int *, const MPI_Aint *, const MPI_Datatype *,
                                  MPI_Datatype *t) { *t = 100; return 0; }
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }

/* Reductions over one rank: in-place is the identity; anything else needs a
 * type size, which this shim does not model. */
inline int MPI_Allreduce(const void *s, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) shim_mpi_refuse("MPI_Allreduce (not in place)");
  return 0;
}

inline int MPI_Alltoall(const void *, int n, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm) {
  if (n != 0) shim_mpi_refuse("MPI_Alltoall");
  return 0;
}
inline int MPI_Alltoallv(const void *, const int *sc, const int *, MPI_Datatype, void *,
                         const int *rc, const int *, MPI_Datatype, MPI_Comm) {
  if (sc[0] != 0 || rc[0] != 0) shim_mpi_refuse("MPI_Alltoallv");
  return 0;
}
inline int MPI_Ialltoallv(const void *, const int *sc, const int *, MPI_Datatype, void *,
                          const int *rc, const int *, MPI_Datatype, MPI_Comm, MPI_Request *) {
  if (sc[0] != 0 || rc[0] != 0) shim_mpi_refuse("MPI_Ialltoallv");
  return 0;
}
inline int MPI_Gather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm) {
  shim_mpi_refuse("MPI_Gather");
}
