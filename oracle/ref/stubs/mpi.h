/* Single-process stand-in for the handful of MPI calls the reference's LBM
 * library makes (TEST INFRASTRUCTURE ONLY).  With one rank every
 * collective is a copy and MPI_Sendrecv to oneself copies the send buffer
 * into the receive buffer. */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_FLOAT 3
#define MPI_SUCCESS 0

static inline int oracle_mpi_size(MPI_Datatype t) {
  return t == MPI_DOUBLE ? (int)sizeof(double) : (t == MPI_FLOAT ? (int)sizeof(float) : (int)sizeof(int));
}
static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int, MPI_Datatype, MPI_Comm) {
  std::memcpy(rb, sb, (size_t)sc * oracle_mpi_size(st));
  return MPI_SUCCESS;
}
static inline int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int, MPI_Datatype, int, MPI_Comm) {
  if (rb) std::memcpy(rb, sb, (size_t)sc * oracle_mpi_size(st));
  return MPI_SUCCESS;
}
static inline int MPI_Sendrecv(const void* sb, int sc, MPI_Datatype st, int, int, void* rb, int, MPI_Datatype, int, int,
                               MPI_Comm, MPI_Status*) {
  std::memmove(rb, sb, (size_t)sc * oracle_mpi_size(st));
  return MPI_SUCCESS;
}
#endif
