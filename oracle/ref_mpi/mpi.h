/* Single-rank MPI stand-in used only to compile the reference MPLA sources
 * for the oracle (oracle/build_ref.py).  One process, a 1x1 Cartesian grid:
 * communicator constructors return their input, and the collectives the
 * reference calls on device buffers (CUDA-aware MPI) become copies with
 * cudaMemcpyDefault, which also accepts host pointers. */
#ifndef MPLA_ORACLE_REF_MPI_H
#define MPLA_ORACLE_REF_MPI_H

#include <cuda_runtime.h>
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_SUM ((MPI_Op)1)
#define MPI_SUCCESS 0

static inline size_t mpi_stub_size(MPI_Datatype t) { return (size_t)t; }
static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Dims_create(int nn, int nd, int* dims) { (void)nn; for (int i = 0; i < nd; ++i) dims[i] = 1; return 0; }
static inline int MPI_Cart_create(MPI_Comm c, int nd, const int* dims, const int* periods, int reorder, MPI_Comm* out) {
  (void)nd; (void)dims; (void)periods; (void)reorder; *out = c; return 0;
}
static inline int MPI_Cart_get(MPI_Comm c, int nd, int* dims, int* periods, int* coords) {
  (void)c; for (int i = 0; i < nd; ++i) { dims[i] = 1; periods[i] = 0; coords[i] = 0; } return 0;
}
static inline int MPI_Cart_sub(MPI_Comm c, const int* remain, MPI_Comm* out) { (void)remain; *out = c; return 0; }
static inline int MPI_Comm_free(MPI_Comm* c) { (void)c; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Allgatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int* rc, const int* displs,
                                 MPI_Datatype rt, MPI_Comm c) {
  (void)rc; (void)st; (void)c;
  cudaMemcpy((char*)rb + (size_t)displs[0] * mpi_stub_size(rt), sb, (size_t)sc * mpi_stub_size(st), cudaMemcpyDefault);
  return 0;
}
static inline int MPI_Allreduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  cudaMemcpy(rb, sb, (size_t)count * mpi_stub_size(t), cudaMemcpyDefault);
  return 0;
}

#endif
