/* Single-process stand-in for the MPI surface that mpla.h exposes.
 *
 * The GB300 build runs one process on one GPU, so the 2-D process grid of the
 * original library is always 1x1 and every collective is an identity.  This
 * header lets unmodified MPLA drivers (MPI_Init / MPI_COMM_WORLD /
 * MPI_Finalize, the MPI_Comm field of mpla_instance) compile and link without
 * an MPI installation.  MPI_Comm is an int, the same size as MPICH's handle.
 */
#ifndef MPLA_GB300_MPI_SHIM_H
#define MPLA_GB300_MPI_SHIM_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#define MPI_COMM_NULL ((MPI_Comm)0x04000000)
#define MPI_DOUBLE ((MPI_Datatype)0x4c00080b)
#define MPI_INT ((MPI_Datatype)0x4c000405)
#define MPI_SUM ((MPI_Op)0x58000003)
#define MPI_SUCCESS 0

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm comm, int* size) { (void)comm; *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm comm, int* rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }

#endif
