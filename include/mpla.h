/* mpla.h — drop-in declaration of the MPLA host API for the GB300 build.
 *
 * Struct layouts and function signatures are identical to the original
 * library's public header (MPLA src/mpla.h:25-126) because callers allocate
 * these structs themselves and read their fields directly; any difference
 * would break binary compatibility.  The header is C++ (bool parameters, no
 * extern "C"), so the symbols keep C++ linkage exactly like the original.
 *
 * On GB300 the process grid is always 1x1: cur_proc_* equals the global size,
 * offsets are 0, and no MPI collective is issued.  Vector and matrix data are
 * plain device pointers (column-major, lda = rows) as before.  All errors
 * keep the original convention: message to stderr and exit(EXIT_FAILURE).
 * The status-returning C ABI in mpla_gb300.h is the non-exiting alternative.
 */
#include "cublas_v2.h"
#include <mpi.h>

#ifndef mpla_h__
#define mpla_h__

struct mpla_instance
{
	MPI_Comm comm;
	int proc_count;
	int proc_rows;
	int proc_cols;
	int cur_proc_coord[2];
	int cur_proc_row;
	int cur_proc_col;
	int cur_proc_rank;
	bool is_parent;
	cublasHandle_t cublas_handle;
};

struct mpla_matrix
{
	double* data;
	int mat_row_count, mat_col_count;
	int cur_proc_row_count;
	int cur_proc_col_count;
	int cur_proc_row_offset;
	int cur_proc_col_offset;
	int** proc_row_count;
	int** proc_col_count;
	int** proc_row_offset;
	int** proc_col_offset;
};

struct mpla_generic_matrix
{
	void* data;
	int mat_row_count, mat_col_count;
	int cur_proc_row_count;
	int cur_proc_col_count;
	int cur_proc_row_offset;
	int cur_proc_col_offset;
	int** proc_row_count;
	int** proc_col_count;
	int** proc_row_offset;
	int** proc_col_offset;
};

struct mpla_vector
{
	double* data;
	int vec_row_count, vec_col_count;
	int cur_proc_row_count;
	int cur_proc_row_offset;
	int** proc_row_count;
	int** proc_row_offset;
};

typedef void (*mpla_dgemv_core_fn)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*, struct mpla_instance*);

extern void info();

extern void mpla_init_instance(struct mpla_instance* instance, MPI_Comm comm);

extern void mpla_init_instance_block_rows(struct mpla_instance* instance, MPI_Comm comm);

extern void mpla_destroy_instance(struct mpla_instance* instance);

extern void mpla_init_matrix(struct mpla_matrix* matrix, struct mpla_instance* instance, int mat_row_count, int mat_col_count);

extern void mpla_init_generic_matrix(struct mpla_generic_matrix* matrix, struct mpla_instance* instance, int mat_row_count, int mat_col_count);

extern void mpla_init_vector(struct mpla_vector* vector, struct mpla_instance* instance, int vec_row_count);

extern void mpla_init_vector_for_block_rows(struct mpla_vector* vector, struct mpla_instance* instance, int vec_row_count);

extern void mpla_redistribute_vector_for_dgesv(struct mpla_vector* b_redist, struct mpla_vector* b, struct mpla_matrix* A, struct mpla_instance* instance);

extern void mpla_redistribute_vector_for_generic_dgesv(struct mpla_vector* b_redist, struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_instance* instance);

extern void mpla_save_vector(struct mpla_vector* x, char* filename, struct mpla_instance* instance);

extern void mpla_load_vector(struct mpla_vector* x, char* filename, struct mpla_instance* instance);

extern void mpla_free_vector(struct mpla_vector* x, struct mpla_instance* instance);

extern void mpla_free_matrix(struct mpla_matrix* A, struct mpla_instance* instance);

extern void mpla_free_generic_matrix(struct mpla_generic_matrix* A, struct mpla_instance* instance);

extern void mpla_dgemv(struct mpla_vector* b, struct mpla_matrix* A, struct mpla_vector* x, struct mpla_instance* instance);

extern void mpla_ddot(double* xy, struct mpla_vector* x, struct mpla_vector* y, struct mpla_instance* instance);

extern void mpla_generic_dgemv(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x, void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*, struct mpla_instance*), struct mpla_instance* instance);

extern void mpla_daxpy(struct mpla_vector* y, double alpha, struct mpla_vector* x, struct mpla_instance* instance);

extern void mpla_vector_set_zero(struct mpla_vector* x, struct mpla_instance* instance);

extern void mpla_generic_conjugate_gradient(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x, int iter_max, double epsilon, void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*, struct mpla_instance*), struct mpla_instance* instance);

extern void mpla_generic_conjugate_gradient_with_checkpoint_restart(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x, int iter_max, double epsilon, void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*, struct mpla_instance*), int iterations_until_checkpoint, bool restart, struct mpla_instance* instance);

extern void mpla_generic_BiCGSTAB_with_checkpoint_restart(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x, int iter_max, double epsilon, void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*, struct mpla_instance*), int iterations_until_checkpoint, bool restart, struct mpla_instance* instance);

extern void mpla_copy_distributed_vector_to_cpu(double* x_cpu, struct mpla_vector* x, struct mpla_instance* instance);

extern void checkCUDAError(const char* msg);

#endif
