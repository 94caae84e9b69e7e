/* kernel.h — Gaussian kernel-matrix cores on a host descriptor (drop-in).
 *
 * Same descriptor and entry points as MPLA src/kernel.h:3-14.  A->data points
 * to a host kernel_matrix_data whose `points` is a device array of `dim`
 * device pointers.  Entry semantics follow MPLA src/kernel.cu:17-50:
 * K(i,j) = exp(-r^2), r = |p_i - p_j|, plus 1e-8 whenever r < 1e-14
 * (the diagonal and duplicate points).  On GB300 both cores run the same
 * fused kernel; max_row_count_per_dgemv is accepted but not needed because
 * no block of the matrix is ever stored.
 */
#ifndef MPLA_GB300_KERNEL_H
#define MPLA_GB300_KERNEL_H

#include <stdio.h>
#include "mpla.h"

struct kernel_matrix_data
{
	double** points;
	int dim;
	int max_row_count_per_dgemv;
};

extern void mpla_set_gaussian_kernel_rhs(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_instance* instance);

extern void mpla_dgemv_core_kernel_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist, struct mpla_instance* instance);
extern void mpla_dgemv_core_kernel_streamed_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist, struct mpla_instance* instance);

/* GB300 addition: dense core for an mpla_matrix cast to mpla_generic_matrix
 * (column-major, lda = cur_proc_row_count), computed by the library's own
 * HBM-streaming dgemv instead of a user-written cuBLAS core. */
extern void mpla_dgemv_core_dense(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist, struct mpla_instance* instance);

#endif
