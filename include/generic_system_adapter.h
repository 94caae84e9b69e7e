/* generic_system_adapter.h — matvec cores for system_assembler objects (drop-in).
 *
 * Same entry points as MPLA src/generic_system_adapter.h:12-14.  Both cores
 * compute b = K x for the assembler in A->data; on GB300 neither allocates or
 * materialises the matrix, so the "streamed" variant and the plain one run
 * the same fused kernel and max_row_count_per_dgemv is accepted but not
 * needed.
 */
#ifndef generic_system_adapter_h__
#define generic_system_adapter_h__

#include <stdio.h>
#include "mpla.h"
#include "system_assembler.h"

extern void mpla_set_generic_system_rhs(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_instance* instance);
extern void mpla_dgemv_core_generic_system_matrix_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist, struct mpla_instance* instance);
extern void mpla_dgemv_core_generic_system_matrix_streamed_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist, struct mpla_instance* instance);

#endif
