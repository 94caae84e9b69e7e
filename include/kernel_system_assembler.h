/* kernel_system_assembler.h — Gaussian-kernel system assembler (drop-in).
 *
 * Field layout matches MPLA src/kernel_system_assembler.h:10-50 (points,
 * dim, regularization after the base class) because callers may build or
 * patch the device object themselves.  Entry semantics follow the same
 * definition:
 *   K(i,j) = exp(-r^2) with r = sqrt(sum_d (p_d[i]-p_d[j])^2),
 *   plus `regularization` when i == j;
 *   rhs(i) = prod_d (sqrt(pi)/2) * (erf(1 - p_d[i]) - erf(-p_d[i])).
 * `points` is a device array of `dim` device pointers (structure of arrays);
 * a length scale l is expressed by passing points pre-scaled by 1/(sqrt(2) l).
 *
 * The factory of the original never sets `regularization`; value
 * initialisation leaves it 0.  This library's factory sets it to 0 explicitly
 * and adds a variant that takes the nugget.
 */
#ifndef kernel_system_assembler_h__
#define kernel_system_assembler_h__

#include "mpla.h"
#include "system_assembler.h"
#include <math.h>

class gaussian_kernel_system_assembler : public system_assembler
{
	public:
		double** points;
		int dim;
		double regularization;

		__device__ double gaussian_kernel(double r)
		{
			return exp(-r * r);
		}

		__device__ double get_matrix_entry(int i, int j)
		{
			double sq = 0.0;
			for (int d = 0; d < dim; d++)
			{
				const double diff = points[d][i] - points[d][j];
				sq += diff * diff;
			}
			const double k = gaussian_kernel(sqrt(sq));
			return (i == j) ? k + regularization : k;
		}

		__device__ double get_rhs_entry(int i)
		{
			const double half_sqrt_pi = 0.88622692545275801365;
			double prod = 1.0;
			for (int d = 0; d < dim; d++)
				prod = prod * half_sqrt_pi * (erf(1.0 - points[d][i]) - erf(0.0 - points[d][i]));
			return prod;
		}
};

extern void create_gaussian_kernel_system_assembler_object(struct gaussian_kernel_system_assembler** assem, double** points, int max_row_count_per_dgemv, int dim);

extern void destroy_gaussian_kernel_system_assembler_object(struct gaussian_kernel_system_assembler** assem);

/* GB300 addition: same as the factory above but also sets the diagonal nugget. */
extern void create_gaussian_kernel_system_assembler_object_with_regularization(struct gaussian_kernel_system_assembler** assem, double** points, int max_row_count_per_dgemv, int dim, double regularization);

#endif
