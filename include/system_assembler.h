/* system_assembler.h — the generic-system plugin interface (drop-in).
 *
 * Same class layout and virtual interface as MPLA src/system_assembler.h:6-12:
 * one int field followed by two pure-virtual device methods.  A subclass
 * object lives in device memory and is handed to the solvers through
 * mpla_generic_matrix::data.  The GB300 cores recognise Gaussian assemblers
 * created by this library's factories and evaluate them with fused tiled
 * kernels; any other subclass is evaluated through its virtual
 * get_matrix_entry inside a fused tiled kernel (no matrix is materialised).
 */
#ifndef system_assembler_h__
#define system_assembler_h__

#include "mpla.h"

#ifndef __CUDACC__
#ifndef __device__
#define __device__
#endif
#endif

class system_assembler
{
	public:
		int max_row_count_per_dgemv;
		virtual __device__ double get_matrix_entry(int i, int j) = 0;
		virtual __device__ double get_rhs_entry(int i) = 0;
};

#endif
