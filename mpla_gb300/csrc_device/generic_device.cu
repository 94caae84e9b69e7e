// Generic system_assembler kernels for device linking into a user's module.
//
// A system_assembler subclass (include/system_assembler.h) is defined and
// constructed in the user's own CUDA module; its virtual get_matrix_entry can
// only be called from a kernel linked into that same module.  MPLA solves
// this by device-linking generic_system_adapter.o with the user's objects
// (src/Makefile:96-114, kernels at src/generic_system_adapter.cu:7-23 and
// :25-37).  This file is the GB300 counterpart: built with -rdc into
// lib/mpla_generic_device.o, linked by the user with -rdc, it registers its
// launchers with libmpla.so from a static constructor
// (mgb_register_generic_device_code), and the generic_system_adapter.h cores
// and the solvers evaluate user assemblers through it.
//
// Kernel: a CTA of 128 threads owns 128 rows and a range of columns; x is
// staged in shared memory 256 columns at a time and every thread sums its
// row's entries K(i, j) x_j in FP64 with one virtual call per entry (the
// matrix is never stored, unlike the reference, which writes row blocks of K
// to device memory and calls cublasDgemv on them).  Column ranges are reduced
// in a fixed order by the last CTA of each row tile, so results are
// bit-reproducible.
#include <cuda_runtime.h>

#include "../../include/mpla_gb300.h"
#include "../../include/system_assembler.h"
#include "../csrc/devutil.cuh"

namespace {

constexpr int kRowsPerCta = 128;
constexpr int kColTile = 256;

__global__ void __launch_bounds__(kRowsPerCta)
    k_user_assembler_matvec(system_assembler* assem, int rows, int cols, int row_offset, int col_offset,
                            const double* __restrict__ x, double* __restrict__ y, int cols_per_split, int nsplit,
                            double* __restrict__ partials, unsigned int* __restrict__ tickets,
                            const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double sx[kColTile];
  __shared__ int s_last;
  const int tile = blockIdx.x / nsplit, split = blockIdx.x % nsplit;
  const int i = tile * kRowsPerCta + threadIdx.x;
  const int cbeg = split * cols_per_split, cend = min(cols, cbeg + cols_per_split);
  double acc = 0.0;
  for (int j0 = cbeg; j0 < cend; j0 += kColTile) {
    const int nj = min(kColTile, cend - j0);
    __syncthreads();
    for (int t = threadIdx.x; t < nj; t += kRowsPerCta) sx[t] = x[j0 + t];
    __syncthreads();
    if (i < rows)
      for (int t = 0; t < nj; ++t) acc = fma(assem->get_matrix_entry(row_offset + i, col_offset + j0 + t), sx[t], acc);
  }
  if (nsplit == 1) {
    if (i < rows) y[i] = acc;
    return;
  }
  if (i < rows) partials[(long long)split * rows + i] = acc;
  if (mgb::last_block_arrival(&tickets[tile], nsplit, &s_last)) {
    if (i < rows) {
      double s = 0.0;
      for (int p = 0; p < nsplit; ++p) s += __ldcg(&partials[(long long)p * rows + i]);
      y[i] = s;
    }
  }
}

__global__ void k_user_assembler_rhs(system_assembler* assem, int rows, int row_offset, double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < rows) b[i] = assem->get_rhs_entry(row_offset + i);
}

int launch_matvec(const void* assembler, int rows, int cols, int row_offset, int col_offset, const double* x,
                  double* y, int cols_per_split, int nsplit, double* partials, unsigned int* tickets,
                  const int* skip, void* stream) {
  if (rows <= 0) return cudaSuccess;
  const int tiles = (rows + kRowsPerCta - 1) / kRowsPerCta;
  k_user_assembler_matvec<<<tiles * nsplit, kRowsPerCta, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<system_assembler*>(const_cast<void*>(assembler)), rows, cols, row_offset, col_offset, x, y,
      cols_per_split, nsplit, partials, tickets, skip);
  return static_cast<int>(cudaGetLastError());
}

int launch_rhs(const void* assembler, int rows, int row_offset, double* b, void* stream) {
  if (rows <= 0) return cudaSuccess;
  k_user_assembler_rhs<<<(rows + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<system_assembler*>(const_cast<void*>(assembler)), rows, row_offset, b);
  return static_cast<int>(cudaGetLastError());
}

const mgb_generic_device_code kCode = {MGB_GENERIC_DEVICE_ABI, &launch_matvec, &launch_rhs};

// Registration when the module is loaded; withdrawn when it is unloaded.
struct Registration {
  Registration() { mgb_register_generic_device_code(&kCode); }
  ~Registration() { mgb_unregister_generic_device_code(&kCode); }
} g_registration;

}  // namespace
