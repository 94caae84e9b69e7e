// Quadrature weights on Halton points: the application MPLA was written for
// (MPLA src/generate_quadrature_weights.cpp), on the GB300 library through
// the unchanged mpla.h API.
//
// The weights w of n points p_i in [0,1]^dim solve K w = b with the Gaussian
// kernel K_ij = exp(-|p_i - p_j|^2) (+1e-8 where |p_i - p_j| < 1e-14, the
// kernel.h rule) and b_i = integral over [0,1]^dim of exp(-|x - p_i|^2), so
// that sum_i w_i f(p_i) integrates f over the unit cube exactly for f in the
// span of the kernel translates.  As in the original: kernel_matrix_data
// with the streamed kernel core, b from mpla_set_gaussian_kernel_rhs, a
// uniform random start vector, the checkpointing CG at relative tolerance
// `tol`, the wall time of the solve printed and the weights written to
// weights.dat in MPLA's vector format.  Differences: the Halton points come
// from this library (mgb_halton) instead of GSL, and the start vector from
// a seeded splitmix64 stream (seed 1235, stream 1: the same numbers as
// mpla_gb300.synth.uniform) instead of cuRAND.
//
//   generate_quadrature_weights [n=1000] [dim=3] [tol=1e-7] [restart=0]
//                               [iterations_until_checkpoint=100]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "mpla.h"
#include "mpi.h"
#include "kernel.h"
#include "mpla_gb300.h"

// value i (0-based) of the counter-based splitmix64 stream (seed, stream):
// mix(base + (i + 1) * golden), base = mix(seed ^ stream * c); uniform
// doubles from the top 53 bits (S. Vigna's splitmix64 finaliser)
static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static double uniform01(uint64_t seed, uint64_t stream, uint64_t i) {
  const uint64_t base = mix64(seed ^ (stream * 0xD1B54A32D192ED03ULL));
  return (double)(mix64(base + (i + 1) * 0x9E3779B97F4A7C15ULL) >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char* argv[]) {
  int n = 1000, dim = 3, restart = 0, iterations_until_checkpoint = 100;
  double tol = 1.0e-7;
  if (argc > 1) n = atoi(argv[1]);
  if (argc > 2) dim = atoi(argv[2]);
  if (argc > 3) tol = atof(argv[3]);
  if (argc > 4) restart = atoi(argv[4]);
  if (argc > 5) iterations_until_checkpoint = atoi(argv[5]);

  MPI_Init(&argc, &argv);
  mpla_instance instance;
  mpla_init_instance(&instance, MPI_COMM_WORLD);

  mpla_generic_matrix A;
  mpla_init_generic_matrix(&A, &instance, n, n);
  mpla_vector x, b;
  mpla_init_vector(&x, &instance, n);
  mpla_init_vector(&b, &instance, n);

  // Halton points, structure of arrays, on the device
  std::vector<double> pts((size_t)dim * n);
  if (mgb_halton(n, dim, 0, pts.data()) != MGB_OK) {
    fprintf(stderr, "%s\n", mgb_last_error());
    return 1;
  }
  std::vector<double*> cols(dim);
  for (int d = 0; d < dim; ++d) {
    cudaMalloc((void**)&cols[d], sizeof(double) * n);
    cudaMemcpy(cols[d], pts.data() + (size_t)d * n, sizeof(double) * n, cudaMemcpyHostToDevice);
  }
  double** points = nullptr;
  cudaMalloc((void**)&points, sizeof(double*) * dim);
  cudaMemcpy(points, cols.data(), sizeof(double*) * dim, cudaMemcpyHostToDevice);

  kernel_matrix_data matrix_data;
  matrix_data.points = points;
  matrix_data.dim = dim;
  matrix_data.max_row_count_per_dgemv = n;  // the fused core stores no matrix block
  A.data = (void*)&matrix_data;

  mpla_set_gaussian_kernel_rhs(&b, &A, &instance);

  std::vector<double> x0(n);
  for (int i = 0; i < n; ++i) x0[i] = uniform01(1235, 1, (uint64_t)i);
  cudaMemcpy(x.data, x0.data(), sizeof(double) * n, cudaMemcpyHostToDevice);

  cudaEvent_t start, stop;
  cudaEventCreate(&start);
  cudaEventCreate(&stop);
  cudaEventRecord(start, 0);
  mpla_generic_conjugate_gradient_with_checkpoint_restart(&b, &A, &x, 100000, tol,
                                                          &mpla_dgemv_core_kernel_streamed_cublas,
                                                          iterations_until_checkpoint, restart != 0, &instance);
  cudaEventRecord(stop, 0);
  cudaEventSynchronize(stop);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, start, stop);
  printf("Time spent: %.10f\n", ms / 1000);

  char filename[] = "weights.dat";
  mpla_save_vector(&x, filename, &instance);
  checkCUDAError("generate_quadrature_weights");

  mpla_free_generic_matrix(&A, &instance);
  mpla_free_vector(&x, &instance);
  mpla_free_vector(&b, &instance);
  for (double* p : cols) cudaFree(p);
  cudaFree(points);
  mpla_destroy_instance(&instance);
  MPI_Finalize();
  return 0;
}
