// C++ drivers that use the drop-in mpla.h API the way MPLA's own test and
// benchmark programs do (test_library.cpp, test_cg.cpp, test_kernel_cg.cpp,
// benchmark_generic_system_cg.cpp): MPI_Init, an instance on
// MPI_COMM_WORLD, containers, user cores that call cuBLAS through
// instance->cublas_handle, the library's own cores, checkpoint/restart.
// Each mode prints "RESULT <key> <value>" lines for the pytest wrapper.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "mpla.h"
#include "mpi.h"
#include "kernel.h"
#include "generic_system_adapter.h"
#include "kernel_system_assembler.h"

static int idx(int i, int j, int m) { return j * m + i; }

// user core in the style of test_library.cpp:37-42 (cuBLAS through the instance)
static void user_cublas_core(mpla_vector* b, mpla_generic_matrix* A, mpla_vector* x_redist, mpla_instance* inst) {
  double one = 1, zero = 0;
  cublasDgemv(inst->cublas_handle, CUBLAS_OP_N, A->cur_proc_row_count, A->cur_proc_col_count, &one,
              (double*)(A->data), A->cur_proc_row_count, x_redist->data, 1, &zero, b->data, 1);
}

static std::vector<double> to_host(mpla_vector* v) {
  std::vector<double> h(v->cur_proc_row_count);
  cudaMemcpy(h.data(), v->data, sizeof(double) * h.size(), cudaMemcpyDeviceToHost);
  return h;
}

static void upload(mpla_vector* v, const std::vector<double>& h) {
  cudaMemcpy(v->data, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice);
}

// --- test_library.cpp: dgemv and ddot known answers
static int mode_kat(mpla_instance* inst, int m, int n) {
  std::vector<double> A_h((size_t)m * n), x_h(n), y_h(n), Ax_h(m, 0.0);
  for (size_t i = 0; i < A_h.size(); ++i) A_h[i] = (double)i;
  for (int j = 0; j < n; ++j) {
    x_h[j] = j;
    y_h[j] = j + 1;
  }
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) Ax_h[i] += A_h[idx(i, j, m)] * x_h[j];
  double xy_h = 0.0;
  for (int j = 0; j < n; ++j) xy_h += x_h[j] * y_h[j];

  mpla_matrix A;
  mpla_init_matrix(&A, inst, m, n);
  mpla_vector x, y, Ax;
  mpla_init_vector(&x, inst, n);
  mpla_init_vector(&y, inst, n);
  mpla_init_vector(&Ax, inst, m);
  upload(&x, x_h);
  upload(&y, y_h);
  cudaMemcpy(A.data, A_h.data(), sizeof(double) * A_h.size(), cudaMemcpyHostToDevice);

  int bad = 0;
  for (int variant = 0; variant < 3; ++variant) {
    if (variant == 0) mpla_dgemv(&Ax, &A, &x, inst);
    if (variant == 1) mpla_generic_dgemv(&Ax, (mpla_generic_matrix*)&A, &x, &user_cublas_core, inst);
    if (variant == 2) mpla_generic_dgemv(&Ax, (mpla_generic_matrix*)&A, &x, &mpla_dgemv_core_dense, inst);
    std::vector<double> got = to_host(&Ax);
    double worst = 0.0;
    for (int i = 0; i < m; ++i) {
      const double d = fabs(Ax_h[i] - got[i]) / (Ax_h[i] != 0.0 ? fabs(Ax_h[i]) : 1.0);
      if (d > worst) worst = d;
    }
    printf("RESULT dgemv_relerr_%d %.3e\n", variant, worst);
    if (worst > 1e-13) bad = 1;
  }
  double xy = 0.0;
  mpla_ddot(&xy, &x, &y, inst);
  const double ddot_err = fabs(xy_h - xy) / (xy_h != 0.0 ? fabs(xy_h) : 1.0);
  printf("RESULT ddot_relerr %.3e\n", ddot_err);
  if (ddot_err > 1e-13) bad = 1;
  // redistribution and copy-to-cpu at the 1x1 grid are copies
  mpla_vector xr;
  mpla_init_vector_for_block_rows(&xr, inst, n);
  mpla_redistribute_vector_for_dgesv(&xr, &x, &A, inst);
  std::vector<double> back(n);
  mpla_copy_distributed_vector_to_cpu(back.data(), &xr, inst);
  for (int j = 0; j < n; ++j)
    if (back[j] != x_h[j]) bad = 1;
  mpla_free_vector(&xr, inst);
  mpla_free_matrix(&A, inst);
  mpla_free_vector(&x, inst);
  mpla_free_vector(&y, inst);
  mpla_free_vector(&Ax, inst);
  printf("RESULT ok %d\n", bad ? 0 : 1);
  return bad;
}

// --- test_cg.cpp: tridiagonal CG with a user cuBLAS core and the dense core
static int mode_cg_tridiag(mpla_instance* inst, int n) {
  std::vector<double> A_h((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    A_h[idx(i, i, n)] = 2;
    if (i > 0) A_h[idx(i, i - 1, n)] = -1;
    if (i + 1 < n) A_h[idx(i, i + 1, n)] = -1;
  }
  mpla_matrix A;
  mpla_init_matrix(&A, inst, n, n);
  cudaMemcpy(A.data, A_h.data(), sizeof(double) * A_h.size(), cudaMemcpyHostToDevice);
  mpla_vector x, b, Ax;
  mpla_init_vector(&x, inst, n);
  mpla_init_vector(&b, inst, n);
  mpla_init_vector(&Ax, inst, n);
  std::vector<double> xs(n), x0(n);
  for (int i = 0; i < n; ++i) {
    xs[i] = 0.5 + 0.5 * sin(0.37 * i);
    x0[i] = 0.25 + 0.25 * cos(0.11 * i);
  }
  int bad = 0;
  for (int variant = 0; variant < 2; ++variant) {
    mpla_dgemv_core_fn core = variant == 0 ? &user_cublas_core : &mpla_dgemv_core_dense;
    upload(&x, xs);
    mpla_generic_dgemv(&b, (mpla_generic_matrix*)&A, &x, core, inst);  // manufactured rhs
    upload(&x, x0);
    mpla_generic_conjugate_gradient(&b, (mpla_generic_matrix*)&A, &x, 1000, 1.0e-10, core, inst);
    mpla_generic_dgemv(&Ax, (mpla_generic_matrix*)&A, &x, core, inst);
    mpla_daxpy(&Ax, -1, &b, inst);
    double norm;
    mpla_ddot(&norm, &Ax, &Ax, inst);
    norm = sqrt(norm / (double)n);
    printf("RESULT rms_residual_%d %.6e\n", variant, norm);
    if (!(norm < 1e-9)) bad = 1;
  }
  mpla_free_matrix(&A, inst);
  mpla_free_vector(&x, inst);
  mpla_free_vector(&b, inst);
  mpla_free_vector(&Ax, inst);
  printf("RESULT ok %d\n", bad ? 0 : 1);
  return bad;
}

// --- checkpoint/restart of the relative-residual CG (mpla.cpp:887-1001)
static int mode_cg_checkpoint(mpla_instance* inst, int n, int restart) {
  std::vector<double> A_h((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    A_h[idx(i, i, n)] = 2.5;
    if (i > 0) A_h[idx(i, i - 1, n)] = -1;
    if (i + 1 < n) A_h[idx(i, i + 1, n)] = -1;
  }
  mpla_matrix A;
  mpla_init_matrix(&A, inst, n, n);
  cudaMemcpy(A.data, A_h.data(), sizeof(double) * A_h.size(), cudaMemcpyHostToDevice);
  mpla_vector x, b;
  mpla_init_vector(&x, inst, n);
  mpla_init_vector(&b, inst, n);
  std::vector<double> ones(n, 1.0), zeros(n, 0.0);
  upload(&b, ones);
  upload(&x, zeros);
  mpla_generic_conjugate_gradient_with_checkpoint_restart(&b, (mpla_generic_matrix*)&A, &x, 1000, 1e-12,
                                                          &mpla_dgemv_core_dense, 5, restart != 0, inst);
  std::vector<double> xh = to_host(&x);
  double r2 = 0.0;
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += A_h[idx(i, j, n)] * xh[j];
    r2 += (1.0 - s) * (1.0 - s);
  }
  printf("RESULT relres %.6e\n", sqrt(r2 / n));
  mpla_free_matrix(&A, inst);
  mpla_free_vector(&x, inst);
  mpla_free_vector(&b, inst);
  printf("RESULT ok %d\n", sqrt(r2 / n) < 1e-10 ? 1 : 0);
  return 0;
}

// points file: int32 n, int32 dim, then dim*n doubles (structure of arrays)
static double** load_points(const char* path, int* n_out, int* dim_out, std::vector<double*>& host_ptrs) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  int n = 0, dim = 0;
  if (fread(&n, 4, 1, f) != 1 || fread(&dim, 4, 1, f) != 1) exit(2);
  std::vector<double> buf((size_t)n * dim);
  if (fread(buf.data(), 8, buf.size(), f) != buf.size()) exit(2);
  fclose(f);
  host_ptrs.resize(dim);
  for (int d = 0; d < dim; ++d) {
    cudaMalloc((void**)&host_ptrs[d], sizeof(double) * n);
    cudaMemcpy(host_ptrs[d], buf.data() + (size_t)d * n, sizeof(double) * n, cudaMemcpyHostToDevice);
  }
  double** points;
  cudaMalloc((void**)&points, sizeof(double*) * dim);
  cudaMemcpy(points, host_ptrs.data(), sizeof(double*) * dim, cudaMemcpyHostToDevice);
  *n_out = n;
  *dim_out = dim;
  return points;
}

// --- kernel systems: kernel.h descriptor core and the assembler plugin
static int mode_kernel(mpla_instance* inst, const char* pts_path, const char* rhs_path, const char* out_path,
                       int which, double nugget) {
  int n, dim;
  std::vector<double*> hp;
  double** points = load_points(pts_path, &n, &dim, hp);
  mpla_generic_matrix A;
  mpla_init_generic_matrix(&A, inst, n, n);
  mpla_vector x, b;
  mpla_init_vector(&x, inst, n);
  mpla_init_vector(&b, inst, n);
  kernel_matrix_data kd;
  gaussian_kernel_system_assembler** assem_d_p = nullptr;
  mpla_dgemv_core_fn core;
  if (which == 0) {  // benchmark_kernel_cg.cpp style
    kd.points = points;
    kd.dim = dim;
    kd.max_row_count_per_dgemv = 1024;
    A.data = &kd;
    core = &mpla_dgemv_core_kernel_streamed_cublas;
  } else {  // benchmark_generic_system_cg.cpp style, with the nugget
    cudaMalloc((void**)&assem_d_p, sizeof(gaussian_kernel_system_assembler*));
    create_gaussian_kernel_system_assembler_object_with_regularization(assem_d_p, points, 1024, dim, nugget);
    gaussian_kernel_system_assembler* assem_d;
    cudaMemcpy(&assem_d, assem_d_p, sizeof(assem_d), cudaMemcpyDeviceToHost);
    A.data = assem_d;
    core = &mpla_dgemv_core_generic_system_matrix_streamed_cublas;
  }
  // rhs: from a file, or the erf right-hand side of the library
  if (rhs_path && strcmp(rhs_path, "-") != 0) {
    FILE* f = fopen(rhs_path, "rb");
    std::vector<double> bh(n);
    if (!f || fread(bh.data(), 8, n, f) != (size_t)n) exit(2);
    fclose(f);
    upload(&b, bh);
  } else if (which == 0) {
    mpla_set_gaussian_kernel_rhs(&b, &A, inst);
  } else {
    mpla_set_generic_system_rhs(&b, &A, inst);
  }
  mpla_vector_set_zero(&x, inst);
  if (which == 2)
    mpla_generic_BiCGSTAB_with_checkpoint_restart(&b, &A, &x, 5000, 1e-10, core, 100000, false, inst);
  else
    mpla_generic_conjugate_gradient_with_checkpoint_restart(&b, &A, &x, 20000, 1e-10, core, 100000, false, inst);
  std::vector<double> xh = to_host(&x);
  std::vector<double> bh = to_host(&b);
  FILE* f = fopen(out_path, "wb");
  fwrite(xh.data(), 8, n, f);
  fwrite(bh.data(), 8, n, f);
  fclose(f);
  if (assem_d_p) {
    destroy_gaussian_kernel_system_assembler_object(assem_d_p);
    cudaFree(assem_d_p);
  }
  for (double* p : hp) cudaFree(p);
  cudaFree(points);
  mpla_free_generic_matrix(&A, inst);
  mpla_free_vector(&x, inst);
  mpla_free_vector(&b, inst);
  printf("RESULT ok 1\n");
  return 0;
}

int main(int argc, char* argv[]) {
  if (argc < 2) return 2;
  MPI_Init(&argc, &argv);
  mpla_instance instance;
  mpla_init_instance(&instance, MPI_COMM_WORLD);
  int rc = 2;
  const char* mode = argv[1];
  if (!strcmp(mode, "kat")) rc = mode_kat(&instance, atoi(argv[2]), atoi(argv[3]));
  else if (!strcmp(mode, "cg_tridiag")) rc = mode_cg_tridiag(&instance, atoi(argv[2]));
  else if (!strcmp(mode, "cg_checkpoint")) rc = mode_cg_checkpoint(&instance, atoi(argv[2]), atoi(argv[3]));
  else if (!strcmp(mode, "kernel")) rc = mode_kernel(&instance, argv[2], argv[3], argv[4], atoi(argv[5]), atof(argv[6]));
  mpla_destroy_instance(&instance);
  MPI_Finalize();
  return rc;
}
