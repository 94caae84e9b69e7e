// Harness around the reference MPLA, compiled together with the reference's
// own sources into oracle/_ref/libmplaref.so by oracle/build_ref.py.  TEST
// INFRASTRUCTURE: it drives the unmodified reference through its public API
// (mpla.h, kernel.h, generic_system_adapter.h, kernel_system_assembler.h)
// so tests can pin the oracle against the reference's outputs and bench.py's
// reference arm can time it.  Nothing in the product links this.
//
// All entry points take host arrays, return 0 on success, and silence the
// reference's stdout progress lines while it runs.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <unistd.h>
#include <fcntl.h>

#include <cuda_runtime.h>

#include "mpla.h"
#include "kernel.h"
#include "generic_system_adapter.h"
#include "kernel_system_assembler.h"

namespace {

mpla_instance g_inst;
bool g_ready = false;
long g_core_calls = 0;
void (*g_inner_core)(mpla_vector*, mpla_generic_matrix*, mpla_vector*, mpla_instance*) = nullptr;

// Counts matvecs, then forwards to the reference core being measured.
void counting_core(mpla_vector* b, mpla_generic_matrix* A, mpla_vector* x, mpla_instance* inst) {
  ++g_core_calls;
  g_inner_core(b, A, x, inst);
}

// The user core of the reference's own tests (test_cg.cpp:38-43).
void cublas_dense_core(mpla_vector* b, mpla_generic_matrix* A, mpla_vector* x, mpla_instance* inst) {
  double one = 1, zero = 0;
  cublasDgemv(inst->cublas_handle, CUBLAS_OP_N, A->cur_proc_row_count, A->cur_proc_col_count, &one,
              (double*)(A->data), A->cur_proc_row_count, x->data, 1, &zero, b->data, 1);
}

struct Quiet {
  int saved = -1;
  Quiet() {
    fflush(stdout);
    saved = dup(1);
    int nul = open("/dev/null", O_WRONLY);
    if (nul >= 0) {
      dup2(nul, 1);
      close(nul);
    }
  }
  ~Quiet() {
    fflush(stdout);
    if (saved >= 0) {
      dup2(saved, 1);
      close(saved);
    }
  }
};

__global__ void set_regularization(gaussian_kernel_system_assembler* a, double reg) { a->regularization = reg; }

struct DevicePoints {
  std::vector<double*> cols;
  double** dev = nullptr;
  DevicePoints(int n, int dim, const double* host_soa) {
    cols.resize(dim);
    for (int d = 0; d < dim; ++d) {
      cudaMalloc((void**)&cols[d], sizeof(double) * n);
      cudaMemcpy(cols[d], host_soa + (size_t)d * n, sizeof(double) * n, cudaMemcpyHostToDevice);
    }
    cudaMalloc((void**)&dev, sizeof(double*) * dim);
    cudaMemcpy(dev, cols.data(), sizeof(double*) * dim, cudaMemcpyHostToDevice);
  }
  ~DevicePoints() {
    for (double* p : cols) cudaFree(p);
    cudaFree(dev);
  }
};

// Rows per materialised block: the int index of gen_generic_system_matrix
// (generic_system_adapter.cu:9-15) must stay below 2^31, and the block must
// fit in 90 % of free memory.
int safe_max_rows(int n) {
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  long long by_mem = (long long)(0.9 * (double)free_b / (8.0 * n));
  long long by_int = (2147483647LL / n) - 1;
  long long r = by_mem < by_int ? by_mem : by_int;
  if (r > n) r = n;
  return (int)(r < 1 ? 1 : r);
}

struct Assembler {
  gaussian_kernel_system_assembler** dp = nullptr;
  gaussian_kernel_system_assembler* obj = nullptr;
  Assembler(double** points, int n, int dim, double reg) {
    cudaMalloc((void**)&dp, sizeof(*dp));
    create_gaussian_kernel_system_assembler_object(dp, points, safe_max_rows(n), dim);
    cudaMemcpy(&obj, dp, sizeof(obj), cudaMemcpyDeviceToHost);
    set_regularization<<<1, 1>>>(obj, reg);
    cudaDeviceSynchronize();
  }
  ~Assembler() {
    destroy_gaussian_kernel_system_assembler_object(dp);
    cudaFree(dp);
  }
};

int check() {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "reference harness: %s\n", cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

void vec_from_host(mpla_vector* v, const double* h, int n) {
  mpla_init_vector(v, &g_inst, n);
  cudaMemcpy(v->data, h, sizeof(double) * n, cudaMemcpyHostToDevice);
}

}  // namespace

extern "C" {

int ref_init(int device) {
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  if (!g_ready) {
    int argc = 0;
    char** argv = nullptr;
    MPI_Init(&argc, &argv);
    mpla_init_instance(&g_inst, MPI_COMM_WORLD);
    g_ready = true;
  }
  return check();
}

// y = A x through mpla_dgemv (mpla.cpp:716-751), `reps` times; mean ms.
int ref_dgemv(int m, int n, const double* A, const double* x, double* y, int reps, double* ms) {
  mpla_matrix Am;
  mpla_init_matrix(&Am, &g_inst, m, n);
  cudaMemcpy(Am.data, A, sizeof(double) * (size_t)m * n, cudaMemcpyHostToDevice);
  mpla_vector xv, yv;
  vec_from_host(&xv, x, n);
  mpla_init_vector(&yv, &g_inst, m);
  mpla_dgemv(&yv, &Am, &xv, &g_inst);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, 0);
  for (int r = 0; r < reps; ++r) mpla_dgemv(&yv, &Am, &xv, &g_inst);
  cudaEventRecord(e1, 0);
  cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = reps > 0 ? t / reps : 0.0;
  cudaMemcpy(y, yv.data, sizeof(double) * m, cudaMemcpyDeviceToHost);
  mpla_free_matrix(&Am, &g_inst);
  mpla_free_vector(&xv, &g_inst);
  mpla_free_vector(&yv, &g_inst);
  return check();
}

// The cuBLAS call inside mpla_dgemv (mpla.cpp:729) on its own: cublasDgemv
// OP_N with the instance's handle on resident A, x, y, `reps` times; mean ms.
int ref_cublas_dgemv(int n, const double* A, int reps, double* ms) {
  double *dA = nullptr, *dx = nullptr, *dy = nullptr;
  cudaMalloc((void**)&dA, sizeof(double) * (size_t)n * n);
  cudaMalloc((void**)&dx, sizeof(double) * n);
  cudaMalloc((void**)&dy, sizeof(double) * n);
  cudaMemcpy(dA, A, sizeof(double) * (size_t)n * n, cudaMemcpyHostToDevice);
  cudaMemset(dx, 0, sizeof(double) * n);
  const double one = 1.0, zero = 0.0;
  cublasDgemv(g_inst.cublas_handle, CUBLAS_OP_N, n, n, &one, dA, n, dx, 1, &zero, dy, 1);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, 0);
  for (int r = 0; r < reps; ++r) cublasDgemv(g_inst.cublas_handle, CUBLAS_OP_N, n, n, &one, dA, n, dx, 1, &zero, dy, 1);
  cudaEventRecord(e1, 0);
  cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = reps > 0 ? t / reps : 0.0;
  cudaFree(dA);
  cudaFree(dx);
  cudaFree(dy);
  return check();
}

int ref_ddot(int n, const double* x, const double* y, double* out) {
  mpla_vector xv, yv;
  vec_from_host(&xv, x, n);
  vec_from_host(&yv, y, n);
  mpla_ddot(out, &xv, &yv, &g_inst);
  mpla_free_vector(&xv, &g_inst);
  mpla_free_vector(&yv, &g_inst);
  return check();
}

// Krylov solve on a dense matrix with the cuBLAS user core.
// solver: 0 = CG with checkpoint/restart entry (relative rule), 1 = CG (RMS rule), 2 = BiCGSTAB.
int ref_solve_dense(int n, const double* A, const double* b, double* x, int iter_max, double eps, int solver,
                    int* matvecs, double* ms) {
  mpla_matrix Am;
  mpla_init_matrix(&Am, &g_inst, n, n);
  cudaMemcpy(Am.data, A, sizeof(double) * (size_t)n * n, cudaMemcpyHostToDevice);
  mpla_vector bv, xv;
  vec_from_host(&bv, b, n);
  vec_from_host(&xv, x, n);
  g_core_calls = 0;
  g_inner_core = &cublas_dense_core;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  {
    Quiet q;
    cudaEventRecord(e0, 0);
    mpla_generic_matrix* G = (mpla_generic_matrix*)&Am;
    if (solver == 0)
      mpla_generic_conjugate_gradient_with_checkpoint_restart(&bv, G, &xv, iter_max, eps, &counting_core, 1 << 30,
                                                              false, &g_inst);
    else if (solver == 1)
      mpla_generic_conjugate_gradient(&bv, G, &xv, iter_max, eps, &counting_core, &g_inst);
    else
      mpla_generic_BiCGSTAB_with_checkpoint_restart(&bv, G, &xv, iter_max, eps, &counting_core, 1 << 30, false,
                                                    &g_inst);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
  }
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  if (matvecs) *matvecs = (int)g_core_calls;
  cudaMemcpy(x, xv.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
  mpla_free_matrix(&Am, &g_inst);
  mpla_free_vector(&bv, &g_inst);
  mpla_free_vector(&xv, &g_inst);
  return check();
}

// y = K x for a Gaussian system through the reference cores:
// rule 0: gaussian_kernel_system_assembler + generic streamed core (nugget on i == j);
// rule 1: kernel_matrix_data + mpla_dgemv_core_kernel_streamed_cublas (kernel.cu rule).
int ref_gauss_matvec(int n, int dim, const double* pts, double nugget, int rule, const double* x, double* y) {
  DevicePoints P(n, dim, pts);
  mpla_generic_matrix A;
  mpla_init_generic_matrix(&A, &g_inst, n, n);
  mpla_vector xv, yv;
  vec_from_host(&xv, x, n);
  mpla_init_vector(&yv, &g_inst, n);
  if (rule == 0) {
    Assembler as(P.dev, n, dim, nugget);
    A.data = as.obj;
    mpla_generic_dgemv(&yv, &A, &xv, &mpla_dgemv_core_generic_system_matrix_streamed_cublas, &g_inst);
    cudaDeviceSynchronize();
  } else {
    kernel_matrix_data kd;
    kd.points = P.dev;
    kd.dim = dim;
    kd.max_row_count_per_dgemv = safe_max_rows(n);
    A.data = &kd;
    mpla_generic_dgemv(&yv, &A, &xv, &mpla_dgemv_core_kernel_streamed_cublas, &g_inst);
    cudaDeviceSynchronize();
  }
  cudaMemcpy(y, yv.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
  mpla_free_generic_matrix(&A, &g_inst);
  mpla_free_vector(&xv, &g_inst);
  mpla_free_vector(&yv, &g_inst);
  return check();
}

// Right-hand side of the reference plugins: rule 0 through the assembler's
// get_rhs_entry (mpla_set_generic_system_rhs), rule 1 through
// gen_gaussian_kernel_rhs (mpla_set_gaussian_kernel_rhs).
int ref_gauss_rhs(int n, int dim, const double* pts, int rule, double* b) {
  DevicePoints P(n, dim, pts);
  mpla_generic_matrix A;
  mpla_init_generic_matrix(&A, &g_inst, n, n);
  mpla_vector bv;
  mpla_init_vector(&bv, &g_inst, n);
  if (rule == 0) {
    Assembler as(P.dev, n, dim, 0.0);
    A.data = as.obj;
    mpla_set_generic_system_rhs(&bv, &A, &g_inst);
  } else {
    kernel_matrix_data kd;
    kd.points = P.dev;
    kd.dim = dim;
    kd.max_row_count_per_dgemv = n;
    A.data = &kd;
    mpla_set_gaussian_kernel_rhs(&bv, &A, &g_inst);
  }
  cudaMemcpy(b, bv.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
  mpla_free_generic_matrix(&A, &g_inst);
  mpla_free_vector(&bv, &g_inst);
  return check();
}

// Gaussian solve with the assembler plugin (nugget on the diagonal).
// solver as in ref_solve_dense.  x holds x0 on entry.
int ref_solve_gauss(int n, int dim, const double* pts, double nugget, const double* b, double* x, int iter_max,
                    double eps, int solver, int* matvecs, double* ms) {
  DevicePoints P(n, dim, pts);
  Assembler as(P.dev, n, dim, nugget);
  mpla_generic_matrix A;
  mpla_init_generic_matrix(&A, &g_inst, n, n);
  A.data = as.obj;
  mpla_vector bv, xv;
  vec_from_host(&bv, b, n);
  vec_from_host(&xv, x, n);
  g_core_calls = 0;
  g_inner_core = &mpla_dgemv_core_generic_system_matrix_streamed_cublas;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  {
    Quiet q;
    cudaEventRecord(e0, 0);
    if (solver == 0)
      mpla_generic_conjugate_gradient_with_checkpoint_restart(&bv, &A, &xv, iter_max, eps, &counting_core, 1 << 30,
                                                              false, &g_inst);
    else if (solver == 1)
      mpla_generic_conjugate_gradient(&bv, &A, &xv, iter_max, eps, &counting_core, &g_inst);
    else
      mpla_generic_BiCGSTAB_with_checkpoint_restart(&bv, &A, &xv, iter_max, eps, &counting_core, 1 << 30, false,
                                                    &g_inst);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
  }
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  if (matvecs) *matvecs = (int)g_core_calls;
  cudaMemcpy(x, xv.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
  mpla_free_generic_matrix(&A, &g_inst);
  mpla_free_vector(&bv, &g_inst);
  mpla_free_vector(&xv, &g_inst);
  return check();
}

// Bounded sample for the benchmark: `iters` CG iterations (iter_max = iters+1)
// of the relative-residual CG from x0 = 0; returns the device ms of the
// whole call and the number of matvecs it ran (the r0 matvec plus one per
// iteration), so that the caller divides the time by the matvecs timed.
int ref_cg_gauss_sample(int n, int dim, const double* pts, double nugget, const double* b, int iters, double eps,
                        double* ms, int* matvecs_run) {
  std::vector<double> x(n, 0.0);
  int mv = 0;
  const int st = ref_solve_gauss(n, dim, pts, nugget, b, x.data(), iters + 1, eps, 0, &mv, ms);
  if (matvecs_run) *matvecs_run = mv;
  return st;
}

}  // extern "C"
