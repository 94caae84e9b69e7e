// The mpla.h API (MPLA src/mpla.h:80-126) on one GB300: the 2-D process grid
// collapses to 1x1, so every Allgatherv / Allreduce of the original
// (mpla.cpp:449-557, 716-804) becomes the identity and no temporary is
// allocated per call.  Containers keep the original field layout and the
// int** block tables so callers that read them keep working.
//
// Error convention of the original: messages to stdout/stderr, then exit().
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "../../include/mpla.h"
#include "../../include/kernel.h"
#include "../../include/generic_system_adapter.h"
#include "internal.h"
#include "matvecs.h"
#include "plugin.h"

using namespace mgb;

namespace {

DeviceContext* ctx_or_exit() {
  DeviceContext* c = nullptr;
  if (context(&c) != MGB_OK) {
    fprintf(stderr, "MPLA: %s\n", mgb_last_error());
    exit(EXIT_FAILURE);
  }
  return c;
}

void die_on(int status) {
  if (status != MGB_OK) {
    fprintf(stderr, "MPLA: %s\n", mgb_last_error());
    exit(EXIT_FAILURE);
  }
}

int** new_table(int value) {
  int** t = new int*[1];
  t[0] = new int[1];
  t[0][0] = value;
  return t;
}

void delete_table(int** t) {
  if (!t) return;
  delete[] t[0];
  delete[] t;
}

// Matvec that calls a user-supplied core each time (not capturable: the
// core may synchronise or call libraries).  At the 1x1 grid x_redist = x.
class ForeignCoreMatvec : public Matvec {
 public:
  ForeignCoreMatvec(mpla_dgemv_core_fn core, mpla_generic_matrix* A, mpla_instance* inst, int n)
      : core_(core), A_(A), inst_(inst), n_(n) {
    memset(&xv_, 0, sizeof(xv_));
    memset(&yv_, 0, sizeof(yv_));
  }
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override {
    (void)skip;
    // The core runs on the legacy default stream; our blocking stream is
    // ordered with it in both directions.
    (void)s;
    fill(&xv_, const_cast<double*>(x));
    fill(&yv_, y);
    core_(&yv_, A_, &xv_, inst_);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "user dgemv core", __FILE__, __LINE__);
    return MGB_OK;
  }
  bool capturable() const override { return false; }
  int n() const override { return n_; }

 private:
  void fill(mpla_vector* v, double* data) {
    v->data = data;
    v->vec_row_count = n_;
    v->vec_col_count = 1;
    v->cur_proc_row_count = n_;
    v->cur_proc_row_offset = 0;
    v->proc_row_count = nullptr;
    v->proc_row_offset = nullptr;
  }
  mpla_dgemv_core_fn core_;
  mpla_generic_matrix* A_;
  mpla_instance* inst_;
  int n_;
  mpla_vector xv_, yv_;
};

// Build the fastest Matvec for a (core, A) pair: the library's own cores are
// recognised by address and replaced by fused device kernels; anything else
// is called as a foreign core.
struct ResolvedMatvec {
  DenseMatvec* dense = nullptr;
  GaussF64Matvec* gauss = nullptr;
  Matvec* generic = nullptr;
  ForeignCoreMatvec* foreign = nullptr;
  Matvec* get() {
    if (dense) return dense;
    if (gauss) return gauss;
    if (generic) return generic;
    return foreign;
  }
  ~ResolvedMatvec() {
    delete dense;
    delete gauss;
    delete generic;
    delete foreign;
  }
};

void resolve(DeviceContext* c, mpla_dgemv_core_fn core, mpla_generic_matrix* A, mpla_instance* inst,
             ResolvedMatvec* out) {
  const int n = A->cur_proc_row_count;
  if (A->cur_proc_row_count != A->cur_proc_col_count) {
    out->foreign = new ForeignCoreMatvec(core, A, inst, n);
    return;
  }
  if (core == &mpla_dgemv_core_dense) {
    out->dense = new DenseMatvec(c, n, static_cast<const double*>(A->data), A->cur_proc_row_count);
    return;
  }
  GaussSystem g;
  if ((core == &mpla_dgemv_core_kernel_streamed_cublas || core == &mpla_dgemv_core_kernel_cublas) &&
      kernel_data_system(static_cast<kernel_matrix_data*>(A->data), A, &g) == MGB_OK) {
    out->gauss = new GaussF64Matvec();
    die_on(out->gauss->init(c, g, c->stream));
    return;
  }
  if (core == &mpla_dgemv_core_generic_system_matrix_streamed_cublas ||
      core == &mpla_dgemv_core_generic_system_matrix_cublas) {
    if (assembler_system(A->data, A, &g) == MGB_OK) {
      out->gauss = new GaussF64Matvec();
      die_on(out->gauss->init(c, g, c->stream));
      return;
    }
    out->generic = new_generic_assembler_matvec(c, A);
    return;
  }
  out->foreign = new ForeignCoreMatvec(core, A, inst, n);
}

void run_cg(mpla_vector* b, mpla_generic_matrix* A, mpla_vector* x, int iter_max, double epsilon,
            mpla_dgemv_core_fn core, mpla_instance* instance, const SolveOptions& o, bool bicgstab) {
  DeviceContext* c = ctx_or_exit();
  ResolvedMatvec rm;
  resolve(c, core, A, instance, &rm);
  mgb_solve_info info;
  memset(&info, 0, sizeof(info));
  SolveOptions opt = o;
  opt.iter_max = iter_max;
  opt.eps = epsilon;
  const int st = bicgstab ? solve_bicgstab(c, *rm.get(), b->data, x->data, opt, &info, c->stream)
                          : solve_cg(c, *rm.get(), b->data, x->data, opt, &info, c->stream);
  if (st != MGB_OK && st != MGB_ERR_NOTCONV && st != MGB_ERR_BREAKDOWN) die_on(st);
  if (st == MGB_ERR_BREAKDOWN) fprintf(stderr, "MPLA: Krylov breakdown after %d iterations.\n", info.iterations);
  if (opt.print_final && instance->is_parent) {
    // The reference reports the loop counter: the converging iteration, or
    // iter_max when the loop ran out.
    const int k = (info.status == MGB_OK) ? info.iterations : iter_max;
    printf("MPLA CG stopped after %d iterations with a final relative residual norm of %le.\n", k,
           info.final_res);
  }
}

}  // namespace

void info() { printf("Hello world\n"); }

static void init_instance_1x1(struct mpla_instance* instance, MPI_Comm comm) {
  instance->comm = comm;
  instance->proc_count = 1;
  instance->proc_rows = 1;
  instance->proc_cols = 1;
  instance->cur_proc_coord[0] = 0;
  instance->cur_proc_coord[1] = 0;
  instance->cur_proc_row = 0;
  instance->cur_proc_col = 0;
  instance->cur_proc_rank = 0;
  instance->is_parent = true;
  ctx_or_exit();
  // kept for user cores that call cuBLAS through the instance
  cublasCreate(&(instance->cublas_handle));
}

void mpla_init_instance(struct mpla_instance* instance, MPI_Comm comm) { init_instance_1x1(instance, comm); }

void mpla_init_instance_block_rows(struct mpla_instance* instance, MPI_Comm comm) {
  init_instance_1x1(instance, comm);
}

void mpla_destroy_instance(struct mpla_instance* instance) { cublasDestroy(instance->cublas_handle); }

void mpla_init_matrix(struct mpla_matrix* matrix, struct mpla_instance* instance, int mat_row_count,
                      int mat_col_count) {
  (void)instance;
  if (mat_row_count < 1) {
    printf("MPLA: There are more process block rows than matrix rows. Exiting...\n");
    exit(1);
  }
  matrix->mat_row_count = mat_row_count;
  matrix->mat_col_count = mat_col_count;
  matrix->cur_proc_row_count = mat_row_count;
  matrix->cur_proc_col_count = mat_col_count;
  matrix->cur_proc_row_offset = 0;
  matrix->cur_proc_col_offset = 0;
  matrix->proc_row_count = new_table(mat_row_count);
  matrix->proc_col_count = new_table(mat_col_count);
  matrix->proc_row_offset = new_table(0);
  matrix->proc_col_offset = new_table(0);
  cudaMalloc((void**)&(matrix->data), sizeof(double) * (size_t)mat_row_count * (size_t)mat_col_count);
  cudaDeviceSynchronize();
  checkCUDAError("cudaMalloc");
}

void mpla_init_generic_matrix(struct mpla_generic_matrix* matrix, struct mpla_instance* instance,
                              int mat_row_count, int mat_col_count) {
  (void)instance;
  if (mat_row_count < 1) {
    printf("MPLA: There are more process block rows than matrix rows. Exiting...\n");
    exit(1);
  }
  matrix->mat_row_count = mat_row_count;
  matrix->mat_col_count = mat_col_count;
  matrix->cur_proc_row_count = mat_row_count;
  matrix->cur_proc_col_count = mat_col_count;
  matrix->cur_proc_row_offset = 0;
  matrix->cur_proc_col_offset = 0;
  matrix->proc_row_count = new_table(mat_row_count);
  matrix->proc_col_count = new_table(mat_col_count);
  matrix->proc_row_offset = new_table(0);
  matrix->proc_col_offset = new_table(0);
  // the user owns matrix->data
}

static void init_vector_1x1(struct mpla_vector* vector, int vec_row_count, const char* what) {
  if (vec_row_count < 1) {
    printf("%s", what);
    exit(1);
  }
  vector->vec_row_count = vec_row_count;
  vector->cur_proc_row_count = vec_row_count;
  vector->cur_proc_row_offset = 0;
  vector->proc_row_count = new_table(vec_row_count);
  vector->proc_row_offset = new_table(0);
  cudaMalloc((void**)&(vector->data), sizeof(double) * (size_t)vec_row_count);
  cudaDeviceSynchronize();
  checkCUDAError("cudaMalloc");
}

void mpla_init_vector(struct mpla_vector* vector, struct mpla_instance* instance, int vec_row_count) {
  (void)instance;
  init_vector_1x1(vector, vec_row_count, "MPLA: There are more process block rows than vector rows. Exiting...\n");
}

void mpla_init_vector_for_block_rows(struct mpla_vector* vector, struct mpla_instance* instance,
                                     int vec_row_count) {
  (void)instance;
  init_vector_1x1(vector, vec_row_count,
                  "MPLA: There are more process block columns than matrix columns. Exiting...\n");
}

void mpla_redistribute_vector_for_dgesv(struct mpla_vector* b_redist, struct mpla_vector* b, struct mpla_matrix* A,
                                        struct mpla_instance* instance) {
  (void)A;
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  cudaMemcpyAsync(b_redist->data, b->data, sizeof(double) * b_redist->cur_proc_row_count, cudaMemcpyDeviceToDevice,
                  c->stream);
}

void mpla_redistribute_vector_for_generic_dgesv(struct mpla_vector* b_redist, struct mpla_vector* b,
                                                struct mpla_generic_matrix* A, struct mpla_instance* instance) {
  mpla_redistribute_vector_for_dgesv(b_redist, b, reinterpret_cast<mpla_matrix*>(A), instance);
}

void mpla_save_vector(struct mpla_vector* x, char* filename, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  die_on(save_vector_file(filename, x->vec_row_count, x->data, c->stream));
}

void mpla_load_vector(struct mpla_vector* x, char* filename, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  const int st = load_vector_file(filename, x->vec_row_count, x->data, c->stream);
  if (st == MGB_ERR_IO && strstr(mgb_last_error(), "expected")) {
    printf("Loaded vector does not fit to vector size required by the program.\n");
    fflush(stdout);
    exit(1);
  }
  die_on(st);
}

void mpla_copy_distributed_vector_to_cpu(double* x_cpu, struct mpla_vector* x, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  cudaMemcpyAsync(x_cpu, x->data, sizeof(double) * x->cur_proc_row_count, cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  checkCUDAError("mpla_copy_distributed_vector_to_cpu");
}

void mpla_free_vector(struct mpla_vector* x, struct mpla_instance* instance) {
  (void)instance;
  cudaFree(x->data);
  delete_table(x->proc_row_count);
  delete_table(x->proc_row_offset);
}

void mpla_free_matrix(struct mpla_matrix* A, struct mpla_instance* instance) {
  (void)instance;
  cudaFree(A->data);
  delete_table(A->proc_row_count);
  delete_table(A->proc_row_offset);
  delete_table(A->proc_col_count);
  delete_table(A->proc_col_offset);
}

void mpla_free_generic_matrix(struct mpla_generic_matrix* A, struct mpla_instance* instance) {
  (void)instance;
  delete_table(A->proc_row_count);
  delete_table(A->proc_row_offset);
  delete_table(A->proc_col_count);
  delete_table(A->proc_col_offset);
}

void mpla_dgemv(struct mpla_vector* b, struct mpla_matrix* A, struct mpla_vector* x, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  die_on(launch_dgemv(c, A->cur_proc_row_count, A->cur_proc_col_count, A->data, A->cur_proc_row_count, x->data,
                      b->data, c->stream, nullptr));
}

void mpla_ddot(double* xy, struct mpla_vector* x, struct mpla_vector* y, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  die_on(mgb_ddot(x->cur_proc_row_count, x->data, y->data, xy, c->stream));
}

void mpla_generic_dgemv(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x,
                        void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*,
                                                struct mpla_instance*),
                        struct mpla_instance* instance) {
  // 1x1 grid: the redistributed x is x itself, and the row Allreduce is the
  // identity.
  mpla_dgemv_core(b, A, x, instance);
}

void mpla_daxpy(struct mpla_vector* y, double alpha, struct mpla_vector* x, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  die_on(launch_axpy(c, x->cur_proc_row_count, alpha, x->data, y->data, c->stream));
}

void mpla_vector_set_zero(struct mpla_vector* x, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx_or_exit();
  cudaMemsetAsync(x->data, 0, sizeof(double) * x->cur_proc_row_count, c->stream);
}

void mpla_generic_conjugate_gradient(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x,
                                     int iter_max, double epsilon,
                                     void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*,
                                                             struct mpla_vector*, struct mpla_instance*),
                                     struct mpla_instance* instance) {
  SolveOptions o;
  o.stop_rule = MGB_STOP_RMS;
  o.print_every = instance->is_parent ? 10 : 0;
  o.print_style = 0;
  run_cg(b, A, x, iter_max, epsilon, mpla_dgemv_core, instance, o, false);
}

void mpla_generic_conjugate_gradient_with_checkpoint_restart(
    struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x, int iter_max, double epsilon,
    void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*,
                            struct mpla_instance*),
    int iterations_until_checkpoint, bool restart, struct mpla_instance* instance) {
  SolveOptions o;
  o.stop_rule = MGB_STOP_RELATIVE;
  o.print_every = instance->is_parent ? 2 : 0;
  o.print_style = 1;
  o.checkpoint_every = iterations_until_checkpoint > 0 ? iterations_until_checkpoint : 0;
  o.restart = restart;
  o.print_final = true;
  run_cg(b, A, x, iter_max, epsilon, mpla_dgemv_core, instance, o, false);
}

void mpla_generic_BiCGSTAB_with_checkpoint_restart(
    struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x, int iter_max, double epsilon,
    void (*mpla_dgemv_core)(struct mpla_vector*, struct mpla_generic_matrix*, struct mpla_vector*,
                            struct mpla_instance*),
    int iterations_until_checkpoint, bool restart, struct mpla_instance* instance) {
  SolveOptions o;
  o.stop_rule = MGB_STOP_RELATIVE;
  o.print_every = instance->is_parent ? 1 : 0;
  o.print_style = 1;
  o.checkpoint_every = iterations_until_checkpoint > 0 ? iterations_until_checkpoint : 0;
  o.restart = restart;
  o.print_final = true;
  run_cg(b, A, x, iter_max, epsilon, mpla_dgemv_core, instance, o, true);
}

void checkCUDAError(const char* msg) {
  cudaError_t err = cudaGetLastError();
  if (cudaSuccess != err) {
    fprintf(stderr, "Cuda error: %s: %s.\n", msg, cudaGetErrorString(err));
    exit(EXIT_FAILURE);
  }
}
