#include <atomic>
// C ABI of the hot path (mpla_gb300.h): dense BLAS, Gaussian matvecs and the
// solver entry points, plus the Matvec adapters the solvers run on.
#include <cmath>
#include <cstring>

#include "internal.h"
#include "matvecs.h"
#include "gauss_sym.h"

namespace mgb {

int DenseMatvec::apply(const double* x, double* y, cudaStream_t s, const int* skip) {
  return launch_dgemv(c_, n_, n_, A_, lda_, x, y, s, skip);
}

static bool symmetric_ok(const GaussSystem& g) {
  return g.rows == g.cols && g.row_offset == 0 && g.col_offset == 0 && g.dim >= 1 && g.dim <= 3 &&
         g.nugget_rule == MGB_NUGGET_DIAGONAL;
}

GaussF64Matvec::~GaussF64Matvec() {
  delete sym_;
  if (c_) release_scaled_coords(c_, &sc_);
}

int GaussF64Matvec::init(DeviceContext* c, const GaussSystem& g, cudaStream_t s) {
  g_ = g;
  if (symmetric_ok(g)) {
    SymF64* m = new SymF64();
    sym_ = m;
    MGB_TRY(m->init(c, g, s));
    evaluated_ = m->evaluated();
    return MGB_OK;
  }
  c_ = c;
  evaluated_ = (long long)g.rows * g.cols;
  return prepare_scaled_coords(c, g, &sc_, s);
}

int GaussF64Matvec::apply(const double* x, double* y, cudaStream_t s, const int* skip) {
  if (sym_) return sym_->apply(x, y, s, skip);
  return launch_gauss_f64_scaled(c_, g_, sc_.ptr, sc_.dev_ptrs, x, y, s, skip);
}

GaussMixedMatvec::~GaussMixedMatvec() { delete impl_; }

namespace {
std::atomic<int> g_mixed_kind{MGB_MIXED_SIMT};
}

int GaussMixedMatvec::init(DeviceContext* c, const GaussSystem& g, cudaStream_t s) {
  n_ = g.rows;
  if (g_mixed_kind.load() == MGB_MIXED_TENSOR) {
    SymTC* m = new SymTC();
    impl_ = m;
    MGB_TRY(m->init(c, g, s));
    evaluated_ = m->evaluated();
    return MGB_OK;
  }
  SymF32* m = new SymF32();
  impl_ = m;
  MGB_TRY(m->init(c, g, s));
  evaluated_ = m->evaluated();
  return MGB_OK;
}

int GaussMixedMatvec::apply(const double* x, double* y, cudaStream_t s, const int* skip) {
  return impl_->apply(x, y, s, skip);
}

int make_gauss_system(int n, int dim, const double* const* coords, double nugget, int rule, GaussSystem* g) {
  if (n <= 0) return set_error(MGB_ERR_ARG, "n must be positive (got %d)", n);
  if (dim < 1 || dim > kMaxGaussDim) return set_error(MGB_ERR_ARG, "dim %d not in [1,%d]", dim, kMaxGaussDim);
  if (!coords) return set_error(MGB_ERR_ARG, "null coordinate array");
  if (rule != MGB_NUGGET_DIAGONAL && rule != MGB_NUGGET_KERNEL_CU)
    return set_error(MGB_ERR_ARG, "unknown nugget rule %d", rule);
  memset(g, 0, sizeof(*g));
  g->rows = g->cols = n;
  g->dim = dim;
  for (int d = 0; d < dim; ++d) {
    if (!coords[d]) return set_error(MGB_ERR_ARG, "null coordinate pointer for dimension %d", d);
    g->coords[d] = coords[d];
  }
  g->nugget = nugget;
  g->nugget_rule = rule;
  return MGB_OK;
}

// Mean device time per launch over `reps` launches, CUDA events on `s`.
template <class Launch>
static int time_launches(cudaStream_t s, int reps, double* ms_per_launch, Launch launch) {
  if (reps <= 0 || !ms_per_launch) return set_error(MGB_ERR_ARG, "reps must be positive");
  cudaEvent_t e0, e1;
  MGB_CUDA(cudaEventCreate(&e0));
  MGB_CUDA(cudaEventCreate(&e1));
  MGB_TRY(launch());  // warm-up (sizes scratch, loads code)
  MGB_CUDA(cudaEventRecord(e0, s));
  for (int r = 0; r < reps; ++r) MGB_TRY(launch());
  MGB_CUDA(cudaEventRecord(e1, s));
  MGB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  MGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_launch = (double)ms / reps;
  return MGB_OK;
}

}  // namespace mgb

using namespace mgb;

#define MGB_CTX(c)                         \
  DeviceContext* c = nullptr;              \
  MGB_TRY(context(&c))

extern "C" {

int mgb_dgemv(int m, int n, const double* A, int lda, const double* x, double* y, void* stream) {
  MGB_CTX(c);
  if ((m > 0 && n > 0) && (!A || !x || !y)) return set_error(MGB_ERR_ARG, "mgb_dgemv: null pointer");
  return launch_dgemv(c, m, n, A, lda, x, y, pick_stream(c, stream), nullptr);
}

int mgb_ddot(int n, const double* x, const double* y, double* result_host, void* stream) {
  MGB_CTX(c);
  if (n < 0 || !result_host) return set_error(MGB_ERR_ARG, "mgb_ddot: bad arguments");
  if (n == 0) {
    *result_host = 0.0;
    return MGB_OK;
  }
  cudaStream_t s = pick_stream(c, stream);
  double* tmp;
  MGB_TRY(pool_alloc(c, sizeof(double), (void**)&tmp));
  int st = launch_dot(c, n, x, y, tmp, s);
  if (st == MGB_OK) {
    cudaError_t e = cudaMemcpyAsync(result_host, tmp, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_error(e, "ddot readback", __FILE__, __LINE__);
  }
  pool_free(c, tmp);
  return st;
}

int mgb_daxpy(int n, double alpha, const double* x, double* y, void* stream) {
  MGB_CTX(c);
  if (n < 0) return set_error(MGB_ERR_ARG, "mgb_daxpy: negative n");
  return launch_axpy(c, n, alpha, x, y, pick_stream(c, stream));
}

int mgb_gauss_matvec_f64(int rows, int cols, int row_offset, int col_offset, int dim,
                         const double* const* coords, double nugget, int rule, const double* x, double* y,
                         void* stream) {
  MGB_CTX(c);
  if (rows < 0 || cols < 0 || row_offset < 0 || col_offset < 0)
    return set_error(MGB_ERR_ARG, "mgb_gauss_matvec_f64: negative size or offset");
  if (rows == 0) return MGB_OK;
  GaussSystem g;
  MGB_TRY(make_gauss_system(1, dim, coords, nugget, rule, &g));
  g.rows = rows;
  g.cols = cols;
  g.row_offset = row_offset;
  g.col_offset = col_offset;
  cudaStream_t s = pick_stream(c, stream);
  if (cols == 0) {
    MGB_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * rows, s));
    return MGB_OK;
  }
  if (symmetric_ok(g)) {
    GaussF64Matvec A;
    MGB_TRY(A.init(c, g, s));
    MGB_TRY(A.apply(x, y, s, nullptr));
    MGB_CUDA(cudaStreamSynchronize(s));  // the pool block of A is released on return
    return MGB_OK;
  }
  return launch_gauss_f64(c, g, x, y, s, nullptr);
}

int mgb_gauss_matvec_mixed(int n, int dim, const double* const* coords, double nugget, const double* x,
                           double* y, void* stream) {
  MGB_CTX(c);
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, nugget, MGB_NUGGET_DIAGONAL, &g));
  cudaStream_t s = pick_stream(c, stream);
  GaussMixedMatvec A;
  MGB_TRY(A.init(c, g, s));
  MGB_TRY(A.apply(x, y, s, nullptr));
  MGB_CUDA(cudaStreamSynchronize(s));  // the pool blocks of A are released on return
  return MGB_OK;
}

int mgb_gauss_entries_f64(int n, int count, const int* i, const int* j, int dim, const double* const* coords,
                            double nugget, int rule, double* out, void* stream) {
  MGB_CTX(c);
  if (count < 0 || n <= 0) return set_error(MGB_ERR_ARG, "bad sizes");
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, nugget, rule, &g));
  return launch_gauss_entries_f64(c, g, count, i, j, out, pick_stream(c, stream));
}

static void fill_options(SolveOptions* o, int iter_max, double eps, int stop_rule) {
  o->iter_max = iter_max;
  o->eps = eps;
  o->stop_rule = stop_rule;
}

int mgb_cg_dense(int n, const double* A, int lda, const double* b, double* x, int iter_max, double eps,
                 int stop_rule, mgb_solve_info* info, void* stream) {
  MGB_CTX(c);
  if (n <= 0 || lda < n || !A || !b || !x) return set_error(MGB_ERR_ARG, "mgb_cg_dense: bad arguments");
  if (stop_rule != MGB_STOP_RELATIVE && stop_rule != MGB_STOP_RMS)
    return set_error(MGB_ERR_ARG, "unknown stop rule %d", stop_rule);
  DenseMatvec M(c, n, A, lda);
  SolveOptions o;
  fill_options(&o, iter_max, eps, stop_rule);
  o.compute_true_residual = true;
  return solve_cg(c, M, b, x, o, info, pick_stream(c, stream));
}

int mgb_bicgstab_dense(int n, const double* A, int lda, const double* b, double* x, int iter_max, double eps,
                       mgb_solve_info* info, void* stream) {
  MGB_CTX(c);
  if (n <= 0 || lda < n || !A || !b || !x) return set_error(MGB_ERR_ARG, "mgb_bicgstab_dense: bad arguments");
  DenseMatvec M(c, n, A, lda);
  SolveOptions o;
  fill_options(&o, iter_max, eps, MGB_STOP_RELATIVE);
  return solve_bicgstab(c, M, b, x, o, info, pick_stream(c, stream));
}

int mgb_cg_gauss(int n, int dim, const double* const* coords, double nugget, int rule, const double* b, double* x,
                 int iter_max, double eps, int stop_rule, int precision, mgb_solve_info* info, void* stream) {
  MGB_CTX(c);
  if (!b || !x) return set_error(MGB_ERR_ARG, "mgb_cg_gauss: null vector");
  if (stop_rule != MGB_STOP_RELATIVE && stop_rule != MGB_STOP_RMS)
    return set_error(MGB_ERR_ARG, "unknown stop rule %d", stop_rule);
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, nugget, rule, &g));
  cudaStream_t s = pick_stream(c, stream);
  SolveOptions o;
  fill_options(&o, iter_max, eps, stop_rule);
  GaussF64Matvec hi;
  MGB_TRY(hi.init(c, g, s));
  if (precision == MGB_PREC_FP64) {
    o.compute_true_residual = true;
    return solve_cg(c, hi, b, x, o, info, s);
  }
  if (precision != MGB_PREC_MIXED) return set_error(MGB_ERR_ARG, "unknown precision %d", precision);
  GaussMixedMatvec lo;
  MGB_TRY(lo.init(c, g, s));
  return solve_cg_mixed(c, hi, lo, b, x, o, info, s);
}

int mgb_bicgstab_gauss(int n, int dim, const double* const* coords, double nugget, int rule, const double* b,
                       double* x, int iter_max, double eps, mgb_solve_info* info, void* stream) {
  MGB_CTX(c);
  if (!b || !x) return set_error(MGB_ERR_ARG, "mgb_bicgstab_gauss: null vector");
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, nugget, rule, &g));
  cudaStream_t s = pick_stream(c, stream);
  SolveOptions o;
  fill_options(&o, iter_max, eps, MGB_STOP_RELATIVE);
  GaussF64Matvec A;
  MGB_TRY(A.init(c, g, s));
  return solve_bicgstab(c, A, b, x, o, info, s);
}

int mgb_cg_gauss_host(int n, int dim, const double* coords_host, double nugget, const double* b_host,
                      double* x_host, int iter_max, double eps, int precision, mgb_solve_info* info) {
  MGB_CTX(c);
  if (n <= 0 || dim < 1 || dim > 3 || !coords_host || !b_host || !x_host)
    return set_error(MGB_ERR_ARG, "mgb_cg_gauss_host: bad arguments");
  cudaStream_t s = c->stream;
  const double t0 = wall_seconds();
  double* buf = nullptr;
  const size_t nd = (size_t)n * dim;
  MGB_TRY(pool_alloc(c, sizeof(double) * (nd + 2 * (size_t)n), (void**)&buf));
  double* b = buf + nd;
  double* x = b + n;
  int st = MGB_OK;
  cudaError_t e = cudaMemcpyAsync(buf, coords_host, sizeof(double) * nd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b, b_host, sizeof(double) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, x_host, sizeof(double) * n, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = cuda_error(e, "host->device copy", __FILE__, __LINE__);
  if (st == MGB_OK) {
    const double* coords[3] = {buf, dim > 1 ? buf + n : nullptr, dim > 2 ? buf + 2 * (size_t)n : nullptr};
    st = mgb_cg_gauss(n, dim, coords, nugget, MGB_NUGGET_DIAGONAL, b, x, iter_max, eps, MGB_STOP_RELATIVE,
                      precision, info, s);
    if (st == MGB_OK || st == MGB_ERR_NOTCONV) {
      e = cudaMemcpyAsync(x_host, x, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) st = cuda_error(e, "device->host copy", __FILE__, __LINE__);
    }
  }
  pool_free(c, buf);
  if (info) info->seconds = wall_seconds() - t0;
  return st;
}

int mgb_time_gauss_matvec(int n, int dim, const double* const* coords, double nugget, int precision,
                          const double* x, double* y, int reps, double* ms_per_launch, void* stream) {
  MGB_CTX(c);
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, nugget, MGB_NUGGET_DIAGONAL, &g));
  cudaStream_t s = pick_stream(c, stream);
  if (precision == MGB_PREC_FP64) {
    GaussF64Matvec A;
    MGB_TRY(A.init(c, g, s));
    return time_launches(s, reps, ms_per_launch, [&]() { return A.apply(x, y, s, nullptr); });
  }
  if (precision != MGB_PREC_MIXED) return set_error(MGB_ERR_ARG, "unknown precision %d", precision);
  GaussMixedMatvec A;
  MGB_TRY(A.init(c, g, s));
  return time_launches(s, reps, ms_per_launch, [&]() { return A.apply(x, y, s, nullptr); });
}

int mgb_gauss_mixed_work(int n, int dim, const double* const* coords, long long* evaluated) {
  MGB_CTX(c);
  if (!evaluated) return set_error(MGB_ERR_ARG, "mgb_gauss_mixed_work: null output");
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, 0.0, MGB_NUGGET_DIAGONAL, &g));
  GaussMixedMatvec A;
  MGB_TRY(A.init(c, g, c->stream));
  *evaluated = A.evaluated();
  return MGB_OK;
}

int mgb_gauss_fp64_work(int n, int dim, const double* const* coords, long long* evaluated) {
  MGB_CTX(c);
  if (!evaluated) return set_error(MGB_ERR_ARG, "mgb_gauss_fp64_work: null output");
  GaussSystem g;
  MGB_TRY(make_gauss_system(n, dim, coords, 0.0, MGB_NUGGET_DIAGONAL, &g));
  GaussF64Matvec A;
  MGB_TRY(A.init(c, g, c->stream));
  *evaluated = A.evaluated();
  return MGB_OK;
}

int mgb_set_mixed_matvec(int kind) {
  if (kind != MGB_MIXED_TENSOR && kind != MGB_MIXED_SIMT)
    return set_error(MGB_ERR_ARG, "unknown mixed matvec kind %d", kind);
  g_mixed_kind.store(kind);
  return MGB_OK;
}

int mgb_get_mixed_matvec(void) { return g_mixed_kind.load(); }

int mgb_time_dgemv(int n, const double* A, const double* x, double* y, int reps, double* ms_per_launch,
                   void* stream) {
  MGB_CTX(c);
  if (n <= 0 || !A || !x || !y) return set_error(MGB_ERR_ARG, "mgb_time_dgemv: bad arguments");
  cudaStream_t s = pick_stream(c, stream);
  return time_launches(s, reps, ms_per_launch, [&]() { return launch_dgemv(c, n, n, A, n, x, y, s, nullptr); });
}

int mgb_save_vector(const char* path, int n, const double* x) {
  MGB_CTX(c);
  if (!path || n < 0) return set_error(MGB_ERR_ARG, "mgb_save_vector: bad arguments");
  return save_vector_file(path, n, x, c->stream);
}

int mgb_load_vector(const char* path, int n, double* x) {
  MGB_CTX(c);
  if (!path || n < 0) return set_error(MGB_ERR_ARG, "mgb_load_vector: bad arguments");
  return load_vector_file(path, n, x, c->stream);
}

}  // extern "C"
