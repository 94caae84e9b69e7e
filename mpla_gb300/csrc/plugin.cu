// The plugin interfaces of MPLA on GB300: the kernel.h cores (host
// descriptor, kernel.cu nugget rule), the generic system_assembler adapter,
// the Gaussian assembler factory, and the right-hand-side generators.
//
// The reference materialises row blocks of K and calls cublasDgemv on them
// (kernel.cu:87-171, generic_system_adapter.cu:53-137).  Here:
//   * Gaussian systems — from a kernel_matrix_data descriptor or from an
//     assembler made by this library's factory — run the fused FP64 kernel
//     (no matrix storage, so max_row_count_per_dgemv has nothing to bound);
//   * any other system_assembler is a user subclass whose device code lives
//     in the user's module; its virtual get_matrix_entry is called per entry
//     by a fused kernel of lib/mpla_generic_device.o, which the user
//     device-links into that module (as MPLA's Makefile:96-114 links
//     generic_system_adapter.o) and which registers itself here
//     (mgb_register_generic_device_code); the matrix is never stored.
#include <cstring>
#include <mutex>
#include <set>

#include "../../include/mpla.h"
#include "../../include/kernel.h"
#include "../../include/generic_system_adapter.h"
#include "../../include/kernel_system_assembler.h"
#include "internal.h"
#include "devutil.cuh"
#include "matvecs.h"
#include "plugin.h"

namespace mgb {

namespace {

std::mutex g_registry_mutex;
std::set<const void*> g_gauss_objects;  // device objects created by our factory

void die(int st) {
  if (st != MGB_OK) {
    fprintf(stderr, "MPLA: %s\n", mgb_last_error());
    exit(EXIT_FAILURE);
  }
}

DeviceContext* ctx() {
  DeviceContext* c = nullptr;
  die(context(&c));
  return c;
}

__global__ void k_create_gauss(gaussian_kernel_system_assembler** out, double** points, int max_rows, int dim,
                               double regularization) {
  gaussian_kernel_system_assembler* a = new gaussian_kernel_system_assembler();
  if (a) {
    a->points = points;
    a->max_row_count_per_dgemv = max_rows;
    a->dim = dim;
    a->regularization = regularization;
  }
  *out = a;
}

// The object lives on the device heap (in-kernel new), which runtime copies
// cannot address, so its fields are read by a kernel into pool memory.
struct GaussFields {
  double** points;
  double regularization;
  int dim;
  int max_rows;
};

__global__ void k_read_gauss(const gaussian_kernel_system_assembler* obj, GaussFields* out) {
  out->points = obj->points;
  out->regularization = obj->regularization;
  out->dim = obj->dim;
  out->max_rows = obj->max_row_count_per_dgemv;
}

__global__ void k_destroy_gauss(gaussian_kernel_system_assembler** obj) {
  delete *obj;
  *obj = nullptr;
}

// Generic kernels of the user's module (lib/mpla_generic_device.o), set by
// its static constructor.
std::mutex g_generic_mutex;
const mgb_generic_device_code* g_generic_code = nullptr;

const mgb_generic_device_code* generic_code() {
  std::lock_guard<std::mutex> lock(g_generic_mutex);
  return g_generic_code;
}

constexpr int kGenRows = 128;  // rows per CTA of the device-linked kernel

bool is_library_gauss(const void* obj) {
  std::lock_guard<std::mutex> lock(g_registry_mutex);
  return obj && g_gauss_objects.count(obj);
}

int no_generic_code() {
  return set_error(MGB_ERR_ARG,
                   "system_assembler object not made by this library's factory, and no device-linked generic "
                   "adapter is registered: link lib/mpla_generic_device.o with -rdc=true into the module that "
                   "constructs the assembler");
}

__global__ void k_generic_rhs(system_assembler* assem, int rows, int row_offset, double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < rows) b[i] = assem->get_rhs_entry(row_offset + i);
}

// rhs_i = prod_d (sqrt(pi)/2) (erf(1 - p_d[i]) - erf(-p_d[i]))   (kernel.cu:52-68)
__global__ void k_gauss_rhs(const double* const* __restrict__ points, int dim, int rows, int row_offset,
                            double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const double half_sqrt_pi = 0.88622692545275801365;
  double prod = 1.0;
  for (int d = 0; d < dim; ++d) {
    const double p = points[d][row_offset + i];
    prod = prod * half_sqrt_pi * (erf(1.0 - p) - erf(0.0 - p));
  }
  b[i] = prod;
}

class GenericAssemblerMatvec : public Matvec {
 public:
  GenericAssemblerMatvec(DeviceContext* c, mpla_generic_matrix* A) : c_(c), A_(A) {}
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override {
    const int rows = A_->cur_proc_row_count, cols = A_->cur_proc_col_count;
    if (rows <= 0) return MGB_OK;
    const mgb_generic_device_code* code = generic_code();
    if (!code) return no_generic_code();
    const int tiles = (rows + kGenRows - 1) / kGenRows;
    int nsplit = (8 * c_->num_sms + tiles - 1) / tiles;
    nsplit = max(1, min(nsplit, (cols + 255) / 256));
    const int cps = (cols + nsplit - 1) / nsplit;
    nsplit = (cols + cps - 1) / cps;
    if (nsplit > 1) {
      MGB_TRY(ensure_split_partials(c_, (size_t)nsplit * rows));
      MGB_TRY(ensure_tickets(c_, tiles + 1));
    }
    const int e = code->matvec(A_->data, rows, cols, A_->cur_proc_row_offset, A_->cur_proc_col_offset, x, y, cps,
                               nsplit, c_->split_partials, c_->tickets + 1, skip, s);
    if (e != 0) return cuda_error(static_cast<cudaError_t>(e), "device-linked generic matvec", __FILE__, __LINE__);
    count_launches(1);
    return MGB_OK;
  }
  int n() const override { return A_->cur_proc_row_count; }

 private:
  DeviceContext* c_;
  mpla_generic_matrix* A_;
};

}  // namespace

int kernel_data_system(const kernel_matrix_data* kd, const mpla_generic_matrix* A, GaussSystem* g) {
  if (!kd || !kd->points) return set_error(MGB_ERR_ARG, "kernel_matrix_data without points");
  if (kd->dim < 1 || kd->dim > kMaxGaussDim)
    return set_error(MGB_ERR_ARG, "kernel_matrix_data.dim = %d not in [1,%d]", kd->dim, kMaxGaussDim);
  memset(g, 0, sizeof(*g));
  g->dim = kd->dim;
  MGB_CUDA(cudaMemcpy(g->coords, kd->points, sizeof(double*) * kd->dim, cudaMemcpyDeviceToHost));
  g->rows = A->cur_proc_row_count;
  g->cols = A->cur_proc_col_count;
  g->row_offset = A->cur_proc_row_offset;
  g->col_offset = A->cur_proc_col_offset;
  g->nugget = 1e-8;
  g->nugget_rule = MGB_NUGGET_KERNEL_CU;
  return MGB_OK;
}

int assembler_system(const void* obj, const mpla_generic_matrix* A, GaussSystem* g) {
  {
    std::lock_guard<std::mutex> lock(g_registry_mutex);
    if (!obj || !g_gauss_objects.count(obj)) return set_error(MGB_ERR_ARG, "not a library Gaussian assembler");
  }
  // Field values are read from the device object on every call, so a caller
  // that patches points or regularization in place is honoured.
  DeviceContext* c = nullptr;
  MGB_TRY(context(&c));
  GaussFields* dev = nullptr;
  MGB_TRY(pool_alloc(c, sizeof(GaussFields), (void**)&dev));
  k_read_gauss<<<1, 1, 0, c->stream>>>(static_cast<const gaussian_kernel_system_assembler*>(obj), dev);
  count_launches(1);
  GaussFields h;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, dev, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  pool_free(c, dev);
  if (e != cudaSuccess) return cuda_error(e, "reading the assembler object", __FILE__, __LINE__);
  if (h.dim < 1 || h.dim > kMaxGaussDim)
    return set_error(MGB_ERR_ARG, "assembler dim %d not in [1,%d]", h.dim, kMaxGaussDim);
  memset(g, 0, sizeof(*g));
  g->dim = h.dim;
  MGB_CUDA(cudaMemcpy(g->coords, h.points, sizeof(double*) * h.dim, cudaMemcpyDeviceToHost));
  g->rows = A->cur_proc_row_count;
  g->cols = A->cur_proc_col_count;
  g->row_offset = A->cur_proc_row_offset;
  g->col_offset = A->cur_proc_col_offset;
  g->nugget = h.regularization;
  g->nugget_rule = MGB_NUGGET_DIAGONAL;
  return MGB_OK;
}

Matvec* new_generic_assembler_matvec(DeviceContext* c, mpla_generic_matrix* A) {
  return new GenericAssemblerMatvec(c, A);
}

}  // namespace mgb

using namespace mgb;

// --------------------------------------------------------- kernel.h cores
void mpla_set_gaussian_kernel_rhs(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx();
  const kernel_matrix_data* kd = static_cast<const kernel_matrix_data*>(A->data);
  const int rows = A->cur_proc_row_count;
  k_gauss_rhs<<<(rows + 255) / 256, 256, 0, c->stream>>>(kd->points, kd->dim, rows, A->cur_proc_row_offset, b->data); count_launches(1);
  cudaStreamSynchronize(c->stream);
  checkCUDAError("gen_gaussian_kernel_rhs");
}

static void gauss_core_kernel_data(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x) {
  DeviceContext* c = ctx();
  GaussSystem g;
  die(kernel_data_system(static_cast<const kernel_matrix_data*>(A->data), A, &g));
  die(launch_gauss_f64(c, g, x->data, b->data, c->stream, nullptr));
}

void mpla_dgemv_core_kernel_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist,
                                   struct mpla_instance* instance) {
  (void)instance;
  gauss_core_kernel_data(b, A, x_redist);
}

void mpla_dgemv_core_kernel_streamed_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A,
                                            struct mpla_vector* x_redist, struct mpla_instance* instance) {
  (void)instance;
  gauss_core_kernel_data(b, A, x_redist);
}

void mpla_dgemv_core_dense(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x_redist,
                           struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx();
  die(launch_dgemv(c, A->cur_proc_row_count, A->cur_proc_col_count, static_cast<const double*>(A->data),
                   A->cur_proc_row_count, x_redist->data, b->data, c->stream, nullptr));
}

// ------------------------------------------- generic_system_adapter.h cores
static void generic_core(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_vector* x) {
  DeviceContext* c = ctx();
  GaussSystem g;
  if (assembler_system(A->data, A, &g) == MGB_OK) {
    die(launch_gauss_f64(c, g, x->data, b->data, c->stream, nullptr));
    return;
  }
  GenericAssemblerMatvec M(c, A);
  die(M.apply(x->data, b->data, c->stream, nullptr));
}

void mpla_dgemv_core_generic_system_matrix_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A,
                                                  struct mpla_vector* x_redist, struct mpla_instance* instance) {
  (void)instance;
  generic_core(b, A, x_redist);
}

void mpla_dgemv_core_generic_system_matrix_streamed_cublas(struct mpla_vector* b, struct mpla_generic_matrix* A,
                                                           struct mpla_vector* x_redist, struct mpla_instance* instance) {
  (void)instance;
  generic_core(b, A, x_redist);
}

void mpla_set_generic_system_rhs(struct mpla_vector* b, struct mpla_generic_matrix* A, struct mpla_instance* instance) {
  (void)instance;
  DeviceContext* c = ctx();
  const int rows = A->cur_proc_row_count;
  if (is_library_gauss(A->data)) {
    // constructed in this module: its virtual get_rhs_entry is callable here
    k_generic_rhs<<<(rows + 255) / 256, 256, 0, c->stream>>>(static_cast<system_assembler*>(A->data), rows,
                                                            A->cur_proc_row_offset, b->data);
    count_launches(1);
  } else {
    const mgb_generic_device_code* code = generic_code();
    if (!code) die(no_generic_code());
    const int e = code->rhs(A->data, rows, A->cur_proc_row_offset, b->data, c->stream);
    if (e != 0) die(cuda_error(static_cast<cudaError_t>(e), "device-linked generic rhs", __FILE__, __LINE__));
    count_launches(1);
  }
  cudaStreamSynchronize(c->stream);
  checkCUDAError("gen_generic_system_rhs");
}

extern "C" int mgb_register_generic_device_code(const mgb_generic_device_code* code) {
  if (code && code->abi_version != MGB_GENERIC_DEVICE_ABI)
    return set_error(MGB_ERR_ARG, "generic device code ABI %d, library expects %d", code->abi_version,
                     MGB_GENERIC_DEVICE_ABI);
  if (code && (!code->matvec || !code->rhs)) return set_error(MGB_ERR_ARG, "generic device code without launchers");
  std::lock_guard<std::mutex> lock(g_generic_mutex);
  g_generic_code = code;
  return MGB_OK;
}

extern "C" int mgb_unregister_generic_device_code(const mgb_generic_device_code* code) {
  std::lock_guard<std::mutex> lock(g_generic_mutex);
  if (g_generic_code == code) g_generic_code = nullptr;
  return MGB_OK;
}

// ------------------------------------------ kernel_system_assembler.h factory
void create_gaussian_kernel_system_assembler_object_with_regularization(struct gaussian_kernel_system_assembler** assem,
                                                                       double** points, int max_row_count_per_dgemv,
                                                                       int dim, double regularization) {
  DeviceContext* c = ctx();
  k_create_gauss<<<1, 1, 0, c->stream>>>(assem, points, max_row_count_per_dgemv, dim, regularization); count_launches(1);
  cudaStreamSynchronize(c->stream);
  checkCUDAError("create_gaussian_kernel_system_assembler_object");
  gaussian_kernel_system_assembler* obj = nullptr;
  cudaMemcpy(&obj, assem, sizeof(obj), cudaMemcpyDeviceToHost);
  checkCUDAError("create_gaussian_kernel_system_assembler_object");
  if (!obj) {
    fprintf(stderr, "MPLA: device heap exhausted creating the assembler\n");
    exit(EXIT_FAILURE);
  }
  std::lock_guard<std::mutex> lock(g_registry_mutex);
  g_gauss_objects.insert(obj);
}

void create_gaussian_kernel_system_assembler_object(struct gaussian_kernel_system_assembler** assem, double** points,
                                                    int max_row_count_per_dgemv, int dim) {
  create_gaussian_kernel_system_assembler_object_with_regularization(assem, points, max_row_count_per_dgemv, dim, 0.0);
}

void destroy_gaussian_kernel_system_assembler_object(struct gaussian_kernel_system_assembler** assem) {
  DeviceContext* c = ctx();
  gaussian_kernel_system_assembler* obj = nullptr;
  cudaMemcpy(&obj, assem, sizeof(obj), cudaMemcpyDeviceToHost);
  {
    std::lock_guard<std::mutex> lock(g_registry_mutex);
    g_gauss_objects.erase(obj);
  }
  k_destroy_gauss<<<1, 1, 0, c->stream>>>(assem); count_launches(1);
  cudaStreamSynchronize(c->stream);
  checkCUDAError("destroy_gaussian_kernel_system_assembler_object");
}
