// A user of the drop-in API with its own system_assembler subclass, written
// the way MPLA's benchmark_generic_system_cg.cpp and its Gaussian assembler
// are (src/kernel_system_assembler.h:10-50, .cu:10-36): an inverse
// multiquadric kernel with a diagonal shift,
//   K(i,j) = 1 / sqrt(c2 + |p_i - p_j|^2) + shift [i == j],
// constructed on the device heap by a kernel of this module, and handed to
// the generic cores through mpla_generic_matrix::data.  Built with -rdc and
// linked with lib/mpla_generic_device.o, as MPLA's Makefile device-links
// generic_system_adapter.o with its users.
//
//   user_assembler matvec <dir> <n> <dim>  writes <dir>/y.bin (K x) and <dir>/rhs.bin
//   user_assembler cg <dir> <n> <dim>      writes <dir>/x.bin (CG on K x = b)
// Inputs: <dir>/pts.bin (dim x n, structure of arrays), x.in.bin or b.bin.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mpla.h"
#include "mpi.h"
#include "system_assembler.h"
#include "generic_system_adapter.h"

class imq_system_assembler : public system_assembler {
 public:
  double** points;
  int dim;
  double c2;
  double shift;

  __device__ double get_matrix_entry(int i, int j) {
    double sq = c2;
    for (int d = 0; d < dim; d++) {
      const double diff = points[d][i] - points[d][j];
      sq = __dadd_rn(sq, __dmul_rn(diff, diff));
    }
    const double k = 1.0 / sqrt(sq);
    return (i == j) ? k + shift : k;
  }

  __device__ double get_rhs_entry(int i) { return 1.0 + points[0][i]; }
};

__global__ void create_imq(imq_system_assembler** out, double** points, int dim, double c2, double shift) {
  imq_system_assembler* a = new imq_system_assembler();
  a->points = points;
  a->dim = dim;
  a->c2 = c2;
  a->shift = shift;
  a->max_row_count_per_dgemv = 1 << 20;
  *out = a;
}

__global__ void destroy_imq(imq_system_assembler** obj) { delete *obj; }

static std::vector<double> read_file(const std::string& path, size_t count) {
  std::vector<double> v(count);
  FILE* f = fopen(path.c_str(), "rb");
  if (!f || fread(v.data(), sizeof(double), count, f) != count) {
    fprintf(stderr, "cannot read %s\n", path.c_str());
    exit(2);
  }
  fclose(f);
  return v;
}

static void write_file(const std::string& path, const std::vector<double>& v) {
  FILE* f = fopen(path.c_str(), "wb");
  fwrite(v.data(), sizeof(double), v.size(), f);
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const std::string mode = argv[1], dir = argv[2];
  const int n = atoi(argv[3]), dim = atoi(argv[4]);
  MPI_Init(&argc, &argv);
  mpla_instance inst;
  mpla_init_instance(&inst, MPI_COMM_WORLD);

  std::vector<double> pts = read_file(dir + "/pts.bin", (size_t)dim * n);
  std::vector<double*> cols(dim);
  for (int d = 0; d < dim; ++d) {
    cudaMalloc((void**)&cols[d], sizeof(double) * n);
    cudaMemcpy(cols[d], pts.data() + (size_t)d * n, sizeof(double) * n, cudaMemcpyHostToDevice);
  }
  double** dpoints = nullptr;
  cudaMalloc((void**)&dpoints, sizeof(double*) * dim);
  cudaMemcpy(dpoints, cols.data(), sizeof(double*) * dim, cudaMemcpyHostToDevice);
  imq_system_assembler** dobj = nullptr;
  cudaMalloc((void**)&dobj, sizeof(*dobj));
  create_imq<<<1, 1>>>(dobj, dpoints, dim, 0.25, 5.0);
  imq_system_assembler* obj = nullptr;
  cudaMemcpy(&obj, dobj, sizeof(obj), cudaMemcpyDeviceToHost);
  checkCUDAError("create_imq");

  mpla_generic_matrix A;
  mpla_init_generic_matrix(&A, &inst, n, n);
  A.data = obj;
  mpla_vector x, y;
  mpla_init_vector(&x, &inst, n);
  mpla_init_vector(&y, &inst, n);

  if (mode == "matvec") {
    std::vector<double> xh = read_file(dir + "/x.in.bin", n), yh(n);
    cudaMemcpy(x.data, xh.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    mpla_generic_dgemv(&y, &A, &x, &mpla_dgemv_core_generic_system_matrix_streamed_cublas, &inst);
    cudaMemcpy(yh.data(), y.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
    write_file(dir + "/y.bin", yh);
    mpla_generic_dgemv(&y, &A, &x, &mpla_dgemv_core_generic_system_matrix_cublas, &inst);
    cudaMemcpy(yh.data(), y.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
    write_file(dir + "/y2.bin", yh);
    mpla_set_generic_system_rhs(&y, &A, &inst);
    cudaMemcpy(yh.data(), y.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
    write_file(dir + "/rhs.bin", yh);
  } else if (mode == "cg") {
    std::vector<double> bh = read_file(dir + "/b.bin", n), xh(n, 0.0);
    cudaMemcpy(y.data, bh.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    mpla_vector_set_zero(&x, &inst);
    mpla_generic_conjugate_gradient_with_checkpoint_restart(&y, &A, &x, 5000, 1e-10,
                                                            &mpla_dgemv_core_generic_system_matrix_streamed_cublas,
                                                            1 << 30, false, &inst);
    cudaMemcpy(xh.data(), x.data, sizeof(double) * n, cudaMemcpyDeviceToHost);
    write_file(dir + "/x.bin", xh);
  } else {
    return 2;
  }
  checkCUDAError("user_assembler");
  destroy_imq<<<1, 1>>>(dobj);
  cudaDeviceSynchronize();
  mpla_free_generic_matrix(&A, &inst);
  mpla_free_vector(&x, &inst);
  mpla_free_vector(&y, &inst);
  for (double* p : cols) cudaFree(p);
  cudaFree(dpoints);
  cudaFree(dobj);
  mpla_destroy_instance(&inst);
  MPI_Finalize();
  printf("RESULT ok 1\n");
  return 0;
}
