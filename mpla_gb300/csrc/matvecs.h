// Matvec adapters used by the solver drivers and the mpla.h cores.
#pragma once

#include "internal.h"

namespace mgb {

// Scaled copy of a Gaussian system's coordinates (gauss_f64.cu).
struct ScaledCoords {
  double* buf = nullptr;
  const double* ptr[3] = {nullptr, nullptr, nullptr};
  const double* const* dev_ptrs = nullptr;
};
int prepare_scaled_coords(DeviceContext* c, const GaussSystem& g, ScaledCoords* out, cudaStream_t s);
void release_scaled_coords(DeviceContext* c, ScaledCoords* sc);
int launch_gauss_f64_scaled(DeviceContext* c, const GaussSystem& g, const double* const* scaled,
                            const double* const* scaled_dev_ptrs, const double* x, double* y,
                            cudaStream_t s, const int* skip);
int make_gauss_system(int n, int dim, const double* const* coords, double nugget, int rule, GaussSystem* g);

// Dense column-major matrix through the library's dgemv.
class DenseMatvec : public Matvec {
 public:
  DenseMatvec(DeviceContext* c, int n, const double* A, int lda) : c_(c), n_(n), A_(A), lda_(lda) {}
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return n_; }
  bool graph_key(std::vector<uintptr_t>* key) const override {
    key->insert(key->end(), {1u, (uintptr_t)n_, (uintptr_t)A_, (uintptr_t)lda_, (uintptr_t)c_->split_partials,
                             (uintptr_t)c_->split_partials_count, (uintptr_t)c_->tickets, (uintptr_t)c_->dev_error});
    return true;
  }

 private:
  DeviceContext* c_;
  int n_;
  const double* A_;
  int lda_;
};

// Gaussian kernel matrix, FP64 fused matvec: the symmetric tile-pair kernel
// for square systems with d <= 3 and the diagonal nugget, the rectangular
// kernel otherwise (kernel.cu nugget rule, d > 3).
class GaussF64Matvec : public Matvec {
 public:
  ~GaussF64Matvec() override;
  int init(DeviceContext* c, const GaussSystem& g, cudaStream_t s);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return g_.rows; }
  // kernel entries one apply evaluates
  long long evaluated() const { return evaluated_; }

 private:
  DeviceContext* c_ = nullptr;
  GaussSystem g_{};
  ScaledCoords sc_;
  Matvec* sym_ = nullptr;
  long long evaluated_ = 0;
};

// Gaussian kernel matrix, FP32/SFU symmetric matvec (square systems).
class GaussMixedMatvec : public Matvec {
 public:
  ~GaussMixedMatvec() override;
  int init(DeviceContext* c, const GaussSystem& g, cudaStream_t s);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return n_; }
  long long evaluated() const { return evaluated_; }

 private:
  Matvec* impl_ = nullptr;
  long long evaluated_ = 0;
  int n_ = 0;
};

}  // namespace mgb
