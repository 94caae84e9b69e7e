// Symmetric tile-pair Gaussian matvecs (gauss_sym.cu) for square systems.
#pragma once

#include "internal.h"

namespace mgb {

int sym_tiles(int n);

// FP64: the plain-CG operator.
class SymF64 : public Matvec {
 public:
  ~SymF64() override;
  int init(DeviceContext* c, const GaussSystem& g);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return g_.rows; }

 private:
  DeviceContext* c_ = nullptr;
  GaussSystem g_{};
  int T_ = 0;
  double* S_ = nullptr;  // T x T x 128 slot partials
};

// FP32 + SFU on Morton-ordered, tile-centred points: the mixed-CG operator.
class SymF32 : public Matvec {
 public:
  ~SymF32() override;
  int init(DeviceContext* c, const GaussSystem& g, cudaStream_t s);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return n_; }

 private:
  DeviceContext* c_ = nullptr;
  int n_ = 0, dim_ = 0, T_ = 0;
  double nugget_ = 0.0;
  float4* pts_ = nullptr;     // T*128 points relative to their tile centre (pool block, also holds centres/perm)
  double* centers_ = nullptr; // 3 per tile
  int* perm_ = nullptr;       // sorted position -> original index
  float* S_ = nullptr;        // T x T x 128 slot partials (pool block, also holds xf_)
  float* xf_ = nullptr;       // x gathered into sorted order, FP32
};

}  // namespace mgb
