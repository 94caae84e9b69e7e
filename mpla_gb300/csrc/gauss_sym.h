// Symmetric tile-pair Gaussian matvecs (gauss_sym.cu) for square systems.
#pragma once

#include <vector>

#include "internal.h"

namespace mgb {

int sym_tiles(int n);
// Morton (Z-order) permutation of n points (dim x n, structure of arrays):
// sorted position -> original index.
std::vector<int> morton_perm(const std::vector<double>& h, int n, int dim);
// k-d tile order: the points split in two at a multiple of `leaf` along the
// widest axis of their bounding box, recursively, down to tiles of `leaf`
// points laid out left to right.  Its tiles are tighter boxes than runs of
// `leaf` Morton-ordered points, which may straddle two Morton cells: at
// n = 65536, d = 2, l = 0.05 it leaves 10.5 % fewer 128-point tile pairs
// within the 2^-40 cut (13 % at n = 131072, d = 3, l = 0.08).
std::vector<int> kd_tile_perm(const std::vector<double>& h, int n, int dim, int leaf);

// FP64: the plain-CG operator (points in k-d tile order, tile pairs below
// 2^-80 left out).
class SymF64 : public Matvec {
 public:
  ~SymF64() override;
  int init(DeviceContext* c, const GaussSystem& g, cudaStream_t s);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return g_.rows; }
  // kernel entries one apply evaluates (each unordered near pair once)
  long long evaluated() const { return (long long)npairs_ * 128LL * 128LL; }

 private:
  DeviceContext* c_ = nullptr;
  GaussSystem g_{};
  int T_ = 0;
  int npairs_ = 0;
  double* S_ = nullptr;    // T x T x 128 slot partials
  double* pts_ = nullptr;  // 3 x T*128 coordinates in tile order (one pool block with the rest)
  int* perm_ = nullptr;    // tile position -> caller index
  int2* pairs_ = nullptr;  // near tile pairs (I <= J)
};

// FP32 + SFU on points in k-d tile order (packed f32x2 arithmetic): the
// default mixed-CG operator.
class SymF32 : public Matvec {
 public:
  ~SymF32() override;
  int init(DeviceContext* c, const GaussSystem& g, cudaStream_t s);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return n_; }
  // kernel entries (exponentials) one apply evaluates
  long long evaluated() const { return pairs_near_ * 128LL * 128LL; }

 private:
  DeviceContext* c_ = nullptr;
  int n_ = 0, dim_ = 0, T_ = 0, GT_ = 0;
  long long ncta_ = 0;
  long long pairs_near_ = 0;  // tile pairs I <= J evaluated (the rest are below 2^-40)
  double nugget_ = 0.0;
  float4* pts_ = nullptr;     // T*128 scaled FP32 points (pool block, also holds map_ and perm_)
  int2* map_ = nullptr;       // CTA -> (column tile, row-tile group | near mask << 16)
  int* perm_ = nullptr;       // sorted position -> original index
  int* near_off_ = nullptr;   // per row tile I: offsets into near_J_
  int* near_J_ = nullptr;     // column tiles J >= I near tile I
  float* S_ = nullptr;        // row slots T x T x 128 (pool block, also holds Scol_ and xf_)
  float* Scol_ = nullptr;     // column slots T x GT x 128
  float* xf_ = nullptr;       // x gathered into sorted order, FP32
};

// FP32 + SFU with the squared distances as a BF16 tensor-core contraction
// (gauss_tc.cu): selectable with mgb_set_mixed_matvec.
class SymTC : public Matvec {
 public:
  ~SymTC() override;
  int init(DeviceContext* c, const GaussSystem& g, cudaStream_t s);
  int apply(const double* x, double* y, cudaStream_t s, const int* skip) override;
  int n() const override { return n_; }
  long long evaluated() const { return (long long)T_ * (T_ + 1) / 2 * 128LL * 128LL; }

 private:
  DeviceContext* c_ = nullptr;
  int n_ = 0, dim_ = 0, T_ = 0, GT_ = 0;
  long long ncta_ = 0;
  double nugget_ = 0.0;
  void* block_ = nullptr;           // pool block holding the arrays below
  unsigned char* btiles_ = nullptr; // T column-tile operands (BF16, canonical layout)
  float4* phi_ = nullptr;           // scaled coordinates, FP32 high part (Morton order, whole tiles)
  float4* plo_ = nullptr;           // ... and low part
  float4* ctr_ = nullptr;           // tile centres (FP32)
  int2* map_ = nullptr;             // CTA -> (column tile, row-tile pair)
  int* perm_ = nullptr;             // sorted position -> original index
  float* S_ = nullptr;              // row slots T x T x 128, then column slots, then xf
  float* Scol_ = nullptr;           // column slots T x GT x 128
  float* xf_ = nullptr;             // x gathered into sorted order, FP32
};

}  // namespace mgb
