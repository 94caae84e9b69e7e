// Matrix-free FP64 Gaussian kernel matvec y = K x over a rectangular block
// (rows x cols with offsets; square systems use the symmetric tile-pair
// kernel of gauss_sym.cu, which evaluates each entry pair once).
//
// Replaces the reference's three-pass core (gen_dis_matrix -> apply_kernel ->
// cublasDgemv, MPLA src/kernel.cu:17-50,118-171, and the virtual-call
// assembly of src/generic_system_adapter.cu:7-23,83-137): no block of K is
// ever written to HBM, so per entry the work is pure FP64 arithmetic.
//
// On GB300 the FP64 pipe (about 2 FMA/clk/SM) is the bound, so the kernel
// minimises FP64 instructions per entry:
//   * distances come from the caller's coordinates (one rounding per
//     difference, as in the reference) and are scaled once into the argument
//     t of the table exponential;
//   * exp(-s) uses the 4096-entry table method (devutil.cuh): round, a
//     degree-3 polynomial and one FMA, with the power of two and the range
//     checks done on the integer pipe;
//   * the diagonal nugget is added once per row after the loop instead of
//     being tested on every entry.
// 3 + 2*DIM + 8 FP64 operations per entry (13 for d = 2).
//
// Work layout: a CTA owns 256 rows (128 threads x 2 rows in registers) and a
// column range; source tiles of 128 points (coordinates + x values) and the
// exp table live in shared memory.  Column ranges are reduced by the
// last-arriving CTA of each row tile in a fixed order.
#include "internal.h"
#include "devutil.cuh"
#include "matvecs.h"

namespace mgb {

namespace {

constexpr int kThreads = 128;
constexpr int kRowsPerThread = 2;
constexpr int kRowsPerCta = kThreads * kRowsPerThread;
constexpr int kTileJ = 128;
constexpr int kMaxDim = 16;

// t = scaled squared distance (t = s * 4096/ln2 for squared distance s).
__device__ __forceinline__ double exp_neg_scaled(double t, const double* __restrict__ table) {
  double kd = t + 6755399441055744.0;
  const int ki = __double2loint(kd);
  kd -= 6755399441055744.0;
  const double u = t - kd;
  const double q = fma(fma(kExpC3, u, kExpC2), u, kExpC1);
  const double p = q * u;
  const double tj = table[ki & 4095];
  const double ts = __longlong_as_double(__double_as_longlong(tj) - ((long long)(ki >> 12) << 52));
  const double r = fma(ts, p, ts);
  // Range handling on the integer pipe: t >= 0, so the bit patterns order
  // like the values.  Beyond t = 708*4096/ln2 the result is below 2^-1021.
  const long long tb = __double_as_longlong(t);
  constexpr long long kLimit = 0x414FEB6C80000000LL;  // bits of 4183769.0 = floor(708 * 4096/ln2)
  constexpr long long kInf = 0x7FF0000000000000LL;
  return (tb <= kLimit) ? r : ((tb > kInf) ? t : 0.0);
}

// kernel.cu nugget rule: + 1e-8 when the unscaled distance is below 1e-14,
// i.e. when t < 1e-28 * 4096/ln2 (compared on the bit pattern, t >= 0).
constexpr long long kKernelCuTinyBits = 0x3AE6DC442F8BC262LL;  // bits of 1e-28 * 4096/ln2
__device__ __forceinline__ bool below_kernel_cu_tiny(double t) {
  return __double_as_longlong(t) < kKernelCuTinyBits;
}

template <int DIM, int RULE>
__global__ void __launch_bounds__(kThreads) gauss_f64_kernel(
    int rows, int cols, int row_offset, int col_offset, int dyn_dim,
    const double* __restrict__ c0, const double* __restrict__ c1, const double* __restrict__ c2,
    const double* const* __restrict__ cgen, double nugget, const double* __restrict__ x,
    double* __restrict__ y, const double* __restrict__ table_g, int cols_per_split, int nsplit,
    double* __restrict__ partials, unsigned int* __restrict__ tickets, const int* __restrict__ skip) {
  if (skip && *skip) return;
  constexpr int D = (DIM > 0) ? DIM : kMaxDim;
  __shared__ double table[kExpTableSize];
  __shared__ double sp[D][kTileJ];
  __shared__ double sx[kTileJ];
  __shared__ int s_last;
  const int dim = (DIM > 0) ? DIM : dyn_dim;

  for (int i = threadIdx.x; i < kExpTableSize; i += kThreads) table[i] = table_g[i];

  const int tile = blockIdx.x / nsplit;
  const int split = blockIdx.x % nsplit;
  const int cbeg = split * cols_per_split;
  const int cend = min(cols, cbeg + cols_per_split);

  auto coord = [&](int d, int idx) -> double {
    if (DIM > 0) return d == 0 ? c0[idx] : (d == 1 ? c1[idx] : c2[idx]);
    return cgen[d][idx];
  };

  double pi[kRowsPerThread][D];
  int li[kRowsPerThread];
#pragma unroll
  for (int q = 0; q < kRowsPerThread; ++q) {
    li[q] = tile * kRowsPerCta + q * kThreads + threadIdx.x;
    const int gi = row_offset + min(li[q], rows - 1);
#pragma unroll
    for (int d = 0; d < D; ++d) pi[q][d] = (d < dim) ? coord(d, gi) : 0.0;
  }
  double acc[kRowsPerThread];
#pragma unroll
  for (int q = 0; q < kRowsPerThread; ++q) acc[q] = 0.0;

  for (int j0 = cbeg; j0 < cend; j0 += kTileJ) {
    const int nj = min(kTileJ, cend - j0);
    __syncthreads();
    for (int t = threadIdx.x; t < kTileJ; t += kThreads) {
      const bool in = t < nj;
      const int gj = col_offset + j0 + (in ? t : 0);
#pragma unroll
      for (int d = 0; d < D; ++d) sp[d][t] = (d < dim) ? coord(d, gj) : 0.0;
      sx[t] = in ? x[j0 + t] : 0.0;
    }
    __syncthreads();
#pragma unroll 2
    for (int t = 0; t < nj; ++t) {
      double pj[D];
#pragma unroll
      for (int d = 0; d < D; ++d) pj[d] = sp[d][t];
      const double xv = sx[t];
#pragma unroll
      for (int q = 0; q < kRowsPerThread; ++q) {
        double s = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          if (d < dim) {
            const double df = pi[q][d] - pj[d];
            s = (d == 0) ? df * df : fma(df, df, s);
          }
        }
        const double ts = s * kExpScale;
        double e = exp_neg_scaled(ts, table);
        if (RULE == MGB_NUGGET_KERNEL_CU) {
          if (below_kernel_cu_tiny(ts)) e += 1e-8;
        }
        acc[q] = fma(e, xv, acc[q]);
      }
    }
  }

  // Diagonal nugget (system_assembler rule): once per row whose diagonal
  // column falls into this CTA's column range.
  if (RULE == MGB_NUGGET_DIAGONAL) {
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int jl = row_offset + li[q] - col_offset;  // local column of the diagonal
      if (li[q] < rows && jl >= cbeg && jl < cend) acc[q] = fma(nugget, x[jl], acc[q]);
    }
  }

  if (nsplit == 1) {
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q)
      if (li[q] < rows) y[li[q]] = acc[q];
    return;
  }
#pragma unroll
  for (int q = 0; q < kRowsPerThread; ++q)
    if (li[q] < rows) partials[(long long)split * rows + li[q]] = acc[q];
  if (last_block_arrival(&tickets[tile], nsplit, &s_last)) {
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      if (li[q] < rows) {
        double s = 0.0;
        for (int p = 0; p < nsplit; ++p) s += __ldcg(&partials[(long long)p * rows + li[q]]);
        y[li[q]] = s;
      }
    }
  }
}

__global__ void scale_coords_kernel(int n, int dim, const double* const* __restrict__ src,
                                    double* __restrict__ dst, double f) {
  const long long total = (long long)n * dim;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int d = (int)(k / n);
    const int i = (int)(k % n);
    dst[k] = src[d][i] * f;
  }
}

__global__ void gauss_entries_kernel(int count, const int* __restrict__ ii, const int* __restrict__ jj,
                                     int dim, const double* const* __restrict__ coords, int stride,
                                     double nugget, int rule, const double* __restrict__ table,
                                     double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int i = ii[k], j = jj[k];
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    const double df = coords[0][(long long)d * stride + i] - coords[0][(long long)d * stride + j];
    s = (d == 0) ? df * df : fma(df, df, s);
  }
  const double ts = s * kExpScale;
  double e = exp_neg_scaled(ts, table);
  if (rule == MGB_NUGGET_KERNEL_CU) {
    if (below_kernel_cu_tiny(ts)) e += 1e-8;
  } else if (i == j) {
    e += nugget;
  }
  out[k] = e;
}

}  // namespace

// Scaled structure-of-arrays copy of the coordinates: one block of n*dim
// doubles from the pool.  Returned pointers index the same global rows.
static int make_scaled_coords(DeviceContext* c, const GaussSystem& g, double** out,
                              const double** dev_ptr_array, cudaStream_t s) {
  const int n = max(g.row_offset + g.rows, g.col_offset + g.cols);
  double* buf = nullptr;
  MGB_TRY(pool_alloc(c, sizeof(double) * (size_t)n * g.dim + sizeof(double*) * kMaxDim, (void**)&buf));
  // pointer array lives after the coordinates
  const double** ptrs = reinterpret_cast<const double**>(buf + (size_t)n * g.dim);
  const double* host_ptrs[kMaxDim];
  for (int d = 0; d < g.dim; ++d) host_ptrs[d] = g.coords[d];
  MGB_CUDA(cudaMemcpyAsync(ptrs, host_ptrs, sizeof(double*) * g.dim, cudaMemcpyHostToDevice, s));
  const double f = 1.0;  // plain copy: distances are formed from the caller's coordinates
  const long long total = (long long)n * g.dim;
  const long long want = (total + 255) / 256, cap = 4LL * c->num_sms;
  const int blocks = (int)(want < cap ? want : cap);
  scale_coords_kernel<<<blocks, 256, 0, s>>>(n, g.dim, ptrs, buf, f); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  *out = buf;
  if (dev_ptr_array) *dev_ptr_array = reinterpret_cast<const double*>(ptrs);
  return MGB_OK;
}

struct GaussF64Plan {
  int nsplit, cols_per_split, grid;
};

static GaussF64Plan plan_gauss_f64(const DeviceContext* c, int rows, int cols) {
  GaussF64Plan p;
  const int tiles = (rows + kRowsPerCta - 1) / kRowsPerCta;
  // About 32 work items per SM so the hardware block scheduler balances the
  // FP64-bound work (a single item is ~1/30 of an SM's share); keep at least
  // 512 columns per split so the cross-split reduction stays negligible.
  int nsplit = (32 * c->num_sms + tiles - 1) / tiles;
  nsplit = max(1, min(nsplit, (cols + 511) / 512));
  p.cols_per_split = ((cols + nsplit - 1) / nsplit + kTileJ - 1) / kTileJ * kTileJ;
  p.nsplit = (cols + p.cols_per_split - 1) / p.cols_per_split;
  p.grid = tiles * p.nsplit;
  return p;
}

template <int DIM, int RULE>
static void launch_typed(const GaussSystem& g, const double* const* sc, const double* const* dev_ptrs,
                         const GaussF64Plan& p, DeviceContext* c, const double* x, double* y,
                         cudaStream_t s, const int* skip) {
  gauss_f64_kernel<DIM, RULE><<<p.grid, kThreads, 0, s>>>(
      g.rows, g.cols, g.row_offset, g.col_offset, g.dim, sc[0], sc[1], sc[2], dev_ptrs, g.nugget, x, y,
      c->exp_table, p.cols_per_split, p.nsplit, c->split_partials, c->tickets + 1, skip); count_launches(1);
}

// Matvec on already-scaled coordinates (used by the solvers, which scale once).
int launch_gauss_f64_scaled(DeviceContext* c, const GaussSystem& g, const double* const* scaled,
                            const double* const* scaled_dev_ptrs, const double* x, double* y,
                            cudaStream_t s, const int* skip) {
  if (g.rows <= 0 || g.cols <= 0) return MGB_OK;
  const GaussF64Plan p = plan_gauss_f64(c, g.rows, g.cols);
  if (p.nsplit > 1) MGB_TRY(ensure_split_partials(c, (size_t)p.nsplit * g.rows));
  const int tiles = (g.rows + kRowsPerCta - 1) / kRowsPerCta;
  MGB_TRY(ensure_tickets(c, tiles + 1));
  const bool kcu = g.nugget_rule == MGB_NUGGET_KERNEL_CU;
  switch (g.dim) {
    case 1: kcu ? launch_typed<1, 1>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip)
                : launch_typed<1, 0>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip); break;
    case 2: kcu ? launch_typed<2, 1>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip)
                : launch_typed<2, 0>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip); break;
    case 3: kcu ? launch_typed<3, 1>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip)
                : launch_typed<3, 0>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip); break;
    default: kcu ? launch_typed<0, 1>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip)
                 : launch_typed<0, 0>(g, scaled, scaled_dev_ptrs, p, c, x, y, s, skip); break;
  }
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

// Scaled coordinates of a system, owned by the caller (release with
// release_scaled_coords).
int prepare_scaled_coords(DeviceContext* c, const GaussSystem& g, ScaledCoords* out, cudaStream_t s) {
  if (g.dim < 1 || g.dim > kMaxDim) return set_error(MGB_ERR_ARG, "dim %d not in [1,%d]", g.dim, kMaxDim);
  const double* devp = nullptr;
  MGB_TRY(make_scaled_coords(c, g, &out->buf, &devp, s));
  const int n = max(g.row_offset + g.rows, g.col_offset + g.cols);
  for (int d = 0; d < 3; ++d) out->ptr[d] = (d < g.dim) ? out->buf + (size_t)d * n : out->buf;
  out->dev_ptrs = reinterpret_cast<const double* const*>(devp);
  // the generic-dim kernel reads cgen[d] = scaled pointers; rewrite them
  const double* host_ptrs[kMaxDim];
  for (int d = 0; d < g.dim; ++d) host_ptrs[d] = out->buf + (size_t)d * n;
  MGB_CUDA(cudaMemcpyAsync((void*)out->dev_ptrs, host_ptrs, sizeof(double*) * g.dim,
                           cudaMemcpyHostToDevice, s));
  // the host array must outlive the async copy
  MGB_CUDA(cudaStreamSynchronize(s));
  return MGB_OK;
}

void release_scaled_coords(DeviceContext* c, ScaledCoords* sc) {
  pool_free(c, sc->buf);
  sc->buf = nullptr;
}

int launch_gauss_f64(DeviceContext* c, const GaussSystem& g, const double* x, double* y,
                     cudaStream_t s, const int* skip) {
  ScaledCoords sc;
  MGB_TRY(prepare_scaled_coords(c, g, &sc, s));
  int st = launch_gauss_f64_scaled(c, g, sc.ptr, sc.dev_ptrs, x, y, s, skip);
  // the pool block may be reused only after the kernel ran
  cudaError_t e = cudaStreamSynchronize(s);
  release_scaled_coords(c, &sc);
  if (st != MGB_OK) return st;
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
  return MGB_OK;
}

int launch_gauss_entries_f64(DeviceContext* c, const GaussSystem& g, int count, const int* i,
                             const int* j, double* out, cudaStream_t s) {
  ScaledCoords sc;
  MGB_TRY(prepare_scaled_coords(c, g, &sc, s));
  const int n = max(g.row_offset + g.rows, g.col_offset + g.cols);
  if (count > 0) {
    gauss_entries_kernel<<<(count + 255) / 256, 256, 0, s>>>(count, i, j, g.dim, sc.dev_ptrs, n,
                                                             g.nugget, g.nugget_rule, c->exp_table, out); count_launches(1);
  }
  cudaError_t e = cudaGetLastError();
  cudaError_t e2 = cudaStreamSynchronize(s);
  release_scaled_coords(c, &sc);
  if (e != cudaSuccess) return cuda_error(e, "gauss_entries_kernel", __FILE__, __LINE__);
  if (e2 != cudaSuccess) return cuda_error(e2, "cudaStreamSynchronize", __FILE__, __LINE__);
  return MGB_OK;
}

}  // namespace mgb
