// Mixed-precision (FP32) matrix-free Gaussian matvec y = K x, the inner
// operator of the mixed CG.  Entries are evaluated in FP32 and the
// exponential runs on the SFU (ex2.approx); x is read in FP64 and rounded
// when a source tile is staged, partial sums are combined in FP64, and the
// diagonal nugget is applied in FP64.  Accuracy is about 1e-6 relative per
// entry; the FP64 residual replacement of the solver removes its effect on
// the final residual.
//
// Coordinates are pre-scaled by sqrt(log2 e) so that K = 2^(-|p_i - p_j|^2)
// and the SFU's base-2 exponential needs no extra multiply:
//   per entry (d = 2): 2 FADD + FMUL + FFMA (negated squared distance),
//   1 MUFU.EX2, 1 FFMA accumulate, plus a quarter of a broadcast LDS.128.
// The kernel is SFU-bound (16 ex2/clk/SM).
#include "internal.h"
#include "devutil.cuh"

namespace mgb {

struct MixedSystem {
  int n = 0;
  int dim = 0;
  double nugget = 0.0;
  float4* pts = nullptr;  // n points {x, y, z, 0} scaled by sqrt(log2 e) (pool block)
};

namespace {

constexpr int kThreads = 256;
constexpr int kRows = 4;  // rows per thread
constexpr int kRowsPerCta = kThreads * kRows;
constexpr int kTileJ = 256;

__device__ __forceinline__ float ex2_approx(float v) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

__global__ void mixed_pack_kernel(int n, int dim, const double* const* __restrict__ coords, double scale,
                                  float4* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float v[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dim && d < 3; ++d) v[d] = (float)(coords[d][i] * scale);
    out[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) gauss_mixed_kernel(int n, const float4* __restrict__ pts,
                                                               const double* __restrict__ x, double nugget,
                                                               double* __restrict__ y, int cols_per_split,
                                                               int nsplit, float* __restrict__ partials,
                                                               unsigned int* __restrict__ tickets,
                                                               const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ float4 sj[kTileJ];
  __shared__ int s_last;
  const int tile = blockIdx.x / nsplit;
  const int split = blockIdx.x % nsplit;
  const int cbeg = split * cols_per_split;
  const int cend = min(n, cbeg + cols_per_split);

  float pi[kRows][3];
  int li[kRows];
#pragma unroll
  for (int q = 0; q < kRows; ++q) {
    li[q] = tile * kRowsPerCta + q * kThreads + threadIdx.x;
    const float4 p = pts[min(li[q], n - 1)];
    pi[q][0] = p.x;
    pi[q][1] = p.y;
    pi[q][2] = p.z;
  }
  float acc[kRows];
#pragma unroll
  for (int q = 0; q < kRows; ++q) acc[q] = 0.f;

  for (int j0 = cbeg; j0 < cend; j0 += kTileJ) {
    const int nj = min(kTileJ, cend - j0);
    __syncthreads();
    for (int t = threadIdx.x; t < kTileJ; t += kThreads) {
      float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
      if (t < nj) {
        p = pts[j0 + t];
        p.w = (float)x[j0 + t];
      }
      sj[t] = p;
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < nj; ++t) {
      const float4 p = sj[t];
#pragma unroll
      for (int q = 0; q < kRows; ++q) {
        const float dx = pi[q][0] - p.x;
        float ns;
        if (DIM == 1) {
          ns = -dx * dx;
        } else if (DIM == 2) {
          const float dy = pi[q][1] - p.y;
          ns = fmaf(-dx, dx, -dy * dy);
        } else {
          const float dy = pi[q][1] - p.y;
          const float dz = pi[q][2] - p.z;
          ns = fmaf(-dx, dx, fmaf(-dy, dy, -dz * dz));
        }
        acc[q] = fmaf(ex2_approx(ns), p.w, acc[q]);
      }
    }
  }

  if (nsplit == 1) {
#pragma unroll
    for (int q = 0; q < kRows; ++q)
      if (li[q] < n) y[li[q]] = (double)acc[q] + nugget * x[li[q]];
    return;
  }
#pragma unroll
  for (int q = 0; q < kRows; ++q)
    if (li[q] < n) partials[(long long)split * n + li[q]] = acc[q];
  if (last_block_arrival(&tickets[tile], nsplit, &s_last)) {
#pragma unroll
    for (int q = 0; q < kRows; ++q) {
      if (li[q] < n) {
        double s = 0.0;
        for (int p = 0; p < nsplit; ++p) s += (double)__ldcg(&partials[(long long)p * n + li[q]]);
        y[li[q]] = fma(nugget, x[li[q]], s);
      }
    }
  }
}

}  // namespace

int mixed_prepare(DeviceContext* c, const GaussSystem& g, MixedSystem** out, cudaStream_t s) {
  if (g.rows != g.cols || g.row_offset != 0 || g.col_offset != 0)
    return set_error(MGB_ERR_ARG, "mixed matvec: square systems only");
  if (g.dim < 1 || g.dim > 3) return set_error(MGB_ERR_ARG, "mixed matvec: dim %d not in [1,3]", g.dim);
  if (g.nugget_rule != MGB_NUGGET_DIAGONAL)
    return set_error(MGB_ERR_ARG, "mixed matvec: only the diagonal nugget rule");
  MixedSystem* m = new MixedSystem();
  m->n = g.rows;
  m->dim = g.dim;
  m->nugget = g.nugget;
  int st = pool_alloc(c, sizeof(float4) * (size_t)m->n + sizeof(double*) * 3, (void**)&m->pts);
  if (st != MGB_OK) {
    delete m;
    return st;
  }
  const double** ptrs = reinterpret_cast<const double**>(m->pts + m->n);
  const double* hp[3] = {g.coords[0], g.dim > 1 ? g.coords[1] : nullptr, g.dim > 2 ? g.coords[2] : nullptr};
  MGB_CUDA(cudaMemcpyAsync(ptrs, hp, sizeof(hp), cudaMemcpyHostToDevice, s));
  const double scale = sqrt(1.4426950408889634);  // sqrt(log2 e)
  mixed_pack_kernel<<<min((m->n + 255) / 256, 8 * c->num_sms), 256, 0, s>>>(m->n, m->dim, ptrs, scale, m->pts); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  MGB_CUDA(cudaStreamSynchronize(s));
  *out = m;
  return MGB_OK;
}

void mixed_release(DeviceContext* c, MixedSystem* m) {
  if (!m) return;
  pool_free(c, m->pts);
  delete m;
}

int launch_gauss_mixed(DeviceContext* c, MixedSystem* m, const double* x, double* y, cudaStream_t s,
                       const int* skip) {
  const int n = m->n;
  const int tiles = (n + kRowsPerCta - 1) / kRowsPerCta;
  int nsplit = (48 * c->num_sms + tiles - 1) / tiles;
  nsplit = max(1, min(nsplit, (n + 1023) / 1024));
  int cps = ((n + nsplit - 1) / nsplit + kTileJ - 1) / kTileJ * kTileJ;
  nsplit = (n + cps - 1) / cps;
  if (nsplit > 1) {
    // float partials share the double split buffer (half the doubles needed)
    MGB_TRY(ensure_split_partials(c, ((size_t)nsplit * n + 1) / 2));
    MGB_TRY(ensure_tickets(c, tiles + 1));
  }
  float* partials = reinterpret_cast<float*>(c->split_partials);
  const int grid = tiles * nsplit;
  switch (m->dim) {
    case 1: gauss_mixed_kernel<1><<<grid, kThreads, 0, s>>>(n, m->pts, x, m->nugget, y, cps, nsplit, partials, c->tickets + 1, skip); count_launches(1); break;
    case 2: gauss_mixed_kernel<2><<<grid, kThreads, 0, s>>>(n, m->pts, x, m->nugget, y, cps, nsplit, partials, c->tickets + 1, skip); count_launches(1); break;
    default: gauss_mixed_kernel<3><<<grid, kThreads, 0, s>>>(n, m->pts, x, m->nugget, y, cps, nsplit, partials, c->tickets + 1, skip); count_launches(1); break;
  }
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

}  // namespace mgb
