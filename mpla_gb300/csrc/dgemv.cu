// Dense FP64 GEMV y = A x for column-major A (the only device compute of
// mpla_dgemv, MPLA src/mpla.cpp:716-751, which calls cublasDgemv OP_N).
//
// 8 bytes of A per 2 flops: HBM-bound on paper, but GB300 issues only ~2
// FP64 FMAs per clock per SM, which at n = 4096 takes longer than streaming A.
// So most products run in FP32 pairs with FP64 accuracy, beside FP64 FMAs on
// the rest (3 columns of every 8), keeping both kinds of pipe busy:
//   * each matrix element a is split exactly by integer operations into
//     ah (its top 24 significand bits, a float) and al (the other 29 bits,
//     converted to float: 2^-53 relative error), x likewise once per CTA;
//   * ah*xh is split exactly into p + e by an FMA (TwoProd), the cross terms
//     ah*xl + al*xh + e are added in FP32 (2^-48 relative);
//   * p is summed with TwoSum into a double-float (S, C) per row, flushed
//     into an FP64 accumulator every 64 columns.
// A product is thus accurate to ~2^-48 relative and integer data below 2^48
// stays exact.  Elements outside [2^-50, 2^58) in magnitude (zeros
// included) take one FP64 FMA instead, and a CTA whose slice of x has a
// nonzero entry outside that range uses FP64 FMAs throughout.
// Layout of the work:
//   * a CTA owns a strip of 32*VEC rows and a chunk of 8*cpw columns;
//   * each of its 8 warps streams cpw columns of the strip with 128-bit
//     (VEC = 2) coalesced, L1-bypassing loads, 8 columns in flight per thread;
//   * the CTA's slice of x is staged in shared memory by one bulk (TMA) copy;
//   * warp partials are summed in shared memory in warp order, and chunk
//     partials across the grid by the last-arriving CTA of each strip in
//     chunk order — a fixed summation order, so results are bit-reproducible.
#include <mutex>

#include "internal.h"
#include "devutil.cuh"

namespace mgb {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

__device__ __forceinline__ double2 ld_stream2(const double* p) {
  double2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}

__device__ __forceinline__ double ld_stream1(const double* p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// Double-float accumulation of a * x into (S, C), or into acc64 when a is out
// of the split's range.
__device__ __forceinline__ void split_fma(double a, float xh, float xl, double x, float& S, float& C,
                                          double& acc64) {
  const uint32_t lo = (uint32_t)__double2loint(a), hi = (uint32_t)__double2hiint(a);
  const uint32_t E = (hi >> 20) & 0x7ffu;
  if (E - 973u > 107u) {  // |a| outside [2^-50, 2^58), zeros and subnormals included
    acc64 = fma(a, x, acc64);
    return;
  }
  const uint32_t sign = hi & 0x80000000u;
  const float ah = __uint_as_float(sign | ((E - 896u) << 23) | (__funnelshift_r(lo, hi, 29) & 0x7fffffu));
  const float al = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu), __uint_as_float(sign | ((E - 948u) << 23)));
  const float p = __fmul_rn(ah, xh);
  const float e = __fmaf_rn(ah, xh, -p);
  const float c = __fmaf_rn(ah, xl, __fmaf_rn(al, xh, e));
  const float t = __fadd_rn(S, p);
  const float bp = __fsub_rn(t, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  S = t;
  C = __fadd_rn(C, __fadd_rn(err, c));
}

__device__ __forceinline__ void split_flush(float& S, float& C, double& acc64) {
  acc64 += (double)S + (double)C;
  S = 0.f;
  C = 0.f;
}

template <int VEC>
__global__ void __launch_bounds__(kThreads) dgemv_kernel(int m, int n, const double* __restrict__ A,
                                                         long long lda, const double* __restrict__ x,
                                                         double* __restrict__ y, int cpw, int nsplit,
                                                         double* __restrict__ partials,
                                                         unsigned int* __restrict__ tickets,
                                                         const int* __restrict__ done,
                                                         unsigned int* __restrict__ err) {
  if (done && *done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // layout: [mbarrier 16 B][x chunk: 8*cpw doubles][warp partials: 8 x 32*VEC doubles]
  //         [x chunk split: 8*cpw float2 (hi, lo)]
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  double* xs = reinterpret_cast<double*>(smem_raw + 16);
  const int chunk = kWarps * cpw;
  double* wpart = xs + chunk;
  float2* xsp = reinterpret_cast<float2*>(wpart + kWarps * 32 * VEC);
  __shared__ int s_last;

  constexpr int kRows = 32 * VEC;
  const int strip = blockIdx.x / nsplit;
  const int split = blockIdx.x % nsplit;
  const int row0 = strip * kRows;
  const int col0 = split * chunk;
  const int ncols = min(chunk, n - col0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // ---- stage x[col0 : col0+ncols) in shared memory
  const bool use_bulk = ((reinterpret_cast<uintptr_t>(x + col0) & 15) == 0) && ((ncols & 1) == 0);
  if (use_bulk) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      fence_proxy_async_smem();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_arrive_expect_tx(bar, ncols * 8);
      bulk_copy_g2s(xs, x + col0, ncols * 8, bar);
    }
  } else {
    for (int j = threadIdx.x; j < ncols; j += kThreads) xs[j] = x[col0 + j];
    __syncthreads();
  }

  // ---- stream A: this warp's columns [wc0, wc1) of the chunk
  const int wc0 = warp * cpw;
  const int wc1 = min(wc0 + cpw, ncols);
  const int r = row0 + lane * VEC;
  double acc0 = 0.0, acc1 = 0.0;
  bool x_ready = true;
  if (use_bulk) x_ready = mbar_wait_bounded(bar, 0, err, DEV_ERR_WAIT_TIMEOUT);
  // split this CTA's x into FP32 (hi, lo) pairs; any entry outside the
  // split's range sends the whole CTA down the FP64 path
  int bad = 0;
  if (x_ready) {
    for (int j = threadIdx.x; j < ncols; j += kThreads) {
      const double xv = xs[j];
      const uint32_t E = ((uint32_t)__double2hiint(xv) >> 20) & 0x7ffu;
      bad |= (xv != 0.0) && (E - 973u > 107u);
      const float h = __double2float_rn(xv);
      xsp[j] = make_float2(h, __double2float_rn(xv - (double)h));
    }
  }
  const bool use_split = !__syncthreads_or(bad);
  if (x_ready && use_split && r < m && wc0 < wc1) {
    // Columns 0-2 of every group of 8 take FP64 FMAs and columns 3-7 the
    // FP32-pair products, so the FP64 pipe and the FP32/integer pipes work
    // side by side (each alone would take longer than streaming A).  The
    // next group's loads are issued before the current group is computed.
    const double* a = A + (long long)(col0 + wc0) * lda + r;
    const bool pair = (VEC == 2) && (r + 1 < m);
    float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
    int j = wc0;
    if (VEC == 2 && pair) {
      double2 v[8];
      if (j + 8 <= wc1) {
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = ld_stream2(a + (long long)u * lda);
      }
      for (; j + 8 <= wc1; j += 8) {
        double2 nv[8];
        const bool more = j + 16 <= wc1;
        if (more) {
#pragma unroll
          for (int u = 0; u < 8; ++u) nv[u] = ld_stream2(a + (long long)(8 + u) * lda);
        }
#pragma unroll
        for (int u = 0; u < 3; ++u) {
          const double x64 = xs[j + u];
          acc0 = fma(v[u].x, x64, acc0);
          acc1 = fma(v[u].y, x64, acc1);
        }
#pragma unroll
        for (int u = 3; u < 8; ++u) {
          const float2 xv = xsp[j + u];
          const double x64 = xs[j + u];
          split_fma(v[u].x, xv.x, xv.y, x64, S0, C0, acc0);
          split_fma(v[u].y, xv.x, xv.y, x64, S1, C1, acc1);
        }
        a += 8 * lda;
        if (((j - wc0) & 63) == 56) {  // every 64 columns
          split_flush(S0, C0, acc0);
          split_flush(S1, C1, acc1);
        }
        if (more) {
#pragma unroll
          for (int u = 0; u < 8; ++u) v[u] = nv[u];
        }
      }
    } else {
      for (; j + 8 <= wc1; j += 8) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = ld_stream1(a + (long long)u * lda);
#pragma unroll
        for (int u = 0; u < 3; ++u) acc0 = fma(v[u], xs[j + u], acc0);
#pragma unroll
        for (int u = 3; u < 8; ++u) {
          const float2 xv = xsp[j + u];
          split_fma(v[u], xv.x, xv.y, xs[j + u], S0, C0, acc0);
        }
        a += 8 * lda;
        if (((j - wc0) & 63) == 56) split_flush(S0, C0, acc0);
      }
    }
    for (; j < wc1; ++j) {
      const float2 xv = xsp[j];
      if (VEC == 2 && pair) {
        const double2 v = ld_stream2(a);
        split_fma(v.x, xv.x, xv.y, xs[j], S0, C0, acc0);
        split_fma(v.y, xv.x, xv.y, xs[j], S1, C1, acc1);
      } else {
        split_fma(ld_stream1(a), xv.x, xv.y, xs[j], S0, C0, acc0);
      }
      a += lda;
    }
    split_flush(S0, C0, acc0);
    split_flush(S1, C1, acc1);
  } else if (x_ready && r < m && wc0 < wc1) {
    const double* a = A + (long long)(col0 + wc0) * lda + r;
    const bool pair = (VEC == 2) && (r + 1 < m);
    int j = wc0;
    for (; j + 8 <= wc1; j += 8) {
      if (VEC == 2 && pair) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = ld_stream2(a + (long long)u * lda);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const double xv = xs[j + u];
          acc0 = fma(v[u].x, xv, acc0);
          acc1 = fma(v[u].y, xv, acc1);
        }
      } else {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = ld_stream1(a + (long long)u * lda);
#pragma unroll
        for (int u = 0; u < 8; ++u) acc0 = fma(v[u], xs[j + u], acc0);
      }
      a += 8 * lda;
    }
    for (; j < wc1; ++j) {
      const double xv = xs[j];
      if (VEC == 2 && pair) {
        const double2 v = ld_stream2(a);
        acc0 = fma(v.x, xv, acc0);
        acc1 = fma(v.y, xv, acc1);
      } else {
        acc0 = fma(ld_stream1(a), xv, acc0);
      }
      a += lda;
    }
  }
  wpart[warp * kRows + lane * VEC] = acc0;
  if (VEC == 2) wpart[warp * kRows + lane * VEC + 1] = acc1;
  __syncthreads();

  // ---- CTA partial for the strip: sum warps in order
  double cta_sum = 0.0;
  const int lr = threadIdx.x;
  if (lr < kRows) {
#pragma unroll
    for (int w = 0; w < kWarps; ++w) cta_sum += wpart[w * kRows + lr];
  }
  if (nsplit == 1) {
    if (lr < kRows && row0 + lr < m) y[row0 + lr] = cta_sum;
    return;
  }
  if (lr < kRows && row0 + lr < m) partials[(long long)split * m + row0 + lr] = cta_sum;
  if (last_block_arrival(&tickets[strip], nsplit, &s_last)) {
    if (lr < kRows && row0 + lr < m) {
      double s = 0.0;
#pragma unroll 8
      for (int q = 0; q < nsplit; ++q) s += __ldcg(&partials[(long long)q * m + row0 + lr]);
      y[row0 + lr] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Scratch of the allocation-free entry point mgb_dgemv_noalloc: the split-K
// partials and the per-strip arrival tickets live in this fixed array, which
// every GPU that loads the library keeps for the life of the process.
constexpr size_t kNoAllocPartials = size_t(1) << 20;  // doubles (8 MiB)
constexpr int kNoAllocTickets = 16384;                // strips + 1
constexpr int kNoAllocMaxChunkCols = 4096;            // 8 warps x 512 columns per CTA
constexpr size_t kNoAllocBytes =
    sizeof(double) * kNoAllocPartials + sizeof(unsigned int) * (kNoAllocTickets + 64);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];
// dynamic shared memory of the widest chunk: mbarrier, x, warp partials, split x
constexpr int kNoAllocMaxSmem = 16 + 8 * (kNoAllocMaxChunkCols + kWarps * 64) + 8 * kNoAllocMaxChunkCols;

}  // namespace

int launch_dgemv(DeviceContext* c, int m, int n, const double* A, int lda, const double* x,
                 double* y, cudaStream_t s, const int* done) {
  if (m < 0 || n < 0 || lda < (m > 1 ? m : 1))
    return set_error(MGB_ERR_ARG, "dgemv: bad sizes m=%d n=%d lda=%d", m, n, lda);
  if (m == 0) return MGB_OK;
  if (n == 0) {
    MGB_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * m, s));
    return MGB_OK;
  }
  const bool vec2 = ((lda & 1) == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  const int rows_per_strip = vec2 ? 64 : 32;
  const int strips = (m + rows_per_strip - 1) / rows_per_strip;
  // Columns per warp: enough CTAs to cover the machine several times over,
  // at least 64 columns per warp, so the per-CTA staging of x is amortised.
  int cpw = 128;
  const long long target = 6LL * c->num_sms;
  while (cpw > 64 && (long long)strips * ((n + kWarps * cpw - 1) / (kWarps * cpw)) < target) cpw >>= 1;
  const int nsplit = (n + kWarps * cpw - 1) / (kWarps * cpw);
  if (nsplit > 1) {
    MGB_TRY(ensure_split_partials(c, (size_t)nsplit * m));
    MGB_TRY(ensure_tickets(c, strips + 1));
  }
  const size_t smem = 16 + sizeof(double) * (kWarps * cpw + kWarps * rows_per_strip) + sizeof(float2) * kWarps * cpw;
  const long long grid = (long long)strips * nsplit;
  if (grid > 0x7fffffffLL) return set_error(MGB_ERR_ARG, "dgemv: grid too large");
  if (vec2) {
    dgemv_kernel<2><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit,
                                                         c->split_partials, c->tickets + 1, done, c->dev_error);
  } else {
    dgemv_kernel<1><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit,
                                                         c->split_partials, c->tickets + 1, done, c->dev_error);
  }
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

}  // namespace mgb

using namespace mgb;

namespace {

// Per-device address of g_noalloc_scratch and SM count, resolved once per
// device with that device current.  In host code the array's name is only a
// host-side stand-in, never a device address.
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[64] = {nullptr};
int g_noalloc_sms[64] = {0};

int noalloc_setup(int dev, unsigned char** scratch, int* sms) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    MGB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    int count = 0;
    MGB_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev));
    // the widest column chunk of this path needs more than the default 48 KB
    // of dynamic shared memory (a launch attribute, not an allocation)
    MGB_CUDA(cudaFuncSetAttribute(dgemv_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNoAllocMaxSmem));
    MGB_CUDA(cudaFuncSetAttribute(dgemv_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNoAllocMaxSmem));
    g_noalloc_sms[dev] = count;
    g_noalloc_ptr[dev] = p;
  }
  *scratch = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
  *sms = g_noalloc_sms[dev];
  return MGB_OK;
}

}  // namespace

extern "C" int mgb_dgemv_noalloc(int m, int n, const double* A, int lda, const double* x, double* y, void* stream) {
  if (m < 0 || n < 0 || lda < (m > 1 ? m : 1))
    return set_error(MGB_ERR_ARG, "dgemv_noalloc: bad sizes m=%d n=%d lda=%d", m, n, lda);
  if (m > 0 && n > 0 && (!A || !x || !y)) return set_error(MGB_ERR_ARG, "dgemv_noalloc: null pointer");
  const bool vec2 = ((lda & 1) == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  const int rows_per_strip = vec2 ? 64 : 32;
  const long long strips = ((long long)m + rows_per_strip - 1) / rows_per_strip;
  if (strips + 1 > kNoAllocTickets)
    return set_error(MGB_ERR_ARG, "dgemv_noalloc: m=%d exceeds the allocation-free maximum of %d rows", m,
                     (kNoAllocTickets - 1) * rows_per_strip);
  const long long min_split = ((long long)n + kNoAllocMaxChunkCols - 1) / kNoAllocMaxChunkCols;
  if (min_split > 1 && min_split * m > (long long)kNoAllocPartials)
    return set_error(MGB_ERR_ARG,
                     "dgemv_noalloc: m x ceil(n/%d) = %lld exceeds the allocation-free scratch of %zu partials",
                     kNoAllocMaxChunkCols, min_split * m, kNoAllocPartials);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamLegacy;
  if (m == 0) return MGB_OK;
  if (n == 0) {
    MGB_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * m, s));
    return MGB_OK;
  }
  int dev = 0;
  MGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(MGB_ERR_ARG, "device index %d out of range", dev);
  unsigned char* scratch = nullptr;
  int sms = 0;
  MGB_TRY(noalloc_setup(dev, &scratch, &sms));
  double* partials = reinterpret_cast<double*>(scratch);
  unsigned int* tickets = reinterpret_cast<unsigned int*>(scratch + sizeof(double) * kNoAllocPartials);
  unsigned int* err = tickets + kNoAllocTickets;
  // same column split as the allocating path, bounded by the fixed scratch
  int cpw = 128;
  const long long target = 6LL * sms;
  while (cpw > 16 && strips * ((n + kWarps * cpw - 1) / (kWarps * cpw)) < target) cpw >>= 1;
  while ((long long)((n + kWarps * cpw - 1) / (kWarps * cpw)) * m > (long long)kNoAllocPartials &&
         kWarps * cpw < kNoAllocMaxChunkCols)
    cpw <<= 1;
  const int nsplit = (n + kWarps * cpw - 1) / (kWarps * cpw);
  // The array keeps the previous call's contents: the arrival tickets must
  // start at zero (the partials are written before they are read).
  MGB_CUDA(cudaMemsetAsync(tickets, 0, sizeof(unsigned int) * (strips + 1), s));
  const size_t smem = 16 + sizeof(double) * (kWarps * cpw + kWarps * rows_per_strip) + sizeof(float2) * kWarps * cpw;
  if (smem > (size_t)kNoAllocMaxSmem) return set_error(MGB_ERR_ARG, "dgemv_noalloc: column chunk too large");
  const long long grid = strips * nsplit;
  if (vec2) {
    dgemv_kernel<2><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit, partials, tickets + 1,
                                                         nullptr, err);
  } else {
    dgemv_kernel<1><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit, partials, tickets + 1,
                                                         nullptr, err);
  }
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}
