// Dense FP64 GEMV y = A x for column-major A (the only device compute of
// mpla_dgemv, MPLA src/mpla.cpp:716-751, which calls cublasDgemv OP_N).
//
// HBM-bound: 8 bytes of A per 2 flops.  Layout of the work:
//   * a CTA owns a strip of 32*VEC rows and a chunk of 8*cpw columns;
//   * each of its 8 warps streams cpw columns of the strip with 128-bit
//     (VEC = 2) coalesced, L1-bypassing loads, 8 columns in flight per thread;
//   * the CTA's slice of x is staged in shared memory by one bulk (TMA) copy;
//   * warp partials are summed in shared memory in warp order, and chunk
//     partials in chunk order: when a strip's chunks fit in one thread-block
//     cluster (at most 8), CTA 0 of the cluster reads the others' partials
//     from their shared memory (no global partials, fences or atomics);
//     otherwise the last-arriving CTA of each strip reads them from global
//     memory.  A fixed summation order either way, so results are
//     bit-reproducible and the same on both paths.
#include <cooperative_groups.h>
#include <mutex>

#include "internal.h"
#include "devutil.cuh"

namespace mgb {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kMaxCluster = 8;  // portable thread-block cluster size

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

// BULK: stage x with one bulk copy and a bounded mbarrier wait (a wait that
// gives up sets DEV_ERR_WAIT_TIMEOUT in *err); otherwise with plain loads.
// CLUSTER: the nsplit chunks of a strip form one cluster (rank = chunk) and
// are reduced through distributed shared memory.
template <int VEC, bool BULK, bool CLUSTER>
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
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  double* xs = reinterpret_cast<double*>(smem_raw + 16);
  const int chunk = kWarps * cpw;
  double* wpart = xs + chunk;
  __shared__ int s_last;

  constexpr int kRows = 32 * VEC;
  const int strip = blockIdx.x / nsplit;
  const int split = blockIdx.x % nsplit;
  const int row0 = strip * kRows;
  const int col0 = split * chunk;
  const int ncols = min(chunk, n - col0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // ---- stage x[col0 : col0+ncols) in shared memory
  const bool use_bulk = BULK && ((reinterpret_cast<uintptr_t>(x + col0) & 15) == 0) && ((ncols & 1) == 0);
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
  if (x_ready && r < m && wc0 < wc1) {
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
  if (CLUSTER) {
    __shared__ double cpart[kRows];
    if (lr < kRows) cpart[lr] = cta_sum;
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    cl.sync();  // every chunk's partials are in its shared memory
    if (split == 0 && lr < kRows && row0 + lr < m) {
      double s = 0.0;
      for (int q = 0; q < nsplit; ++q) s += *cl.map_shared_rank(&cpart[lr], q);
      y[row0 + lr] = s;
    }
    cl.sync();  // keep every CTA's shared memory until CTA 0 has read it
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
  // at least 16 columns per warp so each thread keeps 8 loads in flight.
  int cpw = 128;
  const long long target = 6LL * c->num_sms;
  while (cpw > 16 && (long long)strips * ((n + kWarps * cpw - 1) / (kWarps * cpw)) < target) cpw >>= 1;
  int nsplit = (n + kWarps * cpw - 1) / (kWarps * cpw);
  // Cluster reduction when a strip's chunks fit in a portable cluster (8),
  // widening the chunks if that still leaves >= 2 CTAs per SM.
  int ccpw = cpw;
  while (ccpw < 512 && (n + kWarps * ccpw - 1) / (kWarps * ccpw) > kMaxCluster) ccpw <<= 1;
  const int csplit = (n + kWarps * ccpw - 1) / (kWarps * ccpw);
  const bool cluster = csplit > 1 && csplit <= kMaxCluster && (long long)strips * csplit >= 2LL * c->num_sms;
  if (cluster) {
    cpw = ccpw;
    nsplit = csplit;
  } else if (nsplit > 1) {
    MGB_TRY(ensure_split_partials(c, (size_t)nsplit * m));
    MGB_TRY(ensure_tickets(c, strips + 1));
  }
  const size_t smem = 16 + sizeof(double) * (kWarps * cpw + kWarps * rows_per_strip);
  const long long grid = (long long)strips * nsplit;
  if (grid > 0x7fffffffLL) return set_error(MGB_ERR_ARG, "dgemv: grid too large");
  if (cluster) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)nsplit;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    long long lda_ll = lda;
    double* no_partials = nullptr;
    unsigned int* no_tickets = nullptr;
    if (vec2)
      MGB_CUDA(cudaLaunchKernelEx(&cfg, dgemv_kernel<2, true, true>, m, n, A, lda_ll, x, y, cpw, nsplit, no_partials,
                                  no_tickets, done, c->dev_error));
    else
      MGB_CUDA(cudaLaunchKernelEx(&cfg, dgemv_kernel<1, true, true>, m, n, A, lda_ll, x, y, cpw, nsplit, no_partials,
                                  no_tickets, done, c->dev_error));
  } else if (vec2) {
    dgemv_kernel<2, true, false><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit,
                                                                      c->split_partials, c->tickets + 1, done,
                                                                      c->dev_error);
  } else {
    dgemv_kernel<1, true, false><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit,
                                                                      c->split_partials, c->tickets + 1, done,
                                                                      c->dev_error);
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
  if (stream && s != cudaStreamLegacy && s != cudaStreamPerThread) {
    // the scratch address below belongs to the current device
    int sdev = -1;
    MGB_CUDA(cudaStreamGetDevice(s, &sdev));
    if (sdev != dev)
      return set_error(MGB_ERR_ARG, "dgemv_noalloc: stream belongs to device %d, current device is %d", sdev, dev);
  }
  unsigned char* scratch = nullptr;
  int sms = 0;
  MGB_TRY(noalloc_setup(dev, &scratch, &sms));
  double* partials = reinterpret_cast<double*>(scratch);
  unsigned int* tickets = reinterpret_cast<unsigned int*>(scratch + sizeof(double) * kNoAllocPartials);
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
  const size_t smem = 16 + sizeof(double) * (kWarps * cpw + kWarps * rows_per_strip);
  if (smem > 48 * 1024) return set_error(MGB_ERR_ARG, "dgemv_noalloc: column chunk too large");
  const long long grid = strips * nsplit;
  // x is staged with plain loads: this variant has no device-side wait, so
  // no error word exists that a caller would have to read back.
  if (vec2) {
    dgemv_kernel<2, false, false><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit, partials,
                                                                tickets + 1, nullptr, nullptr);
  } else {
    dgemv_kernel<1, false, false><<<(unsigned)grid, kThreads, smem, s>>>(m, n, A, lda, x, y, cpw, nsplit, partials,
                                                                tickets + 1, nullptr, nullptr);
  }
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}
