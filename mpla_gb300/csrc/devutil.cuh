// Device-side helpers shared by the kernels: deterministic block reductions,
// the "last block finishes" ticket pattern, bounded mbarrier waits for bulk
// (TMA) copies, and the table-driven FP64 exponential.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace mgb {

// --------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of `v` over the block (blockDim.x a multiple of 32, <= 1024).  Fixed
// tree: butterfly within warps, then warp 0 adds the warp sums in order.
// Every thread receives the result.
__device__ __forceinline__ double block_sum(double v, double* smem32) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) smem32[warp] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double t = (threadIdx.x < nw) ? smem32[threadIdx.x] : 0.0;
  if (warp == 0) t = warp_sum(t);
  if (threadIdx.x == 0) smem32[0] = t;
  __syncthreads();
  double r = smem32[0];
  __syncthreads();
  return r;
}

// Block-wide ticket: returns true in every thread of the block that arrives
// last among `nblocks` blocks sharing `ticket`.  The caller must have written
// its partial results before calling.  The last block resets the ticket so
// the counter can be reused by the next launch without a memset.
__device__ __forceinline__ bool last_block_arrival(unsigned int* ticket, unsigned int nblocks,
                                                   int* smem_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(ticket, 1u);
    int last = (prev == nblocks - 1) ? 1 : 0;
    if (last) *ticket = 0u;
    *smem_flag = last;
  }
  __syncthreads();
  const bool last = *smem_flag != 0;
  if (last) __threadfence();
  return last;
}

// ------------------------------------------------- mbarrier + bulk copies
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (and sets `err_bit` in
// the device error word) when the limit is reached instead of spinning
// forever.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, unsigned int* err,
                                                  unsigned int err_bit, uint32_t limit = 1u << 24) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  if (err) atomicOr(err, err_bit);
  return false;
}

// 1-D bulk copy global -> shared (TMA unit), completion counted on `bar`.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ------------------------------------------------- FP64 exponential of -s
// exp(-s) for s >= 0 by the table-driven method of P. T. P. Tang (ACM TOMS
// 15(2), 1989): with t = s * 4096/ln2 and k = round(t), u = t - k,
//   exp(-s) = 2^(-k div 4096) * 2^(-(k mod 4096)/4096) * 2^(-u/4096),
// where the middle factor comes from a 4096-entry table and the last one is
// the degree-3 Taylor polynomial of exp(-u ln2/4096), |u| <= 1/2 (truncation
// below 3e-18 relative).  8 FP64 operations; the power of two is applied by
// integer arithmetic on the exponent field.  Arguments beyond 708 (results
// below 2^-1021) return 0; NaN propagates.
constexpr double kExpScale = 5909.278887481194;             // 4096 / ln 2
constexpr double kExpC1 = -0.0001692253858788929;           // -(ln2/4096)
constexpr double kExpC2 = 1.4318615612930102e-08;           // (ln2/4096)^2 / 2
constexpr double kExpC3 = -8.076910841165457e-13;           // -(ln2/4096)^3 / 6

__device__ __forceinline__ double exp_neg_table(double s, const double* __restrict__ table) {
  const double t = s * kExpScale;
  double kd = t + 6755399441055744.0;  // 1.5 * 2^52: low mantissa bits hold round(t)
  const int ki = __double2loint(kd);
  kd -= 6755399441055744.0;
  const double u = t - kd;
  const double q = fma(fma(kExpC3, u, kExpC2), u, kExpC1);
  const double p = q * u;
  const int e = ki >> 12;
  const double tj = table[ki & 4095];
  const double ts = __longlong_as_double(__double_as_longlong(tj) - ((long long)e << 52));
  const double r = fma(ts, p, ts);
  return (s <= 708.0) ? r : ((s == s) ? 0.0 : s);
}

}  // namespace mgb
