// Accumulation rounding of the tensor cores on this GPU: one CTA issues a
// 128 x 128 x 32 tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in
// tensor memory) on operands whose row sums have known exact values, and
// prints each computed sum beside the exact one.  Every product here is
// exact in FP32, so any difference is the accumulation's rounding.  The
// squared distances of the mixed-precision Gaussian matvec would be such
// sums (norms and cross terms of split-BF16 coordinates); a biased rounding
// there perturbs whole tile pairs of the FP32 operator coherently.
// Every wait is bounded; one CTA, 128 tensor-memory columns.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#include "devutil.cuh"
using namespace mgb;

constexpr int kTB = 128, kK = 32;
constexpr uint32_t kLBO = 128, kSBO = 128 * (kK / 8);
__host__ __device__ inline uint32_t op_offset(int row, int kchunk) {
  return (uint32_t)(row / 8) * kSBO + (uint32_t)kchunk * kLBO + (uint32_t)(row % 8) * 16;
}
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) | (1ull << 46);
}
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTB >> 3) << 17) | ((uint32_t)(kTB >> 4) << 24);

__global__ void probe(const uint16_t* A, const uint16_t* B, float* D, unsigned int* err) {
  __shared__ __align__(1024) unsigned char sA[kTB * kK * 2];
  __shared__ __align__(1024) unsigned char sB[kTB * kK * 2];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  // operands: row tid, 32 BF16 values
  for (int kc = 0; kc < kK / 8; ++kc) {
    uint32_t w[4], v[4];
    for (int m = 0; m < 4; ++m) {
      w[m] = (uint32_t)A[tid * kK + 8 * kc + 2 * m] | ((uint32_t)A[tid * kK + 8 * kc + 2 * m + 1] << 16);
      v[m] = (uint32_t)B[tid * kK + 8 * kc + 2 * m] | ((uint32_t)B[tid * kK + 8 * kc + 2 * m + 1] << 16);
    }
    *reinterpret_cast<uint4*>(sA + op_offset(tid, kc)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(sB + op_offset(tid, kc)) = make_uint4(v[0], v[1], v[2], v[3]);
  }
  if (tid == 0) { mbar_init(&bar, 1); fence_mbar_init(); }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)), "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_proxy_async_smem();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  if (tid == 0) {
    const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
    for (int ks = 0; ks < kK / 16; ++ks) {
      const uint64_t da = smem_desc(a_base + ks * 2 * kLBO), db = smem_desc(b_base + ks * 2 * kLBO);
      const uint32_t acc = ks > 0 ? 1u : 0u;
      asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                   ::"r"(tmem), "l"(da), "l"(db), "r"(kIdesc), "r"(acc));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
  }
  const bool ok = mbar_wait_bounded(&bar, 0, err, 1u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    for (int j0 = 0; j0 < 128; j0 += 16) {
      uint32_t v[16];
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                   : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                     "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                   : "r"(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)j0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      for (int k = 0; k < 16; ++k) D[tid * 128 + j0 + k] = __uint_as_float(v[k]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128));
}

static uint16_t bf(float v) {  // exact BF16 bits (values chosen representable)
  uint32_t u; memcpy(&u, &v, 4);
  if (u & 0xFFFF) { fprintf(stderr, "not bf16-exact: %g\n", v); exit(3); }
  return (uint16_t)(u >> 16);
}

int main() {
  std::vector<uint16_t> A(kTB * kK, 0), B(kTB * kK, 0);
  // B column 0 = all ones (sums), column 1 = ones in k-step 1 only
  for (int k = 0; k < kK; ++k) B[0 * kK + k] = bf(1.f);
  std::vector<std::vector<float>> cases;
  const float u23 = ldexpf(1.f, -23), u24 = ldexpf(1.f, -24), u25 = ldexpf(1.f, -25);
  cases.push_back({1.f, 0.75f * u23});                 // 0: RN 1+2^-23, RZ 1
  cases.push_back({1.f, -0.25f * u24});                // 1: RN 1, RZ 1-2^-24
  cases.push_back({ldexpf(1.f, 30), 1.f, -ldexpf(1.f, 30)});  // 2: exact 1
  { std::vector<float> c = {1.f}; for (int i = 0; i < 16; ++i) c.push_back(u25); cases.push_back(c); }  // 3: exact 1+2^-21
  { std::vector<float> c; for (int i = 0; i < 16; ++i) c.push_back(u25); c.push_back(1.f); cases.push_back(c); }  // 4
  cases.push_back({-1.f, -0.75f * u23});               // 5: RN -(1+2^-23), RZ -1
  cases.push_back({1.f, 0.5f * u23});                  // 6: tie: RNE 1
  cases.push_back({1.f + u23 * 1.0f, 0.5f * u23});     // 7 (1+2^-23 not bf16) -> skipped below
  cases.push_back({3.f, 0.75f * ldexpf(1.f, -22)});    // 8: ulp(3)=2^-22 -> RN 3+2^-22, RZ 3
  cases.push_back({1.f, 0.375f * u23, 0.375f * u23});  // 9: exact 1+0.75ulp
  cases.push_back({ldexpf(1.f, 10), 1.f, -ldexpf(1.f, 10), 0.75f * u23});  // 10
  cases.push_back({1.f, 0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f, 0.75f * u23}); // 11: second k-step
  cases.push_back({1.f, 0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f,0.f, -0.25f * u24}); // 12
  cases.push_back({0.75f * u23, 1.f});                 // 13: order swapped
  int row = 0;
  std::vector<int> rows;
  for (size_t c = 0; c < cases.size(); ++c) {
    bool okc = true;
    for (float v : cases[c]) { uint32_t u; memcpy(&u, &v, 4); if (u & 0xFFFF) okc = false; }
    if (!okc) { rows.push_back(-1); continue; }
    for (size_t k = 0; k < cases[c].size(); ++k) A[row * kK + k] = bf(cases[c][k]);
    rows.push_back(row++);
  }
  uint16_t *dA, *dB; float* dD; unsigned int* dErr;
  cudaMalloc(&dA, A.size() * 2); cudaMalloc(&dB, B.size() * 2); cudaMalloc(&dD, 128 * 128 * 4); cudaMalloc(&dErr, 4);
  cudaMemcpy(dA, A.data(), A.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B.data(), B.size() * 2, cudaMemcpyHostToDevice);
  cudaMemset(dErr, 0, 4); cudaMemset(dD, 0, 128 * 128 * 4);
  probe<<<1, 128>>>(dA, dB, dD, dErr);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned int err = 0; cudaMemcpy(&err, dErr, 4, cudaMemcpyDeviceToHost);
  std::vector<float> D(128 * 128);
  cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
  printf("cuda=%s err=%u\n", cudaGetErrorString(e), err);
  for (size_t c = 0; c < cases.size(); ++c) {
    if (rows[c] < 0) { printf("case %zu skipped\n", c); continue; }
    const float d = D[rows[c] * 128 + 0];
    double exact = 0; for (float v : cases[c]) exact += v;
    uint32_t u; memcpy(&u, &d, 4);
    printf("CASE %zu %.17g %.17g\n", c, (double)d, exact);
  }
  return 0;
}
