// Symmetric FP32 Gaussian matvec with the squared distances on the tensor
// cores (tcgen05, sm_103a): the MGB_MIXED_TENSOR variant of the mixed-CG
// operator (mgb_set_mixed_matvec).  Measured against the default
// (FP32-difference) kernel on GB300 it is slower (1.06 ms against 0.31 ms at
// n = 65536, d = 2: one tile-pair group per CTA leaves the bulk-copy, MMA and
// TMEM-allocation latencies exposed), and its errors -- from norms taken
// relative to a per-tile-pair centre -- are coherent across each 128 x 128
// block, enough at n = 65536 to make the FP32 operator indefinite at a 1e-4
// nugget.  It is kept as the tensor-core form of the operator, tested to the
// same matvec bar on moderate tile extents.  Consistent per-point norms would
// not remove the coherence: tcgen05's FP32 accumulation truncates toward
// zero after aligning the products to the largest (measured by
// tests/test_gpu_tc_accumulation.py), so every distance of a tile pair is
// biased the same way by up to an ulp of its largest term.
//
// Points are in Morton order, in 128-point tiles.  One CTA takes a column
// tile J and two row tiles I0 = 2g, I0 + 1 <= J.  Relative to the column
// tile's centre c_J (an FP32 point), u_i = x_i - c_J and v_j = x_j - c_J, and
//   -s_ij = 2 u_i . v_j - |u_i|^2 - |v_j|^2
// is one K = 32 contraction of BF16 operands with FP32 accumulation: every
// coordinate and squared norm is split into three BF16 parts (24 bits), the
// six significant products of 2 u.v per dimension take one K slot each, and
// the norms pair with ones:
//   A_i = [uh uh um uh um ul]*dim  -|u|^2(h m l)  1 1 1  0...
//   B_j = 2[vh vm vh vl vm vh]*dim  1 1 1  -|v|^2(h m l)  0...
// Coordinates carry sqrt(log2 e), so K_ij = 2^(-s_ij) = ex2(D_ij) on the SFU.
// B operands of every tile are prepared once per system (FP64 on the host);
// A operands are formed per CTA from the FP32 (hi, lo) coordinates.  The
// error of -s is a few FP32 ulps of |u|^2 + |v|^2 with |u - v| small where
// the kernel matters -- no worse than FP32 differences of centred
// coordinates, and far better than differences of global FP32 coordinates.
//
// The MMA writes two 128 x 128 FP32 accumulators into tensor memory (256
// columns, two CTAs per SM).  Each of the 8 warps reads one 32-lane group
// (rows) and one 64-column half with tcgen05.ld, takes ex2 of every entry
// and forms
//   row sums  sum_j K_ij x_j  (per thread: its row, both row tiles, packed)
//   column partials  sum_i K_ij x_i over the two row tiles (per thread),
// then sums the column partials over the warp's 32 rows through shared
// memory and over the 4 lane groups in order.  Each unordered pair of
// points is evaluated once (the diagonal tile J = I keeps j >= i, with
// K_ii = 1), so the operator is exactly symmetric.  Row and column sums go
// to per-pair slots reduced in a fixed order: the matvec is reproducible.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "internal.h"
#include "devutil.cuh"
#include "gauss_sym.h"

namespace mgb {

namespace {

constexpr int kTB = 128;              // points per tile
constexpr int kK = 32;                // contraction length (two K = 16 MMAs)
constexpr int kTcThreads = 256;       // 8 warps
constexpr uint32_t kTmemCols = 256;   // two 128-column FP32 accumulators
constexpr int kOpBytes = kTB * kK * 2;  // one BF16 operand tile: 8 KB
// canonical K-major layout without swizzle: 8 x 16-byte core matrices, the
// next core matrix along K 128 B away (LBO), the next 8-row group 512 B away
// (SBO)
constexpr uint32_t kLBO = 128;
constexpr uint32_t kSBO = 128 * (kK / 8);
constexpr int kTbStride = 20;         // floats per row of the transpose buffer

// shared memory layout (bytes)
constexpr int kSmA = 0;                                   // 2 row-tile operands
constexpr int kSmB = kSmA + 2 * kOpBytes;                 // column-tile operand
constexpr int kSmXj = kSmB + kOpBytes;                    // 128 float2 {x_j, x_j}
constexpr int kSmXi = kSmXj + kTB * 8;                    // 256 floats
constexpr int kSmTb = kSmXi + 2 * kTB * 4;                // 8 warps x 32 x kTbStride floats
constexpr int kSmCol = kSmTb + 8 * 32 * kTbStride * 4;    // [2 halves][4 groups][64] floats
constexpr int kSmRow = kSmCol + 2 * 4 * 64 * 4;           // [2 halves][2 tiles][128] floats
constexpr int kSmBar = kSmRow + 2 * 2 * kTB * 4;          // 2 mbarriers
constexpr int kSmTmem = kSmBar + 16;                      // TMEM base address
constexpr int kSmUsed = kSmTmem + 16;
// requested dynamic shared memory: large enough that no more than two CTAs
// (2 x 256 TMEM columns) are ever resident on one SM
constexpr int kSmRequest = 96 * 1024;
static_assert(kSmUsed <= kSmRequest, "shared memory layout");

__host__ __device__ inline uint32_t op_offset(int row, int kchunk) {
  return (uint32_t)(row / 8) * kSBO + (uint32_t)kchunk * kLBO + (uint32_t)(row % 8) * 16;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) |
         (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both
// K-major, N = 128, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTB >> 3) << 17) |
                            ((uint32_t)(kTB >> 4) << 24);

__device__ __forceinline__ float ex2_approx(float v) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

constexpr uint16_t kBf16One = 0x3F80;

// v = a + b + c (BF16 bits, round to nearest even); the remainders are exact
// in FP32, so a + b + c carries 24 bits of v.
__device__ __forceinline__ void split3(float v, uint16_t& a, uint16_t& b, uint16_t& c) {
  const __nv_bfloat16 x = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(x);
  const __nv_bfloat16 y = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(y);
  const __nv_bfloat16 z = __float2bfloat16_rn(r2);
  a = __bfloat16_as_ushort(x);
  b = __bfloat16_as_ushort(y);
  c = __bfloat16_as_ushort(z);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

// One 16-column chunk of the epilogue.  DIAG0/DIAG1: row tile 0/1 is the
// column tile itself (keep j >= i; the diagonal entry is 1 and counts in the
// row sum only).
template <bool DIAG0, bool DIAG1>
__device__ __forceinline__ void epilogue_chunk(const uint32_t (&d0)[16], const uint32_t (&d1)[16], bool two,
                                               int r, int j0, const float2* __restrict__ xj2, uint64_t xi01,
                                               uint64_t& acc01, float (&cv)[16]) {
#pragma unroll
  for (int jj = 0; jj < 16; ++jj) {
    const int j = j0 + jj;
    float e0 = ex2_approx(__uint_as_float(d0[jj]));
    float e1 = two ? ex2_approx(__uint_as_float(d1[jj])) : 0.f;
    float c0 = e0, c1 = e1;
    if (DIAG0) {
      e0 = j > r ? e0 : (j == r ? 1.f : 0.f);
      c0 = j > r ? c0 : 0.f;
    }
    if (DIAG1) {
      e1 = j > r ? e1 : (j == r ? 1.f : 0.f);
      c1 = j > r ? c1 : 0.f;
    }
    const float2 xj = xj2[j];
    acc01 = f2_fma(f2_pack(e0, e1), f2_pack(xj.x, xj.y), acc01);
    const uint64_t c2 = f2_mul(f2_pack(c0, c1), xi01);
    float a, b;
    f2_unpack(c2, a, b);
    cv[jj] = a + b;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kTcThreads, 2)
    sym_tc_kernel(int n, int T, int GT, const int2* __restrict__ ctamap, const float4* __restrict__ phi,
                  const float4* __restrict__ plo, const float4* __restrict__ centers,
                  const unsigned char* __restrict__ btiles, const float* __restrict__ xf, float* __restrict__ Srow,
                  float* __restrict__ Scol, const int* __restrict__ skip, unsigned int* __restrict__ err) {
  if (skip && *skip) return;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem + kSmA;
  unsigned char* sB = smem + kSmB;
  float2* xj2 = reinterpret_cast<float2*>(smem + kSmXj);
  float* xis = reinterpret_cast<float*>(smem + kSmXi);
  float* tb = reinterpret_cast<float*>(smem + kSmTb);
  float* colp = reinterpret_cast<float*>(smem + kSmCol);
  float* rowp = reinterpret_cast<float*>(smem + kSmRow);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kSmBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kSmTmem);

  const int2 jm = ctamap[blockIdx.x];
  const int J = jm.x, g = jm.y;
  const int I0 = 2 * g;
  const bool two = I0 + 1 <= J;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // column-tile operand: one bulk copy
  if (tid == 0) {
    mbar_arrive_expect_tx(&bars[0], kOpBytes);
    bulk_copy_g2s(sB, btiles + (size_t)J * kOpBytes, kOpBytes, &bars[0]);
  }
  // x of the column tile (duplicated for packed FMAs) and of the row tiles
  if (tid < kTB) {
    const int p = J * kTB + tid;
    const float v = p < n ? xf[p] : 0.f;
    xj2[tid] = make_float2(v, v);
  }
  {
    const int a = tid >> 7, r = tid & 127;
    const int p = (I0 + a) * kTB + r;
    xis[tid] = (a == 0 || two) && p < n ? xf[p] : 0.f;
  }
  // row-tile operands relative to the column tile's centre
  const float4 c = centers[J];
  for (int t = tid; t < 2 * kTB; t += kTcThreads) {
    const int a = t >> 7, r = t & 127;
    const int p = (I0 + a) * kTB + r;
    uint32_t w[kK / 2];  // BF16 pairs (k = 2m low half, 2m + 1 high half)
#pragma unroll
    for (int m = 0; m < kK / 2; ++m) w[m] = 0u;
    if ((a == 0 || two) && p < n) {
      const float4 hp = phi[p], lp = plo[p];
      const float u[3] = {(hp.x - c.x) + lp.x, (hp.y - c.y) + lp.y, (hp.z - c.z) + lp.z};
      float nn = 0.f;
#pragma unroll
      for (int d = DIM - 1; d >= 0; --d) nn = fmaf(u[d], u[d], nn);
      uint16_t row[kK];
#pragma unroll
      for (int k = 0; k < kK; ++k) row[k] = 0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        uint16_t uh, um, ul;
        split3(u[d], uh, um, ul);
        row[6 * d + 0] = uh;
        row[6 * d + 1] = uh;
        row[6 * d + 2] = um;
        row[6 * d + 3] = uh;
        row[6 * d + 4] = um;
        row[6 * d + 5] = ul;
      }
      uint16_t nh, nm, nl;
      split3(-nn, nh, nm, nl);
      row[6 * DIM + 0] = nh;
      row[6 * DIM + 1] = nm;
      row[6 * DIM + 2] = nl;
      row[6 * DIM + 3] = kBf16One;
      row[6 * DIM + 4] = kBf16One;
      row[6 * DIM + 5] = kBf16One;
#pragma unroll
      for (int m = 0; m < kK / 2; ++m) w[m] = (uint32_t)row[2 * m] | ((uint32_t)row[2 * m + 1] << 16);
    }
    unsigned char* base = sA + a * kOpBytes;
#pragma unroll
    for (int kc = 0; kc < kK / 8; ++kc)
      *reinterpret_cast<uint4*>(base + op_offset(r, kc)) = make_uint4(w[4 * kc], w[4 * kc + 1], w[4 * kc + 2], w[4 * kc + 3]);
  }
  fence_proxy_async_smem();  // generic-proxy operand writes -> tensor core reads
  __syncthreads();

  const bool have_b = mbar_wait_bounded(&bars[0], 0, err, DEV_ERR_WAIT_TIMEOUT);
  if (tid == 0 && have_b) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
    for (int a = 0; a < (two ? 2 : 1); ++a) {
#pragma unroll
      for (int ks = 0; ks < kK / 16; ++ks) {
        const uint64_t da = smem_desc(a_base + a * kOpBytes + ks * 2 * kLBO);
        const uint64_t db = smem_desc(b_base + ks * 2 * kLBO);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem + a * kTB),
            "l"(da), "l"(db), "r"(kIdesc), "r"(acc));
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(&bars[1]))
                 : "memory");
  }
  const bool have_d = have_b && mbar_wait_bounded(&bars[1], 0, err, DEV_ERR_WAIT_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue: warp -> (lane group q = rows 32q.., column half h)
  const int q = warp & 3, h = warp >> 2;
  const int r = 32 * q + lane;
  const bool diag0 = (I0 == J), diag1 = two && (I0 + 1 == J);
  uint64_t acc01 = 0ull;
  const uint64_t xi01 = f2_pack(xis[r], xis[kTB + r]);
  float* tbw = tb + warp * 32 * kTbStride;
  if (have_d) {
    for (int ch = 0; ch < 4; ++ch) {
      const int j0 = 64 * h + 16 * ch;
      uint32_t d0[16], d1[16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)j0;
      tmem_ld16(taddr, d0);
      if (two) tmem_ld16(taddr + kTB, d1);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      float cv[16];
      if (diag0) epilogue_chunk<true, false>(d0, d1, two, r, j0, xj2, xi01, acc01, cv);
      else if (diag1) epilogue_chunk<false, true>(d0, d1, two, r, j0, xj2, xi01, acc01, cv);
      else epilogue_chunk<false, false>(d0, d1, two, r, j0, xj2, xi01, acc01, cv);
      // column partials of this chunk: sum over the warp's 32 rows
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4)
        *reinterpret_cast<float4*>(tbw + lane * kTbStride + 4 * k4) =
            make_float4(cv[4 * k4], cv[4 * k4 + 1], cv[4 * k4 + 2], cv[4 * k4 + 3]);
      __syncwarp();
      const int col = lane & 15, rh = lane >> 4;
      float s = 0.f;
#pragma unroll
      for (int rr = 0; rr < 16; ++rr) s += tbw[(16 * rh + rr) * kTbStride + col];
      s += __shfl_down_sync(0xffffffffu, s, 16);
      if (lane < 16) colp[(h * 4 + q) * 64 + 16 * ch + lane] = s;
      __syncwarp();
    }
  }
  float a0, a1;
  f2_unpack(acc01, a0, a1);
  rowp[(h * 2 + 0) * kTB + r] = a0;
  rowp[(h * 2 + 1) * kTB + r] = a1;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (have_d && tid < kTB) {
    // row sums of both row tiles over this column tile
    Srow[((size_t)I0 * T + J) * kTB + tid] = rowp[0 * kTB + tid] + rowp[2 * kTB + tid];
    if (two) Srow[((size_t)(I0 + 1) * T + J) * kTB + tid] = rowp[1 * kTB + tid] + rowp[3 * kTB + tid];
    // column sums over both row tiles: lane groups in order
    const int hh = tid >> 6, cc = tid & 63;
    const float* cp = colp + hh * 4 * 64 + cc;
    Scol[((size_t)J * GT + g) * kTB + tid] = ((cp[0] + cp[64]) + cp[128]) + cp[192];
  }
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// xf[k] = x[perm[k]] rounded to FP32, zero beyond n (whole tiles)
__global__ void tc_gather_kernel(int n, int npad, const int* __restrict__ perm, const double* __restrict__ x,
                                 float* __restrict__ xf, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < npad) xf[k] = k < n ? (float)x[perm[k]] : 0.f;
}

// y[perm[i]] = nugget x + row slots (J >= I) + column slots (groups of the
// column tile I), in FP32 groups of 16 slots added in FP64, in a fixed order.
__global__ void tc_reduce_kernel(int n, int T, int GT, const float* __restrict__ Srow, const float* __restrict__ Scol,
                                 const int* __restrict__ perm, const double* __restrict__ x, double nugget,
                                 double* __restrict__ y, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int I = i / kTB, r = i % kTB;
  double s = 0.0;
  const float* pr = Srow + (size_t)I * T * kTB + r;
  for (int J0 = I; J0 < T; J0 += 16) {
    const int J1 = min(T, J0 + 16);
    float gsum = 0.f;
    for (int J = J0; J < J1; ++J) gsum += __ldcg(pr + (size_t)J * kTB);
    s += (double)gsum;
  }
  const float* pc = Scol + (size_t)I * GT * kTB + r;
  const int ng = I / 2 + 1;
  for (int g0 = 0; g0 < ng; g0 += 16) {
    const int g1 = min(ng, g0 + 16);
    float gsum = 0.f;
    for (int g = g0; g < g1; ++g) gsum += __ldcg(pc + (size_t)g * kTB);
    s += (double)gsum;
  }
  const int o = perm[i];
  y[o] = fma(nugget, x[o], s);
}

// host: round-to-nearest-even BF16 of a float, and the three-part split
uint16_t bf16_bits(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7FFFu + lsb;
  return (uint16_t)(u >> 16);
}
float bf16_value(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float v;
  std::memcpy(&v, &u, 4);
  return v;
}
void split3_host(double v, uint16_t out[3]) {
  double r = v;
  for (int k = 0; k < 3; ++k) {
    out[k] = bf16_bits((float)r);
    r -= (double)bf16_value(out[k]);
  }
}

}  // namespace

// ---------------------------------------------------------------- host side
SymTC::~SymTC() {
  if (c_) {
    pool_free(c_, block_);
    pool_free(c_, S_);
  }
}

int SymTC::init(DeviceContext* c, const GaussSystem& g, cudaStream_t s) {
  if (g.rows != g.cols || g.row_offset || g.col_offset || g.dim < 1 || g.dim > 3 ||
      g.nugget_rule != MGB_NUGGET_DIAGONAL)
    return set_error(MGB_ERR_ARG, "tensor-core mixed matvec: square d<=3 systems with a diagonal nugget only");
  c_ = c;
  n_ = g.rows;
  dim_ = g.dim;
  nugget_ = g.nugget;
  T_ = sym_tiles(n_);
  GT_ = (T_ + 1) / 2;
  std::vector<double> h((size_t)n_ * dim_);
  for (int d = 0; d < dim_; ++d)
    MGB_CUDA(cudaMemcpyAsync(h.data() + (size_t)d * n_, g.coords[d], sizeof(double) * n_, cudaMemcpyDeviceToHost, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  const std::vector<int> perm = morton_perm(h, n_, dim_);
  const double scale = std::sqrt(1.4426950408889634);  // sqrt(log2 e): exp(-s) = 2^(-s log2 e)
  const size_t npad = (size_t)T_ * kTB;
  std::vector<float4> phi(npad, make_float4(0.f, 0.f, 0.f, 0.f)), plo(npad, make_float4(0.f, 0.f, 0.f, 0.f));
  std::vector<float4> ctr(T_, make_float4(0.f, 0.f, 0.f, 0.f));
  std::vector<uint16_t> bt((size_t)T_ * kTB * kK, 0);
  std::vector<int2> map;
  for (int t = 0; t < T_; ++t) {
    const int b0 = t * kTB, b1 = std::min(n_, b0 + kTB);
    double cen[3] = {0, 0, 0};
    for (int k = b0; k < b1; ++k)
      for (int d = 0; d < dim_; ++d) cen[d] += h[(size_t)d * n_ + perm[k]] * scale;
    float cf[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dim_; ++d) cf[d] = (float)(cen[d] / (b1 - b0));
    ctr[t] = make_float4(cf[0], cf[1], cf[2], 0.f);
    for (int k = b0; k < b1; ++k) {
      float hv[3] = {0.f, 0.f, 0.f}, lv[3] = {0.f, 0.f, 0.f};
      double v[3] = {0, 0, 0}, vv = 0.0;
      for (int d = 0; d < dim_; ++d) {
        const double xs = h[(size_t)d * n_ + perm[k]] * scale;
        hv[d] = (float)xs;
        lv[d] = (float)(xs - (double)hv[d]);
        v[d] = xs - (double)cf[d];
        vv += v[d] * v[d];
      }
      phi[k] = make_float4(hv[0], hv[1], hv[2], 0.f);
      plo[k] = make_float4(lv[0], lv[1], lv[2], 0.f);
      // column-tile operand row of point k (position k - b0 of tile t)
      uint16_t row[kK] = {0};
      for (int d = 0; d < dim_; ++d) {
        uint16_t sp[3];
        split3_host(2.0 * v[d], sp);  // 2 v: exact scaling of the split
        row[6 * d + 0] = sp[0];
        row[6 * d + 1] = sp[1];
        row[6 * d + 2] = sp[0];
        row[6 * d + 3] = sp[2];
        row[6 * d + 4] = sp[1];
        row[6 * d + 5] = sp[0];
      }
      uint16_t ns[3];
      split3_host(-vv, ns);
      const uint16_t one = bf16_bits(1.f);
      row[6 * dim_ + 0] = one;
      row[6 * dim_ + 1] = one;
      row[6 * dim_ + 2] = one;
      row[6 * dim_ + 3] = ns[0];
      row[6 * dim_ + 4] = ns[1];
      row[6 * dim_ + 5] = ns[2];
      unsigned char* tile = reinterpret_cast<unsigned char*>(bt.data()) + (size_t)t * kOpBytes;
      for (int kc = 0; kc < kK / 8; ++kc)
        std::memcpy(tile + op_offset(k - b0, kc), &row[8 * kc], 16);
    }
    for (int gg = 0; gg <= t / 2; ++gg) map.push_back(make_int2(t, gg));
  }
  ncta_ = (long long)map.size();
  if (ncta_ > 0x7fffffffLL) return set_error(MGB_ERR_ARG, "system too large for one grid");
  const size_t bytes_b = bt.size() * sizeof(uint16_t);
  const size_t bytes_pts = sizeof(float4) * npad;
  const size_t bytes_ctr = sizeof(float4) * T_;
  const size_t bytes_map = sizeof(int2) * map.size();
  const size_t bytes_perm = sizeof(int) * (size_t)n_;
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  MGB_TRY(pool_alloc(c, up(bytes_b) + 2 * up(bytes_pts) + up(bytes_ctr) + up(bytes_map) + up(bytes_perm),
                     (void**)&block_));
  char* p = reinterpret_cast<char*>(block_);
  btiles_ = reinterpret_cast<unsigned char*>(p);
  p += up(bytes_b);
  phi_ = reinterpret_cast<float4*>(p);
  p += up(bytes_pts);
  plo_ = reinterpret_cast<float4*>(p);
  p += up(bytes_pts);
  ctr_ = reinterpret_cast<float4*>(p);
  p += up(bytes_ctr);
  map_ = reinterpret_cast<int2*>(p);
  p += up(bytes_map);
  perm_ = reinterpret_cast<int*>(p);
  MGB_CUDA(cudaMemcpyAsync(btiles_, bt.data(), bytes_b, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(phi_, phi.data(), bytes_pts, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(plo_, plo.data(), bytes_pts, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(ctr_, ctr.data(), bytes_ctr, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(map_, map.data(), bytes_map, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(perm_, perm.data(), bytes_perm, cudaMemcpyHostToDevice, s));
  const size_t nrow = (size_t)T_ * T_ * kTB, ncol = (size_t)T_ * GT_ * kTB;
  MGB_TRY(pool_alloc(c, sizeof(float) * (nrow + ncol + npad), (void**)&S_));
  Scol_ = S_ + nrow;
  xf_ = Scol_ + ncol;
  // the kernels' shared-memory limit, once per device (a function attribute
  // of the current device; cheap and idempotent, so a race only repeats it)
  static std::atomic<bool> attr_set[64];
  if (c->device >= 0 && c->device < 64 && !attr_set[c->device].load()) {
    MGB_CUDA(cudaFuncSetAttribute(sym_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmRequest));
    MGB_CUDA(cudaFuncSetAttribute(sym_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmRequest));
    MGB_CUDA(cudaFuncSetAttribute(sym_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmRequest));
    attr_set[c->device].store(true);
  }
  MGB_CUDA(cudaStreamSynchronize(s));
  return MGB_OK;
}

int SymTC::apply(const double* x, double* y, cudaStream_t s, const int* skip) {
  const int npad = T_ * kTB;
  tc_gather_kernel<<<(npad + 255) / 256, 256, 0, s>>>(n_, npad, perm_, x, xf_, skip);
  const unsigned grid = (unsigned)ncta_;
  switch (dim_) {
    case 1:
      sym_tc_kernel<1><<<grid, kTcThreads, kSmRequest, s>>>(n_, T_, GT_, map_, phi_, plo_, ctr_, btiles_, xf_, S_,
                                                            Scol_, skip, c_->dev_error);
      break;
    case 2:
      sym_tc_kernel<2><<<grid, kTcThreads, kSmRequest, s>>>(n_, T_, GT_, map_, phi_, plo_, ctr_, btiles_, xf_, S_,
                                                            Scol_, skip, c_->dev_error);
      break;
    default:
      sym_tc_kernel<3><<<grid, kTcThreads, kSmRequest, s>>>(n_, T_, GT_, map_, phi_, plo_, ctr_, btiles_, xf_, S_,
                                                            Scol_, skip, c_->dev_error);
      break;
  }
  tc_reduce_kernel<<<(n_ + 255) / 256, 256, 0, s>>>(n_, T_, GT_, S_, Scol_, perm_, x, nugget_, y, skip);
  count_launches(3);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

}  // namespace mgb
