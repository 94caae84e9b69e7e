// Symmetric tile-pair Gaussian matvec y = K x for square systems, in FP64
// (plain CG) and FP32 (mixed CG).
//
// K is symmetric, so each 128 x 128 tile pair (I, J) with I <= J is
// evaluated once and used twice: its row sums go to tile I and, for I < J,
// its column sums go to tile J.  That halves the exponentials per matvec
// compared with the reference, which builds and multiplies every entry
// (MPLA src/kernel.cu:118-171, src/generic_system_adapter.cu:83-137).
//
// FP64 (the plain-CG operator and the mixed CG's true residual):
//   pair kernel   a fixed grid strides over the tile pairs; 256 threads in a
//                 16 x 16 grid, each thread an 8 x 8 register block of
//                 entries, with row and column accumulators in registers.
//                 Row sums reduce across a half-warp with shuffles, column
//                 sums across the CTA in shared memory.  Each contribution is
//                 written to its own slot S[tile][other tile][row]: no
//                 atomics.
//   reduce kernel y_i = sum over the T slots of row i in tile order (FP64),
//                 + nugget x_i: a fixed order, so the product is
//                 bit-reproducible.
//   Entries exp(-s) with the table exponential (devutil.cuh) on the squared
//   distance of the caller's coordinates (copied once in k-d tile order);
//   15 FP64 operations per evaluated entry, 7.5 per matrix entry (d = 2).
//   Tile pairs whose entries are all below 2^-80 are left out (60 % of the
//   pairs are evaluated at n = 65536, d = 2, l = 0.05).
//
// FP32 (the mixed CG's operator, MGB_MIXED_SIMT):
//   group kernel  one CTA per column tile and group of 4 row tiles, packed
//                 f32x2 arithmetic on (row, column pair) operands, tile
//                 pairs whose entries are all below 2^-40 left out (see the
//                 kernel);
//   reduce kernel row slots of the near column tiles and the column slots of
//                 the groups, in a fixed order.
//   Points are in k-d tile order (compact tiles, kd_tile_perm) and rounded
//   to FP32 once per point, so the FP32 operator is the Gaussian kernel
//   matrix of a slightly perturbed point set and stays symmetric positive
//   definite.  (A per-tile-pair centring, with the difference of the two
//   tile centres rounded once per pair, perturbs every tile pair
//   differently; at n = 65536 that operator made the mixed solve stagnate at
//   relres 1.4e-10, so coordinates are global.)  Exponentials on the SFU
//   (ex2.approx, with coordinates pre-scaled by sqrt(log2 e)).  3 packed
//   FMA-pipe instructions (6 FP32 lane operations) and 1 MUFU per evaluated
//   entry (d = 2).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "internal.h"
#include "devutil.cuh"
#include "matvecs.h"
#include "gauss_sym.h"

namespace mgb {

namespace {

constexpr int kB = 128;        // tile edge
constexpr int kThreads = 256;  // 16 x 16
constexpr int kR = 8;          // rows per thread
constexpr int kC = 8;          // columns per thread

__device__ __forceinline__ float ex2_approx(float v) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

// Write the CTA's row sums (acc_r, one per thread row) and column sums.
template <typename AccT>
__device__ __forceinline__ void store_sums(AccT (&acc_r)[kR], AccT (&acc_c)[kC], AccT* slot_row, AccT* slot_col,
                                           AccT* colbuf, int ty, int tx) {
  // rows: reduce across the 16 lanes that share ty (a half-warp)
#pragma unroll
  for (int a = 0; a < kR; ++a) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) acc_r[a] += __shfl_xor_sync(0xffffffffu, acc_r[a], o, 16);
  }
  if (tx < kR) {
    AccT v = acc_r[0];
#pragma unroll
    for (int a = 1; a < kR; ++a)
      if (tx == a) v = acc_r[a];
    slot_row[ty + 16 * tx] = v;
  }
  if (slot_col) {
    // columns: 16 partial sums per column (one per ty), summed in ty order;
    // colbuf may alias data the other threads were still reading
    __syncthreads();
#pragma unroll
    for (int b = 0; b < kC; ++b) colbuf[ty * kB + tx + 16 * b] = acc_c[b];
    __syncthreads();
    if (threadIdx.x < kB) {
      AccT v = 0;
#pragma unroll
      for (int q = 0; q < 16; ++q) v += colbuf[q * kB + threadIdx.x];
      slot_col[threadIdx.x] = v;
    }
  }
}

// ----------------------------------------------------------------- FP64
template <int DIM>
__global__ void __launch_bounds__(kThreads) sym_f64_pair_kernel(int n, int T, const double* __restrict__ c0,
                                                                const double* __restrict__ c1,
                                                                const double* __restrict__ c2,
                                                                const double* __restrict__ x,
                                                                const int* __restrict__ perm,
                                                                const double* __restrict__ table_g,
                                                                double* __restrict__ S,
                                                                const int2* __restrict__ pairs, int npairs,
                                                                const int* __restrict__ skip) {
  // A fixed grid strides over the list of near tile pairs (I <= J), so that
  // a launch whose skip flag is set (the mixed CG's true-residual node on
  // most iterations) costs a few hundred CTA starts, not one per tile pair.
  // Coordinates are in tile order, padded to whole tiles; x is the caller's,
  // read through perm (tile position -> caller index).
  if (skip && *skip) return;
  // the exp table is dead once a pair's entries are evaluated; the column
  // reduction buffer (16 x 128 doubles) reuses its storage, and the table is
  // reloaded (from L2) for the next pair
  __shared__ double table[kExpTableSize];
  __shared__ double sp[2][DIM][kB];
  __shared__ double sxv[2][kB];
  double* colbuf = table;
  static_assert(16 * kB <= kExpTableSize, "column buffer must fit in the table storage");
  for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
  const int2 ij = pairs[pair];
  const int I = ij.x, J = ij.y;
  __syncthreads();  // the previous pair's column reduction is done with colbuf
  for (int i = threadIdx.x; i < kExpTableSize; i += kThreads) table[i] = table_g[i];
  for (int t = threadIdx.x; t < 2 * kB; t += kThreads) {
    const int side = t / kB, k = t % kB;
    const int g = (side ? J : I) * kB + k;
#pragma unroll
    for (int d = 0; d < DIM; ++d) sp[side][d][k] = (d == 0 ? c0 : (d == 1 ? c1 : c2))[g];
    sxv[side][k] = g < n ? x[perm[g]] : 0.0;
  }
  __syncthreads();
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  double ri[kR][DIM], xi[kR];
#pragma unroll
  for (int a = 0; a < kR; ++a) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) ri[a][d] = sp[0][d][ty + 16 * a];
    xi[a] = sxv[0][ty + 16 * a];
  }
  double acc_r[kR], acc_c[kC];
#pragma unroll
  for (int a = 0; a < kR; ++a) acc_r[a] = 0.0;
#pragma unroll
  for (int b = 0; b < kC; ++b) acc_c[b] = 0.0;
  const bool diag = (I == J);
#pragma unroll
  for (int b = 0; b < kC; ++b) {
    double cj[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) cj[d] = sp[1][d][tx + 16 * b];
    const double xj = sxv[1][tx + 16 * b];
#pragma unroll
    for (int a = 0; a < kR; ++a) {
      double s = 0.0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const double df = ri[a][d] - cj[d];
        s = (d == 0) ? df * df : fma(df, df, s);
      }
      const double e = exp_neg_table(s, table);
      acc_r[a] = fma(e, xj, acc_r[a]);
      acc_c[b] = fma(e, xi[a], acc_c[b]);
    }
  }
  double* slot_row = S + ((long long)I * T + J) * kB;
  double* slot_col = diag ? nullptr : S + ((long long)J * T + I) * kB;
  store_sums<double>(acc_r, acc_c, slot_row, slot_col, colbuf, ty, tx);
  }
}

// y[perm[i]] = sum_K S[tile(i)][K][i % B] + nugget x[perm[i]], the slots in
// tile order (the slots of far pairs hold zeros)
__global__ void sym_f64_reduce_kernel(int n, int T, const double* __restrict__ S, const int* __restrict__ perm,
                                      const double* __restrict__ x, double nugget, double* __restrict__ y,
                                      const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int tile = i / kB, r = i % kB;
  const double* p = S + (long long)tile * T * kB + r;
  double s = 0.0;
#pragma unroll 4
  for (int k = 0; k < T; ++k) s += __ldcg(p + (long long)k * kB);
  const int o = perm[i];
  y[o] = fma(nugget, x[o], s);
}

// ----------------------------------------------------------------- FP32
// Warp layout for FP32: a CTA of 4 warps evaluates one 128 x 128 tile pair;
// warp w owns columns [32w, 32w+32) of tile J, lane l owns rows
// {l, l+32, l+64, l+96} of tile I.  Per entry: FADDs and one FMUL/FFMA for
// the negated squared distance, one MUFU.EX2, an FFMA into the row sum and an
// FFMA into the lane's partial of that column.  The 32 column partials of a
// lane are summed across the warp by a butterfly reduce-scatter (31 shuffles
// and adds per lane for 4096 entries), after which lane l holds column
// 32w + l complete (the warp saw all 128 rows).  Row sums combine the 4 warps
// in shared memory in warp order.
constexpr int kF32Threads = 128;

__device__ __forceinline__ void warp_reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int half = 16; half >= 1; half >>= 1) {
    const bool upper = (lane & half) != 0;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      const float send = upper ? v[k] : v[k + half];
      const float keep = upper ? v[k + half] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, send, half);
    }
  }
}

// Packed FP32 pairs (Blackwell f32x2 instructions): one instruction applies
// the same operation to two rows.
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
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

// One CTA takes a column tile J and a group of up to kGroup row tiles
// I = kGroup*g .. min(kGroup*g + kGroup - 1, J).  Warp w owns columns
// 32w .. 32w+31 and, for every row tile of the group, lane l owns rows l,
// l+32, l+64, l+96.  A packed pair is one row and two adjacent columns
// (b, b+1): the column tile is staged once in shared memory as column pairs,
// cxy[t] = {x_2t, x_2t+1, y_2t, y_2t+1} and czw[t] = {z_2t, z_2t+1, w_2t,
// w_2t+1} (w the FP32 vector entry), so one broadcast 128-bit load gives the
// packed column operands of 8 entries of a lane.  Per pair of entries: packed
// subtractions, a packed multiply and FMA for the squared distance, two
// MUFU.EX2, a packed FMA into the row's two half-sums (even and odd columns)
// and a packed FMA into the pair of column partials -- both halves of every
// packed accumulator belong to one sum, so no repacking per entry.  (Pairing
// two rows of one column instead needs a MOV and an FADD per column to fold
// the column halves: 7 issue slots per entry against 6.25, and 0.269 against
// 0.213 ms for the whole matvec at n = 65536, d = 2 on GB300.)
// Column partials accumulate over the whole group in registers, and one
// butterfly reduce-scatter per CTA (31 shuffles and adds per lane) leaves
// lane l with column 32w + l complete (the warp saw every row of the group).
// The diagonal tile I = J is evaluated in full for its row sums and adds
// nothing to the column partials (its row weights are zero there), so every
// unordered pair of points counts once per direction.  Row sums of each row
// tile combine the 4 warps in shared memory in warp order.
//
// Tile pairs whose bounding boxes are more than kFarLog2 apart (squared
// distance in the kernel's log2 units) are not evaluated: every entry there
// is below 2^-40, so even summed over all n columns a row loses less than
// n * 2^-40 (6e-8 at n = 65536) -- far below the FP32 rounding of its sum and
// the nugget.  The CTA map lists only groups with a near row tile, and a
// 4-bit mask per CTA marks which of its row tiles are near; the slots of
// far pairs are zeroed once and never written.
//
// The kernel is bound by its FMA pipe (3 packed instructions per entry, each
// two pipe cycles), so occupancy is not what it lacks: with a minimum of one
// CTA per SM in its launch bounds the compiler keeps more entries in flight
// per warp (112 registers at d = 2, 4 CTAs per SM), 4 % faster on GB300 than
// with registers capped for 6 or 7 CTAs per SM (0.207 against 0.215 ms for
// the matvec at n = 65536, d = 2).
constexpr int kGroup = 4;
constexpr double kFarLog2 = 40.0;

template <int DIM>
__global__ void __launch_bounds__(kF32Threads, 1) sym_f32_group_kernel(int n, int T, int GT,
                                                                    const int2* __restrict__ map,
                                                                    const float4* __restrict__ pts,
                                                                    const float* __restrict__ xf,
                                                                    float* __restrict__ Srow,
                                                                    float* __restrict__ Scol,
                                                                    const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ float4 cxy[kB / 2];  // {x_2t, x_2t+1, y_2t, y_2t+1}
  __shared__ float4 czw[kB / 2];  // {z_2t, z_2t+1, w_2t, w_2t+1}
  __shared__ float rowacc[kGroup][4][kB];
  const int2 jm = map[blockIdx.x];
  const int J = jm.x, g = jm.y & 0xFFFF, near = jm.y >> 16;
  const int I0 = kGroup * g, I1 = min(I0 + kGroup - 1, J);
  {
    const int t = threadIdx.x;  // 128 threads, 128 columns
    const int gi = J * kB + t;
    const float4 p = pts[gi];  // padded to whole tiles
    const float w = gi < n ? xf[gi] : 0.f;
    float* fxy = reinterpret_cast<float*>(cxy);
    float* fzw = reinterpret_cast<float*>(czw);
    const int o = 4 * (t >> 1) + (t & 1);
    fxy[o] = p.x;
    fxy[o + 2] = p.y;
    fzw[o] = p.z;
    fzw[o + 2] = w;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t col2[16];  // columns (2b, 2b+1) of the warp's 32
#pragma unroll
  for (int b = 0; b < 16; ++b) col2[b] = 0ull;
#pragma unroll 1
  for (int I = I0; I <= I1; ++I) {
    if (!((near >> (I - I0)) & 1)) continue;
    const bool diag = I == J;
    float rx[4], ry[4], rz[4];
    uint64_t xi2[4], acc2[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int r = I * kB + lane + 32 * a;
      const float4 p = pts[r];
      const float w = (!diag && r < n) ? xf[r] : 0.f;
      rx[a] = p.x;
      ry[a] = p.y;
      rz[a] = p.z;
      xi2[a] = f2_pack(w, w);
      acc2[a] = 0ull;  // +0.0f in both halves
    }
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      const float4 P = cxy[16 * warp + b];
      const float4 Z = czw[16 * warp + b];
      const uint64_t wq = f2_pack(Z.z, Z.w);
      uint64_t c2 = col2[b];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const uint64_t dx = f2_sub(f2_pack(rx[a], rx[a]), f2_pack(P.x, P.y));
        uint64_t s2;
        if (DIM == 1) {
          s2 = f2_mul(dx, dx);
        } else {
          const uint64_t dy = f2_sub(f2_pack(ry[a], ry[a]), f2_pack(P.z, P.w));
          if (DIM == 2) {
            s2 = f2_fma(dx, dx, f2_mul(dy, dy));
          } else {
            const uint64_t dz = f2_sub(f2_pack(rz[a], rz[a]), f2_pack(Z.x, Z.y));
            s2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_mul(dz, dz)));
          }
        }
        float s0, s1;
        f2_unpack(s2, s0, s1);
        const uint64_t e2 = f2_pack(ex2_approx(-s0), ex2_approx(-s1));
        acc2[a] = f2_fma(e2, wq, acc2[a]);
        c2 = f2_fma(e2, xi2[a], c2);
      }
      col2[b] = c2;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      float lo, hi;
      f2_unpack(acc2[a], lo, hi);
      rowacc[I - I0][warp][lane + 32 * a] = lo + hi;
    }
  }
  float col[32];
#pragma unroll
  for (int b = 0; b < 16; ++b) f2_unpack(col2[b], col[2 * b], col[2 * b + 1]);
  warp_reduce_scatter32(col, lane);
  Scol[((long long)J * GT + g) * kB + 32 * warp + lane] = col[0];
  __syncthreads();
  const int r = threadIdx.x;
  for (int I = I0; I <= I1; ++I) {
    const int i = I - I0;
    if (!((near >> i) & 1)) continue;
    Srow[((long long)I * T + J) * kB + r] = ((rowacc[i][0][r] + rowacc[i][1][r]) + rowacc[i][2][r]) + rowacc[i][3][r];
  }
}

// xf[k] = x[perm[k]] rounded to FP32 (once per matvec, not once per tile pair)
__global__ void sym_f32_gather_kernel(int n, const int* __restrict__ perm, const double* __restrict__ x,
                                      float* __restrict__ xf, const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) xf[k] = (float)x[perm[k]];
}

// y[perm[i]] = nugget x + row slots of the near column tiles J >= I (a
// per-row-tile list) + column slots (groups of the column tile I): FP32 sums
// of 8 consecutive slots added in FP64, in a fixed order.  kRedSplit threads
// share a row (warp q of a CTA takes the 8-slot groups q, q + kRedSplit, ...
// of 32 consecutive rows, so every load of a warp is one 128-byte line), and
// their FP64 sums combine in thread order: with one thread per row the loads
// of a row were too few in flight to cover their latency (0.150 ms for the
// slots of n = 131072, d = 3, which stream from HBM at 6.7 TB/s in 0.03 ms).
constexpr int kRedRows = 32, kRedSplit = 8, kRedGroup = 8;

__global__ void __launch_bounds__(kRedRows * kRedSplit) sym_f32_reduce_kernel(
    int n, int T, int GT, const float* __restrict__ Srow, const float* __restrict__ Scol,
    const int* __restrict__ near_off, const int* __restrict__ near_J, const int* __restrict__ perm,
    const double* __restrict__ x, double nugget, double* __restrict__ y, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double part[kRedSplit][kRedRows];
  const int rl = threadIdx.x & (kRedRows - 1), q = threadIdx.x / kRedRows;
  const int i = blockIdx.x * kRedRows + rl;
  double s = 0.0;
  if (i < n) {
    const int I = i / kB, r = i % kB;
    const float* pr = Srow + (long long)I * T * kB + r;
    const int k0 = near_off[I], k1 = near_off[I + 1];
    for (int a = k0 + kRedGroup * q; a < k1; a += kRedGroup * kRedSplit) {
      const int b = min(k1, a + kRedGroup);
      float gsum = 0.f;
#pragma unroll 8
      for (int k = a; k < b; ++k) gsum += __ldcg(pr + (long long)__ldg(&near_J[k]) * kB);
      s += (double)gsum;
    }
    const float* pc = Scol + (long long)I * GT * kB + r;
    const int ng = I / kGroup + 1;
    for (int g0 = kRedGroup * q; g0 < ng; g0 += kRedGroup * kRedSplit) {
      const int g1 = min(ng, g0 + kRedGroup);
      float gsum = 0.f;
#pragma unroll 8
      for (int g = g0; g < g1; ++g) gsum += __ldcg(pc + (long long)g * kB);
      s += (double)gsum;
    }
  }
  part[q][rl] = s;
  __syncthreads();
  if (q == 0 && i < n) {
    double t = part[0][rl];
#pragma unroll
    for (int k = 1; k < kRedSplit; ++k) t += part[k][rl];
    const int o = perm[i];
    y[o] = fma(nugget, x[o], t);
  }
}

// Morton (Z-order) key of a point quantised to 21 bits per axis.
uint64_t spread3(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

uint64_t spread2(uint64_t v) {
  v &= 0xffffffffULL;
  v = (v | v << 16) & 0x0000ffff0000ffffULL;
  v = (v | v << 8) & 0x00ff00ff00ff00ffULL;
  v = (v | v << 4) & 0x0f0f0f0f0f0f0f0fULL;
  v = (v | v << 2) & 0x3333333333333333ULL;
  v = (v | v << 1) & 0x5555555555555555ULL;
  return v;
}

}  // namespace

// ---------------------------------------------------------------- host side
int sym_tiles(int n) { return (n + kB - 1) / kB; }

std::vector<int> kd_tile_perm(const std::vector<double>& h, int n, int dim, int leaf) {
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  struct Range {
    int lo, hi;
  };
  std::vector<Range> stack{{0, n}};
  while (!stack.empty()) {
    const Range r = stack.back();
    stack.pop_back();
    const int cnt = r.hi - r.lo;
    if (cnt <= leaf) {
      std::sort(perm.begin() + r.lo, perm.begin() + r.hi);  // original order inside a tile
      continue;
    }
    int axis = 0;
    double widest = -1.0;
    for (int d = 0; d < dim; ++d) {
      double lo = 1e300, hi = -1e300;
      for (int k = r.lo; k < r.hi; ++k) {
        const double v = h[(size_t)d * n + perm[k]];
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
      if (hi - lo > widest) {
        widest = hi - lo;
        axis = d;
      }
    }
    const double* c = h.data() + (size_t)axis * n;
    const int tiles = (cnt + leaf - 1) / leaf;
    const int mid = r.lo + (tiles / 2) * leaf;
    // a total order (coordinate, then index): the left part is the same set
    // of points on every machine, and each tile is sorted by index at the end
    std::nth_element(perm.begin() + r.lo, perm.begin() + mid, perm.begin() + r.hi,
                     [c](int a, int b) { return c[a] < c[b] || (c[a] == c[b] && a < b); });
    // the right half first on the stack, so the left half is laid out first
    stack.push_back({mid, r.hi});
    stack.push_back({r.lo, mid});
  }
  return perm;
}

std::vector<int> morton_perm(const std::vector<double>& h, int n, int dim) {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    lo[d] = hi[d] = h[(size_t)d * n];
    for (int i = 0; i < n; ++i) {
      lo[d] = std::min(lo[d], h[(size_t)d * n + i]);
      hi[d] = std::max(hi[d], h[(size_t)d * n + i]);
    }
  }
  std::vector<uint64_t> key(n);
  for (int i = 0; i < n; ++i) {
    uint64_t q[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      const double span = hi[d] > lo[d] ? hi[d] - lo[d] : 1.0;
      const double u = (h[(size_t)d * n + i] - lo[d]) / span;
      const double bits = dim == 3 ? 2097151.0 : 4294967295.0;
      q[d] = (uint64_t)std::min(bits, std::max(0.0, u * bits));
    }
    key[i] = dim == 3 ? (spread3(q[0]) | spread3(q[1]) << 1 | spread3(q[2]) << 2)
                      : (dim == 2 ? (spread2(q[0]) | spread2(q[1]) << 1) : q[0]);
  }
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
  return perm;
}

SymF64::~SymF64() {
  if (c_) {
    pool_free(c_, S_);
    pool_free(c_, pts_);
  }
}

// Tile pairs whose entries are all below 2^-80 are left out of the FP64
// operator: summed over all n <= 2^31 columns they change a row by less than
// 2^-49 |x|_max, and in practice (the entries fall off as exp(-s) beyond
// the cut) by far less than one rounding of the row's FP64 sum.
constexpr double kFarF64 = 80.0 * 0.69314718055994531;  // exp(-s) < 2^-80

int SymF64::init(DeviceContext* c, const GaussSystem& g, cudaStream_t s) {
  if (g.rows != g.cols || g.row_offset || g.col_offset || g.dim < 1 || g.dim > 3 ||
      g.nugget_rule != MGB_NUGGET_DIAGONAL)
    return set_error(MGB_ERR_ARG, "symmetric FP64 matvec: square d<=3 systems with a diagonal nugget only");
  c_ = c;
  g_ = g;
  const int n = g.rows, dim = g.dim;
  T_ = sym_tiles(n);
  std::vector<double> h((size_t)n * dim);
  for (int d = 0; d < dim; ++d)
    MGB_CUDA(cudaMemcpyAsync(h.data() + (size_t)d * n, g.coords[d], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  const std::vector<int> perm = kd_tile_perm(h, n, dim, kB);
  const size_t np = (size_t)T_ * kB;
  std::vector<double> pts(3 * np, 0.0);  // tile order, padded with zeros
  for (int d = 0; d < dim; ++d)
    for (int k = 0; k < n; ++k) pts[d * np + k] = h[(size_t)d * n + perm[k]];
  std::vector<double> blo((size_t)3 * T_, 0.0), bhi((size_t)3 * T_, 0.0);
  for (int t = 0; t < T_; ++t) {
    const int b0 = t * kB, b1 = std::min(n, b0 + kB);
    for (int d = 0; d < dim; ++d) {
      double lo = 1e300, hi = -1e300;
      for (int k = b0; k < b1; ++k) {
        lo = std::min(lo, pts[d * np + k]);
        hi = std::max(hi, pts[d * np + k]);
      }
      blo[3 * t + d] = lo;
      bhi[3 * t + d] = hi;
    }
  }
  std::vector<int2> pairs;
  for (int I = 0; I < T_; ++I)
    for (int J = I; J < T_; ++J) {
      double d2 = 0.0;
      for (int d = 0; d < dim; ++d) {
        const double gap = std::max({0.0, blo[3 * J + d] - bhi[3 * I + d], blo[3 * I + d] - bhi[3 * J + d]});
        d2 += gap * gap;
      }
      if (d2 <= kFarF64) pairs.push_back(make_int2(I, J));
    }
  if (pairs.size() > 0x7fffffffULL) return set_error(MGB_ERR_ARG, "system too large for one pair list");
  npairs_ = (int)pairs.size();
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t b_pts = sizeof(double) * 3 * np, b_perm = sizeof(int) * (size_t)n;
  const size_t b_pairs = sizeof(int2) * std::max<size_t>(1, pairs.size());
  MGB_TRY(pool_alloc(c, up(b_pts) + up(b_perm) + up(b_pairs), (void**)&pts_));
  perm_ = reinterpret_cast<int*>(reinterpret_cast<char*>(pts_) + up(b_pts));
  pairs_ = reinterpret_cast<int2*>(reinterpret_cast<char*>(perm_) + up(b_perm));
  MGB_CUDA(cudaMemcpyAsync(pts_, pts.data(), b_pts, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(perm_, perm.data(), b_perm, cudaMemcpyHostToDevice, s));
  if (!pairs.empty())
    MGB_CUDA(cudaMemcpyAsync(pairs_, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, s));
  const size_t b_slots = sizeof(double) * (size_t)T_ * T_ * kB;
  MGB_TRY(pool_alloc(c, b_slots, (void**)&S_));
  // slots of far pairs are never written: zero them once
  MGB_CUDA(cudaMemsetAsync(S_, 0, b_slots, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  return MGB_OK;
}

int SymF64::apply(const double* x, double* y, cudaStream_t s, const int* skip) {
  const int n = g_.rows;
  const size_t np = (size_t)T_ * kB;
  const double* c0 = pts_;
  const double* c1 = pts_ + np;
  const double* c2 = pts_ + 2 * np;
  const unsigned grid = (unsigned)std::max(1, std::min(npairs_, 4 * c_->num_sms));
  const double* tab = c_->exp_table;
  switch (g_.dim) {
    case 1: sym_f64_pair_kernel<1><<<grid, kThreads, 0, s>>>(n, T_, c0, c1, c2, x, perm_, tab, S_, pairs_, npairs_, skip); break;
    case 2: sym_f64_pair_kernel<2><<<grid, kThreads, 0, s>>>(n, T_, c0, c1, c2, x, perm_, tab, S_, pairs_, npairs_, skip); break;
    default: sym_f64_pair_kernel<3><<<grid, kThreads, 0, s>>>(n, T_, c0, c1, c2, x, perm_, tab, S_, pairs_, npairs_, skip); break;
  }
  sym_f64_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, T_, S_, perm_, x, g_.nugget, y, skip);
  count_launches(2);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

SymF32::~SymF32() {
  if (c_) {
    pool_free(c_, S_);
    pool_free(c_, pts_);
  }
}

int SymF32::init(DeviceContext* c, const GaussSystem& g, cudaStream_t s) {
  if (g.rows != g.cols || g.row_offset || g.col_offset || g.dim < 1 || g.dim > 3 ||
      g.nugget_rule != MGB_NUGGET_DIAGONAL)
    return set_error(MGB_ERR_ARG, "mixed matvec: square d<=3 systems with a diagonal nugget only");
  c_ = c;
  n_ = g.rows;
  dim_ = g.dim;
  nugget_ = g.nugget;
  T_ = sym_tiles(n_);
  // coordinates to the host once per system: k-d tile order, tile boxes
  std::vector<double> h((size_t)n_ * dim_);
  for (int d = 0; d < dim_; ++d)
    MGB_CUDA(cudaMemcpyAsync(h.data() + (size_t)d * n_, g.coords[d], sizeof(double) * n_, cudaMemcpyDeviceToHost, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  const double scale = std::sqrt(1.4426950408889634);  // sqrt(log2 e): exp(-s) = 2^(-s log2 e)
  const std::vector<int> perm = kd_tile_perm(h, n_, dim_, kB);
  // global FP32 coordinates (one rounding per point: the FP32 operator is the
  // kernel matrix of a slightly perturbed point set)
  std::vector<float4> pts((size_t)T_ * kB, make_float4(0.f, 0.f, 0.f, 0.f));
  for (int k = 0; k < n_; ++k) {
    float v[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dim_; ++d) v[d] = (float)(h[(size_t)d * n_ + perm[k]] * scale);
    pts[k] = make_float4(v[0], v[1], v[2], 0.f);
  }
  GT_ = T_ / kGroup + 1;
  // tile bounding boxes in the kernel's (log2-scaled FP32) coordinates
  std::vector<double> blo((size_t)3 * T_, 0.0), bhi((size_t)3 * T_, 0.0);
  for (int t = 0; t < T_; ++t) {
    const int b0 = t * kB, b1 = std::min(n_, b0 + kB);
    for (int d = 0; d < 3; ++d) {
      double lo = 1e300, hi = -1e300;
      for (int k = b0; k < b1; ++k) {
        const float4 q = pts[k];
        const double v = d == 0 ? q.x : (d == 1 ? q.y : q.z);
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
      blo[3 * t + d] = lo;
      bhi[3 * t + d] = hi;
    }
  }
  auto far = [&](int a, int b) {
    double d2 = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double gap = std::max({0.0, blo[3 * b + d] - bhi[3 * a + d], blo[3 * a + d] - bhi[3 * b + d]});
      d2 += gap * gap;
    }
    return d2 > kFarLog2;
  };
  std::vector<int2> map;
  pairs_near_ = 0;
  for (int J = 0; J < T_; ++J)
    for (int g = 0; g <= J / kGroup; ++g) {
      int near = 0;
      for (int i = 0; i < kGroup && kGroup * g + i <= J; ++i)
        if (!far(kGroup * g + i, J)) {
          near |= 1 << i;
          ++pairs_near_;
        }
      if (near) map.push_back(make_int2(J, g | (near << 16)));
    }
  // per row tile I: the column tiles J >= I it is near, ascending
  std::vector<int> near_off(T_ + 1, 0), near_J;
  for (int I = 0; I < T_; ++I) {
    for (int J = I; J < T_; ++J)
      if (!far(I, J)) near_J.push_back(J);
    near_off[I + 1] = (int)near_J.size();
  }
  ncta_ = (long long)map.size();
  if (ncta_ > 0x7fffffffLL) return set_error(MGB_ERR_ARG, "system too large for one grid");
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t bytes_pts = sizeof(float4) * pts.size();
  const size_t bytes_map = sizeof(int2) * map.size();
  const size_t bytes_perm = sizeof(int) * (size_t)n_;
  const size_t bytes_off = sizeof(int) * near_off.size(), bytes_nj = sizeof(int) * std::max<size_t>(1, near_J.size());
  MGB_TRY(pool_alloc(c, up(bytes_pts) + up(bytes_map) + up(bytes_perm) + up(bytes_off) + up(bytes_nj), (void**)&pts_));
  map_ = reinterpret_cast<int2*>(reinterpret_cast<char*>(pts_) + up(bytes_pts));
  perm_ = reinterpret_cast<int*>(reinterpret_cast<char*>(map_) + up(bytes_map));
  near_off_ = reinterpret_cast<int*>(reinterpret_cast<char*>(perm_) + up(bytes_perm));
  near_J_ = reinterpret_cast<int*>(reinterpret_cast<char*>(near_off_) + up(bytes_off));
  MGB_CUDA(cudaMemcpyAsync(near_off_, near_off.data(), bytes_off, cudaMemcpyHostToDevice, s));
  if (!near_J.empty())
    MGB_CUDA(cudaMemcpyAsync(near_J_, near_J.data(), sizeof(int) * near_J.size(), cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(pts_, pts.data(), bytes_pts, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(map_, map.data(), bytes_map, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaMemcpyAsync(perm_, perm.data(), bytes_perm, cudaMemcpyHostToDevice, s));
  const size_t nrow = (size_t)T_ * T_ * kB, ncol = (size_t)T_ * GT_ * kB;
  MGB_TRY(pool_alloc(c, sizeof(float) * (nrow + ncol + (size_t)T_ * kB), (void**)&S_));
  Scol_ = S_ + nrow;
  xf_ = Scol_ + ncol;
  // slots of far pairs and groups are never written: zero them once
  MGB_CUDA(cudaMemsetAsync(S_, 0, sizeof(float) * (nrow + ncol), s));
  MGB_CUDA(cudaStreamSynchronize(s));
  return MGB_OK;
}

int SymF32::apply(const double* x, double* y, cudaStream_t s, const int* skip) {
  sym_f32_gather_kernel<<<(n_ + 255) / 256, 256, 0, s>>>(n_, perm_, x, xf_, skip);
  const unsigned grid = (unsigned)ncta_;
  switch (dim_) {
    case 1: sym_f32_group_kernel<1><<<grid, kF32Threads, 0, s>>>(n_, T_, GT_, map_, pts_, xf_, S_, Scol_, skip); break;
    case 2: sym_f32_group_kernel<2><<<grid, kF32Threads, 0, s>>>(n_, T_, GT_, map_, pts_, xf_, S_, Scol_, skip); break;
    default: sym_f32_group_kernel<3><<<grid, kF32Threads, 0, s>>>(n_, T_, GT_, map_, pts_, xf_, S_, Scol_, skip); break;
  }
  sym_f32_reduce_kernel<<<(n_ + kRedRows - 1) / kRedRows, kRedRows * kRedSplit, 0, s>>>(
      n_, T_, GT_, S_, Scol_, near_off_, near_J_, perm_, x, nugget_, y, skip);
  count_launches(3);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

}  // namespace mgb
