// Batched Gaussian-kernel CG: many independent systems, each with several
// right-hand sides, advanced together by one graph-captured step.
//
// A "lane" is one right-hand side of one system: its own CG (the iteration of
// mpla_generic_conjugate_gradient, mpla.cpp:888-1010) with its own scalars.
// Vectors of a system are stored interleaved, element (i, k) of the n x R
// block at i*R + k, so a matvec reads the R values of a point together and
// reuses every kernel entry for all R lanes.
//
// One step (captured once into a CUDA graph, replayed until every lane is
// done):
//   mv32    persistent kernel over (system, 128 rows, 1024-column chunk)
//           items of mixed systems: partial K~ d per chunk, entries in FP32
//           with the exponential on the SFU, summed in FP32 per chunk
//   mv64    the same items of FP64 systems: partial K d in FP64
//   true    one slice of every FP64 true-residual round in progress (below)
//           (the launches of this phase, per class and kind, run as
//           concurrent graph branches)
//   alpha   persistent kernel over (system, 1024-row) items: z = nugget d +
//           the chunk partials in chunk order, per-item <d,z>; the last item
//           of a system to finish sums the items in order and sets alpha
//   update  x += alpha d, r -= alpha z, <r,r>; the last item sets beta, the
//           stop test, and for mixed lanes whether the FP64 true residual is
//           due (such a lane then waits for a true-residual round)
//   replace r = b - K x for the lanes of a completed round, convergence test
//           on the FP64 true residual, restart of the direction
//   dir     d = beta d + r (and its FP32 copy)
//   count   lanes still running per system, systems still running; starts
//           and advances the true-residual rounds
// True residuals run in the background of the other systems' iterations.
// A round serves the lanes of one system that were waiting when it started
// (they stop iterating until it ends; the system's other lanes go on).  It
// splits the columns into streams of kTrueSpan 128-column tiles; in each
// step every (row tile, stream) item adds the next column tile of its stream
// to its double-double sums, so the round takes min(tiles, kTrueSpan) steps,
// each step's FP64 work is one tile pair per item (it overlaps the FP32
// matvecs, which use other pipes), and the sums are added in an order fixed
// by the system alone.  (Computing a whole residual inside one step, as
// before, stalled every system for the ~30 ms a n = 15000 residual takes on
// GB300's FP64 pipe, and most steps of a 512-system batch held one.)
// Work is split so that one large system still spreads over the whole GPU,
// and every sum runs in an order fixed by the system's own size: a system's
// result is bitwise the same alone and in any mix.  Systems and item lists
// live in device memory, so systems are added and retired between replays
// (the serving loop) without re-capturing.
//
// Mixed precision.  K~ is the FP32 operator: every scaled coordinate is
// rounded once to FP32, so K~ is the Gaussian kernel matrix of a slightly
// perturbed point set (positive definite again, exactly symmetric) up to the
// rounding of each entry.  The outer iteration is iterative refinement with
// reliable residual replacement: when the recursive residual has fallen
// 100x since the last FP64 true residual, when it claims convergence, or at
// the iteration cap, r = b - K x in FP64 replaces it and the search
// direction restarts from r (the FP32 operator's perturbation makes the old
// direction's conjugacy unusable once r jumps).  Convergence is declared only
// on the FP64 true residual.
//
// Rows per thread of the FP32 matvec (2 or 4) are chosen per (dim, R)
// class by timing each variant on the class's items at first use.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "devutil.cuh"
#include "batch.h"

namespace mgb {

namespace {

constexpr int kTile = 128;        // rows per item and threads per matvec CTA
constexpr int kColTile = 128;     // columns staged per shared-memory round
constexpr int kChunkCols = 1024;  // columns per matvec item
constexpr int kVecThreads = 256;  // threads of the vector-phase CTAs
constexpr int kVecRows = 1024;    // rows per vector-phase item
constexpr int kTrueSpan = 32;     // column tiles per stream of a true-residual round

enum LaneDone : int { LANE_RUNNING = 0, LANE_CONVERGED = 1, LANE_CAPPED = 2, LANE_BROKE = 3 };
enum QueueMode : int { Q_MV32 = 0, Q_MV64 = 1 };

__device__ __forceinline__ float ex2_approx(float v) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

__device__ __forceinline__ bool sys_active(const BatchSys& s) { return s.in_use && s.active_lanes > 0; }
// a lane that iterates this step: running and not waiting for a true residual
__device__ __forceinline__ bool lane_live(const BatchLane& L) { return L.done == LANE_RUNNING && L.hi == 0; }

// Persistent work loop shared by the matvec kernels: items are claimed with
// an atomic counter that the last CTA to finish resets for the next launch.
struct WorkQueue {
  const BatchItem* items;
  const int* count;
  int* counter;
  unsigned int* finished;
};

__device__ __forceinline__ int claim(const WorkQueue& q, int* s_item) {
  __syncthreads();
  if (threadIdx.x == 0) *s_item = atomicAdd(q.counter, 1);
  __syncthreads();
  return *s_item;
}

__device__ __forceinline__ void queue_done(const WorkQueue& q) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int prev = atomicAdd(q.finished, 1u);
    if (prev == gridDim.x - 1) {
      *q.counter = 0;
      *q.finished = 0u;
      __threadfence();
    }
  }
}

// ------------------------------------------------------- FP32 matvec
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
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// Partial (K~ d) over one column chunk for the R lanes of mixed systems of one
// class, into P[chunk].  A thread owns RPT rows (RPT/2 packed pairs: rows r
// and r + 128 of a pair of tiles); column values are staged in shared memory
// twice over so that one load gives a packed operand.  Per 128-column tile
// the products are summed in FP32, the tile sums of the chunk in FP32 as
// well (no FP64 work inside the chunk: GB300's FP64 pipe issues ~2 operations
// per clock per SM), and each chunk partial is stored in FP64.
template <int DIM, int R, int RPT>
__global__ void __launch_bounds__(kTile) k_bmv32(WorkQueue q, const BatchSys* __restrict__ sys) {
  constexpr int NP = RPT / 2;  // packed row pairs per thread
  __shared__ float4 shx[kColTile];  // {x, x, y, y}
  __shared__ float2 sz[kColTile];   // {z, z}
  __shared__ float2 sd[kColTile * R];
  __shared__ int s_item;
  for (;;) {
    const int it = claim(q, &s_item);
    if (it >= *q.count) break;
    const BatchItem w = q.items[it];
    const BatchSys& S = sys[w.sys];
    if (!sys_active(S) || S.live_lanes == 0 || S.precision != MGB_PREC_MIXED || S.dim != DIM || S.R != R) continue;
    // items are 128-row tiles; a variant with RPT rows per thread covers
    // RPT consecutive tiles and takes only every RPT-th item
    if ((w.row0 / kTile) % RPT != 0) continue;
    const int n = S.n;
    uint64_t hx[NP], hy[NP], hz[NP];
    int row[RPT];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      row[2 * p] = w.row0 + threadIdx.x + kTile * (2 * p);
      row[2 * p + 1] = row[2 * p] + kTile;
      const float4 h0 = S.pts_hi[min(row[2 * p], n - 1)], h1 = S.pts_hi[min(row[2 * p + 1], n - 1)];
      hx[p] = f2_pack(h0.x, h1.x);
      hy[p] = f2_pack(h0.y, h1.y);
      hz[p] = f2_pack(h0.z, h1.z);
    }
    uint64_t acc[NP][R];  // chunk sums, packed FP32
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int k = 0; k < R; ++k) acc[p][k] = 0ull;
    const int c0 = w.chunk * kChunkCols, c1 = min(n, c0 + kChunkCols);
    for (int j0 = c0; j0 < c1; j0 += kColTile) {
      const int nj = min(kColTile, c1 - j0);
      __syncthreads();
      for (int t = threadIdx.x; t < kColTile; t += kTile) {
        const bool in = t < nj;
        const float4 h = in ? S.pts_hi[j0 + t] : make_float4(0.f, 0.f, 0.f, 0.f);
        shx[t] = make_float4(h.x, h.x, h.y, h.y);
        sz[t] = make_float2(h.z, h.z);
#pragma unroll
        for (int k = 0; k < R; ++k) {
          const float v = in ? S.d32[(long long)(j0 + t) * R + k] : 0.f;
          sd[t * R + k] = make_float2(v, v);
        }
      }
      __syncthreads();
      uint64_t part[NP][R];
#pragma unroll
      for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int k = 0; k < R; ++k) part[p][k] = 0ull;
#pragma unroll 2
      for (int t = 0; t < nj; ++t) {
        const float4 H = shx[t];
        const uint64_t qhx = f2_pack(H.x, H.y), qhy = f2_pack(H.z, H.w);
        uint64_t qhz = 0ull;
        if (DIM == 3) {
          const float2 Z = sz[t];
          qhz = f2_pack(Z.x, Z.y);
        }
        uint64_t dv[R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
          const float2 v = sd[t * R + k];
          dv[k] = f2_pack(v.x, v.y);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const uint64_t dx = f2_sub(hx[p], qhx);
          const uint64_t dy = f2_sub(hy[p], qhy);
          uint64_t s2;
          if (DIM == 2) {
            s2 = f2_fma(dx, dx, f2_mul(dy, dy));
          } else {
            const uint64_t dz = f2_sub(hz[p], qhz);
            s2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_mul(dz, dz)));
          }
          float s0, s1;
          f2_unpack(s2, s0, s1);
          const uint64_t e2 = f2_pack(ex2_approx(-s0), ex2_approx(-s1));
#pragma unroll
          for (int k = 0; k < R; ++k) part[p][k] = f2_fma(e2, dv[k], part[p][k]);
        }
      }
#pragma unroll
      for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int k = 0; k < R; ++k) acc[p][k] = f2_add(acc[p][k], part[p][k]);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        float a0, a1;
        f2_unpack(acc[p][k], a0, a1);
        if (row[2 * p] < n) S.P[((long long)w.chunk * n + row[2 * p]) * R + k] = (double)a0;
        if (row[2 * p + 1] < n) S.P[((long long)w.chunk * n + row[2 * p + 1]) * R + k] = (double)a1;
      }
    }
  }
  queue_done(q);
}

// ------------------------------------------------------- FP64 matvec
// Partial K d over one column chunk of FP64 systems, into P[chunk] (the
// reference's FP64 iteration).
template <int DIM, int R>
__global__ void __launch_bounds__(kTile) k_bmv64(WorkQueue q, const BatchSys* __restrict__ sys,
                                                 const double* __restrict__ table_g) {
  __shared__ double table[kExpTableSize];
  __shared__ double sp[DIM][kColTile];
  __shared__ double sv[kColTile * R];
  __shared__ int s_item;
  bool have_table = false;  // loaded on the first item with work (most launches have none)
  for (;;) {
    const int it = claim(q, &s_item);
    if (it >= *q.count) break;
    const BatchItem w = q.items[it];
    const BatchSys& S = sys[w.sys];
    if (!sys_active(S) || S.dim != DIM || S.R != R || S.precision != MGB_PREC_FP64) continue;
    if (!have_table) {
      for (int i = threadIdx.x; i < kExpTableSize; i += kTile) table[i] = table_g[i];
      have_table = true;  // the __syncthreads of the column staging below orders it
    }
    const int n = S.n;
    const int i = w.row0 + threadIdx.x;
    const int c0 = w.chunk * kChunkCols, c1 = min(n, c0 + kChunkCols);
    double pi[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) pi[d] = S.pts64[(long long)d * n + min(i, n - 1)];
    double acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = 0.0;
    for (int j0 = c0; j0 < c1; j0 += kColTile) {
      const int nj = min(kColTile, c1 - j0);
      __syncthreads();
      for (int t = threadIdx.x; t < kColTile; t += kTile) {
        const bool in = t < nj;
#pragma unroll
        for (int d = 0; d < DIM; ++d) sp[d][t] = in ? S.pts64[(long long)d * n + j0 + t] : 0.0;
#pragma unroll
        for (int k = 0; k < R; ++k) sv[t * R + k] = in ? S.d[(long long)(j0 + t) * R + k] : 0.0;
      }
      __syncthreads();
      double tile[R];
#pragma unroll
      for (int k = 0; k < R; ++k) tile[k] = 0.0;
      for (int t = 0; t < nj; ++t) {
        double s = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const double df = pi[d] - sp[d][t];
          s = (d == 0) ? df * df : fma(df, df, s);
        }
        const double e = exp_neg_table(s, table);
#pragma unroll
        for (int k = 0; k < R; ++k) tile[k] = fma(e, sv[t * R + k], tile[k]);
      }
#pragma unroll
      for (int k = 0; k < R; ++k) acc[k] += tile[k];
    }
    if (i < n) {
#pragma unroll
      for (int k = 0; k < R; ++k) S.P[((long long)w.chunk * n + i) * R + k] = acc[k];
    }
  }
  queue_done(q);
}

// ---------------------------------------------------- FP64 true residuals
// The true residual z = b - (K x + nugget x) of the mixed lanes in a round.
// On these systems x reaches ~1e4 ||b||, and a plain FP64 sum of K_ij x_j
// over a row carries noise of about u * sum_j |K_ij x_j|, i.e. ~1e-10
// relative: the very tolerance the mixed iteration must certify (points are
// in the caller's order, so even a 128-column tile mixes far-apart large
// terms).  So every product is split exactly by an FMA and summed in
// double-double (TwoSum, Knuth, TAOCP vol. 2, 4.2.2): the compensated dot
// product of Ogita, Rump and Oishi.
__device__ __forceinline__ void dd_add(double& s, double& c, double p, double pe) {
  const double t = __dadd_rn(s, p);
  const double bp = __dsub_rn(t, s);
  const double e = __dadd_rn(__dsub_rn(s, __dsub_rn(t, bp)), __dsub_rn(p, bp));
  s = t;
  c = __dadd_rn(c, __dadd_rn(e, pe));
}

// One step of every round in progress: item (row tile I, stream c) of a
// system adds column tile J = c * kTrueSpan + hi_step of its stream to the
// double-double sums of its 128 rows (zt[c], zero at the round's first
// step).  The systems come from the list the count phase builds; the items
// of all of them are dealt round-robin to the CTAs of the launch.
template <int DIM, int R>
__global__ void __launch_bounds__(kTile) k_btrue(const int* __restrict__ pending, const int* __restrict__ npending,
                                                 BatchSys* __restrict__ sys, const double* __restrict__ table_g) {
  __shared__ double table[kExpTableSize];
  __shared__ double sp[DIM][kTile];
  __shared__ double sv[kTile * R];
  bool have_table = false;
  const int np = *npending;
  long long base = 0;  // index of the current system's first item
  for (int p = 0; p < np; ++p) {
    BatchSys& S = sys[pending[p]];
    if (S.dim != DIM || S.R != R) continue;
    const int n = S.n, T = (n + kTile - 1) / kTile, step = S.hi_step;
    const long long nitems = (long long)T * S.nstream;
    long long k = ((long long)blockIdx.x - base) % gridDim.x;
    if (k < 0) k += gridDim.x;
    base += nitems;
    bool on[R];
#pragma unroll
    for (int l = 0; l < R; ++l) on[l] = S.lanes[l].done == LANE_RUNNING && S.lanes[l].hi == 2;
    for (; k < nitems; k += gridDim.x) {
      const int I = (int)(k % T), c = (int)(k / T);
      const int J = c * kTrueSpan + step;
      if (J >= T) continue;
      if (!have_table) {
        for (int t = threadIdx.x; t < kExpTableSize; t += kTile) table[t] = table_g[t];
        have_table = true;  // ordered by the __syncthreads below
      }
      const int i = I * kTile + threadIdx.x;
      const int j0 = J * kTile, nj = min(kTile, n - j0);
      double* zs = S.zt + (size_t)c * n * R * 2;
      double acc[R], cmp[R];
#pragma unroll
      for (int l = 0; l < R; ++l) {
        acc[l] = cmp[l] = 0.0;
        if (step > 0 && i < n && on[l]) {
          acc[l] = zs[((size_t)i * R + l) * 2];
          cmp[l] = zs[((size_t)i * R + l) * 2 + 1];
        }
      }
      __syncthreads();  // the previous item is done with sp / sv
      for (int t = threadIdx.x; t < kTile; t += kTile) {
        const bool in = t < nj;
#pragma unroll
        for (int d = 0; d < DIM; ++d) sp[d][t] = in ? S.pts64[(long long)d * n + j0 + t] : 0.0;
#pragma unroll
        for (int l = 0; l < R; ++l) sv[t * R + l] = in ? S.x[(long long)(j0 + t) * R + l] : 0.0;
      }
      __syncthreads();
      double pi[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) pi[d] = S.pts64[(long long)d * n + min(i, n - 1)];
      for (int t = 0; t < nj; ++t) {
        double s2 = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const double df = pi[d] - sp[d][t];
          s2 = (d == 0) ? df * df : fma(df, df, s2);
        }
        const double e = exp_neg_table(s2, table);
#pragma unroll
        for (int l = 0; l < R; ++l) {
          if (!on[l]) continue;
          const double vl = sv[t * R + l];
          const double pr = __dmul_rn(e, vl);
          dd_add(acc[l], cmp[l], pr, fma(e, vl, -pr));
        }
      }
      if (i < n) {
#pragma unroll
        for (int l = 0; l < R; ++l) {
          if (!on[l]) continue;
          zs[((size_t)i * R + l) * 2] = acc[l];
          zs[((size_t)i * R + l) * 2 + 1] = cmp[l];
        }
      }
    }
  }
}

// ---------------------------------------------------------- vector phases
// Persistent kernels over (system, kVecRows rows) items.  Each item writes
// its R partial sums to S.vpart in item order; the last item of a system to
// arrive sums them in that order and runs the lane scalars.
template <int R>
__device__ __forceinline__ void block_sums(double (&v)[R], double* smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < R; ++k) smem[warp * 8 + k] = v[k];
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      double t = threadIdx.x < (kVecThreads >> 5) ? smem[threadIdx.x * 8 + k] : 0.0;
      t = warp_sum(t);
      if (threadIdx.x == 0) smem[64 + k] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = smem[64 + k];
  __syncthreads();
}

// Writes this item's partials, and returns true in the last item of the
// system with tot[k] = the system-wide sums (item order).
template <int R>
__device__ bool finish_item(BatchSys& S, int vi, double (&v)[R], double* smem, int* s_last, double (&tot)[8]) {
  block_sums<R>(v, smem);
  if (threadIdx.x < R) S.vpart[vi * 8 + threadIdx.x] = v[threadIdx.x];
  if (!last_block_arrival(S.ticket, (unsigned)S.nvec, s_last)) return false;
#pragma unroll
  for (int k = 0; k < 8; ++k) tot[k] = 0.0;
  for (int c = 0; c < S.nvec; ++c)
#pragma unroll
    for (int k = 0; k < R; ++k) tot[k] += __ldcg(&S.vpart[c * 8 + k]);
  return true;
}

template <int R>
__device__ void vec_alpha(BatchSys& S, int row0, double* smem, int* s_last) {
  double v[R];
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = 0.0;
  const int n = S.n, row1 = min(n, row0 + kVecRows);
  for (int i = row0 + threadIdx.x; i < row1; i += kVecThreads) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const long long o = (long long)i * R + k;
      double z = 0.0;
      for (int c = 0; c < S.nchunks; ++c) z += S.P[(long long)c * n * R + o];
      const double dv = S.d[o];
      z = fma(S.nugget, dv, z);
      S.z[o] = z;
      v[k] = fma(dv, z, v[k]);
    }
  }
  double tot[8];
  if (!finish_item<R>(S, row0 / kVecRows, v, smem, s_last, tot)) return;
  if (threadIdx.x < R) {
    BatchLane& L = S.lanes[threadIdx.x];
    if (lane_live(L)) {
      const double a = L.rr / tot[threadIdx.x];
      if (!(tot[threadIdx.x] > 0.0) || !isfinite(a)) L.done = LANE_BROKE;
      else L.alpha = a;
    }
  }
}

template <int R>
__device__ void vec_update(BatchSys& S, int row0, double* smem, int* s_last, double delta2) {
  __shared__ double s_alpha[8];
  __shared__ int s_run[8];
  if (threadIdx.x < R) {
    s_alpha[threadIdx.x] = S.lanes[threadIdx.x].alpha;
    s_run[threadIdx.x] = lane_live(S.lanes[threadIdx.x]);
  }
  __syncthreads();
  double v[R];
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = 0.0;
  const int row1 = min(S.n, row0 + kVecRows);
  for (int i = row0 + threadIdx.x; i < row1; i += kVecThreads) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const long long o = (long long)i * R + k;
      if (s_run[k]) {
        S.x[o] = fma(s_alpha[k], S.d[o], S.x[o]);
        const double ri = fma(-s_alpha[k], S.z[o], S.r[o]);
        S.r[o] = ri;
        v[k] = fma(ri, ri, v[k]);
      }
    }
  }
  double tot[8];
  if (!finish_item<R>(S, row0 / kVecRows, v, smem, s_last, tot)) return;
  if (threadIdx.x == 0) {
    for (int k = 0; k < R; ++k) {
      BatchLane& L = S.lanes[k];
      if (!s_run[k]) continue;
      L.k += 1;
      const double rr_new = tot[k];
      if (S.precision == MGB_PREC_MIXED) {
        const bool replace = (rr_new < delta2 * L.rr_ref) || (sqrt(rr_new) / L.bnorm < S.eps) ||
                             (L.k + 1 >= S.iter_max) || !(rr_new == rr_new);
        L.rr_new = rr_new;
        if (replace) {
          L.hi = 1;  // waits (does not iterate) until a true-residual round has served it
        } else {
          L.beta = rr_new / L.rr;
          L.rr = rr_new;
        }
      } else {
        L.beta = rr_new / L.rr;
        L.rr = rr_new;
        L.res = sqrt(rr_new) / L.bnorm;
        if (L.res < S.eps) L.done = LANE_CONVERGED;
        else if (!(L.res == L.res)) L.done = LANE_BROKE;
        else if (L.k + 1 >= S.iter_max) L.done = LANE_CAPPED;
      }
    }
  }
}

// Lanes of a completed true-residual round: r = b - (sum of the streams in
// order + nugget x), all in double-double, then the convergence test and a
// restart of the direction from the true residual.
template <int R>
__device__ void vec_replace(BatchSys& S, int row0, double* smem, int* s_last) {
  __shared__ int s_flag[8];
  if (threadIdx.x < R) s_flag[threadIdx.x] = S.lanes[threadIdx.x].done == LANE_RUNNING && S.lanes[threadIdx.x].hi == 2;
  __syncthreads();
  double v[R];
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = 0.0;
  const int n = S.n, row1 = min(n, row0 + kVecRows);
  for (int i = row0 + threadIdx.x; i < row1; i += kVecThreads) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      if (!s_flag[k]) continue;
      const long long o = (long long)i * R + k;
      double acc = 0.0, cmp = 0.0;
      for (int c = 0; c < S.nstream; ++c) {
        const double* zs = S.zt + ((size_t)c * n * R + o) * 2;
        dd_add(acc, cmp, zs[0], zs[1]);
      }
      const double xv = S.x[o];
      const double p = __dmul_rn(S.nugget, xv);
      dd_add(acc, cmp, p, fma(S.nugget, xv, -p));
      // b and acc agree to a few digits, so b - acc is (nearly) exact
      const double ri = __dsub_rn(__dsub_rn(S.b[o], acc), cmp);
      S.r[o] = ri;
      v[k] = fma(ri, ri, v[k]);
    }
  }
  double tot[8];
  if (!finish_item<R>(S, row0 / kVecRows, v, smem, s_last, tot)) return;
  if (threadIdx.x == 0) {
    for (int k = 0; k < R; ++k) {
      if (!s_flag[k]) continue;
      BatchLane& L = S.lanes[k];
      L.res = sqrt(tot[k]) / L.bnorm;
      L.replacements += 1;
      L.beta = 0.0;  // restart the direction from the true residual
      L.rr = tot[k];
      L.rr_ref = tot[k];
      L.hi = 0;
      if (L.res < S.eps) L.done = LANE_CONVERGED;
      else if (!(L.res == L.res)) L.done = LANE_BROKE;
      else if (L.k + 1 >= S.iter_max) L.done = LANE_CAPPED;
    }
    S.hi_ready = 0;
  }
}

template <int R>
__device__ void vec_direction(BatchSys& S, int row0) {
  __shared__ double s_beta[8];
  __shared__ int s_run[8];
  if (threadIdx.x < R) {
    s_beta[threadIdx.x] = S.lanes[threadIdx.x].beta;
    s_run[threadIdx.x] = lane_live(S.lanes[threadIdx.x]);
  }
  __syncthreads();
  const int row1 = min(S.n, row0 + kVecRows);
  for (int i = row0 + threadIdx.x; i < row1; i += kVecThreads) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const long long o = (long long)i * R + k;
      const double dn = s_run[k] ? __dadd_rn(__dmul_rn(s_beta[k], S.d[o]), S.r[o]) : 0.0;
      S.d[o] = dn;
      if (S.d32) S.d32[o] = (float)dn;
    }
  }
}

// One persistent kernel per phase; the R dispatch is a runtime switch over
// templated bodies.  Phase 2 (replace) touches only systems with a completed
// true-residual round; every item of such a system takes part, so the
// last-arrival count is complete.
template <int PHASE>
__global__ void __launch_bounds__(kVecThreads) k_bvec(WorkQueue q, const VecItem* __restrict__ vitems,
                                                      BatchSys* sys, double delta2) {
  __shared__ double smem[80];
  __shared__ int s_item, s_last;
  for (;;) {
    const int it = claim(q, &s_item);
    if (it >= *q.count) break;
    const VecItem w = vitems[it];
    BatchSys& S = sys[w.sys];
    if (!sys_active(S)) continue;
    if (PHASE == 2 && (S.precision != MGB_PREC_MIXED || !S.hi_ready)) continue;
    switch (S.R) {
#define MGB_BVEC_CASE(RR)                                             \
  case RR:                                                            \
    if (PHASE == 0) vec_alpha<RR>(S, w.row0, smem, &s_last);          \
    if (PHASE == 1) vec_update<RR>(S, w.row0, smem, &s_last, delta2); \
    if (PHASE == 2) vec_replace<RR>(S, w.row0, smem, &s_last);        \
    if (PHASE == 3) vec_direction<RR>(S, w.row0);                     \
    break;
      MGB_BVEC_CASE(1)
      MGB_BVEC_CASE(2)
      MGB_BVEC_CASE(3)
      MGB_BVEC_CASE(4)
      MGB_BVEC_CASE(6)
      MGB_BVEC_CASE(8)
#undef MGB_BVEC_CASE
      default:
        break;
    }
  }
  queue_done(q);
}

// Initial state with x0 = 0: r = d = b, <r,r> and ||b|| per lane (one CTA,
// once per admitted system).
__global__ void __launch_bounds__(kVecThreads) k_binit(BatchSys* sys, int slot) {
  __shared__ double smem[80];
  BatchSys& S = sys[slot];
  const int R = S.R;
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = 0.0;
  for (int i = threadIdx.x; i < S.n; i += kVecThreads)
    for (int k = 0; k < R; ++k) {
      const long long o = (long long)i * R + k;
      const double bv = S.b[o];
      S.x[o] = 0.0;
      S.r[o] = bv;
      S.d[o] = bv;
      if (S.d32) S.d32[o] = (float)bv;
      v[k] = fma(bv, bv, v[k]);
    }
  block_sums<8>(v, smem);
  if (threadIdx.x == 0) {
    int act = 0;
    for (int k = 0; k < 8; ++k) {
      BatchLane& L = S.lanes[k];
      L = BatchLane{};
      L.rr = v[k];
      L.rr_ref = v[k];
      L.bnorm = sqrt(v[k]);
      L.res = (L.bnorm > 0.0) ? 1.0 : 0.0;
      if (k >= S.nrhs || L.bnorm == 0.0) L.done = LANE_CONVERGED;  // padding lanes and b = 0
      else if (S.iter_max <= 1) L.done = LANE_CAPPED;
      act += L.done == LANE_RUNNING;
    }
    S.active_lanes = act;
    S.live_lanes = act;
    S.hi_step = -1;
    S.hi_ready = 0;
    *S.ticket = 0u;
  }
}

// End of a step: advances the true-residual rounds (the one in progress took
// its step in this step's matvec phase; a finished one is replaced in the
// next step; a new one starts for the lanes that wait), counts the lanes
// still running and iterating per system and the systems still running, and
// lists the systems with a round in progress in slot order (for the next
// step's true-residual launches).  One CTA of 256 threads.
__global__ void __launch_bounds__(256) k_bcount(BatchSys* sys, int nslots, int* active, int* pending,
                                                int* npending) {
  __shared__ int sm[8];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int a = 0;
  for (int s = threadIdx.x; s < nslots; s += blockDim.x) {
    BatchSys& S = sys[s];
    if (!S.in_use) continue;
    if (S.precision == MGB_PREC_MIXED) {
      if (S.hi_step >= 0) {
        const int T = (S.n + kTile - 1) / kTile;
        S.hi_step += 1;
        if (S.hi_step >= min(T, kTrueSpan)) {
          S.hi_step = -1;
          S.hi_ready = 1;
        }
      }
      if (S.hi_step < 0 && !S.hi_ready) {
        int due = 0;
        for (int k = 0; k < S.R; ++k)
          if (S.lanes[k].done == LANE_RUNNING && S.lanes[k].hi == 1) {
            S.lanes[k].hi = 2;
            ++due;
          }
        if (due) S.hi_step = 0;
      }
    }
    int act = 0, live = 0;
    for (int k = 0; k < S.R; ++k) {
      act += S.lanes[k].done == LANE_RUNNING;
      live += lane_live(S.lanes[k]);
    }
    S.active_lanes = act;
    S.live_lanes = live;
    a += act > 0 ? 1 : 0;
  }
  a = __reduce_add_sync(0xffffffffu, a);
  if (lane == 0) sm[warp] = a;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
    *active = t;
  }
  __syncthreads();
  // compaction in slot order (each thread re-reads the slots it updated)
  for (int s0 = 0; s0 < nslots; s0 += blockDim.x) {
    const int s = s0 + threadIdx.x;
    const bool pend = s < nslots && sys[s].in_use && sys[s].precision == MGB_PREC_MIXED && sys[s].hi_step >= 0;
    const unsigned int m = __ballot_sync(0xffffffffu, pend);
    if (lane == 0) sm[warp] = __popc(m);
    __syncthreads();
    int off = s_base;
    for (int w = 0; w < warp; ++w) off += sm[w];
    if (pend) pending[off + __popc(m & ((1u << lane) - 1u))] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
      s_base += t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *npending = s_base;
}

// Right-hand-side widths with their own kernels: 5 runs as 6 and 7 as 8.
int padded_rhs(int r) { return r <= 4 ? (r < 1 ? 1 : r) : (r <= 6 ? 6 : 8); }
constexpr int kWidths[6] = {1, 2, 3, 4, 6, 8};

}  // namespace

// --------------------------------------------------------------- engine
int BatchEngine::init(DeviceContext* c, int max_systems, cudaStream_t s) {
  c_ = c;
  if (!s) {
    MGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    own_stream_ = true;
  }
  s_ = s;
  max_ = max_systems;
  host_.assign(max_systems, BatchSys{});
  blocks_.assign(max_systems, nullptr);
  MGB_TRY(pool_alloc(c, sizeof(BatchSys) * max_systems, (void**)&dev_sys_));
  MGB_CUDA(cudaMemsetAsync(dev_sys_, 0, sizeof(BatchSys) * max_systems, s));
  max_items_ = 1 << 18;  // 128 systems of n = 16384 in one class
  listed_.assign(max_systems, 0);
  listed_count_ = 0;
  for (int l = 0; l < kLists; ++l)
    for (int q = 0; q < kClasses; ++q)
      MGB_TRY(pool_alloc(c, sizeof(BatchItem) * list_capacity(l), (void**)&items_[l][q]));
  for (int q = 0; q < kClasses; ++q) items_host_[q].clear();
  MGB_TRY(pool_alloc(c, sizeof(VecItem) * max_items_, (void**)&vitems_));
  MGB_TRY(pool_alloc(c, sizeof(int) * max_systems, (void**)&pending_));
  vitems_host_.clear();
  MGB_TRY(pool_alloc(c, sizeof(int) * kCounterInts, (void**)&counters_));
  MGB_CUDA(cudaMemsetAsync(counters_, 0, sizeof(int) * kCounterInts, s));
  MGB_CUDA(cudaMallocHost(&active_host_, sizeof(int)));
  MGB_CUDA(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
  for (int i = 0; i < kBranches; ++i) {
    MGB_CUDA(cudaStreamCreateWithFlags(&side_[i], cudaStreamNonBlocking));
    MGB_CUDA(cudaEventCreateWithFlags(&join_ev_[i], cudaEventDisableTiming));
  }
  for (int k = 0; k < kClasses; ++k) rpt_[k] = 0;
  MGB_CUDA(cudaStreamSynchronize(s));
  return MGB_OK;
}

BatchEngine::~BatchEngine() {
  if (!c_) return;
  cudaStreamSynchronize(s_);
  for (int i = 0; i < max_; ++i)
    if (host_[i].in_use) pool_free(c_, blocks_[i]);
  for (int l = 0; l < kLists; ++l)
    for (int q = 0; q < kClasses; ++q)
      if (items_[l][q]) pool_free(c_, items_[l][q]);
  if (vitems_) pool_free(c_, vitems_);
  if (pending_) pool_free(c_, pending_);
  if (counters_) pool_free(c_, counters_);
  if (dev_sys_) pool_free(c_, dev_sys_);
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  if (graph_) cudaGraphDestroy(graph_);
  if (active_host_) cudaFreeHost(active_host_);
  for (int i = 0; i < kBranches; ++i) {
    if (side_[i]) cudaStreamDestroy(side_[i]);
    if (join_ev_[i]) cudaEventDestroy(join_ev_[i]);
  }
  if (fork_ev_) cudaEventDestroy(fork_ev_);
  if (own_stream_) cudaStreamDestroy(s_);
}

int BatchEngine::class_of(int dim, int R) {
  int r = 0;
  while (r < 5 && kWidths[r] != R) ++r;
  return (dim == 2 ? 0 : 6) + r;
}

static int chunks_of(int n) { return (n + kChunkCols - 1) / kChunkCols; }
static int streams_of(int n) { return ((n + kTile - 1) / kTile + kTrueSpan - 1) / kTrueSpan; }
static int vec_items_of(int n) { return (n + kVecRows - 1) / kVecRows; }

size_t BatchEngine::bytes_needed(int n, int dim, int nrhs, int precision) {
  const int R = padded_rhs(nrhs);
  const size_t nv = (size_t)n * R;
  const size_t pad = 256;
  size_t b = 5 * (sizeof(double) * nv + pad) + sizeof(double) * (size_t)n * dim + pad + sizeof(BatchLane) * 8 + pad;
  b += sizeof(double) * nv * chunks_of(n) + pad;        // matvec partials
  b += sizeof(double) * 8 * vec_items_of(n) + pad;      // vector-phase partials
  b += sizeof(unsigned int) + pad;                      // ticket
  if (precision == MGB_PREC_MIXED)
    b += (sizeof(float4) * (size_t)n + pad) + sizeof(float) * nv + pad + sizeof(double) * 2 * nv * streams_of(n) + pad;
  return b;
}

int BatchEngine::add(int n, int dim, const double* coords_host, double nugget, int nrhs, const double* b_host,
                     int precision, double eps, int iter_max, size_t reserve_bytes, int* handle) {
  if (n <= 0 || (dim != 2 && dim != 3) || nrhs < 1 || nrhs > 8 || !coords_host || !b_host || iter_max < 1)
    return set_error(MGB_ERR_ARG, "batch add: n > 0, dim in {2,3}, 1 <= nrhs <= 8, iter_max >= 1 required");
  if (precision != MGB_PREC_FP64 && precision != MGB_PREC_MIXED)
    return set_error(MGB_ERR_ARG, "batch add: unknown precision %d", precision);
  int slot = -1;
  for (int i = 0; i < max_; ++i)
    if (!host_[i].in_use) {
      slot = i;
      break;
    }
  if (slot < 0) return set_error(MGB_ERR_NOMEM, "batch add: all %d system slots in use", max_);
  const int R = padded_rhs(nrhs);
  const int cls = class_of(dim, R);
  const int nchunks = chunks_of(n), nvec = vec_items_of(n);
  {
    const long long tiles = (n + kTile - 1) / kTile;
    const long long add_items[kLists] = {tiles * nchunks, (tiles + 1) / 2 * nchunks, (tiles + 3) / 4 * nchunks};
    long long have[kLists] = {};
    for (const BatchItem& w : items_host_[cls]) {
      const int t = w.row0 / kTile;
      have[kListAll] += 1;
      have[kListRpt2] += t % 2 == 0;
      have[kListRpt4] += t % 4 == 0;
    }
    bool fits = (long long)vitems_host_.size() + nvec <= max_items_;
    for (int l = 0; l < kLists; ++l) fits = fits && have[l] + add_items[l] <= list_capacity(l);
    if (!fits) return set_error(MGB_ERR_NOMEM, "batch add: more than %d work items", max_items_);
  }
  // admission by free device memory
  const size_t need = bytes_needed(n, dim, nrhs, precision);
  size_t free_b = 0, total_b = 0;
  MGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (reserve_bytes > free_b || need > free_b - reserve_bytes)
    return set_error(MGB_ERR_NOMEM, "batch add: %zu bytes needed, %zu free (reserve %zu)", need, free_b,
                     reserve_bytes);
  BatchSys S{};
  S.in_use = 1;
  S.n = n;
  S.dim = dim;
  S.R = R;
  S.nrhs = nrhs;
  S.precision = precision;
  S.iter_max = iter_max;
  S.eps = eps;
  S.nugget = nugget;
  S.nchunks = nchunks;
  S.nvec = nvec;
  S.nstream = streams_of(n);
  S.hi_step = -1;
  char* base = nullptr;
  MGB_TRY(pool_alloc(c_, need, (void**)&base));
  blocks_[slot] = base;
  auto take = [&](size_t bytes) {
    char* p = base;
    base += (bytes + 255) & ~size_t(255);
    return p;
  };
  const size_t nv = (size_t)n * R;
  S.x = (double*)take(sizeof(double) * nv);
  S.r = (double*)take(sizeof(double) * nv);
  S.d = (double*)take(sizeof(double) * nv);
  S.z = (double*)take(sizeof(double) * nv);
  S.b = (double*)take(sizeof(double) * nv);
  S.P = (double*)take(sizeof(double) * nv * nchunks);
  S.vpart = (double*)take(sizeof(double) * 8 * nvec);
  S.ticket = (unsigned int*)take(sizeof(unsigned int));
  S.pts64 = (const double*)take(sizeof(double) * (size_t)n * dim);
  S.lanes = (BatchLane*)take(sizeof(BatchLane) * 8);
  if (precision == MGB_PREC_MIXED) {
    S.pts_hi = (const float4*)take(sizeof(float4) * (size_t)n);
    S.d32 = (float*)take(sizeof(float) * nv);
    S.zt = (double*)take(sizeof(double) * 2 * nv * S.nstream);
  }
  // host staging: interleave b; scaled coordinates rounded once to FP32
  std::vector<double> bh(nv, 0.0);
  for (int k = 0; k < nrhs; ++k)
    for (int i = 0; i < n; ++i) bh[(size_t)i * R + k] = b_host[(size_t)k * n + i];
  MGB_CUDA(cudaMemcpyAsync(S.b, bh.data(), sizeof(double) * nv, cudaMemcpyHostToDevice, s_));
  MGB_CUDA(cudaMemcpyAsync((void*)S.pts64, coords_host, sizeof(double) * (size_t)n * dim, cudaMemcpyHostToDevice,
                           s_));
  std::vector<float4> ph;
  if (precision == MGB_PREC_MIXED) {
    ph.resize(n);
    const double sc = std::sqrt(1.4426950408889634);  // exp(-s) = 2^(-s log2 e)
    for (int i = 0; i < n; ++i) {
      float h[3] = {0.f, 0.f, 0.f};
      for (int d = 0; d < dim; ++d) h[d] = (float)(coords_host[(size_t)d * n + i] * sc);
      ph[i] = make_float4(h[0], h[1], h[2], 0.f);
    }
    MGB_CUDA(cudaMemcpyAsync((void*)S.pts_hi, ph.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s_));
  }
  host_[slot] = S;
  MGB_CUDA(cudaMemcpyAsync(dev_sys_ + slot, &host_[slot], sizeof(BatchSys), cudaMemcpyHostToDevice, s_));
  k_binit<<<1, kVecThreads, 0, s_>>>(dev_sys_, slot);
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  // the host staging buffers must outlive the async copies
  MGB_CUDA(cudaStreamSynchronize(s_));
  for (int r0 = 0; r0 < n; r0 += kTile)
    for (int c = 0; c < nchunks; ++c) items_host_[cls].push_back(BatchItem{slot, r0, c});
  for (int r0 = 0; r0 < n; r0 += kVecRows) vitems_host_.push_back(VecItem{slot, r0});
  listed_[slot] = 1;
  listed_count_ += 1;
  items_dirty_ = true;
  nslots_ = std::max(nslots_, slot + 1);
  *handle = slot;
  return MGB_OK;
}

// Takes the work items of the slots marked in `drop` out of the lists (their
// systems are finished or released: every kernel would skip them).
void BatchEngine::unlist(const std::vector<char>& drop) {
  for (int q = 0; q < kClasses; ++q) {
    auto& v = items_host_[q];
    v.erase(std::remove_if(v.begin(), v.end(), [&](const BatchItem& w) { return drop[w.sys] != 0; }), v.end());
  }
  vitems_host_.erase(std::remove_if(vitems_host_.begin(), vitems_host_.end(),
                                    [&](const VecItem& w) { return drop[w.sys] != 0; }),
                     vitems_host_.end());
  for (int i = 0; i < max_; ++i)
    if (drop[i] && listed_[i]) {
      listed_[i] = 0;
      listed_count_ -= 1;
    }
  items_dirty_ = true;
}

void BatchEngine::release_slot(int slot) {
  pool_free(c_, blocks_[slot]);
  blocks_[slot] = nullptr;
  if (listed_[slot]) {
    std::vector<char> drop(max_, 0);
    drop[slot] = 1;
    unlist(drop);
  }
  host_[slot] = BatchSys{};
}

// After a replay in which systems finished: read their lane state and drop
// the finished systems' items, so that later steps no longer claim and skip
// them (their results stay in place until read).
int BatchEngine::prune_finished() {
  std::vector<BatchSys> snap(nslots_);
  MGB_CUDA(cudaMemcpyAsync(snap.data(), dev_sys_, sizeof(BatchSys) * nslots_, cudaMemcpyDeviceToHost, s_));
  MGB_CUDA(cudaStreamSynchronize(s_));
  std::vector<char> drop(max_, 0);
  bool any = false;
  for (int i = 0; i < nslots_; ++i)
    if (listed_[i] && snap[i].in_use && snap[i].active_lanes == 0) drop[i] = 1, any = true;
  if (any) unlist(drop);
  return MGB_OK;
}

int BatchEngine::sync_items() {
  if (!items_dirty_) return MGB_OK;
  for (int q = 0; q < kClasses; ++q) {
    for (int l = 0; l < kLists; ++l) list_host_[l][q].clear();
    for (const BatchItem& w : items_host_[q]) {
      const int t = w.row0 / kTile;
      list_host_[kListAll][q].push_back(w);
      if (t % 2 == 0) list_host_[kListRpt2][q].push_back(w);
      if (t % 4 == 0) list_host_[kListRpt4][q].push_back(w);
    }
    for (int l = 0; l < kLists; ++l) {
      const int cnt = (int)list_host_[l][q].size();
      if (cnt)
        MGB_CUDA(cudaMemcpyAsync(items_[l][q], list_host_[l][q].data(), sizeof(BatchItem) * cnt,
                                 cudaMemcpyHostToDevice, s_));
      count_host_[l][q] = cnt;
    }
  }
  for (int q = 0; q < kClasses; ++q) has_mixed_[q] = has_fp64_[q] = false;
  for (int i = 0; i < nslots_; ++i) {
    if (!host_[i].in_use || !listed_[i]) continue;
    const int cls = class_of(host_[i].dim, host_[i].R);
    (host_[i].precision == MGB_PREC_MIXED ? has_mixed_ : has_fp64_)[cls] = true;
  }
  vcount_host_ = (int)vitems_host_.size();
  if (vcount_host_)
    MGB_CUDA(cudaMemcpyAsync(vitems_, vitems_host_.data(), sizeof(VecItem) * vcount_host_, cudaMemcpyHostToDevice,
                             s_));
  MGB_CUDA(cudaMemcpyAsync(counters_ + kOffCount, count_host_, sizeof(int) * kLists * kClasses,
                           cudaMemcpyHostToDevice, s_));
  MGB_CUDA(cudaMemcpyAsync(counters_ + kOffVecCount, &vcount_host_, sizeof(int), cudaMemcpyHostToDevice, s_));
  MGB_CUDA(cudaStreamSynchronize(s_));
  items_dirty_ = false;
  return MGB_OK;
}

// Matvec queue of class `cls` and mode over item list `list`: (claim,
// finished) counters at kOffMv + (cls * 3 + mode) * 2, item count at
// kOffCount + list * kClasses + cls.
static WorkQueue make_queue(const BatchItem* items, int* counters, int cls, int mode, int list) {
  WorkQueue q;
  q.items = items;
  q.count = counters + BatchEngine::kOffCount + list * BatchEngine::kClasses + cls;
  q.counter = counters + BatchEngine::kOffMv + (cls * 3 + mode) * 2;
  q.finished = reinterpret_cast<unsigned int*>(q.counter + 1);
  return q;
}

template <int DIM, int R>
static void launch_mv32(const WorkQueue& q, const BatchSys* sys, int rpt, int sms, cudaStream_t s) {
  // persistent grid: as many CTAs as fit on every SM at once (the light
  // variants hold up to 16 CTAs per SM, the R = 8 four-row one 4), so that
  // the latency of each item's dependent chains is hidden by other CTAs
  static int per_sm[2] = {0, 0};
  int& occ = per_sm[rpt == 4 ? 1 : 0];
  if (occ == 0) {
    int b = 0;
    if (rpt == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bmv32<DIM, R, 4>, kTile, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bmv32<DIM, R, 2>, kTile, 0);
    occ = b > 0 ? b : 4;
  }
  const int grid = occ * sms;
  if (rpt == 4) k_bmv32<DIM, R, 4><<<grid, kTile, 0, s>>>(q, sys);
  else k_bmv32<DIM, R, 2><<<grid, kTile, 0, s>>>(q, sys);
}

// class index -> (DIM, R) for the templated launches
#define MGB_CLASS_SWITCH(cls, CALL)                 \
  switch (cls) {                                    \
    case 0: CALL(2, 1); break;                      \
    case 1: CALL(2, 2); break;                      \
    case 2: CALL(2, 3); break;                      \
    case 3: CALL(2, 4); break;                      \
    case 4: CALL(2, 6); break;                      \
    case 5: CALL(2, 8); break;                      \
    case 6: CALL(3, 1); break;                      \
    case 7: CALL(3, 2); break;                      \
    case 8: CALL(3, 3); break;                      \
    case 9: CALL(3, 4); break;                      \
    case 10: CALL(3, 6); break;                     \
    default: CALL(3, 8); break;                     \
  }

int BatchEngine::enqueue_mv32(int cls, int rpt, cudaStream_t s) {
  const int list = rpt == 4 ? kListRpt4 : kListRpt2;
  const WorkQueue q = make_queue(items_[list][cls], counters_, cls, Q_MV32, list);
#define MGB_MV32(D, R) launch_mv32<D, R>(q, dev_sys_, rpt, c_->num_sms, s)
  MGB_CLASS_SWITCH(cls, MGB_MV32)
#undef MGB_MV32
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

template <int DIM, int R>
static void launch_mv64(const WorkQueue& q, const BatchSys* sys, const double* table, int grid, cudaStream_t s) {
  k_bmv64<DIM, R><<<grid, kTile, 0, s>>>(q, sys, table);
}

int BatchEngine::enqueue_mv64(int cls, int mode, cudaStream_t s) {
  const WorkQueue q = make_queue(items_[kListAll][cls], counters_, cls, mode, kListAll);
  const int grid = 2 * c_->num_sms;
  const double* t = c_->exp_table;
#define MGB_MV64(D, R) launch_mv64<D, R>(q, dev_sys_, t, grid, s)
  MGB_CLASS_SWITCH(cls, MGB_MV64)
#undef MGB_MV64
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

// One step of the true-residual rounds of class `cls` (systems listed by the
// previous step's count phase).
int BatchEngine::enqueue_true(int cls, cudaStream_t s) {
  const int grid = 2 * c_->num_sms;
  const int* np = counters_ + kOffPending;
  const double* t = c_->exp_table;
#define MGB_TRUE(D, R) k_btrue<D, R><<<grid, kTile, 0, s>>>(pending_, np, dev_sys_, t)
  MGB_CLASS_SWITCH(cls, MGB_TRUE)
#undef MGB_TRUE
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

int BatchEngine::enqueue_vec(int phase) {
  WorkQueue q;
  q.items = nullptr;
  q.count = counters_ + kOffVecCount;
  q.counter = counters_ + kOffVec + 2 * phase;
  q.finished = reinterpret_cast<unsigned int*>(q.counter + 1);
  const int grid = 2 * c_->num_sms;
  const double delta2 = 1e-4;  // replacement when the recursive residual fell 100x
  switch (phase) {
    case 0: k_bvec<0><<<grid, kVecThreads, 0, s_>>>(q, vitems_, dev_sys_, delta2); break;
    case 1: k_bvec<1><<<grid, kVecThreads, 0, s_>>>(q, vitems_, dev_sys_, delta2); break;
    case 2: k_bvec<2><<<grid, kVecThreads, 0, s_>>>(q, vitems_, dev_sys_, delta2); break;
    default: k_bvec<3><<<grid, kVecThreads, 0, s_>>>(q, vitems_, dev_sys_, delta2); break;
  }
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

// The matvec launches of one phase (one per class and mode) touch disjoint
// systems and queues, so they run as parallel branches: each on its own side
// stream, forked from and joined back into the engine stream.  Under stream
// capture this becomes a fan-out / fan-in of graph nodes, and the GPU fills
// the tail of one class's launch with the items of the others.
int BatchEngine::fork_branches(int nb) {
  MGB_CUDA(cudaEventRecord(fork_ev_, s_));
  for (int i = 0; i < nb; ++i) MGB_CUDA(cudaStreamWaitEvent(side_[i], fork_ev_, 0));
  return MGB_OK;
}

int BatchEngine::join_branches(int nb) {
  for (int i = 0; i < nb; ++i) {
    MGB_CUDA(cudaEventRecord(join_ev_[i], side_[i]));
    MGB_CUDA(cudaStreamWaitEvent(s_, join_ev_[i], 0));
  }
  return MGB_OK;
}

int BatchEngine::enqueue_step() {
  int nb = 0;
  for (int cls = 0; cls < kClasses; ++cls) nb += 2 * (int)has_mixed_[cls] + (int)has_fp64_[cls];
  MGB_TRY(fork_branches(nb));
  nb = 0;
  for (int cls = 0; cls < kClasses; ++cls) {
    if (has_mixed_[cls]) {
      MGB_TRY(enqueue_mv32(cls, rpt_[cls] ? rpt_[cls] : 2, side_[nb++]));
      MGB_TRY(enqueue_true(cls, side_[nb++]));
    }
    if (has_fp64_[cls]) MGB_TRY(enqueue_mv64(cls, Q_MV64, side_[nb++]));
  }
  MGB_TRY(join_branches(nb));
  MGB_TRY(enqueue_vec(0));
  MGB_TRY(enqueue_vec(1));
  MGB_TRY(enqueue_vec(2));
  MGB_TRY(enqueue_vec(3));
  k_bcount<<<1, 256, 0, s_>>>(dev_sys_, nslots_, counters_ + kOffActive, pending_, counters_ + kOffPending);
  count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

// Autotuner: for each class with mixed work and no choice yet, time one FP32
// matvec of each rows-per-thread variant (outside any capture; the matvec
// only rewrites z, which every step recomputes) and keep the fastest.
int BatchEngine::autotune() {
  cudaEvent_t e0, e1;
  MGB_CUDA(cudaEventCreate(&e0));
  MGB_CUDA(cudaEventCreate(&e1));
  int st = MGB_OK;
  for (int cls = 0; cls < kClasses && st == MGB_OK; ++cls) {
    if (!count_host_[kListAll][cls] || rpt_[cls]) continue;
    bool mixed = false;
    for (const BatchItem& w : items_host_[cls]) mixed |= host_[w.sys].precision == MGB_PREC_MIXED;
    if (!mixed) continue;
    float best = 1e30f;
    int best_rpt = 2;
    for (int v = 1; v < 3 && st == MGB_OK; ++v) {
      const int rpt = 1 << v;
      st = enqueue_mv32(cls, rpt, s_);  // warm-up
      if (st != MGB_OK) break;
      if (cudaEventRecord(e0, s_) != cudaSuccess) {
        st = set_error(MGB_ERR_CUDA, "batch autotune: event failure");
        break;
      }
      st = enqueue_mv32(cls, rpt, s_);
      if (st != MGB_OK) break;
      if (cudaEventRecord(e1, s_) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
        st = set_error(MGB_ERR_CUDA, "batch autotune: event failure");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      tune_ms_[cls][v] = ms;
      if (ms < best) {
        best = ms;
        best_rpt = rpt;
      }
    }
    rpt_[cls] = best_rpt;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

// (Re)captures the step graph when the set of non-empty classes, the slot
// range or a tuning choice changed.
int BatchEngine::prepare_graph() {
  unsigned long long sig = 1469598103934665603ULL;  // FNV-1a over everything the capture bakes in
  auto fold = [&](unsigned long long v) { sig = (sig ^ v) * 1099511628211ULL; };
  for (int q = 0; q < kClasses; ++q) fold((has_mixed_[q] ? 1u : 0u) | (has_fp64_[q] ? 2u : 0u) | (unsigned)rpt_[q] << 2);
  fold((unsigned long long)nslots_);
  if (graph_exec_ && sig == graph_sig_) return MGB_OK;
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  if (graph_) cudaGraphDestroy(graph_);
  graph_exec_ = nullptr;
  graph_ = nullptr;
  MGB_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
  begin_capture_count();
  int st = MGB_OK;
  for (int i = 0; i < kStepsPerGraph && st == MGB_OK; ++i) st = enqueue_step();
  graph_kernels_ = end_capture_count();
  cudaError_t e = cudaStreamEndCapture(s_, &graph_);
  if (st != MGB_OK) return st;
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  MGB_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
  graph_sig_ = sig;
  return MGB_OK;
}

int BatchEngine::run_steps(int steps, int* active_out) {
  MGB_TRY(sync_items());
  MGB_TRY(autotune());
  int done_steps = 0;
  int active = listed_count_;
  while (active > 0 && done_steps < steps) {
    MGB_TRY(prepare_graph());
    MGB_CUDA(cudaGraphLaunch(graph_exec_, s_));
    count_launches(graph_kernels_);
    done_steps += kStepsPerGraph;
    MGB_CUDA(cudaMemcpyAsync(active_host_, counters_ + kOffActive, sizeof(int), cudaMemcpyDeviceToHost, s_));
    MGB_CUDA(cudaStreamSynchronize(s_));
    active = *active_host_;
    if (active < listed_count_) {  // systems finished in this replay
      MGB_TRY(prune_finished());
      MGB_TRY(sync_items());
    }
  }
  if (active_out) *active_out = active;
  return MGB_OK;
}

int BatchEngine::run_async(int steps) {
  MGB_TRY(sync_items());
  MGB_TRY(autotune());
  if (listed_count_ == 0 || steps <= 0) return MGB_OK;
  for (int done_steps = 0; done_steps < steps; done_steps += kStepsPerGraph) {
    MGB_TRY(prepare_graph());
    MGB_CUDA(cudaGraphLaunch(graph_exec_, s_));
    count_launches(graph_kernels_);
  }
  MGB_CUDA(cudaMemcpyAsync(active_host_, counters_ + kOffActive, sizeof(int), cudaMemcpyDeviceToHost, s_));
  launched_ = true;
  return MGB_OK;
}

int BatchEngine::wait(int* active_out) {
  MGB_CUDA(cudaStreamSynchronize(s_));
  const int active = launched_ ? *active_host_ : listed_count_;
  launched_ = false;
  if (active < listed_count_) {  // systems finished in these replays
    MGB_TRY(prune_finished());
    MGB_TRY(sync_items());
  }
  if (active_out) *active_out = active;
  return MGB_OK;
}

int BatchEngine::ready(int* ready_out) {
  const cudaError_t e = cudaStreamQuery(s_);
  if (e == cudaErrorNotReady) {
    *ready_out = 0;
    return MGB_OK;
  }
  MGB_CUDA(e);
  *ready_out = 1;
  return MGB_OK;
}

int BatchEngine::result(int handle, double* x_host, mgb_solve_info* info, bool release) {
  if (handle < 0 || handle >= max_ || !host_[handle].in_use)
    return set_error(MGB_ERR_ARG, "bad batch handle %d", handle);
  const BatchSys& H = host_[handle];
  BatchLane lanes[8];
  MGB_CUDA(cudaMemcpyAsync(lanes, H.lanes, sizeof(lanes), cudaMemcpyDeviceToHost, s_));
  std::vector<double> xi((size_t)H.n * H.R);
  MGB_CUDA(cudaMemcpyAsync(xi.data(), H.x, sizeof(double) * xi.size(), cudaMemcpyDeviceToHost, s_));
  MGB_CUDA(cudaStreamSynchronize(s_));
  if (x_host)
    for (int k = 0; k < H.nrhs; ++k)
      for (int i = 0; i < H.n; ++i) x_host[(size_t)k * H.n + i] = xi[(size_t)i * H.R + k];
  int status = MGB_OK;
  for (int k = 0; k < H.nrhs; ++k) {
    const int st = lanes[k].done == LANE_CONVERGED ? MGB_OK
                   : lanes[k].done == LANE_BROKE   ? MGB_ERR_BREAKDOWN
                                                   : MGB_ERR_NOTCONV;
    if (st != MGB_OK && status == MGB_OK) status = st;
    if (!info) continue;
    mgb_solve_info& f = info[k];
    memset(&f, 0, sizeof(f));
    f.iterations = lanes[k].k;
    f.status = st;
    f.final_res = lanes[k].res;
    f.true_relres = H.precision == MGB_PREC_MIXED ? lanes[k].res : -1.0;
    f.fp64_matvecs = H.precision == MGB_PREC_MIXED ? lanes[k].replacements : lanes[k].k;
    f.low_matvecs = H.precision == MGB_PREC_MIXED ? lanes[k].k : 0;
  }
  if (release) {
    BatchSys empty{};
    MGB_CUDA(cudaMemcpyAsync(dev_sys_ + handle, &empty, sizeof(BatchSys), cudaMemcpyHostToDevice, s_));
    MGB_CUDA(cudaStreamSynchronize(s_));
    release_slot(handle);
  }
  if (status != MGB_OK) set_error(status, "batch system %d: a right-hand side did not converge", handle);
  return status;
}

int BatchEngine::done_handles(std::vector<int>* out) {
  out->clear();
  if (nslots_ == 0) return MGB_OK;
  std::vector<BatchSys> snap(nslots_);
  MGB_CUDA(cudaMemcpyAsync(snap.data(), dev_sys_, sizeof(BatchSys) * nslots_, cudaMemcpyDeviceToHost, s_));
  MGB_CUDA(cudaStreamSynchronize(s_));
  for (int i = 0; i < nslots_; ++i)
    if (host_[i].in_use && snap[i].active_lanes == 0) out->push_back(i);
  return MGB_OK;
}

}  // namespace mgb

// ------------------------------------------------------------------ C ABI
struct mgb_batch {
  mgb::BatchEngine engine;
};

using namespace mgb;

extern "C" {

int mgb_batch_create(int max_systems, mgb_batch** out) {
  if (!out || max_systems <= 0) return set_error(MGB_ERR_ARG, "mgb_batch_create: bad arguments");
  DeviceContext* c = nullptr;
  MGB_TRY(context(&c));
  mgb_batch* b = new mgb_batch();
  const int st = b->engine.init(c, max_systems, nullptr);  // a stream of its own
  if (st != MGB_OK) {
    delete b;
    return st;
  }
  *out = b;
  return MGB_OK;
}

int mgb_batch_add(mgb_batch* b, int n, int dim, const double* coords_host, double nugget, int nrhs,
                  const double* b_host, int precision, double eps, int iter_max, size_t reserve_bytes, int* handle) {
  if (!b || !handle) return set_error(MGB_ERR_ARG, "mgb_batch_add: null argument");
  return b->engine.add(n, dim, coords_host, nugget, nrhs, b_host, precision, eps, iter_max, reserve_bytes, handle);
}

int mgb_batch_run(mgb_batch* b, int max_steps, int* active) {
  if (!b) return set_error(MGB_ERR_ARG, "mgb_batch_run: null batch");
  return b->engine.run_steps(max_steps, active);
}

int mgb_batch_run_async(mgb_batch* b, int max_steps) {
  if (!b) return set_error(MGB_ERR_ARG, "mgb_batch_run_async: null batch");
  return b->engine.run_async(max_steps);
}

int mgb_batch_wait(mgb_batch* b, int* active) {
  if (!b) return set_error(MGB_ERR_ARG, "mgb_batch_wait: null batch");
  return b->engine.wait(active);
}

int mgb_batch_ready(mgb_batch* b, int* ready) {
  if (!b || !ready) return set_error(MGB_ERR_ARG, "mgb_batch_ready: null argument");
  return b->engine.ready(ready);
}

int mgb_batch_finished(mgb_batch* b, int* handles, int capacity, int* count) {
  if (!b || !count || (capacity > 0 && !handles)) return set_error(MGB_ERR_ARG, "mgb_batch_finished: null argument");
  std::vector<int> h;
  MGB_TRY(b->engine.done_handles(&h));
  const int m = (int)h.size() < capacity ? (int)h.size() : capacity;
  for (int i = 0; i < m; ++i) handles[i] = h[i];
  *count = m;
  return MGB_OK;
}

int mgb_batch_result(mgb_batch* b, int handle, double* x_host, mgb_solve_info* info, int release) {
  if (!b) return set_error(MGB_ERR_ARG, "mgb_batch_result: null batch");
  return b->engine.result(handle, x_host, info, release != 0);
}

int mgb_batch_tuning(mgb_batch* b, int* rows_per_thread, float* ms) {
  if (!b) return set_error(MGB_ERR_ARG, "mgb_batch_tuning: null batch");
  for (int c = 0; c < BatchEngine::kClasses; ++c) {
    if (rows_per_thread) rows_per_thread[c] = b->engine.rows_per_thread()[c];
    if (ms)
      for (int v = 0; v < 3; ++v) ms[3 * c + v] = b->engine.tune_ms(c)[v];
  }
  return MGB_OK;
}

int mgb_batch_destroy(mgb_batch* b) {
  delete b;
  return MGB_OK;
}

}  // extern "C"
