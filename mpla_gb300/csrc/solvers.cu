// Device-resident Krylov solvers: CG with the two stopping rules of MPLA,
// BiCGSTAB, and the mixed-precision CG with FP64 residual replacement.
//
// The operation order follows MPLA src/mpla.cpp:817-1183 (same recurrences,
// same scalar formulas, same stopping tests and iteration numbering), but the
// host no longer drives every BLAS-1 call:
//   * all scalars (alpha, beta, omega, norms, iteration count, stop flag) live
//     in a SolverState in device memory;
//   * each iteration is a matvec plus three fused kernels (axpys and dot
//     products in one pass, warp-shuffle + block reductions, the last CTA
//     finishing the scalar algebra), instead of 3 blocking cublasDdot calls
//     and 7 daxpy/memset calls per iteration;
//   * iterations are captured once into a CUDA graph and replayed in chunks;
//     after convergence every kernel returns at its first instruction, so the
//     host only checks the stop flag once per chunk.
// Dot products use a fixed reduction tree, so a solve is bit-reproducible.
#include <cmath>
#include <cstring>

#include "internal.h"
#include "devutil.cuh"

namespace mgb {

namespace {

constexpr int T = kReduceThreads;
constexpr int kChunk = 16;  // iterations per graph launch

struct RedCtx {
  double* partials;       // kMaxReduceBlocks * 4
  unsigned int* ticket;   // one counter
};

__device__ __forceinline__ double stop_measure(const SolverState* st, double rr) {
  return (st->stop_rule == MGB_STOP_RMS) ? sqrt(rr / (double)st->n) : sqrt(rr) / st->bnorm;
}

// Reduce up to 3 per-thread values over the grid.  Returns true in the last
// block, where out[q] holds the grid totals (summed over blocks in order).
template <int Q>
__device__ __forceinline__ bool grid_reduce(double (&v)[Q], RedCtx rc, double (&out)[Q]) {
  __shared__ double sm[32];
  __shared__ int s_last;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    double b = block_sum(v[q], sm);
    if (threadIdx.x == 0) rc.partials[q * kMaxReduceBlocks + blockIdx.x] = b;
  }
  if (!last_block_arrival(rc.ticket, gridDim.x, &s_last)) return false;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    // block totals in block order: each thread sums a strided subset in
    // order, then the fixed block tree combines them.
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) t += __ldcg(&rc.partials[q * kMaxReduceBlocks + b]);
    out[q] = block_sum(t, sm);
  }
  return true;
}

// ----------------------------------------------------------------- CG
__global__ void __launch_bounds__(T) k_cg_init(int n, const double* __restrict__ b, const double* __restrict__ z,
                                               double* __restrict__ r, double* __restrict__ d, SolverState* st,
                                               double* hist, RedCtx rc) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    const double ri = b[i] - z[i];
    r[i] = ri;
    d[i] = ri;
    v[0] = fma(ri, ri, v[0]);
    v[1] = fma(b[i], b[i], v[1]);
  }
  double tot[2];
  if (grid_reduce<2>(v, rc, tot) && threadIdx.x == 0) {
    st->rr = tot[0];
    st->bnorm = sqrt(tot[1]);
    st->k = 0;
    const double res = stop_measure(st, tot[0]);
    st->res = res;
    if (hist) hist[0] = res;
    st->done = (res < st->eps) ? CONVERGED : ((st->iter_max <= 1) ? CAPPED : RUNNING);
  }
}

// alpha = <r,r> / <d,z>  (mpla.cpp:944-946)
__global__ void __launch_bounds__(T) k_cg_alpha(int n, const double* __restrict__ d, const double* __restrict__ z,
                                                SolverState* st, RedCtx rc) {
  if (st->done) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) v[0] = fma(d[i], z[i], v[0]);
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    st->t2 = tot[0];
    const double a = st->rr / tot[0];
    if (!(tot[0] > 0.0) || !isfinite(a)) st->done = BROKE_DOWN;
    else st->alpha = a;
  }
}

// x += alpha d; r -= alpha z; beta = <r,r>_new / <r,r>_old; stop test
// (mpla.cpp:948-968 and 849-871).
__global__ void __launch_bounds__(T) k_cg_update(int n, const double* __restrict__ d, const double* __restrict__ z,
                                                 double* __restrict__ x, double* __restrict__ r, SolverState* st,
                                                 double* hist, RedCtx rc) {
  if (st->done) return;
  const double a = st->alpha;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    x[i] = fma(a, d[i], x[i]);
    const double ri = fma(-a, z[i], r[i]);
    r[i] = ri;
    v[0] = fma(ri, ri, v[0]);
  }
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    const int k = st->k + 1;
    st->k = k;
    st->beta = tot[0] / st->rr;
    st->rr = tot[0];
    const double res = stop_measure(st, tot[0]);
    st->res = res;
    if (hist) hist[k] = res;
    if (res < st->eps) st->done = CONVERGED;
    else if (!(res == res)) st->done = BROKE_DOWN;
    else if (k + 1 >= st->iter_max) st->done = CAPPED;
  }
}

// d = beta d + r, rounded as the reference's two daxpys into a zeroed
// temporary: fl(fl(beta*d) + r)  (mpla.cpp:970-975)
__global__ void __launch_bounds__(T) k_cg_direction(int n, const double* __restrict__ r, double* __restrict__ d,
                                                    const SolverState* st) {
  if (st->done) return;
  const double be = st->beta;
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) d[i] = __dadd_rn(__dmul_rn(be, d[i]), r[i]);
}

// <r,r> after a restart load (the reference recomputes it in the loop).
__global__ void __launch_bounds__(T) k_rr(int n, const double* __restrict__ r, SolverState* st, RedCtx rc) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) v[0] = fma(r[i], r[i], v[0]);
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) st->rr = tot[0];
}

// ---------------------------------------------------------- mixed CG
// Iteration: z = A_lo d (FP32 kernel); alpha; k_mx_update; z = A_hi x
// (skipped unless a replacement is due); k_mx_replace; direction.
// Replacement (reliable update) when the recursive residual has dropped by
// `delta` since the last true residual, when it claims convergence, or at
// the iteration cap; the search direction then restarts from the true
// residual (iterative refinement with a CG inner solve that keeps x).
// Convergence is only ever declared on the FP64 true residual
// ||b - A_hi x|| / ||b||.
__global__ void __launch_bounds__(T) k_mx_update(int n, const double* __restrict__ d, const double* __restrict__ z,
                                                 double* __restrict__ x, double* __restrict__ r, SolverState* st,
                                                 double delta2, RedCtx rc) {
  if (st->done) return;
  const double a = st->alpha;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    x[i] = fma(a, d[i], x[i]);
    const double ri = fma(-a, z[i], r[i]);
    r[i] = ri;
    v[0] = fma(ri, ri, v[0]);
  }
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    const int k = st->k + 1;
    st->k = k;
    const double rr_new = tot[0];
    const bool replace = (rr_new < delta2 * st->rr_ref) || (sqrt(rr_new) / st->bnorm < st->eps) ||
                         (k + 1 >= st->iter_max) || !(rr_new == rr_new);
    st->t3 = rr_new;
    if (replace) {
      st->flag = 0;  // run the FP64 matvec and the replacement
    } else {
      st->flag = 1;
      st->beta = rr_new / st->rr;
      st->rr = rr_new;
    }
  }
}

__global__ void __launch_bounds__(T) k_mx_replace(int n, const double* __restrict__ b, const double* __restrict__ z,
                                                  double* __restrict__ r, SolverState* st, double* hist,
                                                  int* replacements, RedCtx rc) {
  if (st->done || st->flag) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    const double ri = b[i] - z[i];
    r[i] = ri;
    v[0] = fma(ri, ri, v[0]);
  }
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    const double rr_true = tot[0];
    const double res = sqrt(rr_true) / st->bnorm;
    st->res = res;
    if (hist) hist[st->k] = res;
    *replacements += 1;
    // restart the direction from the true residual: the FP32 operator's
    // perturbation leaves the old direction's conjugacy unusable once r jumps
    st->beta = 0.0;
    st->rr = rr_true;
    st->rr_ref = rr_true;
    st->flag = 1;
    if (res < st->eps) st->done = CONVERGED;
    else if (!(res == res)) st->done = BROKE_DOWN;
    else if (st->k + 1 >= st->iter_max) st->done = CAPPED;
  }
}

// ------------------------------------------------------------ BiCGSTAB
// Follows mpla.cpp:1030-1150.  rho = <r_hat, r> of the current iteration.
__global__ void __launch_bounds__(T) k_bi_init(int n, const double* __restrict__ b, const double* __restrict__ z,
                                               double* __restrict__ r, double* __restrict__ rh, double* __restrict__ p,
                                               SolverState* st, double* hist, RedCtx rc) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    const double ri = b[i] - z[i];
    r[i] = ri;
    rh[i] = ri;
    p[i] = ri;
    v[0] = fma(ri, ri, v[0]);
    v[1] = fma(b[i], b[i], v[1]);
  }
  double tot[2];
  if (grid_reduce<2>(v, rc, tot) && threadIdx.x == 0) {
    st->rr = tot[0];  // <r_hat, r> = <r0, r0>
    st->bnorm = sqrt(tot[1]);
    st->k = 0;
    const double res = sqrt(tot[0]) / st->bnorm;
    st->res = res;
    if (hist) hist[0] = res;
    st->done = (res < st->eps) ? CONVERGED : ((st->iter_max <= 1) ? CAPPED : RUNNING);
  }
}

// alpha = rho / <z, r_hat>, then s = r - alpha z   (mpla.cpp:1091-1103)
__global__ void __launch_bounds__(T) k_bi_alpha(int n, const double* __restrict__ z, const double* __restrict__ rh,
                                                SolverState* st, RedCtx rc) {
  if (st->done) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) v[0] = fma(z[i], rh[i], v[0]);
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    const double a = st->rr / tot[0];
    if (!isfinite(a) || tot[0] == 0.0) st->done = BROKE_DOWN;
    else st->alpha = a;
  }
}

__global__ void __launch_bounds__(T) k_bi_s(int n, const double* __restrict__ r, const double* __restrict__ z,
                                            double* __restrict__ s, const SolverState* st) {
  if (st->done) return;
  const double a = st->alpha;
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) s[i] = fma(-a, z[i], r[i]);
}

// omega = <zz, s> / <zz, zz>   (mpla.cpp:1105-1110)
__global__ void __launch_bounds__(T) k_bi_omega(int n, const double* __restrict__ zz, const double* __restrict__ s,
                                                SolverState* st, RedCtx rc) {
  if (st->done) return;
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    v[0] = fma(zz[i], s[i], v[0]);
    v[1] = fma(zz[i], zz[i], v[1]);
  }
  double tot[2];
  if (grid_reduce<2>(v, rc, tot) && threadIdx.x == 0) {
    const double w = tot[0] / tot[1];
    if (!isfinite(w) || w == 0.0) st->done = BROKE_DOWN;
    else st->omega = w;
  }
}

// x += alpha p + omega s; r = s - omega zz; beta = (alpha/omega)(<r,r_hat>/rho)
// (mpla.cpp:1112-1123)
__global__ void __launch_bounds__(T) k_bi_update(int n, const double* __restrict__ p, const double* __restrict__ s,
                                                 const double* __restrict__ zz, const double* __restrict__ rh,
                                                 double* __restrict__ x, double* __restrict__ r, SolverState* st,
                                                 RedCtx rc) {
  if (st->done) return;
  const double a = st->alpha, w = st->omega;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    x[i] = fma(w, s[i], fma(a, p[i], x[i]));
    const double ri = fma(-w, zz[i], s[i]);
    r[i] = ri;
    v[0] = fma(ri, rh[i], v[0]);
  }
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    const double be = (a / w) * (tot[0] / st->rr);
    if (!isfinite(be)) st->done = BROKE_DOWN;
    st->beta = be;
    st->rr = tot[0];
  }
}

// p = r + beta (p - omega z)   (mpla.cpp:1125-1131)
__global__ void __launch_bounds__(T) k_bi_p(int n, const double* __restrict__ r, const double* __restrict__ z,
                                            double* __restrict__ p, const SolverState* st) {
  if (st->done) return;
  const double be = st->beta, w = st->omega;
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    const double t = fma(-w, z[i], p[i]);
    p[i] = fma(be, t, r[i]);
  }
}

// true residual zz = b - A x and its relative norm   (mpla.cpp:1133-1150)
__global__ void __launch_bounds__(T) k_bi_true(int n, const double* __restrict__ b, const double* __restrict__ z,
                                               double* __restrict__ zz, SolverState* st, double* hist, RedCtx rc) {
  if (st->done) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) {
    const double t = b[i] - z[i];
    zz[i] = t;
    v[0] = fma(t, t, v[0]);
  }
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) {
    const int k = st->k + 1;
    st->k = k;
    const double res = sqrt(tot[0]) / st->bnorm;
    st->res = res;
    if (hist) hist[k] = res;
    if (res < st->eps) st->done = CONVERGED;
    else if (!(res == res)) st->done = BROKE_DOWN;
    else if (k + 1 >= st->iter_max) st->done = CAPPED;
  }
}

// ------------------------------------------------------------- BLAS-1
__global__ void __launch_bounds__(T) k_dot(int n, const double* __restrict__ x, const double* __restrict__ y,
                                           double* out, RedCtx rc) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) v[0] = fma(x[i], y[i], v[0]);
  double tot[1];
  if (grid_reduce<1>(v, rc, tot) && threadIdx.x == 0) *out = tot[0];
}

__global__ void __launch_bounds__(T) k_axpy(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (int i = blockIdx.x * T + threadIdx.x; i < n; i += gridDim.x * T) y[i] = fma(a, x[i], y[i]);
}

__global__ void k_set_state(SolverState* st, double eps, int iter_max, int stop_rule, int n) {
  st->eps = eps;
  st->iter_max = iter_max;
  st->stop_rule = stop_rule;
  st->n = n;
  st->k = 0;
  st->done = RUNNING;
  st->flag = 1;
}

int vec_blocks(const DeviceContext* c, int n) {
  int b = (n + T * 4 - 1) / (T * 4);
  b = b < 1 ? 1 : b;
  const int cap = 2 * c->num_sms < kMaxReduceBlocks ? 2 * c->num_sms : kMaxReduceBlocks;
  return b > cap ? cap : b;
}

RedCtx red_ctx(DeviceContext* c) { return RedCtx{c->partials, c->tickets}; }

}  // namespace

// ---------------------------------------------------------------- BLAS-1 API
int launch_dot(DeviceContext* c, int n, const double* x, const double* y, double* out_dev, cudaStream_t s) {
  k_dot<<<vec_blocks(c, n), T, 0, s>>>(n, x, y, out_dev, red_ctx(c)); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

int launch_axpy(DeviceContext* c, int n, double alpha, const double* x, double* y, cudaStream_t s) {
  if (n <= 0) return MGB_OK;
  k_axpy<<<vec_blocks(c, n), T, 0, s>>>(n, alpha, x, y); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  return MGB_OK;
}

// --------------------------------------------------------------- drivers
namespace {

// Workspace of one solve: vectors and state from the pool, freed on exit.
struct Workspace {
  DeviceContext* c;
  std::vector<void*> blocks;
  explicit Workspace(DeviceContext* ctx) : c(ctx) {}
  ~Workspace() {
    for (void* p : blocks) pool_free(c, p);
  }
  int get(size_t bytes, void** out) {
    MGB_TRY(pool_alloc(c, bytes, out));
    blocks.push_back(*out);
    return MGB_OK;
  }
};

struct GraphHolder {
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  long long kernels = 0;  // kernel nodes per replay
  ~GraphHolder() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

// Capture `iters` iterations produced by `body` into an executable graph.
template <class Body>
int capture_iterations(cudaStream_t s, int iters, Body body, GraphHolder* g) {
  MGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  begin_capture_count();
  int st = MGB_OK;
  for (int i = 0; i < iters && st == MGB_OK; ++i) st = body();
  g->kernels = end_capture_count();
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (st != MGB_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  g->graph = graph;
  MGB_CUDA(cudaGraphInstantiate(&g->exec, graph, 0));
  return MGB_OK;
}

void print_history(const SolveOptions& o, const double* hist_host, int from_k, int to_k, double n_for_rms) {
  (void)n_for_rms;
  if (!o.print_every) return;
  for (int k = from_k; k <= to_k; ++k) {
    if (k <= 0 || k % o.print_every) continue;
    if (o.print_style == 0) printf("%d: %e\n", k, hist_host[k]);
    else printf("Iteration: %d\t Relative residual norm: %le\n", k, hist_host[k]);
  }
}

int finish_info(DeviceContext* c, SolverState* st_dev, mgb_solve_info* info, double t0, cudaStream_t s) {
  MGB_CUDA(cudaMemcpyAsync(c->state_host, st_dev, sizeof(SolverState), cudaMemcpyDeviceToHost, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  const SolverState& h = *c->state_host;
  int status = MGB_OK;
  if (h.done == BROKE_DOWN) status = MGB_ERR_BREAKDOWN;
  else if (h.done != CONVERGED) status = MGB_ERR_NOTCONV;
  if (info) {
    info->iterations = h.k;
    info->status = status;
    info->final_res = h.res;
    info->seconds = wall_seconds() - t0;
  }
  return status;
}

// Generic chunked loop: runs `one_iter` (which enqueues one iteration) until
// the device stop flag is set.  Graph-captured when possible.
// The kChunk-iteration graph of an earlier solve whose launches baked in the
// same values (`key`), or null.
DeviceContext::CachedGraph* cached_graph(DeviceContext* c, const std::vector<uintptr_t>& key) {
  for (auto& g : c->graph_cache)
    if (g.key == key) {
      g.last_use = ++c->graph_clock;
      return &g;
    }
  return nullptr;
}

// Keep an instantiated graph for later solves (at most 8, least recently
// used evicted); takes ownership of g's graph and exec.
void keep_graph(DeviceContext* c, const std::vector<uintptr_t>& key, GraphHolder* g) {
  if (c->graph_cache.size() >= 8) {
    auto lru = c->graph_cache.begin();
    for (auto it = c->graph_cache.begin(); it != c->graph_cache.end(); ++it)
      if (it->last_use < lru->last_use) lru = it;
    cudaGraphExecDestroy(lru->exec);
    cudaGraphDestroy(lru->graph);
    c->graph_cache.erase(lru);
  }
  DeviceContext::CachedGraph e;
  e.key = key;
  e.graph = g->graph;
  e.exec = g->exec;
  e.kernels = g->kernels;
  e.last_use = ++c->graph_clock;
  c->graph_cache.push_back(e);
  g->graph = nullptr;
  g->exec = nullptr;
}

template <class OneIter, class AfterChunk>
int run_loop(DeviceContext* c, Matvec& A, SolverState* st_dev, const SolveOptions& o, double* hist_dev,
             std::vector<double>& hist_host, cudaStream_t s, OneIter one_iter, AfterChunk after_chunk,
             const std::vector<uintptr_t>* cache_key = nullptr) {
  GraphHolder g_chunk, g_one;
  DeviceContext::CachedGraph* cached = cache_key ? cached_graph(c, *cache_key) : nullptr;
  const bool graphs = A.capturable();
  // A plain solve (no printing, checkpoints or restart) starts at k = 0, and
  // its kernels return at once if the entry test already stopped it: the
  // first chunk is queued behind the set-up kernels without a round trip to
  // the host.
  bool blind = graphs && !hist_dev && o.checkpoint_every <= 0 && !o.restart;
  int k_printed = 0;
  for (;;) {
    SolverState h;
    if (blind) {
      memset(&h, 0, sizeof(h));
      blind = false;
    } else {
      MGB_CUDA(cudaMemcpyAsync(c->state_host, st_dev, sizeof(SolverState), cudaMemcpyDeviceToHost, s));
      MGB_CUDA(cudaStreamSynchronize(s));
      h = *c->state_host;
    }
    if (hist_dev && h.k > k_printed) {
      MGB_CUDA(cudaMemcpy(hist_host.data() + k_printed + 1, hist_dev + k_printed + 1,
                          sizeof(double) * (h.k - k_printed), cudaMemcpyDeviceToHost));
      print_history(o, hist_host.data(), k_printed + 1, h.k, 0.0);
      k_printed = h.k;
    }
    MGB_TRY(after_chunk(h));
    if (h.done) break;
    // iterations until the next checkpoint boundary / cap
    int todo = kChunk;
    if (o.checkpoint_every > 0) {
      const int to_ckpt = o.checkpoint_every - (h.k % o.checkpoint_every);
      todo = todo < to_ckpt ? todo : to_ckpt;
    }
    if (!graphs) {
      // foreign matvec: one iteration at a time, stop flag checked each time
      MGB_TRY(one_iter());
      continue;
    }
    if (todo == kChunk) {
      if (!cached && !g_chunk.exec) {
        MGB_TRY(capture_iterations(s, kChunk, one_iter, &g_chunk));
        if (cache_key) {
          keep_graph(c, *cache_key, &g_chunk);
          cached = cached_graph(c, *cache_key);
        }
      }
      cudaGraphExec_t exec = cached ? cached->exec : g_chunk.exec;
      const long long kernels = cached ? cached->kernels : g_chunk.kernels;
      MGB_CUDA(cudaGraphLaunch(exec, s));
      count_launches(kernels);
      if (!hist_dev && o.checkpoint_every <= 0 && h.k >= 2 * kChunk) {
        // A long solve without printing or checkpoints: keep the next chunk
        // queued while the host reads the state of the previous one, so the
        // GPU never waits for the host between chunks.  Iterations after
        // convergence return at once (the done flag), so the one queued
        // chunk that follows the last costs only its empty launches.
        int i = 0;
        MGB_CUDA(cudaMemcpyAsync(&c->state_ahead[0], st_dev, sizeof(SolverState), cudaMemcpyDeviceToHost, s));
        MGB_CUDA(cudaEventRecord(c->state_ev[0], s));
        for (;;) {
          MGB_CUDA(cudaGraphLaunch(exec, s));
          count_launches(kernels);
          MGB_CUDA(cudaMemcpyAsync(&c->state_ahead[(i + 1) & 1], st_dev, sizeof(SolverState),
                                   cudaMemcpyDeviceToHost, s));
          MGB_CUDA(cudaEventRecord(c->state_ev[(i + 1) & 1], s));
          MGB_CUDA(cudaEventSynchronize(c->state_ev[i & 1]));
          if (c->state_ahead[i & 1].done) break;
          ++i;
        }
        MGB_CUDA(cudaStreamSynchronize(s));
        return MGB_OK;
      }
    } else {
      if (!g_one.exec) MGB_TRY(capture_iterations(s, 1, one_iter, &g_one));
      for (int i = 0; i < todo; ++i) {
        MGB_CUDA(cudaGraphLaunch(g_one.exec, s));
        count_launches(g_one.kernels);
      }
    }
  }
  return MGB_OK;
}

}  // namespace

int solve_cg(DeviceContext* c, Matvec& A, const double* b, double* x, const SolveOptions& o,
             mgb_solve_info* info, cudaStream_t s) {
  const double t0 = wall_seconds();
  const int n = A.n();
  if (n <= 0) return set_error(MGB_ERR_ARG, "cg: n must be positive");
  Workspace ws(c);
  double *r, *d, *z, *hist = nullptr;
  SolverState* st;
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&r));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&d));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&z));
  MGB_TRY(ws.get(sizeof(SolverState), (void**)&st));
  std::vector<double> hist_host;
  if (o.print_every) {
    MGB_TRY(ws.get(sizeof(double) * ((size_t)o.iter_max + 2), (void**)&hist));
    hist_host.resize((size_t)o.iter_max + 2);
  }
  const int nb = vec_blocks(c, n);
  const RedCtx rc = red_ctx(c);
  k_set_state<<<1, 1, 0, s>>>(st, o.eps, o.iter_max, o.stop_rule, n); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  // r0 = b - A x0, d0 = r0   (mpla.cpp:904-915)
  MGB_TRY(A.apply(x, z, s, nullptr));
  k_cg_init<<<nb, T, 0, s>>>(n, b, z, r, d, st, hist, rc); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  if (o.restart) {
    // mpla.cpp:922-933: iterates loaded after r0 and the entry test.
    MGB_CUDA(cudaStreamSynchronize(s));
    MGB_TRY(load_vector_file("x.dat", n, x, s));
    MGB_TRY(load_vector_file("r.dat", n, r, s));
    MGB_TRY(load_vector_file("d.dat", n, d, s));
    MGB_TRY(load_vector_file("z.dat", n, z, s));
    k_rr<<<nb, T, 0, s>>>(n, r, st, rc); count_launches(1);
    MGB_CUDA(cudaGetLastError());
  }
  int* done = &st->done;
  auto one_iter = [&]() -> int {
    MGB_TRY(A.apply(d, z, s, done));
    k_cg_alpha<<<nb, T, 0, s>>>(n, d, z, st, rc); count_launches(1);
    k_cg_update<<<nb, T, 0, s>>>(n, d, z, x, r, st, hist, rc); count_launches(1);
    k_cg_direction<<<nb, T, 0, s>>>(n, r, d, st); count_launches(1);
    MGB_CUDA(cudaGetLastError());
    return MGB_OK;
  };
  auto after_chunk = [&](const SolverState& h) -> int {
    if (o.checkpoint_every > 0 && h.k > 0 && !h.done && h.k % o.checkpoint_every == 0) {
      if (o.print_every) printf("Checkpointing...\n");
      MGB_TRY(save_vector_file("x.dat", n, x, s));
      MGB_TRY(save_vector_file("r.dat", n, r, s));
      MGB_TRY(save_vector_file("d.dat", n, d, s));
      // the reference's z holds the new direction at this point
      MGB_TRY(save_vector_file("z.dat", n, d, s));
    }
    return MGB_OK;
  };
  // plain solves reuse the iteration graph of an earlier solve that baked in
  // the same pointers and sizes (repeated solves get the same pool blocks)
  std::vector<uintptr_t> key;
  const bool reuse = !o.print_every && !o.checkpoint_every && !o.restart && A.graph_key(&key);
  if (reuse)
    key.insert(key.end(), {2u, (uintptr_t)n, (uintptr_t)x, (uintptr_t)r, (uintptr_t)d, (uintptr_t)z, (uintptr_t)st,
                           (uintptr_t)s, (uintptr_t)c->partials, (uintptr_t)c->tickets, (uintptr_t)o.stop_rule});
  MGB_TRY(run_loop(c, A, st, o, hist, hist_host, s, one_iter, after_chunk, reuse ? &key : nullptr));
  int status = finish_info(c, st, info, t0, s);
  if (info) {
    info->fp64_matvecs = info->iterations + 1;
    info->low_matvecs = 0;
    info->true_relres = -1.0;
  }
  if (o.compute_true_residual && info) {
    MGB_TRY(A.apply(x, z, s, nullptr));
    double* tmp;
    MGB_TRY(ws.get(sizeof(double) * 2, (void**)&tmp));
    k_axpy<<<nb, T, 0, s>>>(n, -1.0, b, z); count_launches(1);  // z = Ax - b
    k_dot<<<nb, T, 0, s>>>(n, z, z, tmp, rc); count_launches(1);
    k_dot<<<nb, T, 0, s>>>(n, b, b, tmp + 1, rc); count_launches(1);
    MGB_CUDA(cudaGetLastError());
    double hv[2];
    MGB_CUDA(cudaMemcpyAsync(hv, tmp, sizeof(hv), cudaMemcpyDeviceToHost, s));
    MGB_CUDA(cudaStreamSynchronize(s));
    info->true_relres = sqrt(hv[0]) / sqrt(hv[1]);
  }
  MGB_TRY(check_device_error(c, s));
  return status;
}

int solve_cg_mixed(DeviceContext* c, Matvec& hi, Matvec& lo, const double* b, double* x,
                   const SolveOptions& o, mgb_solve_info* info, cudaStream_t s) {
  const double t0 = wall_seconds();
  const int n = hi.n();
  if (n <= 0 || lo.n() != n) return set_error(MGB_ERR_ARG, "mixed cg: bad sizes");
  Workspace ws(c);
  double *r, *d, *z, *hist = nullptr;
  SolverState* st;
  int* repl;
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&r));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&d));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&z));
  MGB_TRY(ws.get(sizeof(SolverState), (void**)&st));
  MGB_TRY(ws.get(sizeof(int), (void**)&repl));
  std::vector<double> hist_host;
  if (o.print_every) {
    MGB_TRY(ws.get(sizeof(double) * ((size_t)o.iter_max + 2), (void**)&hist));
    hist_host.resize((size_t)o.iter_max + 2);
  }
  const int nb = vec_blocks(c, n);
  const RedCtx rc = red_ctx(c);
  MGB_CUDA(cudaMemsetAsync(repl, 0, sizeof(int), s));
  k_set_state<<<1, 1, 0, s>>>(st, o.eps, o.iter_max, MGB_STOP_RELATIVE, n); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  // FP64 true residual r0 = b - A x0
  MGB_TRY(hi.apply(x, z, s, nullptr));
  k_cg_init<<<nb, T, 0, s>>>(n, b, z, r, d, st, hist, rc); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  // rr_ref = rr0
  MGB_CUDA(cudaMemcpyAsync(&st->rr_ref, &st->rr, sizeof(double), cudaMemcpyDeviceToDevice, s));
  // One uncaptured call sizes the low-precision matvec's scratch before the
  // iteration graph is captured (z is overwritten by the first iteration).
  MGB_TRY(lo.apply(d, z, s, nullptr));
  const double delta = 1e-2;  // replacement when the recursive residual fell by 100x
  int* done = &st->done;
  int* skip_hi = &st->flag;
  auto one_iter = [&]() -> int {
    MGB_TRY(lo.apply(d, z, s, done));
    k_cg_alpha<<<nb, T, 0, s>>>(n, d, z, st, rc); count_launches(1);
    k_mx_update<<<nb, T, 0, s>>>(n, d, z, x, r, st, delta * delta, rc); count_launches(1);
    MGB_TRY(hi.apply(x, z, s, skip_hi));
    k_mx_replace<<<nb, T, 0, s>>>(n, b, z, r, st, hist, repl, rc); count_launches(1);
    k_cg_direction<<<nb, T, 0, s>>>(n, r, d, st); count_launches(1);
    MGB_CUDA(cudaGetLastError());
    return MGB_OK;
  };
  auto after_chunk = [&](const SolverState&) -> int { return MGB_OK; };
  // the hi matvec must be skipped when done is set too: the update kernel
  // leaves flag = 1 unless a replacement is due, and k_set_state starts at 1.
  MGB_TRY(run_loop(c, hi, st, o, hist, hist_host, s, one_iter, after_chunk));
  int status = finish_info(c, st, info, t0, s);
  int nrep = 0;
  MGB_CUDA(cudaMemcpy(&nrep, repl, sizeof(int), cudaMemcpyDeviceToHost));
  if (info) {
    info->fp64_matvecs = 1 + nrep;
    info->low_matvecs = info->iterations;
    info->true_relres = info->final_res;
  }
  MGB_TRY(check_device_error(c, s));
  return status;
}

int solve_bicgstab(DeviceContext* c, Matvec& A, const double* b, double* x, const SolveOptions& o,
                   mgb_solve_info* info, cudaStream_t s) {
  const double t0 = wall_seconds();
  const int n = A.n();
  if (n <= 0) return set_error(MGB_ERR_ARG, "bicgstab: n must be positive");
  Workspace ws(c);
  double *r, *rh, *p, *z, *zz, *sv, *hist = nullptr;
  SolverState* st;
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&r));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&rh));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&p));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&z));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&zz));
  MGB_TRY(ws.get(sizeof(double) * n, (void**)&sv));
  MGB_TRY(ws.get(sizeof(SolverState), (void**)&st));
  std::vector<double> hist_host;
  if (o.print_every) {
    MGB_TRY(ws.get(sizeof(double) * ((size_t)o.iter_max + 2), (void**)&hist));
    hist_host.resize((size_t)o.iter_max + 2);
  }
  const int nb = vec_blocks(c, n);
  const RedCtx rc = red_ctx(c);
  k_set_state<<<1, 1, 0, s>>>(st, o.eps, o.iter_max, MGB_STOP_RELATIVE, n); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  MGB_TRY(A.apply(x, z, s, nullptr));
  k_bi_init<<<nb, T, 0, s>>>(n, b, z, r, rh, p, st, hist, rc); count_launches(1);
  MGB_CUDA(cudaGetLastError());
  if (o.restart) {
    MGB_CUDA(cudaStreamSynchronize(s));
    MGB_TRY(load_vector_file("x.dat", n, x, s));
    MGB_TRY(load_vector_file("r.dat", n, r, s));
    MGB_TRY(load_vector_file("r_hat.dat", n, rh, s));
    MGB_TRY(load_vector_file("z.dat", n, z, s));
    MGB_TRY(load_vector_file("zz.dat", n, zz, s));
    MGB_TRY(load_vector_file("s.dat", n, sv, s));
    MGB_TRY(load_vector_file("p.dat", n, p, s));
    // rho = <r_hat, r> of the loaded vectors
    k_dot<<<nb, T, 0, s>>>(n, rh, r, &st->rr, rc); count_launches(1);
    MGB_CUDA(cudaGetLastError());
  }
  int* done = &st->done;
  auto one_iter = [&]() -> int {
    MGB_TRY(A.apply(p, z, s, done));
    k_bi_alpha<<<nb, T, 0, s>>>(n, z, rh, st, rc); count_launches(1);
    k_bi_s<<<nb, T, 0, s>>>(n, r, z, sv, st); count_launches(1);
    MGB_TRY(A.apply(sv, zz, s, done));
    k_bi_omega<<<nb, T, 0, s>>>(n, zz, sv, st, rc); count_launches(1);
    k_bi_update<<<nb, T, 0, s>>>(n, p, sv, zz, rh, x, r, st, rc); count_launches(1);
    k_bi_p<<<nb, T, 0, s>>>(n, r, z, p, st); count_launches(1);
    MGB_TRY(A.apply(x, z, s, done));
    k_bi_true<<<nb, T, 0, s>>>(n, b, z, zz, st, hist, rc); count_launches(1);
    MGB_CUDA(cudaGetLastError());
    return MGB_OK;
  };
  auto after_chunk = [&](const SolverState& h) -> int {
    if (o.checkpoint_every > 0 && h.k > 0 && !h.done && h.k % o.checkpoint_every == 0) {
      if (o.print_every) printf("Checkpointing...\n");
      MGB_TRY(save_vector_file("x.dat", n, x, s));
      MGB_TRY(save_vector_file("r.dat", n, r, s));
      MGB_TRY(save_vector_file("r_hat.dat", n, rh, s));
      MGB_TRY(save_vector_file("z.dat", n, z, s));
      MGB_TRY(save_vector_file("zz.dat", n, zz, s));
      MGB_TRY(save_vector_file("s.dat", n, sv, s));
      MGB_TRY(save_vector_file("p.dat", n, p, s));
    }
    return MGB_OK;
  };
  MGB_TRY(run_loop(c, A, st, o, hist, hist_host, s, one_iter, after_chunk));
  int status = finish_info(c, st, info, t0, s);
  if (info) {
    info->fp64_matvecs = 1 + 3 * info->iterations;
    info->low_matvecs = 0;
    info->true_relres = info->final_res;
  }
  MGB_TRY(check_device_error(c, s));
  return status;
}

// ------------------------------------------------------- checkpoint files
int save_vector_file(const char* path, int n, const double* x_dev, cudaStream_t s) {
  std::vector<double> h((size_t)n);
  MGB_CUDA(cudaMemcpyAsync(h.data(), x_dev, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(MGB_ERR_IO, "cannot open %s for writing", path);
  int32_t nn = n;
  size_t w = fwrite(&nn, sizeof(int32_t), 1, f);
  w += fwrite(h.data(), sizeof(double), (size_t)n, f);
  fclose(f);
  if (w != (size_t)n + 1) return set_error(MGB_ERR_IO, "short write to %s", path);
  return MGB_OK;
}

int load_vector_file(const char* path, int n, double* x_dev, cudaStream_t s) {
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(MGB_ERR_IO, "cannot open %s", path);
  int32_t nn = -1;
  if (fread(&nn, sizeof(int32_t), 1, f) != 1) {
    fclose(f);
    return set_error(MGB_ERR_IO, "%s: missing header", path);
  }
  if (nn != n) {
    fclose(f);
    return set_error(MGB_ERR_IO, "%s holds %d entries, expected %d", path, (int)nn, n);
  }
  std::vector<double> h((size_t)n);
  const size_t got = fread(h.data(), sizeof(double), (size_t)n, f);
  fclose(f);
  if (got != (size_t)n) return set_error(MGB_ERR_IO, "%s: short file (%zu of %d values)", path, got, n);
  MGB_CUDA(cudaMemcpyAsync(x_dev, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  return MGB_OK;
}

}  // namespace mgb
