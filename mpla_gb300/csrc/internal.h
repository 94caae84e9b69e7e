// Internal host-side declarations shared by the translation units of the
// GB300 MPLA library.  Nothing here is part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <map>
#include <vector>

#include "../../include/mpla_gb300.h"

namespace mgb {

// ---------------------------------------------------------------- errors
// Records a formatted message for mgb_last_error() and returns `code`.
int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* expr, const char* file, int line);

#define MGB_CUDA(expr)                                                     \
  do {                                                                     \
    cudaError_t mgb_e_ = (expr);                                           \
    if (mgb_e_ != cudaSuccess)                                             \
      return ::mgb::cuda_error(mgb_e_, #expr, __FILE__, __LINE__);         \
  } while (0)

#define MGB_TRY(expr)                                                      \
  do {                                                                     \
    int mgb_s_ = (expr);                                                   \
    if (mgb_s_ != MGB_OK) return mgb_s_;                                   \
  } while (0)

// Device-side error word bits (written by kernels, read by the host).
enum DeviceErrorBits : unsigned int {
  DEV_ERR_WAIT_TIMEOUT = 1u,   // a bounded mbarrier / flag wait gave up
  DEV_ERR_BAD_INDEX = 2u,      // an index check failed (bounds-checked builds)
};

// ------------------------------------------------------------- constants
constexpr int kExpTableBits = 12;                  // 4096-entry 2^(-j/4096) table
constexpr int kExpTableSize = 1 << kExpTableBits;
constexpr int kReduceThreads = 256;                // block size of reductions
constexpr int kMaxReduceBlocks = 1024;             // partials capacity per reduction
constexpr int kMaxGaussDim = 16;                   // dimensions accepted by the Gaussian kernels

// Scalars of one Krylov solve, resident in device memory for the whole
// solve so that no iteration needs the host.
struct SolverState {
  double rr;       // <r,r> of the current residual (CG), <r_hat,r> (BiCGSTAB)
  double alpha;
  double beta;
  double omega;
  double bnorm;    // ||b||
  double res;      // current value of the stopping measure
  double eps;
  double t1, t2, t3;  // reduction results of the current iteration
  double rr_ref;   // mixed CG: <r,r> at the last residual replacement
  int k;           // iterations completed
  int iter_max;
  int done;        // 0 running, 1 converged, 2 iteration cap, 3 breakdown, 4 replace residual
  int stop_rule;   // MGB_STOP_RELATIVE or MGB_STOP_RMS
  int n;
  int flag;        // solver-specific request flag read by the host loop
};

enum SolveDone : int { RUNNING = 0, CONVERGED = 1, CAPPED = 2, BROKE_DOWN = 3 };

// ------------------------------------------------------- device context
// One per device: the library stream, the exp table, a caching pool for
// vectors, and the persistent reduction scratch (partials + tickets).
struct DeviceContext {
  int device = -1;
  int num_sms = 0;
  cudaStream_t stream = nullptr;       // blocking stream: ordered with the legacy default stream
  double* exp_table = nullptr;         // kExpTableSize doubles, 2^(-j/4096)
  double* partials = nullptr;          // reduction partials, kMaxReduceBlocks * 4 doubles
  unsigned int* tickets = nullptr;     // self-resetting arrival counters
  int n_tickets = 0;
  unsigned int* dev_error = nullptr;   // device error word
  SolverState* state_host = nullptr;   // pinned mirror of one SolverState
  SolverState* state_ahead = nullptr;  // pinned mirrors of the solver loop's two chunks in flight
  cudaEvent_t state_ev[2] = {nullptr, nullptr};
  std::map<size_t, std::vector<void*>> free_blocks;   // caching pool: size -> blocks
  std::map<void*, size_t> live_blocks;
  // split-K partials for dgemv / matvecs (grown on demand, never shrunk)
  double* split_partials = nullptr;
  size_t split_partials_count = 0;
  // instantiated iteration graphs of earlier solves, keyed by every value
  // their launches bake in (least recently used evicted)
  struct CachedGraph {
    std::vector<uintptr_t> key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;
    long long last_use = 0;
  };
  std::vector<CachedGraph> graph_cache;
  long long graph_clock = 0;
};

// Context of the current device (created on first use).
int context(DeviceContext** out);
// Pool allocation of device memory without per-call cudaMalloc after warm-up.
int pool_alloc(DeviceContext* c, size_t bytes, void** out);
void pool_free(DeviceContext* c, void* p);
int ensure_split_partials(DeviceContext* c, size_t count);
int ensure_tickets(DeviceContext* c, int count);
// Resolve a user stream argument (NULL -> library stream).
inline cudaStream_t pick_stream(DeviceContext* c, void* s) {
  return s ? static_cast<cudaStream_t>(s) : c->stream;
}
// Read and clear the device error word; returns MGB_ERR_TIMEOUT etc.
int check_device_error(DeviceContext* c, cudaStream_t s);

// Kernel launch accounting.  While a stream capture is in progress on this
// thread, launches are counted into the graph being built instead; each
// replay of that graph then adds its kernel count.
void count_launches(long long n);
void begin_capture_count();
long long end_capture_count();

// ---------------------------------------------------------- kernels API
// Dense y = A x (column-major).  Deterministic split-K reduction.
int launch_dgemv(DeviceContext* c, int m, int n, const double* A, int lda, const double* x,
                 double* y, cudaStream_t s, const int* done);

// Gaussian matvec descriptor used by the FP64 and mixed kernels.
struct GaussSystem {
  int rows, cols, row_offset, col_offset;
  int dim;                       // 1..3 on the fast kernels, up to kMaxGaussDim
  const double* coords[16];      // device pointers (SoA), one per dimension
  double nugget;
  int nugget_rule;               // MGB_NUGGET_*
};
int launch_gauss_f64(DeviceContext* c, const GaussSystem& g, const double* x, double* y,
                     cudaStream_t s, const int* done);
int launch_gauss_entries_f64(DeviceContext* c, const GaussSystem& g, int count, const int* i,
                             const int* j, double* out, cudaStream_t s);

// BLAS-1 and fused Krylov vector kernels (blas1.cu).
int launch_dot(DeviceContext* c, int n, const double* x, const double* y, double* out_dev,
               cudaStream_t s);
int launch_axpy(DeviceContext* c, int n, double alpha, const double* x, double* y,
                cudaStream_t s);

// Matvec abstraction for the solver drivers.
struct Matvec {
  virtual ~Matvec() {}
  // y = A x on stream s; kernels return immediately when *done != 0.
  virtual int apply(const double* x, double* y, cudaStream_t s, const int* done) = 0;
  // True when apply() only enqueues device work (so it can be graph-captured).
  virtual bool capturable() const { return true; }
  virtual int n() const = 0;
  // Appends every value apply() bakes into captured launches (pointers,
  // sizes) and returns true, when a captured iteration graph may be reused
  // by a later solve with the same values; false: never reuse.
  virtual bool graph_key(std::vector<uintptr_t>* key) const {
    (void)key;
    return false;
  }
};

// Krylov drivers (solvers.cu).
struct SolveOptions {
  int iter_max = 1000;
  double eps = 1e-10;
  int stop_rule = MGB_STOP_RELATIVE;
  int print_every = 0;              // mpla.h printing: 0 none, else every k iterations
  int print_style = 0;              // 0: "%d: %e", 1: "Iteration: %d\t Relative residual norm: %le"
  int checkpoint_every = 0;         // 0: never
  bool restart = false;             // load x,r,d,z before the loop
  bool print_final = false;
  bool compute_true_residual = false;
};
int solve_cg(DeviceContext* c, Matvec& A, const double* b, double* x, const SolveOptions& o,
             mgb_solve_info* info, cudaStream_t s);
int solve_bicgstab(DeviceContext* c, Matvec& A, const double* b, double* x,
                   const SolveOptions& o, mgb_solve_info* info, cudaStream_t s);
// Mixed precision: FP32 matvec `lo`, FP64 matvec `hi` for residual replacement.
int solve_cg_mixed(DeviceContext* c, Matvec& hi, Matvec& lo, const double* b, double* x,
                   const SolveOptions& o, mgb_solve_info* info, cudaStream_t s);

// Checkpoint I/O in the MPLA vector file format.
int save_vector_file(const char* path, int n, const double* x_dev, cudaStream_t s);
int load_vector_file(const char* path, int n, double* x_dev, cudaStream_t s);

double wall_seconds();

}  // namespace mgb
