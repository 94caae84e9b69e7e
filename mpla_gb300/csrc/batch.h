// Batched multi-system, multi-RHS Gaussian-kernel CG engine (internal).
#pragma once

#include <cuda_runtime.h>
#include <vector>

#include "internal.h"

namespace mgb {

// CG scalars of one right-hand side ("lane") of one system.
struct BatchLane {
  double rr;        // <r,r> of the current (recursive) residual
  double rr_new;    // <r,r> after this iteration's update (mixed lanes)
  double rr_ref;    // <r,r> at the last FP64 true residual (mixed lanes)
  double alpha, beta;
  double bnorm;     // ||b||
  double res;       // last stopping measure: ||r|| / ||b||
  int k;            // iterations done
  int done;         // 0 running, 1 converged, 2 capped, 3 broke down
  int hi;           // mixed: 0 iterating, 1 waiting for a true-residual round, 2 in the current round
  int replacements; // mixed: FP64 true residuals computed
};

// One system, resident in device memory.  Vectors are n x R interleaved
// (element (i, k) at i * R + k); R is nrhs, or 6 for 5 and 8 for 7.
struct BatchSys {
  int in_use;
  int n, dim, R, nrhs;
  int precision;     // MGB_PREC_FP64 or MGB_PREC_MIXED
  int iter_max;
  int active_lanes;  // lanes still running (updated at the end of a step)
  int live_lanes;    // running lanes not waiting for a true residual (end of a step)
  int hi_step;       // mixed: steps of the current true-residual round done (-1: no round)
  int hi_ready;      // mixed: the round's sums are complete; its lanes are replaced this step
  int nstream;       // mixed: column streams of a true-residual round
  int nchunks;       // column chunks of the matvec items
  int nvec;          // row chunks of the vector phases
  double eps, nugget;
  double *x, *r, *d, *z, *b;
  double* zt;            // mixed: true-residual sums, nstream x n x R double-double (hi, lo)
  double* P;             // matvec partials: nchunks x n x R (chunk-major)
  double* vpart;         // vector-phase partial sums: nvec x 8
  unsigned int* ticket;  // last-arrival counter of the vector phases
  const double* pts64;   // dim x n, structure of arrays
  const float4* pts_hi;  // mixed: coordinates x sqrt(log2 e), rounded to FP32
  float* d32;            // mixed: FP32 copy of d
  BatchLane* lanes;      // 8 lanes
};

// Matvec work item: 128 rows x one column chunk of one system.
struct BatchItem {
  int sys;
  int row0;
  int chunk;
};

// Vector-phase work item: a chunk of rows of one system.
struct VecItem {
  int sys;
  int row0;
};

class BatchEngine {
 public:
  static constexpr int kClasses = MGB_BATCH_CLASSES;  // (dim 2|3) x (R 1|2|3|4|6|8)
  static constexpr int kStepsPerGraph = 8;  // CG iterations per graph replay
  static constexpr int kBranches = 3 * kClasses;  // concurrent launches of the matvec phase
  // Matvec item lists per class: every item (FP64 matvecs), the items whose
  // row tile is even / a multiple of 4 (FP32 variants with 2 / 4 rows per
  // thread cover 2 / 4 consecutive row tiles).
  static constexpr int kListAll = 0, kListRpt2 = 1, kListRpt4 = 2, kLists = 3;
  // device counters: matvec queues (claim, finished) per class and mode,
  // item counts per list and class, the active-system count, vector-phase
  // queues (claim, finished) per phase and the vector item count
  static_assert(kClasses == 12, "class layout");
  static constexpr int kOffMv = 0;
  static constexpr int kOffCount = 6 * kClasses;
  static constexpr int kOffActive = kOffCount + kLists * kClasses;
  static constexpr int kOffVec = kOffActive + 1;
  static constexpr int kOffVecCount = kOffVec + 8;
  static constexpr int kOffPending = kOffVecCount + 4;  // systems with a true-residual round in progress
  static constexpr int kCounterInts = kOffPending + 4;

  ~BatchEngine();
  int init(DeviceContext* c, int max_systems, cudaStream_t s);
  int add(int n, int dim, const double* coords_host, double nugget, int nrhs, const double* b_host,
          int precision, double eps, int iter_max, size_t reserve_bytes, int* handle);
  int run_steps(int steps, int* active_out);
  // Enqueue up to `steps` iterations (whole graph replays) without waiting;
  // wait() then synchronises, retires finished systems from the work lists
  // and reports the systems still running.
  int run_async(int steps);
  int wait(int* active_out);
  // 1 when the enqueued iterations have finished (wait() then does not block)
  int ready(int* ready_out);
  int done_handles(std::vector<int>* out);
  int result(int handle, double* x_host, mgb_solve_info* info, bool release);
  const int* rows_per_thread() const { return rpt_; }
  const float* tune_ms(int cls) const { return tune_ms_[cls]; }

 private:
  static int class_of(int dim, int R);
  long long list_capacity(int l) const { return l == kListAll ? max_items_ : max_items_ / 2; }
  static size_t bytes_needed(int n, int dim, int nrhs, int precision);
  void release_slot(int slot);
  void unlist(const std::vector<char>& drop);
  int prune_finished();
  int prepare_graph();
  int sync_items();
  int autotune();
  int enqueue_step();
  int fork_branches(int nb);
  int join_branches(int nb);
  int enqueue_mv32(int cls, int rpt, cudaStream_t s);
  int enqueue_mv64(int cls, int mode, cudaStream_t s);
  int enqueue_true(int cls, cudaStream_t s);
  int enqueue_vec(int phase);

  DeviceContext* c_ = nullptr;
  cudaStream_t s_ = nullptr;
  bool own_stream_ = false;  // s_ created by init (destroyed with the engine)
  bool launched_ = false;    // replays enqueued since the last wait()
  int max_ = 0;
  int nslots_ = 0;
  std::vector<BatchSys> host_;
  std::vector<void*> blocks_;
  BatchSys* dev_sys_ = nullptr;
  BatchItem* items_[kLists][kClasses] = {};
  std::vector<BatchItem> items_host_[kClasses];  // every item; the other lists are derived
  std::vector<BatchItem> list_host_[kLists][kClasses];
  int count_host_[kLists][kClasses] = {};
  std::vector<char> listed_;  // slot's items are in the lists (admitted and not seen finished)
  int listed_count_ = 0;
  bool has_mixed_[kClasses] = {};  // classes holding mixed / FP64 systems
  bool has_fp64_[kClasses] = {};
  VecItem* vitems_ = nullptr;
  int* pending_ = nullptr;  // slots with a true-residual round in progress (device, slot order)
  std::vector<VecItem> vitems_host_;
  int vcount_host_ = 0;
  int max_items_ = 0;
  bool items_dirty_ = false;
  int* counters_ = nullptr;
  int* active_host_ = nullptr;
  int rpt_[kClasses] = {};
  float tune_ms_[kClasses][3] = {};
  cudaStream_t side_[kBranches] = {};
  cudaEvent_t join_ev_[kBranches] = {};
  cudaEvent_t fork_ev_ = nullptr;
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  unsigned long long graph_sig_ = 0;
  long long graph_kernels_ = 0;
};

}  // namespace mgb
