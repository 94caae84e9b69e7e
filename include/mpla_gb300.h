/* mpla_gb300.h — C ABI of the GB300 MPLA hot path.
 *
 * Plain C linkage, plain pointers and sizes, integer status codes.  This is
 * the boundary that foreign-language bindings (ctypes, cgo, JNI) load; the
 * C++ drop-in API of mpla.h is implemented on the same internals.  Each entry
 * names the MPLA interface it replaces (file:line in the original sources).
 *
 * Conventions
 *  - Pointers named *_dev are device pointers; *_host are host pointers.
 *  - `stream` is a cudaStream_t passed as void*; NULL selects the library's
 *    own stream for the current device.
 *  - Every function returns MGB_OK (0) or an MGB_ERR_* code; the message of
 *    the last failure on the calling thread is returned by mgb_last_error().
 *  - Vectors and matrices are FP64, column-major (lda >= rows), as in MPLA.
 *  - Gaussian systems: K(i,j) = exp(-|p_i - p_j|^2) (+ nugget on i == j, or
 *    + 1e-8 when |p_i - p_j| < 1e-14 under MGB_NUGGET_KERNEL_CU), points in
 *    structure-of-arrays form, already scaled by 1/(sqrt(2) l) for a length
 *    scale l.
 */
#ifndef MPLA_GB300_H
#define MPLA_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MGB_OK 0
#define MGB_ERR_CUDA 1       /* a CUDA runtime call failed */
#define MGB_ERR_ARG 2        /* invalid argument (size, pointer, alignment) */
#define MGB_ERR_NOMEM 3      /* device allocation failed or admission refused */
#define MGB_ERR_BREAKDOWN 4  /* Krylov breakdown: zero or negative curvature, non-finite scalar */
#define MGB_ERR_NOTCONV 5    /* iteration cap reached before the tolerance */
#define MGB_ERR_NODEV 6      /* no CUDA device */
#define MGB_ERR_TIMEOUT 7    /* a bounded device-side wait gave up */
#define MGB_ERR_IO 8         /* checkpoint file missing, short or of the wrong size */

/* nugget rules for Gaussian systems */
#define MGB_NUGGET_DIAGONAL 0   /* + nugget when i == j (kernel_system_assembler.h:24-38) */
#define MGB_NUGGET_KERNEL_CU 1  /* + 1e-8 when distance < 1e-14 (kernel.cu:39-50) */

/* stopping rules of the CG variants */
#define MGB_STOP_RELATIVE 0  /* ||r|| / ||b|| < eps  (mpla.cpp:963-968) */
#define MGB_STOP_RMS 1       /* sqrt(<r,r>/n) < eps  (mpla.cpp:868-871) */

/* inner matvec precision of the Gaussian solvers */
#define MGB_PREC_FP64 0   /* plain FP64 CG */
#define MGB_PREC_MIXED 1  /* FP32 matvec (kernel chosen by mgb_set_mixed_matvec), FP64 vectors, dots, scalars and true residuals */

/* ---------------------------------------------------------------- runtime */
int mgb_version(void);
const char* mgb_last_error(void);
/* Select and initialise a device (creates the library stream and tables). */
int mgb_init(int device);
/* Release all device memory and the stream of the current device. */
int mgb_shutdown(void);
int mgb_device_sync(void);

/* Convenience memory helpers so bindings need no other CUDA wrapper. */
int mgb_malloc(void** ptr_dev, size_t bytes);
int mgb_free(void* ptr_dev);
int mgb_memcpy_htod(void* dst_dev, const void* src_host, size_t bytes);
int mgb_memcpy_dtoh(void* dst_host, const void* src_dev, size_t bytes);
int mgb_memset(void* ptr_dev, int value, size_t bytes);
/* Pinned host buffers for the end-to-end (host-buffer) entry points. */
int mgb_host_alloc(void** ptr_host, size_t bytes);
int mgb_host_free(void* ptr_host);

/* ------------------------------------------------------------ dense BLAS */
/* y = A x, A m x n column-major.  Replaces the cublasDgemv of mpla_dgemv
 * (mpla.cpp:716-751) at the 1x1 process grid. */
int mgb_dgemv(int m, int n, const double* A_dev, int lda, const double* x_dev, double* y_dev, void* stream);
/* y = A x like mgb_dgemv, for callers that cannot allocate device memory.
 * No counterpart in the reference.  Some hosts of this code may not call
 * cudaMalloc: plugins whose host framework owns every device allocation
 * (its pool must account for all memory), and latency-critical paths that
 * cannot take the allocator's implicit device synchronisation.  This entry
 * point calls no cudaMalloc, cudaFree or allocating library routine and
 * never creates the library context.  Its scratch (split-K partials and
 * arrival counters) is a fixed 8.1 MiB device array that every GPU loading
 * the library holds until the process exits.  Limits: m <= 1,048,512 rows
 * (16383 strips of 64; half that when lda is odd or A is not 16-byte
 * aligned) and m * ceil(n / 4096) <= 1,048,576; larger sizes return
 * MGB_ERR_ARG with a message naming the limit.
 * All calls share that array and it keeps the last call's contents (each
 * call clears the counters it uses): calls that overlap on the GPU
 * (different streams, or several host threads) race and must be serialised
 * by the caller.  The first call on a device resolves the array's device
 * address (cudaGetSymbolAddress with that device current); make that first
 * call before any stream capture.  `stream` must belong to the current
 * device (MGB_ERR_ARG otherwise); NULL is the legacy default stream.
 * This variant stages x with plain loads and has no device-side wait, so it
 * has no timeout to report: MGB_OK means the work was enqueued. */
int mgb_dgemv_noalloc(int m, int n, const double* A_dev, int lda, const double* x_dev, double* y_dev,
                      void* stream);
/* *result_host = <x, y>.  Replaces mpla_ddot (mpla.cpp:753-770). */
int mgb_ddot(int n, const double* x_dev, const double* y_dev, double* result_host, void* stream);
/* y += alpha x.  Replaces mpla_daxpy (mpla.cpp:806-810). */
int mgb_daxpy(int n, double alpha, const double* x_dev, double* y_dev, void* stream);

/* --------------------------------------------------- Gaussian kernel matvec */
/* y[i] = sum_j K(row_offset+i, col_offset+j) x[j] over a rows x cols block,
 * FP64 throughout, no matrix stored.  coords_dev is a HOST array of `dim`
 * device pointers (each of length >= max(row_offset+rows, col_offset+cols)).
 * Replaces mpla_dgemv_core_kernel[_streamed]_cublas (kernel.cu:87-171) and
 * mpla_dgemv_core_generic_system_matrix[_streamed]_cublas
 * (generic_system_adapter.cu:53-137) for the Gaussian assembler. */
int mgb_gauss_matvec_f64(int rows, int cols, int row_offset, int col_offset, int dim,
                         const double* const* coords_dev, double nugget, int nugget_rule,
                         const double* x_dev, double* y_dev, void* stream);
/* Same product with the mixed-precision kernel chosen by
 * mgb_set_mixed_matvec: FP32 arithmetic (by default squared distances from
 * FP32 coordinate differences; MGB_MIXED_TENSOR forms them on the tensor
 * cores), exponentials on the SFU.  x and y stay FP64.  Square systems only
 * (rows == cols, offsets 0). */
int mgb_gauss_matvec_mixed(int n, int dim, const double* const* coords_dev, double nugget,
                           const double* x_dev, double* y_dev, void* stream);
/* Evaluate single entries K(i,j), 0 <= i,j < n, with the FP64 kernel's
 * arithmetic (used by the entry-accuracy tests). */
int mgb_gauss_entries_f64(int n, int count, const int* i_dev, const int* j_dev, int dim,
                          const double* const* coords_dev, double nugget, int nugget_rule,
                          double* out_dev, void* stream);

/* ----------------------------------------------------------------- solvers */
typedef struct mgb_solve_info {
  int iterations;     /* Krylov iterations executed (matvecs in the loop) */
  int status;         /* MGB_OK, MGB_ERR_NOTCONV or MGB_ERR_BREAKDOWN */
  double final_res;   /* value of the stopping measure at exit */
  double true_relres; /* ||b - A x|| / ||b|| recomputed in FP64 at exit (mixed: always; fp64: if requested) */
  int fp64_matvecs;   /* FP64 matvecs spent (mixed: true-residual replacements) */
  int low_matvecs;    /* FP32 matvecs spent (mixed only) */
  double seconds;     /* host wall time of the call */
} mgb_solve_info;

/* CG on a dense SPD matrix (column-major, lda = n).  Follows
 * mpla_generic_conjugate_gradient[_with_checkpoint_restart] (mpla.cpp:817-1001)
 * with the given stopping rule; x holds x0 on entry and the solution on exit. */
int mgb_cg_dense(int n, const double* A_dev, int lda, const double* b_dev, double* x_dev,
                 int iter_max, double eps, int stop_rule, mgb_solve_info* info, void* stream);
/* BiCGSTAB on a dense matrix; follows mpla_generic_BiCGSTAB_with_checkpoint_restart
 * (mpla.cpp:1003-1183): true relative residual as the stopping measure. */
int mgb_bicgstab_dense(int n, const double* A_dev, int lda, const double* b_dev, double* x_dev,
                       int iter_max, double eps, mgb_solve_info* info, void* stream);
/* CG on a Gaussian kernel system held on the device.  precision selects the
 * plain FP64 iteration or the mixed form (FP32 matvec inside FP64 reliable
 * residual replacement; the stopping rule is then always the FP64 true
 * relative residual). */
int mgb_cg_gauss(int n, int dim, const double* const* coords_dev, double nugget, int nugget_rule,
                 const double* b_dev, double* x_dev, int iter_max, double eps, int stop_rule,
                 int precision, mgb_solve_info* info, void* stream);
int mgb_bicgstab_gauss(int n, int dim, const double* const* coords_dev, double nugget, int nugget_rule,
                       const double* b_dev, double* x_dev, int iter_max, double eps,
                       mgb_solve_info* info, void* stream);
/* End-to-end entry: points (n x dim, structure of arrays, already scaled),
 * b and x0 in HOST memory; copies in, solves, copies x back. */
int mgb_cg_gauss_host(int n, int dim, const double* coords_host, double nugget,
                      const double* b_host, double* x_host, int iter_max, double eps,
                      int precision, mgb_solve_info* info);

/* Kernel of the mixed-precision Gaussian matvec, for matvecs and solvers set
 * up after the call (no counterpart in the reference):
 *   MGB_MIXED_TENSOR  squared distances as a split-BF16 tcgen05 contraction,
 *                     exponentials on the SFU (sm_103a tensor cores);
 *   MGB_MIXED_SIMT    squared distances from FP32 coordinate differences
 *                     (the default).
 * Both are symmetric FP32 operators of the same kernel matrix. */
#define MGB_MIXED_TENSOR 0
#define MGB_MIXED_SIMT 1
int mgb_set_mixed_matvec(int kind);
/* Kernel entries (exponentials) one mixed matvec of this system evaluates:
 * each unordered pair once, tile pairs whose entries are all below 2^-40
 * left out (MGB_MIXED_SIMT).  The work figure of the roofline. */
int mgb_gauss_mixed_work(int n, int dim, const double* const* coords_dev, long long* evaluated);
/* Kernel entries one FP64 matvec of this system (diagonal nugget) evaluates:
 * for d <= 3 each unordered pair once, tile pairs whose entries are all
 * below 2^-80 left out; n^2 otherwise. */
int mgb_gauss_fp64_work(int n, int dim, const double* const* coords_dev, long long* evaluated);
int mgb_get_mixed_matvec(void);

/* ------------------------------------------------------------ measurement */
/* Kernels this library has launched so far in this process (a kernel node
 * replayed by a CUDA graph counts once per replay). */
long long mgb_kernel_launches(void);
/* Mean device time of one launch of the Gaussian matvec kernel (precision
 * MGB_PREC_FP64 or MGB_PREC_MIXED) over `reps` back-to-back launches on
 * prepared operands, measured with CUDA events on `stream`. */
int mgb_time_gauss_matvec(int n, int dim, const double* const* coords_dev, double nugget, int precision,
                          const double* x_dev, double* y_dev, int reps, double* ms_per_launch, void* stream);
/* Same for the dense dgemv on an n x n column-major matrix. */
int mgb_time_dgemv(int n, const double* A_dev, const double* x_dev, double* y_dev, int reps,
                   double* ms_per_launch, void* stream);

/* ------------------------------------------------ batched multi-system CG */
/* Many independent Gaussian kernel systems, each with 1..8 right-hand sides,
 * advanced together by one graph-captured step.  No counterpart in the
 * reference: MPLA solves one system per call (mpla.cpp:888-1010); each
 * right-hand side here runs that same CG iteration on its own scalars. */
typedef struct mgb_batch mgb_batch;
/* A batch with room for `max_systems` systems resident at once. */
int mgb_batch_create(int max_systems, mgb_batch** out);
/* Admit a system: n points of dimension 2 or 3 (structure of arrays,
 * scaled so that K_ij = exp(-|x_i - x_j|^2) + nugget delta_ij), nrhs columns
 * of b (column-major, n x nrhs) in host memory, x0 = 0.  Refused with
 * MGB_ERR_NOMEM when its buffers plus `reserve_bytes` do not fit in free
 * device memory or every slot is taken.  Returns a handle. */
int mgb_batch_add(mgb_batch* b, int n, int dim, const double* coords_host, double nugget, int nrhs,
                  const double* b_host, int precision, double eps, int iter_max, size_t reserve_bytes,
                  int* handle);
/* Advance every admitted system by up to max_steps iterations (whole
 * graph replays); *active = systems with a right-hand side still running. */
int mgb_batch_run(mgb_batch* b, int max_steps, int* active);
/* The same in two halves, so that several batches run at once: run_async
 * enqueues up to max_steps iterations on the batch's own stream (every batch
 * has one) and returns; wait synchronises with it, retires finished systems
 * from the work lists and sets *active.  A serving loop keeps FP64 and mixed
 * requests in separate batches and overlaps their steps this way (FP64 work
 * uses the FP64 pipe, mixed work the FP32 and SFU pipes), each batch
 * starting its next slice as soon as its last one has finished. */
int mgb_batch_run_async(mgb_batch* b, int max_steps);
int mgb_batch_wait(mgb_batch* b, int* active);
/* *ready = 1 when the iterations enqueued by run_async have finished (so
 * that mgb_batch_wait returns without blocking), else 0. */
int mgb_batch_ready(mgb_batch* b, int* ready);
/* Handles of systems whose right-hand sides have all finished. */
int mgb_batch_finished(mgb_batch* b, int* handles, int capacity, int* count);
/* Copy x (column-major, n x nrhs) and one mgb_solve_info per right-hand side
 * to the host; release != 0 frees the slot and its device memory. */
int mgb_batch_result(mgb_batch* b, int handle, double* x_host, mgb_solve_info* info, int release);
/* Systems are grouped in classes by dimension (2, 3) and right-hand-side
 * width R (nrhs, with 5 padded to 6 and 7 to 8): class = (dim == 3 ? 6 : 0)
 * + position of R in {1, 2, 3, 4, 6, 8}.  Autotuner choice per class:
 * rows_per_thread[MGB_BATCH_CLASSES] and the timed ms of the 1/2/4 variants
 * (ms[3 * MGB_BATCH_CLASSES]). */
#define MGB_BATCH_CLASSES 12
int mgb_batch_tuning(mgb_batch* b, int* rows_per_thread, float* ms);
int mgb_batch_destroy(mgb_batch* b);

/* ------------------------------------ device-linked generic assemblers */
/* A user subclass of system_assembler (system_assembler.h) lives in the
 * device code of the user's own module, so only a kernel device-linked into
 * that module can call its virtual get_matrix_entry / get_rhs_entry -- the
 * constraint of MPLA's own build, which device-links
 * generic_system_adapter.o with the user's objects (src/Makefile:96-114).
 * lib/mpla_generic_device.o (relocatable device code, built with libmpla.so)
 * holds those kernels; linked into the user's module with -rdc it registers
 * them here from a static constructor, and the generic_system_adapter.h
 * cores and the solvers then evaluate user assemblers with them.  Factory
 * Gaussian assemblers never need it.  Callers do not use this directly. */
#define MGB_GENERIC_DEVICE_ABI 1
typedef struct mgb_generic_device_code {
  int abi_version; /* MGB_GENERIC_DEVICE_ABI */
  /* y[i] = sum_{j < cols} K(row_offset + i, col_offset + j) x[j], i < rows;
   * columns split in nsplit ranges of cols_per_split, partials (nsplit x rows)
   * and tickets (one per 128-row tile, zero on entry and on exit) reduced in
   * a fixed order; the launch returns at once when *skip_dev != 0.
   * Returns a cudaError_t value. */
  int (*matvec)(const void* assembler_dev, int rows, int cols, int row_offset, int col_offset,
                const double* x_dev, double* y_dev, int cols_per_split, int nsplit, double* partials_dev,
                unsigned int* tickets_dev, const int* skip_dev, void* stream);
  /* b[i] = get_rhs_entry(row_offset + i), i < rows.  Returns a cudaError_t. */
  int (*rhs)(const void* assembler_dev, int rows, int row_offset, double* b_dev, void* stream);
} mgb_generic_device_code;
/* Register the generic kernels of a module (the last registration wins;
 * MGB_ERR_ARG on an ABI mismatch), and withdraw them when that module is
 * unloaded (no effect unless `code` is the one registered). */
int mgb_register_generic_device_code(const mgb_generic_device_code* code);
int mgb_unregister_generic_device_code(const mgb_generic_device_code* code);

/* ---------------------------------------------------------- checkpoint I/O */
/* File format of mpla_save_vector (mpla.cpp:605-652): int32 n, then n float64. */
int mgb_save_vector(const char* path, int n, const double* x_dev);
int mgb_load_vector(const char* path, int n, double* x_dev);

/* ------------------------------------------------------ quadrature points */
/* Halton points (host code, no device needed): point i (0-based) has
 * coordinate d = the radical inverse of start + i + 1 in the d-th prime base
 * (2, 3, 5, ...), written structure-of-arrays, points_host[d * n + i],
 * 1 <= dim <= 16.  The point set of MPLA's quadrature-weight application
 * (generate_quadrature_weights.cpp:107-173), which takes it from GSL's
 * gsl_qrng_halton; GSL is not part of this library. */
int mgb_halton(int n, int dim, long long start, double* points_host);

#ifdef __cplusplus
}
#endif

#endif
