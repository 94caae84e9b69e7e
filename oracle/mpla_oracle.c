/* CPU oracle for the GB300 MPLA hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference algorithms on the hot path,
 * used by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * leg, to check results against.  The product never links, loads or calls
 * this code.
 *
 * Every function names the reference code it restates (paths inside the
 * MPLA source tree).  Floating-point contraction is disabled at build time
 * (-ffp-contract=off) and fused multiply-adds are written explicitly where
 * the reference's cuBLAS calls are modelled as FMA-based, so results are the
 * same on x86-64 and AArch64 hosts.  Loops over rows are parallel (OpenMP);
 * each row's reduction runs in a fixed order, so results do not depend on the
 * thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mpla_oracle.h"

/* ------------------------------------------------------------- dense BLAS */

/* y = A x, A m x n column-major with leading dimension lda.
 * Restates the local product of mpla_dgemv (src/mpla.cpp:716-751, the
 * cublasDgemv OP_N call at :729) on a 1x1 process grid, where the
 * Allgatherv/Allreduce around it are identities.  Summation over columns in
 * increasing order. */
void orc_dgemv(int m, int n, const double* A, long lda, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < m; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s = fma(A[(long)j * lda + i], x[j], s);
    y[i] = s;
  }
}

/* <x, y>: mpla_ddot (src/mpla.cpp:753-770). */
double orc_ddot(int n, const double* x, const double* y) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s = fma(x[i], y[i], s);
  return s;
}

/* ------------------------------------------------------- Gaussian entries */

/* Entry of gaussian_kernel_system_assembler::get_matrix_entry
 * (src/kernel_system_assembler.h:24-38): r = sqrt(sum_d (p_d[i]-p_d[j])^2),
 * K = exp(-r*r), plus `reg` on the diagonal.  coords is structure of arrays
 * with stride `ld` between dimensions. */
double orc_gauss_entry_assembler(const double* coords, long ld, int dim, int i, int j, double reg) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    const double df = coords[d * ld + i] - coords[d * ld + j];
    s += df * df;
  }
  const double r = sqrt(s);
  const double k = exp(-r * r);
  return (i == j) ? k + reg : k;
}

/* Entry of the kernel.cu path: gen_dis_matrix (src/kernel.cu:17-37) then
 * apply_kernel (src/kernel.cu:39-50): exp(-r^2), plus 1e-8 when r < 1e-14. */
double orc_gauss_entry_kernelcu(const double* coords, long ld, int dim, int i, int j) {
  double s = 0.0;
  for (int d = 0; d < dim; ++d) {
    const double df = coords[d * ld + i] - coords[d * ld + j];
    s = s + df * df;
  }
  const double r = sqrt(s);
  return (fabs(r) >= 1.0e-14) ? exp(-r * r) : exp(-r * r) + 1.0e-8;
}

/* y[i] = sum_j K(roff+i, coff+j) x[j] for a rows x cols block: the product
 * computed by mpla_dgemv_core_kernel[_streamed]_cublas (src/kernel.cu:87-171)
 * for rule 1 and by mpla_dgemv_core_generic_system_matrix[_streamed]_cublas
 * (src/generic_system_adapter.cu:53-137) with the Gaussian assembler for
 * rule 0.  Column order increasing, FMA accumulation. */
void orc_gauss_matvec(int rows, int cols, int roff, int coff, int dim, const double* coords, long ld,
                      double nugget, int rule, const double* x, double* y) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < rows; ++i) {
    double acc = 0.0;
    for (int j = 0; j < cols; ++j) {
      const double e = (rule == ORC_RULE_KERNEL_CU)
                           ? orc_gauss_entry_kernelcu(coords, ld, dim, roff + i, coff + j)
                           : orc_gauss_entry_assembler(coords, ld, dim, roff + i, coff + j, nugget);
      acc = fma(e, x[j], acc);
    }
    y[i] = acc;
  }
}

/* rhs_i = prod_d (sqrt(pi)/2)(erf(1 - p_d[i]) - erf(-p_d[i])): the integral of
 * the Gaussian kernel over the unit cube, gen_gaussian_kernel_rhs
 * (src/kernel.cu:52-68) and get_rhs_entry (src/kernel_system_assembler.h:40-48). */
void orc_gauss_rhs(int rows, int roff, int dim, const double* coords, long ld, double* b) {
  const double half_sqrt_pi = sqrt(M_PI) / 2.0;
  for (int i = 0; i < rows; ++i) {
    double prod = 1.0;
    for (int d = 0; d < dim; ++d) {
      const double p = coords[d * ld + roff + i];
      prod = prod * half_sqrt_pi * (erf(1.0 - p) - erf(0.0 - p));
    }
    b[i] = prod;
  }
}

/* ----------------------------------------------------------------- Krylov */

static void mv(const orc_operator* op, const double* x, double* y) {
  if (op->kind == ORC_OP_DENSE)
    orc_dgemv(op->n, op->n, op->A, op->lda, x, y);
  else
    orc_gauss_matvec(op->n, op->n, 0, 0, op->dim, op->coords, op->ld, op->nugget, op->rule, x, y);
}

/* CG of src/mpla.cpp, both variants:
 *   stop_rule 0: mpla_generic_conjugate_gradient_with_checkpoint_restart
 *                (src/mpla.cpp:887-1001), ||r||/||b|| < eps;
 *   stop_rule 1: mpla_generic_conjugate_gradient (src/mpla.cpp:817-885),
 *                sqrt(<r,r>/n) < eps.
 * Same recurrences and update order: r0 = b - A x0 (:904-908); d0 = r0;
 * per iteration z = A d, t1 = <r,r>, t2 = <d,z>, alpha = t1/t2,
 * x += alpha d, r -= alpha z, t2 = <r,r>, beta = t2/t1, stop test, then
 * d = beta d + r (:936-975).  The loop runs k = 1 .. iter_max-1.
 * Returns the number of iterations executed; *status is 0 converged,
 * 2 iteration cap, 3 breakdown (non-positive curvature or a non-finite
 * scalar, which the reference would carry on with).  hist[k] (optional,
 * iter_max+1 entries) receives the stopping measure after iteration k. */
int orc_cg(const orc_operator* op, const double* b, double* x, int iter_max, double eps, int stop_rule,
           double* final_res, int* status, double* hist) {
  const int n = op->n;
  double* r = (double*)malloc(sizeof(double) * n);
  double* d = (double*)malloc(sizeof(double) * n);
  double* z = (double*)malloc(sizeof(double) * n);
  const double bnorm = sqrt(orc_ddot(n, b, b));
  mv(op, x, z);
  for (int i = 0; i < n; ++i) {
    r[i] = b[i] - z[i];
    d[i] = r[i];
  }
  double rr = orc_ddot(n, r, r);
  double res = (stop_rule == 1) ? sqrt(rr / (double)n) : sqrt(rr) / bnorm;
  if (hist) hist[0] = res;
  int k = 0, st = 2;
  if (res < eps) st = 0;
  else if (iter_max <= 1) st = 2;
  else {
    for (k = 1; k < iter_max; ++k) {
      mv(op, d, z);
      const double t1 = rr;
      const double t2 = orc_ddot(n, d, z);
      const double alpha = t1 / t2;
      if (!(t2 > 0.0) || !isfinite(alpha)) {
        st = 3;
        --k;
        break;
      }
      for (int i = 0; i < n; ++i) {
        x[i] = fma(alpha, d[i], x[i]);
        r[i] = fma(-alpha, z[i], r[i]);
      }
      const double rr_new = orc_ddot(n, r, r);
      const double beta = rr_new / t1;
      res = (stop_rule == 1) ? sqrt(rr_new / (double)n) : sqrt(rr_new) / bnorm;
      if (hist) hist[k] = res;
      rr = rr_new;
      if (res < eps) {
        st = 0;
        break;
      }
      if (!(res == res)) {
        st = 3;
        break;
      }
      for (int i = 0; i < n; ++i) d[i] = beta * d[i] + r[i];
    }
    if (k >= iter_max) k = iter_max - 1;
  }
  if (final_res) *final_res = res;
  if (status) *status = st;
  free(r);
  free(d);
  free(z);
  return k;
}

/* BiCGSTAB of mpla_generic_BiCGSTAB_with_checkpoint_restart
 * (src/mpla.cpp:1003-1183): r0 = b - A x0, r_hat = p = r0; per iteration
 * alpha = <r_hat,r>/<A p, r_hat>, s = r - alpha z, omega = <A s, s>/<A s, A s>,
 * x += alpha p + omega s, r = s - omega A s,
 * beta = (alpha/omega) <r, r_hat>/<r_hat, r_old>, p = r + beta (p - omega z),
 * then the true residual ||b - A x|| / ||b|| is the stopping measure
 * (:1133-1150).  Returns iterations executed; status as orc_cg. */
int orc_bicgstab(const orc_operator* op, const double* b, double* x, int iter_max, double eps, double* final_res,
                 int* status, double* hist) {
  const int n = op->n;
  double* r = (double*)malloc(sizeof(double) * n);
  double* rh = (double*)malloc(sizeof(double) * n);
  double* p = (double*)malloc(sizeof(double) * n);
  double* z = (double*)malloc(sizeof(double) * n);
  double* zz = (double*)malloc(sizeof(double) * n);
  double* s = (double*)malloc(sizeof(double) * n);
  const double bnorm = sqrt(orc_ddot(n, b, b));
  mv(op, x, z);
  for (int i = 0; i < n; ++i) {
    r[i] = b[i] - z[i];
    rh[i] = r[i];
    p[i] = r[i];
  }
  double rho = orc_ddot(n, r, r);
  double res = sqrt(rho) / bnorm;
  if (hist) hist[0] = res;
  int k = 0, st = 2;
  if (res < eps) st = 0;
  else if (iter_max > 1) {
    for (k = 1; k < iter_max; ++k) {
      mv(op, p, z);
      const double t2 = orc_ddot(n, z, rh);
      const double alpha = rho / t2;
      if (t2 == 0.0 || !isfinite(alpha)) {
        st = 3;
        --k;
        break;
      }
      for (int i = 0; i < n; ++i) s[i] = fma(-alpha, z[i], r[i]);
      mv(op, s, zz);
      const double o1 = orc_ddot(n, zz, s), o2 = orc_ddot(n, zz, zz);
      const double omega = o1 / o2;
      if (omega == 0.0 || !isfinite(omega)) {
        st = 3;
        --k;
        break;
      }
      for (int i = 0; i < n; ++i) {
        x[i] = fma(omega, s[i], fma(alpha, p[i], x[i]));
        r[i] = fma(-omega, zz[i], s[i]);
      }
      const double rho_new = orc_ddot(n, r, rh);
      const double beta = (alpha / omega) * (rho_new / rho);
      rho = rho_new;
      for (int i = 0; i < n; ++i) p[i] = fma(beta, fma(-omega, z[i], p[i]), r[i]);
      mv(op, x, z);
      for (int i = 0; i < n; ++i) zz[i] = b[i] - z[i];
      res = sqrt(orc_ddot(n, zz, zz)) / bnorm;
      if (hist) hist[k] = res;
      if (res < eps) {
        st = 0;
        break;
      }
      if (!(res == res)) {
        st = 3;
        break;
      }
    }
    if (k >= iter_max) k = iter_max - 1;
  }
  if (final_res) *final_res = res;
  if (status) *status = st;
  free(r);
  free(rh);
  free(p);
  free(z);
  free(zz);
  free(s);
  return k;
}

/* ||b - A x|| / ||b|| in FP64: the true relative residual against which the
 * mixed-precision solver is checked. */
double orc_true_relres(const orc_operator* op, const double* b, const double* x) {
  const int n = op->n;
  double* z = (double*)malloc(sizeof(double) * n);
  mv(op, x, z);
  double rr = 0.0, bb = 0.0;
  for (int i = 0; i < n; ++i) {
    const double t = b[i] - z[i];
    rr = fma(t, t, rr);
    bb = fma(b[i], b[i], bb);
  }
  free(z);
  return sqrt(rr) / sqrt(bb);
}

/* ||b - A x|| / ||b|| with each residual entry b_i - sum_j A_ij x_j formed in
 * double-double arithmetic (products split exactly by fma, sums by TwoSum):
 * the compensated dot product Dot2 of Ogita, Rump and Oishi ("Accurate sum
 * and dot product", SIAM J. Sci. Comput. 26(6), 2005), with b_i as the first
 * summand.  The only errors left are those of the FP64 entries A_ij, so the
 * value does not carry the summation noise u * sum_j |A_ij x_j| that a plain
 * FP64 residual has on ill-conditioned kernel systems. */
static inline void two_sum(double a, double b, double* s, double* e) {
  const double t = a + b;
  const double bp = t - a;
  *e = (a - (t - bp)) + (b - bp);
  *s = t;
}

static double residual_entry(const orc_operator* op, const double* b, const double* x, int i) {
  double s = b[i], c = 0.0;
  for (int j = 0; j < op->n; ++j) {
    double a;
    if (op->kind == ORC_OP_DENSE)
      a = op->A[(long)j * op->lda + i];
    else
      a = (op->rule == ORC_RULE_KERNEL_CU) ? orc_gauss_entry_kernelcu(op->coords, op->ld, op->dim, i, j)
                                           : orc_gauss_entry_assembler(op->coords, op->ld, op->dim, i, j, op->nugget);
    const double p = -a * x[j];
    const double pe = fma(-a, x[j], -p);
    double e;
    two_sum(s, p, &s, &e);
    c += e + pe;
  }
  return s + c;
}

double orc_true_relres_accurate(const orc_operator* op, const double* b, const double* x) {
  const int n = op->n;
  double rr = 0.0, bb = 0.0;
#pragma omp parallel for reduction(+ : rr, bb) schedule(dynamic, 16)
  for (int i = 0; i < n; ++i) {
    const double t = residual_entry(op, b, x, i);
    rr += t * t;
    bb += b[i] * b[i];
  }
  return sqrt(rr) / sqrt(bb);
}

/* Operator matvec exposed for the tests. */
void orc_apply(const orc_operator* op, const double* x, double* y) { mv(op, x, y); }

/* File format of mpla_save_vector (src/mpla.cpp:605-652): int32 n followed by
 * n float64 in host byte order.  Returns 0 on success. */
int orc_save_vector(const char* path, int n, const double* x) {
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  int32_t nn = n;
  size_t w = fwrite(&nn, sizeof(nn), 1, f) + fwrite(x, sizeof(double), (size_t)n, f);
  fclose(f);
  return (w == (size_t)n + 1) ? 0 : -1;
}

/* Reader with the checks of mpla_load_vector (src/mpla.cpp:686-713):
 * returns 0, -1 (open/short) or -2 (size mismatch). */
int orc_load_vector(const char* path, int n, double* x) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  int32_t nn = -1;
  if (fread(&nn, sizeof(nn), 1, f) != 1) {
    fclose(f);
    return -1;
  }
  if (nn != n) {
    fclose(f);
    return -2;
  }
  size_t got = fread(x, sizeof(double), (size_t)n, f);
  fclose(f);
  return (got == (size_t)n) ? 0 : -1;
}
