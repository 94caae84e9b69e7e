/* CPU oracle for the GB300 MPLA hot path — test infrastructure only
 * (see mpla_oracle.c).  Nothing in the product includes this header. */
#ifndef MPLA_ORACLE_H
#define MPLA_ORACLE_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_RULE_DIAGONAL 0
#define ORC_RULE_KERNEL_CU 1
#define ORC_OP_DENSE 0
#define ORC_OP_GAUSS 1

typedef struct orc_operator {
  int kind;              /* ORC_OP_DENSE or ORC_OP_GAUSS */
  int n;
  const double* A;       /* dense: column-major */
  long lda;
  int dim;               /* gauss: points in structure-of-arrays form */
  const double* coords;
  long ld;               /* stride between dimensions */
  double nugget;
  int rule;
} orc_operator;

void orc_dgemv(int m, int n, const double* A, long lda, const double* x, double* y);
double orc_ddot(int n, const double* x, const double* y);
double orc_gauss_entry_assembler(const double* coords, long ld, int dim, int i, int j, double reg);
double orc_gauss_entry_kernelcu(const double* coords, long ld, int dim, int i, int j);
void orc_gauss_matvec(int rows, int cols, int roff, int coff, int dim, const double* coords, long ld,
                      double nugget, int rule, const double* x, double* y);
void orc_gauss_rhs(int rows, int roff, int dim, const double* coords, long ld, double* b);
int orc_cg(const orc_operator* op, const double* b, double* x, int iter_max, double eps, int stop_rule,
           double* final_res, int* status, double* hist);
int orc_bicgstab(const orc_operator* op, const double* b, double* x, int iter_max, double eps, double* final_res,
                 int* status, double* hist);
double orc_true_relres(const orc_operator* op, const double* b, const double* x);
double orc_true_relres_accurate(const orc_operator* op, const double* b, const double* x);
void orc_apply(const orc_operator* op, const double* x, double* y);
int orc_save_vector(const char* path, int n, const double* x);
int orc_load_vector(const char* path, int n, double* x);

#ifdef __cplusplus
}
#endif

#endif
