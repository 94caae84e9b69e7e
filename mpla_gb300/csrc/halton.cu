// Halton point sets for the quadrature-weight application of MPLA
// (generate_quadrature_weights.cpp:107-173, which draws them from GSL's
// gsl_qrng_halton).  Host code: the radical inverse of the point index in
// the d-th prime base, the definition of J. H. Halton (Numer. Math. 2, 1960).
#include "internal.h"

namespace {

constexpr int kPrimes[16] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53};

// sum_k digit_k(i) base^-(k+1), digits of i in `base`, least significant
// first (the same operation order as the oracle's restatement)
double radical_inverse(long long i, int base) {
  const double inv = 1.0 / base;
  double f = inv, x = 0.0;
  while (i > 0) {
    x += f * (double)(i % base);
    i /= base;
    f *= inv;
  }
  return x;
}

}  // namespace

extern "C" int mgb_halton(int n, int dim, long long start, double* points_host) {
  if (n < 0 || dim < 1 || dim > 16 || start < 0 || (n > 0 && !points_host))
    return mgb::set_error(MGB_ERR_ARG, "mgb_halton: n >= 0, 1 <= dim <= 16, start >= 0 and a buffer required");
  for (int d = 0; d < dim; ++d)
    for (int i = 0; i < n; ++i) points_host[(size_t)d * n + i] = radical_inverse(start + i + 1, kPrimes[d]);
  return MGB_OK;
}
