/*
 * getf2.c — CPU restatement of the unblocked right-looking LU recurrence
 * (LAPACK dgetf2), the arithmetic that jax.scipy.linalg.lu_factor asks of
 * LAPACK at lineax/_solver/lu.py:53.  TEST INFRASTRUCTURE ONLY: used by the
 * tests as the bit-exact twin of the GPU plain-FP64 LU.
 *
 * Row-major n×n matrix, in place.  For k = 0..n-1:
 *   p = first i >= k of maximal |a(i,k)| (idamax; NaN never wins)
 *   if a(p,k) != 0: swap rows k and p (whole rows),
 *                   scale a(i,k), i > k, by 1/a(k,k) (divide when
 *                   |a(k,k)| < DBL_MIN)
 *   else info = k+1 (first time only)
 *   a(i,j) = fma(-a(i,k), a(k,j), a(i,j)) for i > k, j > k
 * piv[k] = p (0-based).  Returns info.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>

int oracle_getf2_f64(int n, double* a, int32_t* piv) {
  int info = 0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double v = -1.0;
    for (int i = k; i < n; ++i) {
      const double x = fabs(a[(int64_t)i * n + k]);
      if (x > v) { v = x; p = i; }
    }
    piv[k] = p;
    const double akk = a[(int64_t)p * n + k];
    if (akk != 0.0) {
      if (p != k) {
        for (int j = 0; j < n; ++j) {
          const double t = a[(int64_t)k * n + j];
          a[(int64_t)k * n + j] = a[(int64_t)p * n + j];
          a[(int64_t)p * n + j] = t;
        }
      }
      if (fabs(akk) >= DBL_MIN) {
        const double r = 1.0 / akk;
        for (int i = k + 1; i < n; ++i) a[(int64_t)i * n + k] *= r;
      } else {
        for (int i = k + 1; i < n; ++i) a[(int64_t)i * n + k] /= akk;
      }
    } else if (info == 0) {
      info = k + 1;
    }
    for (int i = k + 1; i < n; ++i) {
      const double l = a[(int64_t)i * n + k];
      for (int j = k + 1; j < n; ++j)
        a[(int64_t)i * n + j] = fma(-l, a[(int64_t)k * n + j], a[(int64_t)i * n + j]);
    }
  }
  return info;
}

void oracle_getf2_batched_f64(int64_t batch, int n, double* a, int32_t* piv, int32_t* info) {
  for (int64_t b = 0; b < batch; ++b)
    info[b] = oracle_getf2_f64(n, a + b * (int64_t)n * n, piv + b * (int64_t)n);
}
