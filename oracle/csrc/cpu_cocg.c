/* CPU baseline of the Krylov solve (test / measurement infrastructure only,
 * never part of the product): complex-symmetric COCG with symmetric Jacobi
 * scaling, the same algorithm as the library's FP64 COCG, on all host cores
 * (OpenMP), in FP64.  It stands in for the KSPSolve of petgem/solver.py:584-594
 * (PETSc is not installed) as the "compiled CPU" reference point for the
 * ms-per-RHS half of the metric.
 *
 * pg_cpu_cocg(n, rowptr, col, vals (re, im interleaved), b, x, max_it, rtol,
 *             &iterations, &relres): returns 0 converged, 1 max_it, 2 breakdown.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

static void spmv(int64_t n, const int64_t* rp, const int32_t* col, const cplx* a, const cplx* x, cplx* y) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    cplx s = 0.0;
    for (int64_t k = rp[r]; k < rp[r + 1]; ++k) s += a[k] * x[col[k]];
    y[r] = s;
  }
}

static cplx bdot(int64_t n, const cplx* u, const cplx* v) {   /* u^T v, no conjugate */
  double re = 0.0, im = 0.0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const cplx t = u[i] * v[i];
    re += creal(t);
    im += cimag(t);
  }
  return re + I * im;
}

static double nrm2(int64_t n, const cplx* u) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += creal(u[i]) * creal(u[i]) + cimag(u[i]) * cimag(u[i]);
  return sqrt(s);
}

int pg_cpu_cocg(int64_t n, const int64_t* rp, const int32_t* col, const double* vals, const double* bb, double* xx,
                int64_t max_it, double rtol, int64_t* iterations, double* relres) {
  const cplx* A = (const cplx*)vals;
  const cplx* b = (const cplx*)bb;
  cplx* x = (cplx*)xx;
  cplx* S = malloc(sizeof(cplx) * n);
  cplx* r = malloc(sizeof(cplx) * n);
  cplx* p = malloc(sizeof(cplx) * n);
  cplx* q = malloc(sizeof(cplx) * n);
  cplx* t = malloc(sizeof(cplx) * n);
  int status = 1;
  /* S = diag(A)^(-1/2) */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    cplx d = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k)
      if (col[k] == i) d = A[k];
    S[i] = 1.0 / csqrt(d);
  }
  const double bn = nrm2(n, b);
  /* scaled system: (S A S) y = S b, x = S y; start from x = 0 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    x[i] = 0.0;
    r[i] = S[i] * b[i];
    p[i] = r[i];
  }
  cplx rho = bdot(n, r, r);
  int64_t it = 0;
  double res = bn;
  while (it < max_it) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) t[i] = S[i] * p[i];
    spmv(n, rp, col, A, t, q);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) q[i] *= S[i];
    const cplx mu = bdot(n, p, q);
    if (mu == 0.0) {
      status = 2;
      break;
    }
    const cplx alpha = rho / mu;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];   /* x holds y until the end */
      r[i] -= alpha * q[i];
    }
    ++it;
    const cplx rho1 = bdot(n, r, r);
    /* residual of the original system: b - A x = S^-1 r */
    double s2 = 0.0;
#pragma omp parallel for reduction(+ : s2) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const cplx v = r[i] / S[i];
      s2 += creal(v) * creal(v) + cimag(v) * cimag(v);
    }
    res = sqrt(s2);
    if (res <= rtol * bn) {
      status = 0;
      break;
    }
    if (rho == 0.0) {
      status = 2;
      break;
    }
    const cplx beta = rho1 / rho;
    rho = rho1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) p[i] = r[i] + beta * p[i];
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) x[i] *= S[i];
  *iterations = it;
  *relres = bn > 0 ? res / bn : 0.0;
  free(S);
  free(r);
  free(p);
  free(q);
  free(t);
  return status;
}
