/* CPU baseline of petgem's own Krylov solve (test / measurement
 * infrastructure only, never part of the product): restarted GMRES(m) with
 * Jacobi preconditioning, the KSPSolve of petgem/solver.py:584-594 with
 * -ksp_type gmres -pc_type jacobi (PETSc is not installed), restated in C on
 * all host cores (OpenMP), in complex128.  It follows the library's FP64
 * GMRES step for step: right preconditioning (A D^-1 y = b, x = D^-1 y, so
 * the Arnoldi residual is the true one), classical Gram-Schmidt (PETSc's
 * default; reorth = 1 repeats it once), Hermitian inner products, Givens
 * rotations, and at every restart the true residual b - A x decides
 * convergence (||r|| <= rtol ||b||); inside a cycle the Arnoldi estimate ends
 * it early.
 *
 * pg_cpu_gmres(n, rowptr, col, vals (re, im interleaved), b, x, restart
 *              (1..128), max_it, rtol, reorth, &iterations, &relres): returns
 * 0 converged, 1 max_it, 2 breakdown, 3 bad argument or out of memory.
 * iterations counts Arnoldi steps.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define G_MAX_M 128

typedef double complex cplx;

static void g_spmv(int64_t n, const int64_t* rp, const int32_t* col, const cplx* a, const cplx* x, cplx* y) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    cplx s = 0.0;
    for (int64_t k = rp[r]; k < rp[r + 1]; ++k) s += a[k] * x[col[k]];
    y[r] = s;
  }
}

static double g_nrm2(int64_t n, const cplx* u) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += creal(u[i]) * creal(u[i]) + cimag(u[i]) * cimag(u[i]);
  return sqrt(s);
}

/* h[i] = conj(V_i) . w for i = 0..j in one pass over w (PETSc's VecMDot);
 * each thread sums its static chunk into its own row of part, and the rows
 * are added in thread order, so the result does not depend on scheduling */
static void g_dots(int64_t n, int j, const cplx* V, const cplx* w, cplx* h, cplx* part, int nthreads) {
  /* rows of threads the runtime does not start stay zero */
  for (int t = 0; t < nthreads; ++t)
    for (int i = 0; i <= j; ++i) part[(size_t)t * (G_MAX_M + 1) + i] = 0.0;
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    cplx loc[G_MAX_M + 1];
    for (int i = 0; i <= j; ++i) loc[i] = 0.0;
#pragma omp for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
      const cplx wk = w[k];
      for (int i = 0; i <= j; ++i) loc[i] += conj(V[(int64_t)i * n + k]) * wk;
    }
    for (int i = 0; i <= j; ++i) part[(size_t)tid * (G_MAX_M + 1) + i] = loc[i];
  }
  for (int i = 0; i <= j; ++i) {
    cplx s = 0.0;
    for (int t = 0; t < nthreads; ++t) s += part[(size_t)t * (G_MAX_M + 1) + i];
    h[i] = s;
  }
}

/* true residual r = b - A x, returns ||r|| */
static double g_resid(int64_t n, const int64_t* rp, const int32_t* col, const cplx* A, const cplx* b, const cplx* x,
                      cplx* r) {
  g_spmv(n, rp, col, A, x, r);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
  return g_nrm2(n, r);
}

int pg_cpu_gmres(int64_t n, const int64_t* rp, const int32_t* col, const double* vals, const double* bb, double* xx,
                 int m, int64_t max_it, double rtol, int reorth, int64_t* iterations, double* relres) {
  if (n <= 0 || m < 1 || m > G_MAX_M || max_it < 0 || !rp || !col || !vals || !bb || !xx || !iterations || !relres)
    return 3;
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  const cplx* A = (const cplx*)vals;
  const cplx* b = (const cplx*)bb;
  cplx* x = (cplx*)xx;
  cplx* Dinv = malloc(sizeof(cplx) * n);
  cplx* V = malloc(sizeof(cplx) * n * (size_t)(m + 1));
  cplx* w = malloc(sizeof(cplx) * n);
  cplx* t = malloc(sizeof(cplx) * n);
  cplx* H = malloc(sizeof(cplx) * (size_t)(m + 1) * m); /* column j: H[j * (m + 1) + i] */
  cplx* h = malloc(sizeof(cplx) * (size_t)(m + 1));
  cplx* g = malloc(sizeof(cplx) * (size_t)(m + 1));
  cplx* sn = malloc(sizeof(cplx) * (size_t)m);
  double* cs = malloc(sizeof(double) * (size_t)m);
  cplx* y = malloc(sizeof(cplx) * (size_t)m);
  cplx* part = malloc(sizeof(cplx) * (size_t)nthreads * (G_MAX_M + 1));
  int status = 3;
  int64_t it = 0;
  double res = 0.0, bn = 0.0;
  if (!Dinv || !V || !w || !t || !H || !h || !g || !sn || !cs || !y || !part) goto done;
  /* D = diag(A) (PETSc's -pc_type jacobi); a zero diagonal keeps 1 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    cplx d = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k)
      if (col[k] == i) d = A[k];
    Dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
  }
  bn = g_nrm2(n, b);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) x[i] = 0.0;
  status = 1;
  for (;;) {
    res = g_resid(n, rp, col, A, b, x, w);
    if (res <= rtol * bn) {
      status = 0;
      break;
    }
    if (it >= max_it) break;
    const double beta = res;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) V[i] = w[i] / beta;
    for (int i = 0; i <= m; ++i) g[i] = 0.0;
    g[0] = beta;
    int k = 0; /* Arnoldi steps in this cycle */
    int brk = 0;
    for (int j = 0; j < m && it < max_it; ++j) {
      cplx* vj = V + (int64_t)j * n;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) t[i] = Dinv[i] * vj[i];
      g_spmv(n, rp, col, A, t, w);
      cplx* Hj = H + (size_t)j * (m + 1);
      for (int i = 0; i <= j; ++i) Hj[i] = 0.0;
      for (int pass = 0; pass < (reorth ? 2 : 1); ++pass) {
        g_dots(n, j, V, w, h, part, nthreads);
        for (int i = 0; i <= j; ++i) Hj[i] += h[i];
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n; ++q) {
          cplx s = w[q];
          for (int i = 0; i <= j; ++i) s -= h[i] * V[(int64_t)i * n + q];
          w[q] = s;
        }
      }
      const double hn = g_nrm2(n, w);
      Hj[j + 1] = hn;
      ++it;
      k = j + 1;
      /* earlier rotations on the new column */
      for (int i = 0; i < j; ++i) {
        const cplx a0 = Hj[i], a1 = Hj[i + 1];
        Hj[i] = cs[i] * a0 + sn[i] * a1;
        Hj[i + 1] = -conj(sn[i]) * a0 + cs[i] * a1;
      }
      /* the rotation that zeroes H[j + 1][j] */
      const cplx a = Hj[j];
      const double an = cabs(a), den = sqrt(an * an + hn * hn);
      if (den == 0.0) {
        brk = 1;
        k = j;
        break;
      }
      if (an == 0.0) {
        cs[j] = 0.0;
        sn[j] = 1.0;
      } else {
        cs[j] = an / den;
        sn[j] = (a / an) * hn / den;
      }
      Hj[j] = cs[j] * a + sn[j] * hn;
      Hj[j + 1] = 0.0;
      g[j + 1] = -conj(sn[j]) * g[j];
      g[j] = cs[j] * g[j];
      if (hn == 0.0) break; /* lucky breakdown: the solution lies in the space */
      cplx* vn = V + (int64_t)(j + 1) * n;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) vn[i] = w[i] / hn;
      if (cabs(g[j + 1]) <= rtol * bn) break;
    }
    if (k == 0) {
      status = brk ? 2 : 1;
      break;
    }
    /* y = H(0:k, 0:k)^-1 g(0:k) (upper triangular), x += D^-1 V y */
    for (int i = k - 1; i >= 0; --i) {
      cplx s = g[i];
      for (int l = i + 1; l < k; ++l) s -= H[(size_t)l * (m + 1) + i] * y[l];
      y[i] = s / H[(size_t)i * (m + 1) + i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) {
      cplx s = 0.0;
      for (int i = 0; i < k; ++i) s += y[i] * V[(int64_t)i * n + q];
      x[q] += Dinv[q] * s;
    }
    if (brk) {
      res = g_resid(n, rp, col, A, b, x, w);
      status = res <= rtol * bn ? 0 : 2;
      break;
    }
  }
done:
  *iterations = it;
  *relres = bn > 0 ? res / bn : 0.0;
  free(Dinv);
  free(V);
  free(w);
  free(t);
  free(H);
  free(h);
  free(g);
  free(sn);
  free(cs);
  free(y);
  free(part);
  return status;
}
