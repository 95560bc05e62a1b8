/*
 * CPU baseline and test infrastructure (oracle): complex128 CSR sparse
 * matrix-vector product and unpreconditioned BiCGSTAB on all host cores
 * (OpenMP).  The matrix is the oracle's assembled A = Cm*Ce - w^2*Peps
 * (the reference's create_A, src/model/model.jl:238-259, which Julia then
 * applies with its single-threaded SparseArrays SpMV and solves with A\b).
 * The recurrence is the one in fdfd_oracle.bicgstab (van der Vorst 1992):
 *   rho = <rh, r>, beta = (rho/rho_old)(alpha/omega), p = r + beta(p - omega v),
 *   v = A p, alpha = rho/<rh, v>, s = r - alpha v, t = A s,
 *   omega = <t, s>/<t, t>, x += alpha p + omega s, r = s - omega t
 * with <a, b> = sum conj(a) b.  Complex values are interleaved doubles.
 * Never part of the product path: only the tests and the benchmark's CPU
 * baseline load it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cplx cdiv(cplx a, cplx b) {
  const double d = b.re * b.re + b.im * b.im;
  cplx r = {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
  return r;
}

int csr_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

void csr_spmv(int64_t n, const int64_t *indptr, const int32_t *indices, const double *data, const double *x,
              double *y) {
  const cplx *A = (const cplx *)data, *X = (const cplx *)x;
  cplx *Y = (cplx *)y;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double re = 0.0, im = 0.0;
    for (int64_t q = indptr[i]; q < indptr[i + 1]; ++q) {
      const cplx a = A[q], v = X[indices[q]];
      re += a.re * v.re - a.im * v.im;
      im += a.re * v.im + a.im * v.re;
    }
    Y[i].re = re;
    Y[i].im = im;
  }
}

/* <a, b> = sum conj(a) b */
static cplx dotc(int64_t n, const cplx *a, const cplx *b) {
  double re = 0.0, im = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : re, im)
  for (int64_t i = 0; i < n; ++i) {
    re += a[i].re * b[i].re + a[i].im * b[i].im;
    im += a[i].re * b[i].im - a[i].im * b[i].re;
  }
  cplx r = {re, im};
  return r;
}

static double nrm2(int64_t n, const cplx *a) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (int64_t i = 0; i < n; ++i) s += a[i].re * a[i].re + a[i].im * a[i].im;
  return sqrt(s);
}

/* Runs until ||r||/||b|| < tol or maxit iterations; returns the iterations
 * done (-1 on allocation failure) and the final recursive relative residual
 * in *relres.  x holds the initial guess on entry. */
int64_t csr_bicgstab(int64_t n, const int64_t *indptr, const int32_t *indices, const double *data, const double *b,
                     double *x, double tol, int64_t maxit, double *relres) {
  cplx *r = malloc(n * sizeof(cplx)), *rh = malloc(n * sizeof(cplx)), *p = calloc(n, sizeof(cplx));
  cplx *v = calloc(n, sizeof(cplx)), *s = malloc(n * sizeof(cplx)), *t = malloc(n * sizeof(cplx));
  cplx *X = (cplx *)x;
  const cplx *B = (const cplx *)b;
  int64_t it = -1;
  if (!r || !rh || !p || !v || !s || !t) goto done;
  csr_spmv(n, indptr, indices, data, x, (double *)r);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    r[i].re = B[i].re - r[i].re;
    r[i].im = B[i].im - r[i].im;
    rh[i] = r[i];
  }
  const double nb = nrm2(n, B);
  cplx rho = {1.0, 0.0}, alpha = {1.0, 0.0}, om = {1.0, 0.0};
  double rel = nrm2(n, r) / nb;
  for (it = 1; it <= maxit; ++it) {
    const cplx rho_new = dotc(n, rh, r);
    const cplx beta = cmul(cdiv(rho_new, rho), cdiv(alpha, om));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const cplx q = {p[i].re - (om.re * v[i].re - om.im * v[i].im), p[i].im - (om.re * v[i].im + om.im * v[i].re)};
      const cplx bq = cmul(beta, q);
      p[i].re = r[i].re + bq.re;
      p[i].im = r[i].im + bq.im;
    }
    csr_spmv(n, indptr, indices, data, (const double *)p, (double *)v);
    alpha = cdiv(rho_new, dotc(n, rh, v));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const cplx av = cmul(alpha, v[i]);
      s[i].re = r[i].re - av.re;
      s[i].im = r[i].im - av.im;
    }
    csr_spmv(n, indptr, indices, data, (const double *)s, (double *)t);
    om = cdiv(dotc(n, t, s), dotc(n, t, t));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const cplx ap = cmul(alpha, p[i]), os = cmul(om, s[i]), ot = cmul(om, t[i]);
      X[i].re += ap.re + os.re;
      X[i].im += ap.im + os.im;
      r[i].re = s[i].re - ot.re;
      r[i].im = s[i].im - ot.im;
    }
    rho = rho_new;
    rel = nrm2(n, r) / nb;
    if (rel < tol) break;
  }
  if (it > maxit) it = maxit;
  if (relres) *relres = rel;
done:
  free(r); free(rh); free(p); free(v); free(s); free(t);
  return it;
}
