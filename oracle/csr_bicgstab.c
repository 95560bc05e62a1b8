/*
 * CPU baseline and test infrastructure (oracle): complex128 CSR sparse
 * matrix-vector product, unpreconditioned BiCGSTAB and BiCGStab(l)
 * (Sleijpen & Fokkema 1993) on all host cores (OpenMP).  The matrix is the oracle's assembled A = Cm*Ce - w^2*Peps
 * (the reference's create_A, src/model/model.jl:225-246, which Julia then
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

static void axpy(int64_t n, cplx a, const cplx *x, cplx *y) { /* y += a x */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const cplx t = cmul(a, x[i]);
    y[i].re += t.re;
    y[i].im += t.im;
  }
}
static void xpay(int64_t n, const cplx *x, cplx a, cplx *y) { /* y = x + a y */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const cplx t = cmul(a, y[i]);
    y[i].re = x[i].re + t.re;
    y[i].im = x[i].im + t.im;
  }
}
static inline cplx csub_(cplx a, cplx b) { cplx r = {a.re - b.re, a.im - b.im}; return r; }
static inline cplx cadd_(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }

/* Shadow vector of the GPU solver: r̂_i = (a + i b)/32768 with a, b the two
 * 16-bit halves (signed) of Chris Wellons' "lowbias32" hash of i. */
static uint32_t shadow_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

/* BiCGStab(l), l <= 8, with the modified Gram-Schmidt minimal-residual part
 * of the original algorithm and the GPU solver's generated shadow vector;
 * same stopping rule as csr_bicgstab (recursive residual).  Returns the
 * operator applications done (-1 on allocation failure). */
int64_t csr_bicgstabl(int64_t n, const int64_t *indptr, const int32_t *indices, const double *data, const double *b,
                      double *x, int l, double tol, int64_t maxmv, double *relres) {
  enum { LM = 8 };
  if (l < 1 || l > LM) return -1;
  cplx *r[LM + 1], *u[LM + 1], *rh = malloc(n * sizeof(cplx));
  int ok = rh != NULL;
  for (int i = 0; i <= l; ++i) {
    r[i] = malloc(n * sizeof(cplx));
    u[i] = calloc(n, sizeof(cplx));
    ok = ok && r[i] && u[i];
  }
  int64_t mv = -1;
  cplx *X = (cplx *)x;
  const cplx *B = (const cplx *)b;
  if (ok) {
    csr_spmv(n, indptr, indices, data, x, (double *)r[0]);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      r[0][i].re = B[i].re - r[0][i].re;
      r[0][i].im = B[i].im - r[0][i].im;
      const uint32_t hsh = shadow_hash((uint32_t)i);
      rh[i].re = (double)(int16_t)(hsh & 0xffffu) / 32768.0;
      rh[i].im = (double)(int16_t)(hsh >> 16) / 32768.0;
    }
    const double nb = nrm2(n, B);
    cplx rho0 = {1, 0}, alpha = {0, 0}, om = {1, 0};
    double rel = nrm2(n, r[0]) / nb;
    mv = 0;
    while (mv < maxmv && rel >= tol) {
      const cplx mom = {-om.re, -om.im};
      rho0 = cmul(mom, rho0);
      for (int j = 0; j < l; ++j) {
        const cplx rho1 = dotc(n, rh, r[j]);
        const cplx beta = cmul(alpha, cdiv(rho1, rho0));
        rho0 = rho1;
        const cplx mb = {-beta.re, -beta.im};
        for (int i = 0; i <= j; ++i) xpay(n, r[i], mb, u[i]);
        csr_spmv(n, indptr, indices, data, (const double *)u[j], (double *)u[j + 1]);
        ++mv;
        alpha = cdiv(rho0, dotc(n, rh, u[j + 1]));
        const cplx ma = {-alpha.re, -alpha.im};
        for (int i = 0; i <= j; ++i) axpy(n, ma, u[i + 1], r[i]);
        csr_spmv(n, indptr, indices, data, (const double *)r[j], (double *)r[j + 1]);
        ++mv;
        axpy(n, alpha, u[0], X);
      }
      cplx tau[LM + 1][LM + 1], gp[LM + 1], gam[LM + 1], gpp[LM + 1];
      double sig[LM + 1];
      for (int j = 1; j <= l; ++j) {
        for (int i = 1; i < j; ++i) {
          const cplx d = dotc(n, r[i], r[j]);
          tau[i][j].re = d.re / sig[i];
          tau[i][j].im = d.im / sig[i];
          const cplx mt = {-tau[i][j].re, -tau[i][j].im};
          axpy(n, mt, r[i], r[j]);
        }
        sig[j] = dotc(n, r[j], r[j]).re;
        const cplx g = dotc(n, r[j], r[0]);
        gp[j].re = g.re / sig[j];
        gp[j].im = g.im / sig[j];
      }
      gam[l] = gp[l];
      om = gam[l];
      for (int j = l - 1; j >= 1; --j) {
        cplx t = gp[j];
        for (int i = j + 1; i <= l; ++i) t = csub_(t, cmul(tau[j][i], gam[i]));
        gam[j] = t;
      }
      for (int j = 1; j < l; ++j) {
        cplx t = gam[j + 1];
        for (int i = j + 1; i < l; ++i) t = cadd_(t, cmul(tau[j][i], gam[i + 1]));
        gpp[j] = t;
      }
      axpy(n, gam[1], r[0], X);
      const cplx mg = {-gp[l].re, -gp[l].im}, mgl = {-gam[l].re, -gam[l].im};
      axpy(n, mg, r[l], r[0]);
      axpy(n, mgl, u[l], u[0]);
      for (int j = 1; j < l; ++j) {
        const cplx mgj = {-gam[j].re, -gam[j].im}, mgpj = {-gp[j].re, -gp[j].im};
        axpy(n, mgj, u[j], u[0]);
        axpy(n, gpp[j], r[j], X);
        axpy(n, mgpj, r[j], r[0]);
      }
      rel = nrm2(n, r[0]) / nb;
    }
    if (relres) *relres = rel;
  }
  free(rh);
  for (int i = 0; i <= l; ++i) {
    free(r[i]);
    free(u[i]);
  }
  return mv;
}
