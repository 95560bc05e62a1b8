// Adjoint sensitivities of the FDFD solution with respect to ε.
//
// For A(ε) e = b with A = Cₘ·Cₑ − ω²·Pε (src/model/model.jl:225-246) and a
// real objective L(e), write g = ∂L/∂e for the Wirtinger derivative
// ½(∂/∂Re e − i ∂/∂Im e), so that dL = 2·Re(gᵀ de).  Since ∂A/∂ε_cc = −ω²
// at the E_c sample (pinned wall DOFs included: their row is −ω²ε_cc),
//     de/dε_cc = ω²·A⁻¹ (e_c u_c)   ⇒   dL/dε_cc = 2·Re(ω²·λ_c·e_c),
// with the adjoint field λ = A⁻ᵀ g, solved by the transposed BiCGSTAB.  The
// reference has no adjoint (its users differentiate A\b by hand); the
// formula follows from the operator it assembles.
//
// The design-cell chain follows the per-cell ε convention of the design
// region: ε_ww at an E_w sample touching the region is the mean of the four
// cells around its edge (index clamped at a symmetry wall, wrapped on a
// Bloch axis), so each design cell collects ¼ of dL/dε_ww from every
// sample whose average includes it.  It runs as a gather (one thread per
// design cell, fixed summation order), so the result is deterministic.
#include <cuda_runtime.h>

#include "fdfd_internal.cuh"

namespace fdfd {

int solve_dev_impl(fdfd_handle *h, const double2 *b, double2 *x, const fdfd_solve_opts *o, fdfd_stats *st);

__global__ void k_eps_grad(const double2 *__restrict__ lam, const double2 *__restrict__ e, double2 w2,
                           double *__restrict__ grad, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 l = lam[i], v = e[i];
    // Re(w2 · l · v)
    const double pr = l.x * v.x - l.y * v.y, pi = l.x * v.y + l.y * v.x;
    grad[i] = 2.0 * (w2.x * pr - w2.y * pi);
  }
}

struct RegionDev {
  int lo[3], hi[3];
  int N[3];
  int bloch[3];
};

// Sample indices t along one axis whose clamped/wrapped neighbour t + s
// (s ∈ {−1, 0}) is cell c; returns how many (at most 3).
__device__ __forceinline__ int sources_along(int c, int N, int bloch, int t[3]) {
  int n = 0;
  t[n++] = c;                                  // s = 0
  if (bloch) t[n++] = (c + 1 == N) ? 0 : c + 1;  // s = −1, wrapped
  else {
    if (c + 1 < N) t[n++] = c + 1;             // s = −1
    if (c == 0) t[n++] = 0;                    // s = −1 clamped onto 0
  }
  return n;
}

__global__ void k_design_grad(RegionDev r, const double *__restrict__ grad, double *__restrict__ out) {
  const int e0 = r.hi[0] - r.lo[0], e1 = r.hi[1] - r.lo[1], e2 = r.hi[2] - r.lo[2];
  const long long ne = (long long)e0 * e1 * e2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ne; q += (long long)gridDim.x * blockDim.x) {
    const int c[3] = {r.lo[0] + (int)(q % e0), r.lo[1] + (int)((q / e0) % e1), r.lo[2] + (int)(q / ((long long)e0 * e1))};
    double acc = 0.0;
    for (int w = 0; w < 3; ++w) {
      const int u0 = (w == 0) ? 1 : 0, u1 = (w == 2) ? 1 : 2;
      int t0[3], t1[3];
      const int n0 = sources_along(c[u0], r.N[u0], r.bloch[u0], t0);
      const int n1 = sources_along(c[u1], r.N[u1], r.bloch[u1], t1);
      for (int a = 0; a < n0; ++a)
        for (int b = 0; b < n1; ++b) {
          int t[3] = {c[0], c[1], c[2]};
          t[u0] = t0[a];
          t[u1] = t1[b];
          const long long cell = t[0] + (long long)r.N[0] * (t[1] + (long long)r.N[1] * t[2]);
          acc += 0.25 * grad[3 * cell + w];
        }
    }
    out[q] = acc;
  }
}

int eps_grad_dev_impl(fdfd_handle *h, const double2 *e, const double2 *g, double2 *lam, double *grad,
                      const fdfd_solve_opts *opts, fdfd_stats *stats) {
  fdfd_solve_opts o = *opts;
  o.transpose = 1;
  const int rc = solve_dev_impl(h, g, lam, &o, stats);
  if (rc != FDFD_OK) return rc;
  const long long n = 3 * h->ncell;
  k_eps_grad<<<152 * 8, 256, 0, h->stream>>>(lam, e, make_double2(h->w2[0], h->w2[1]), grad, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_eps_grad");
}

int design_grad_dev_impl(fdfd_handle *h, const double *grad, double *out) {
  if (!h->has_design) return set_error(h, FDFD_ERR_ARG, "no design region (set one with fdfd_smooth_objects)");
  RegionDev r;
  for (int a = 0; a < 3; ++a) {
    r.lo[a] = h->design_lo[a];
    r.hi[a] = h->design_hi[a];
    r.N[a] = h->N[a];
    r.bloch[a] = h->bloch[a];
  }
  k_design_grad<<<152 * 2, 256, 0, h->stream>>>(r, grad, out);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_design_grad");
}

}  // namespace fdfd
