// Krylov solvers for A x = b (the reference leaves the solve to the user's
// A\b on the assembled SparseMatrixCSC, src/model/model.jl:209-220).
//
// Two precisions share one driver:
//   FDFD_PREC_FP64   plain complex128 iteration (the comparison baseline);
//   FDFD_PREC_MIXED  complex64 operator and Krylov vectors, ≈48-bit reductions,
//                    and reliable updates: whenever the recursive residual
//                    has dropped by δ since the last update, the complex64
//                    correction is folded into the FP64 solution x64 and the
//                    residual is recomputed in FP64, r = b − A·x64, then
//                    rounded back — the Krylov space is kept (no restart).
// Convergence is always decided on the true FP64 residual ‖b − A x64‖/‖b‖.
//
// The scalars of the recurrences live on the device (KScalars); a batch of
// `check_every` iterations is one CUDA graph replay with no host sync;
// kernels become no-ops once a stop condition is reached inside a batch.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <vector>

#include "krylov_fin.cuh"

namespace fdfd {

template <typename R>
int bicg_p(fdfd_handle *, const typename CT<R>::C *, typename CT<R>::C *, const typename CT<R>::C *, long long,
           const KScalars *);
template <typename R>
int bicg_s(fdfd_handle *, const typename CT<R>::C *, const typename CT<R>::C *, typename CT<R>::C *, long long,
           const KScalars *);
template <typename R>
int bicg_xr(fdfd_handle *, typename CT<R>::C *, const typename CT<R>::C *, const typename CT<R>::C *,
            const typename CT<R>::C *, typename CT<R>::C *, const typename CT<R>::C *, long long, KScalars *);
template <typename R>
int cocg_xr(fdfd_handle *, typename CT<R>::C *, const typename CT<R>::C *, const typename CT<R>::C *,
            typename CT<R>::C *, const typename CT<R>::C *, const typename CT<R>::C *, long long, KScalars *);
template <typename R>
int cocg_p(fdfd_handle *, const typename CT<R>::C *, const typename CT<R>::C *, typename CT<R>::C *, long long,
           const KScalars *);
template <typename R>
int vmul(fdfd_handle *, typename CT<R>::C *, const typename CT<R>::C *, const typename CT<R>::C *, long long);
template <typename R>
int dot(fdfd_handle *, const typename CT<R>::C *, const typename CT<R>::C *, long long, KScalars *);
template <typename R>
int dot_u(fdfd_handle *, const typename CT<R>::C *, const typename CT<R>::C *, const typename CT<R>::C *, long long,
          int, KScalars *);
template <typename R>
int copy(fdfd_handle *, typename CT<R>::C *, const typename CT<R>::C *, long long);
int accum(fdfd_handle *, double2 *, float2 *, long long);
int accum64(fdfd_handle *, double2 *, double2 *, long long);
int demote(fdfd_handle *, float2 *, const double2 *, long long);
int promote(fdfd_handle *, double2 *, const float2 *, long long);
int build_weights(fdfd_handle *h, double2 *w64, float2 *w32, double2 *d64, float2 *d32);
template <typename R>
int bl_cycle(fdfd_handle *, typename CT<R>::C *, typename CT<R>::C *const *, typename CT<R>::C *const *, long long,
             int, KScalars *, bool);
template <typename R>
int bl_redo(fdfd_handle *, const typename CT<R>::C *, long long, int, KScalars *);

#define TRY(x)              \
  do {                      \
    int _rc = (x);          \
    if (_rc) return _rc;    \
  } while (0)

struct Workspace {
  long long n = 0;
  double2 *x64 = nullptr, *r64 = nullptr;
  float2 *f[12] = {nullptr};   // inner vectors: BiCGSTAB 7, COCG 4, BiCGStab(ℓ) 2ℓ+4
  double2 *d[12] = {nullptr};
  double2 *w64 = nullptr, *dj64 = nullptr;  // COCG: S weights and Jacobi factors 1/diag(A)
  double2 *bt = nullptr, *lt = nullptr;     // transposed solves: V⁻¹ b and V μ
  float2 *w32 = nullptr, *dj32 = nullptr;
  KScalars *sc = nullptr, *scu = nullptr;
  KScalars *host = nullptr;  // pinned mirror
  cudaGraphExec_t gexec[2][3][2] = {};  // [precision][method][transpose]
  cudaGraph_t graph[2][3][2] = {};      // the captured batches (child graphs of a multi-system round)
  int gbatch[2][3][2] = {};
  int gell[2][3][2] = {};               // ℓ the BiCGStab(ℓ) graph was captured with
  long long gkern[2][3][2] = {};        // kernels per graph replay
};

void free_workspace(fdfd_handle *h) {
  Workspace *ws = h->ws;
  if (!ws) return;
  cudaFree(ws->x64);
  cudaFree(ws->r64);
  for (int i = 0; i < 12; ++i) {
    cudaFree(ws->f[i]);
    cudaFree(ws->d[i]);
  }
  cudaFree(ws->bt);
  cudaFree(ws->lt);
  cudaFree(ws->w64);
  cudaFree(ws->w32);
  cudaFree(ws->dj64);
  cudaFree(ws->dj32);
  cudaFree(ws->sc);
  cudaFree(ws->scu);
  if (ws->host) cudaFreeHost(ws->host);
  for (auto &a : ws->gexec)
    for (auto &b : a)
      for (auto &g : b)
        if (g) cudaGraphExecDestroy(g);
  for (auto &a : ws->graph)
    for (auto &b : a)
      for (auto &g : b)
        if (g) cudaGraphDestroy(g);
  delete ws;
  h->ws = nullptr;
}

void drop_graphs(fdfd_handle *h) {
  Workspace *ws = h->ws;
  if (!ws) return;
  for (auto &a : ws->gexec)
    for (auto &b : a)
      for (auto &g : b)
        if (g) {
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
  for (auto &a : ws->graph)
    for (auto &b : a)
      for (auto &g : b)
        if (g) {
          cudaGraphDestroy(g);
          g = nullptr;
        }
}

static int alloc(fdfd_handle *h, void **p, size_t bytes, const char *what) {
  if (*p) return FDFD_OK;
  cudaError_t e = dev_malloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(h, FDFD_ERR_NOMEM, std::string("cudaMalloc failed for ") + what);
  }
  return FDFD_OK;
}

static int ensure_ws(fdfd_handle *h, bool mixed, int method, int ell) {
  if (!h->ws) {
    h->ws = new Workspace();
    h->ws->n = 3 * h->ncell;
  }
  Workspace *ws = h->ws;
  const size_t n = (size_t)ws->n;
  TRY(alloc(h, (void **)&ws->x64, n * sizeof(double2), "x64"));
  TRY(alloc(h, (void **)&ws->r64, n * sizeof(double2), "r64"));
  const int nv = method == FDFD_COCG ? 4 : method == FDFD_BICGSTABL ? 2 * ell + 4 : 7;
  for (int i = 0; i < nv; ++i) {
    if (mixed) TRY(alloc(h, (void **)&ws->f[i], n * sizeof(float2), "inner vector (c64)"));
    else TRY(alloc(h, (void **)&ws->d[i], n * sizeof(double2), "inner vector (c128)"));
  }
  if (method == FDFD_COCG) {
    // rebuilt on every solve: the Jacobi factors follow the current ε
    if (mixed) {
      TRY(alloc(h, (void **)&ws->w32, n * sizeof(float2), "weights"));
      TRY(alloc(h, (void **)&ws->dj32, n * sizeof(float2), "Jacobi factors"));
    } else {
      TRY(alloc(h, (void **)&ws->w64, n * sizeof(double2), "weights"));
      TRY(alloc(h, (void **)&ws->dj64, n * sizeof(double2), "Jacobi factors"));
    }
    TRY(build_weights(h, mixed ? nullptr : ws->w64, mixed ? ws->w32 : nullptr, mixed ? nullptr : ws->dj64,
                      mixed ? ws->dj32 : nullptr));
  }
  TRY(alloc(h, (void **)&ws->sc, sizeof(KScalars), "scalars"));
  TRY(alloc(h, (void **)&ws->scu, sizeof(KScalars), "scalars"));
  if (!ws->host) {
    if (cudaHostAlloc((void **)&ws->host, 2 * sizeof(KScalars), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaHostAlloc(scalars) failed");
    }
    std::memset(ws->host, 0, 2 * sizeof(KScalars));
    TRY(cuda_check(h, cudaMemcpyAsync(ws->scu, ws->host + 1, sizeof(KScalars), cudaMemcpyHostToDevice, h->stream),
                   "init scu"));
  }
  return FDFD_OK;
}

template <typename R> static typename CT<R>::C *vec(Workspace *ws, int i);
template <> float2 *vec<float>(Workspace *ws, int i) { return ws->f[i]; }
template <> double2 *vec<double>(Workspace *ws, int i) { return ws->d[i]; }
template <typename R> static typename CT<R>::C *wvec(Workspace *ws);
template <> float2 *wvec<float>(Workspace *ws) { return ws->w32; }
template <> double2 *wvec<double>(Workspace *ws) { return ws->w64; }
template <typename R> static typename CT<R>::C *jvec(Workspace *ws);
template <> float2 *jvec<float>(Workspace *ws) { return ws->dj32; }
template <> double2 *jvec<double>(Workspace *ws) { return ws->dj64; }

static int read_scalars(fdfd_handle *h, const KScalars *dev, KScalars *host) {
  TRY(cuda_check(h, cudaMemcpyAsync(host, dev, sizeof(KScalars), cudaMemcpyDeviceToHost, h->stream), "read scalars"));
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}
static int write_scalars(fdfd_handle *h, KScalars *dev, const KScalars *host) {
  TRY(cuda_check(h, cudaMemcpyAsync(dev, host, sizeof(KScalars), cudaMemcpyHostToDevice, h->stream),
                 "write scalars"));
  // the pinned source must stay unchanged until the copy has run
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

// r64 = b − A x64 (FP64), returns ‖r64‖² on the host
static int true_residual(fdfd_handle *h, const double2 *b, bool tr, double *rr) {
  Workspace *ws = h->ws;
  TRY(launch_apply_fin<double>(h, ws->x64, ws->r64, EPI_RESID, b, FIN_NONE, ws->scu, tr));
  TRY(read_scalars(h, ws->scu, ws->host + 1));
  *rr = ws->host[1].dot0.x;
  return FDFD_OK;
}

// One BiCGSTAB iteration (5 kernels, 2 operator applications).
template <typename R>
static int bicg_iter(fdfd_handle *h, Workspace *ws, bool tr) {
  using C = typename CT<R>::C;
  const long long n = ws->n;
  C *xi = vec<R>(ws, 0), *r = vec<R>(ws, 1), *rh = vec<R>(ws, 2), *p = vec<R>(ws, 3), *v = vec<R>(ws, 4),
    *s = vec<R>(ws, 5), *t = vec<R>(ws, 6);
  TRY(bicg_p<R>(h, r, p, v, n, ws->sc));
  TRY(launch_apply_fin<R>(h, p, v, EPI_DOT_AUX, rh, FIN_ALPHA, ws->sc, tr));
  TRY(bicg_s<R>(h, r, v, s, n, ws->sc));
  TRY(launch_apply_fin<R>(h, s, t, EPI_DOT_TS, nullptr, FIN_OMEGA, ws->sc, tr));
  TRY(bicg_xr<R>(h, xi, p, s, t, r, rh, n, ws->sc));
  return FDFD_OK;
}

// One Jacobi-preconditioned COCG iteration on the S-symmetric operator
// (1 application, 3 kernels), z = D⁻¹ r with D = diag(A):
//   q = A p and pᵀ S q (fused) ; α = ρ/(pᵀ S q) ; x += α p ; r −= α q ;
//   ρ' = rᵀ S z ; β = ρ'/ρ ; p = z + β p
template <typename R>
static int cocg_iter(fdfd_handle *h, Workspace *ws, bool tr) {
  using C = typename CT<R>::C;
  const long long n = ws->n;
  C *xi = vec<R>(ws, 0), *r = vec<R>(ws, 1), *p = vec<R>(ws, 2), *q = vec<R>(ws, 3);
  TRY(launch_apply_fin<R>(h, p, q, EPI_DOT_SU, nullptr, FIN_COCG_A, ws->sc, tr));
  TRY(cocg_xr<R>(h, xi, p, q, r, wvec<R>(ws), jvec<R>(ws), n, ws->sc));
  TRY(cocg_p<R>(h, r, jvec<R>(ws), p, n, ws->sc));
  return FDFD_OK;
}

// One BiCGStab(ℓ) cycle.  Vectors: 0 x (correction), 2 … 2+ℓ r_0 … r_ℓ,
// 3+ℓ … 3+2ℓ u_0 … u_ℓ (slot 1 unused: r̂ is generated).
template <typename R>
static int bl_iter(fdfd_handle *h, Workspace *ws, int ell, bool tr) {
  using C = typename CT<R>::C;
  C *r[5], *u[5];
  for (int i = 0; i <= ell; ++i) {
    r[i] = vec<R>(ws, 2 + i);
    u[i] = vec<R>(ws, 3 + ell + i);
  }
  return bl_cycle<R>(h, vec<R>(ws, 0), r, u, ws->n, ell, ws->sc, tr);
}

// ρ = rᵀ S D⁻¹ r of the current residual (q is used as scratch for D⁻¹ r)
template <typename R>
static int cocg_rho(fdfd_handle *h, Workspace *ws, double2 *rho) {
  const long long n = ws->n;
  TRY(vmul<R>(h, vec<R>(ws, 3), jvec<R>(ws), vec<R>(ws, 1), n));
  TRY(dot_u<R>(h, vec<R>(ws, 1), vec<R>(ws, 3), wvec<R>(ws), n, FIN_NONE, ws->scu));
  KScalars tmp;
  TRY(read_scalars(h, ws->scu, &tmp));
  *rho = tmp.dot0;
  return FDFD_OK;
}

// Capture (once) a batch of `batch` iterations as a CUDA graph on the
// handle's stream; *gout receives the graph (kept for multi-system rounds)
// and the instantiated executable is kept too.
template <typename R>
static int batch_graph(fdfd_handle *h, Workspace *ws, int method, int ell, bool tr, int batch,
                       cudaGraphExec_t **geout, cudaGraph_t *gout) {
  const int pi = sizeof(R) == 4 ? 1 : 0;
  const int mi = method == FDFD_COCG ? 1 : method == FDFD_BICGSTABL ? 2 : 0;
  const int ti = tr ? 1 : 0;
  // lazily-sized buffers must exist before any capture (the Gram kernel of
  // BiCGStab(ℓ) keeps up to 16 partials per block)
  TRY(ensure_red(h, std::max(apply_blocks(h), method == FDFD_BICGSTABL ? 8 * 152 * 4 : 0)));
  cudaGraphExec_t &ge = ws->gexec[pi][mi][ti];
  cudaGraph_t &gg = ws->graph[pi][mi][ti];
  if (ge && (ws->gbatch[pi][mi][ti] != batch || ws->gell[pi][mi][ti] != ell)) {
    cudaGraphExecDestroy(ge);
    ge = nullptr;
    if (gg) cudaGraphDestroy(gg);
    gg = nullptr;
  }
  if (!ge) {
    cudaGraph_t g;
    TRY(cuda_check(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture"));
    const long long l0 = h->launches;
    int rc = FDFD_OK;
    for (int i = 0; i < batch && rc == FDFD_OK; ++i) {
      if (method == FDFD_COCG) rc = cocg_iter<R>(h, ws, tr);
      else if (method == FDFD_BICGSTABL) rc = bl_iter<R>(h, ws, ell, tr);
      else rc = bicg_iter<R>(h, ws, tr);
    }
    ws->gkern[pi][mi][ti] = h->launches - l0;
    h->launches = l0;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) return rc;
    TRY(cuda_check(h, e, "end capture"));
    e = cudaGraphInstantiate(&ge, g, 0);
    if (e != cudaSuccess) cudaGraphDestroy(g);
    TRY(cuda_check(h, e, "graph instantiate"));
    gg = g;
    ws->gbatch[pi][mi][ti] = batch;
    ws->gell[pi][mi][ti] = ell;
  }
  if (geout) *geout = &ge;
  if (gout) *gout = gg;
  return FDFD_OK;
}

template <typename R>
static long long batch_kernels(Workspace *ws, int method, bool tr) {
  const int pi = sizeof(R) == 4 ? 1 : 0;
  const int mi = method == FDFD_COCG ? 1 : method == FDFD_BICGSTABL ? 2 : 0;
  return ws->gkern[pi][mi][tr ? 1 : 0];
}

template <typename R>
static int run_batch(fdfd_handle *h, Workspace *ws, int method, int ell, bool tr, int batch, bool use_graph) {
  if (!use_graph) {
    TRY(ensure_red(h, std::max(apply_blocks(h), method == FDFD_BICGSTABL ? 8 * 152 * 4 : 0)));
    for (int i = 0; i < batch; ++i) {
      if (method == FDFD_COCG) TRY(cocg_iter<R>(h, ws, tr));
      else if (method == FDFD_BICGSTABL) TRY(bl_iter<R>(h, ws, ell, tr));
      else TRY(bicg_iter<R>(h, ws, tr));
    }
    return FDFD_OK;
  }
  cudaGraphExec_t *ge = nullptr;
  TRY(batch_graph<R>(h, ws, method, ell, tr, batch, &ge, nullptr));
  h->launches += batch_kernels<R>(ws, method, tr);
  return cuda_check(h, cudaGraphLaunch(*ge, h->stream), "graph launch");
}

// (Re)initialise the inner iteration from the FP64 residual r64.
template <typename R>
static int init_inner(fdfd_handle *h, Workspace *ws, int method, int ell, double rr, KScalars *hs) {
  using C = typename CT<R>::C;
  const long long n = ws->n;
  const size_t bytes = (size_t)n * sizeof(C);
  if (method == FDFD_BICGSTABL) {
    // r_0 = r64, u_0 = 0, x = 0; ρ₀ = (r̂, r_0) with the generated shadow
    // vector r̂; α = 0 so the first β is 0
    C *r0 = vec<R>(ws, 2);
    if constexpr (sizeof(R) == 4) TRY(demote(h, r0, ws->r64, n));
    else TRY(copy<double>(h, r0, ws->r64, n));
    TRY(cuda_check(h, cudaMemsetAsync(vec<R>(ws, 0), 0, bytes, h->stream), "memset x"));
    TRY(cuda_check(h, cudaMemsetAsync(vec<R>(ws, 3 + ell), 0, bytes, h->stream), "memset u0"));
    TRY(bl_redo<R>(h, r0, n, FIN_NONE, ws->scu));
    KScalars tmp;
    TRY(read_scalars(h, ws->scu, &tmp));
    hs->rho = tmp.dot0;
    hs->alpha = make_double2(0.0, 0.0);
    hs->omega = make_double2(1.0, 0.0);
    hs->beta = make_double2(0.0, 0.0);
    hs->rho_pre = make_double2(-1.0, 0.0);
    hs->rr = rr;
    hs->rr_max = rr;
    hs->done = 0;
    hs->reason = 0;
    return FDFD_OK;
  }
  C *r = vec<R>(ws, 1);
  if constexpr (sizeof(R) == 4) TRY(demote(h, r, ws->r64, n));
  else TRY(copy<double>(h, r, ws->r64, n));
  TRY(cuda_check(h, cudaMemsetAsync(vec<R>(ws, 0), 0, bytes, h->stream), "memset x"));
  if (method == FDFD_COCG) {
    // p = z = D⁻¹ r ; ρ = rᵀ S z
    TRY(vmul<R>(h, vec<R>(ws, 2), jvec<R>(ws), r, n));
    TRY(cocg_rho<R>(h, ws, &hs->rho));
  } else {
    TRY(copy<R>(h, vec<R>(ws, 2), r, n));  // r̂ = r₀
    TRY(cuda_check(h, cudaMemsetAsync(vec<R>(ws, 3), 0, bytes, h->stream), "memset p"));
    TRY(cuda_check(h, cudaMemsetAsync(vec<R>(ws, 4), 0, bytes, h->stream), "memset v"));
    hs->rho = make_double2(rr, 0.0);
  }
  hs->alpha = make_double2(1.0, 0.0);
  hs->omega = make_double2(1.0, 0.0);
  hs->beta = make_double2(0.0, 0.0);
  hs->rr = rr;
  hs->rr_max = rr;
  hs->done = 0;
  hs->reason = 0;
  return FDFD_OK;
}

// One system's solve as a resumable state machine: begin() up to the first
// batch, after_batch() after each replayed batch of iterations (reliable
// updates, restarts, stop tests), end() for the result and the stats.  The
// single-system driver alternates run_batch and after_batch; the
// multi-system driver replays the batches of every unfinished system as
// child graphs of one parent graph per round.
template <typename R>
struct Solve {
  fdfd_handle *h = nullptr;
  const double2 *b = nullptr;
  double2 *x = nullptr;
  fdfd_solve_opts o{};
  fdfd_stats *st = nullptr;
  Workspace *ws = nullptr;
  bool tr = false, done = false;
  int ell = 1, per = 1, batch = 1, mv_per_it = 2, status = FDFD_ERR_NOT_CONVERGED, restarts = 0;
  long long n = 0, iters = 0, launches0 = 0;
  double bb = 0.0, tol2 = 0.0, rr = 0.0;

  int begin(fdfd_handle *h_, const double2 *b_, double2 *x_, const fdfd_solve_opts &o_, fdfd_stats *st_) {
    h = h_;
    b = b_;
    x = x_;
    o = o_;
    st = st_;
    const bool mixed = sizeof(R) == 4;
    tr = o.transpose != 0;
    ell = o.method == FDFD_BICGSTABL ? o.ell : 1;
    TRY(ensure_ws(h, mixed, o.method, ell));
    ws = h->ws;
    n = ws->n;
    TRY(cuda_check(h, cudaEventRecord(h->ev0, h->stream), "event"));
    launches0 = h->launches;
    if (o.x0_given) TRY(cuda_check(h, cudaMemcpyAsync(ws->x64, x, n * sizeof(double2), cudaMemcpyDeviceToDevice,
                                                      h->stream), "copy x0"));
    else TRY(cuda_check(h, cudaMemsetAsync(ws->x64, 0, n * sizeof(double2), h->stream), "memset x64"));
    // ‖b‖²
    TRY(dot<double>(h, b, b, n, ws->scu));
    KScalars tmp;
    TRY(read_scalars(h, ws->scu, &tmp));
    bb = tmp.dot1.x;
    *st = fdfd_stats{};
    if (!std::isfinite(bb)) {
      st->status = status = FDFD_ERR_NONFINITE;
      done = true;
      return set_error(h, FDFD_ERR_NONFINITE, "the right-hand side holds a NaN or Inf");
    }
    if (!(bb > 0.0)) {
      TRY(cuda_check(h, cudaMemsetAsync(x, 0, n * sizeof(double2), h->stream), "zero x"));
      st->status = FDFD_OK;
      status = FDFD_OK;
      done = true;
      bb = 0.0;
      return FDFD_OK;
    }
    tol2 = o.tol * o.tol * bb;
    TRY(true_residual(h, b, tr, &rr));
    st->matvecs = 1;
    if (!std::isfinite(rr)) {
      st->status = status = FDFD_ERR_NONFINITE;
      done = true;
      return set_error(h, FDFD_ERR_NONFINITE, "the initial residual holds a NaN or Inf (check x0)");
    }
    KScalars &hs = ws->host[0];
    std::memset(&hs, 0, sizeof(KScalars));
    hs.bb = bb;
    // recursive-residual target a little below the true target; mixed also
    // stops every δ-drop for a reliable update
    hs.stop2 = tol2 * 0.25;
    hs.upd2 = mixed ? o.delta * o.delta : 0.0;
    // a BiCGStab(ℓ) cycle counts as ℓ iterations (2ℓ operator applications)
    per = o.method == FDFD_BICGSTABL ? ell : 1;
    batch = std::max(1, (o.check_every > 0 ? o.check_every : 50) / per);
    mv_per_it = o.method == FDFD_COCG ? 1 : 2;
    if (rr <= tol2) {
      status = FDFD_OK;
      done = true;
      return FDFD_OK;
    }
    TRY(init_inner<R>(h, ws, o.method, ell, rr, &hs));
    TRY(write_scalars(h, ws->sc, &hs));
    return FDFD_OK;
  }

  int after_batch() {
    KScalars &hs = ws->host[0];
    TRY(read_scalars(h, ws->sc, &hs));
    iters = hs.iter * per;
    if (hs.done) {
      if (hs.reason == 4) {
        status = FDFD_ERR_NONFINITE;
        done = true;
        return FDFD_OK;
      }
      // fold the correction into x64 and recompute the true residual
      if constexpr (sizeof(R) == 4) TRY(accum(h, ws->x64, vec<R>(ws, 0), n));
      else TRY(accum64(h, ws->x64, vec<R>(ws, 0), n));
      TRY(true_residual(h, b, tr, &rr));
      st->matvecs += 1;
      st->refinements += 1;
      if (rr <= tol2) {
        status = FDFD_OK;
        done = true;
        return FDFD_OK;
      }
      if (hs.reason == 3) {
        if (++restarts > 50) {
          status = FDFD_ERR_BREAKDOWN;
          done = true;
          return FDFD_OK;
        }
        const long long it_keep = hs.iter;
        TRY(init_inner<R>(h, ws, o.method, ell, rr, &hs));
        hs.iter = it_keep;
      } else {
        // reliable update: replace the recursive residual, keep the Krylov state
        using C = typename CT<R>::C;
        C *r = vec<R>(ws, o.method == FDFD_BICGSTABL ? 2 : 1);
        if constexpr (sizeof(R) == 4) TRY(demote(h, r, ws->r64, n));
        else TRY(copy<double>(h, r, ws->r64, n));
        hs.rr = rr;
        hs.rr_max = rr;
        hs.done = 0;
        hs.reason = 0;
        if (o.method == FDFD_COCG) {
          // COCG's ρ = rᵀ S D⁻¹ r must describe the replaced residual
          TRY(cocg_rho<R>(h, ws, &hs.rho));
        } else if (o.method == FDFD_BICGSTABL) {
          // ρ₁ = (r̂, r_0) and β of the next cycle for the replaced r_0
          TRY(write_scalars(h, ws->sc, &hs));
          TRY(bl_redo<R>(h, r, n, FIN_BL_REDO, ws->sc));
          TRY(read_scalars(h, ws->sc, &hs));
        }
      }
      TRY(write_scalars(h, ws->sc, &hs));
    }
    if (iters >= o.maxit) {
      // fold what we have and report
      if constexpr (sizeof(R) == 4) TRY(accum(h, ws->x64, vec<R>(ws, 0), n));
      else TRY(accum64(h, ws->x64, vec<R>(ws, 0), n));
      TRY(true_residual(h, b, tr, &rr));
      st->matvecs += 1;
      status = rr <= tol2 ? FDFD_OK : FDFD_ERR_NOT_CONVERGED;
      done = true;
    }
    return FDFD_OK;
  }

  int end() {
    st->matvecs += iters * mv_per_it;
    if (bb > 0.0)
      TRY(cuda_check(h, cudaMemcpyAsync(x, ws->x64, n * sizeof(double2), cudaMemcpyDeviceToDevice, h->stream),
                     "copy x"));
    TRY(cuda_check(h, cudaEventRecord(h->ev1, h->stream), "event"));
    TRY(cuda_check(h, cudaEventSynchronize(h->ev1), "event sync"));
    TRY(check_dev_err(h));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    st->iterations = iters;
    st->relres = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    st->time_ms = ms;
    st->status = status;
    st->launches = h->launches - launches0;
    if (status == FDFD_ERR_NOT_CONVERGED)
      return set_error(h, status, "solver reached maxit before the tolerance");
    if (status == FDFD_ERR_BREAKDOWN) return set_error(h, status, "Krylov breakdown persisted after restarts");
    if (status == FDFD_ERR_NONFINITE) return set_error(h, status, "non-finite value in the iteration");
    return FDFD_OK;
  }
};

template <typename R>
static int solve_impl(fdfd_handle *h, const double2 *b, double2 *x, const fdfd_solve_opts &o, fdfd_stats &st) {
  Solve<R> sv;
  const int rc = sv.begin(h, b, x, o, &st);
  if (rc) return rc;
  while (!sv.done) {
    TRY(run_batch<R>(h, sv.ws, o.method, sv.ell, sv.tr, sv.batch, o.use_graph != 0));
    TRY(sv.after_batch());
  }
  return sv.end();
}

// Several systems at once (handles hs[i], each with its own stream and
// workspace): every round replays, as ONE parent CUDA graph, the captured
// iteration batch of each system still iterating (child graph nodes, which
// the GPU runs concurrently), then does each system's host-side step.
template <typename R>
static int solve_multi(fdfd_handle *const *hs, int nsys, const double2 *const *b, double2 *const *x,
                       const fdfd_solve_opts &o, fdfd_stats *st) {
  std::vector<Solve<R>> sv(nsys);
  int first_rc = FDFD_OK;
  for (int i = 0; i < nsys; ++i) {
    const int rc = sv[i].begin(hs[i], b[i], x[i], o, &st[i]);
    if (rc) {
      if (!sv[i].done) return rc;  // a CUDA or allocation failure
      if (first_rc == FDFD_OK) first_rc = rc;
    }
  }
  fdfd_handle *h0 = hs[0];
  cudaStream_t master = nullptr;
  TRY(cuda_check(h0, cudaStreamCreateWithFlags(&master, cudaStreamNonBlocking), "stream"));
  std::vector<cudaEvent_t> evs(nsys + 1, nullptr);
  int rc = FDFD_OK;
  for (auto &e : evs)
    if (rc == FDFD_OK) rc = cuda_check(h0, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  cudaGraphExec_t pexec = nullptr;
  std::vector<int> prev;
  while (rc == FDFD_OK) {
    std::vector<int> act;
    for (int i = 0; i < nsys; ++i)
      if (!sv[i].done) act.push_back(i);
    if (act.empty()) break;
    if (act != prev || !o.use_graph) {
      if (pexec) cudaGraphExecDestroy(pexec);
      pexec = nullptr;
      cudaGraph_t parent = nullptr;
      rc = cuda_check(h0, cudaGraphCreate(&parent, 0), "graph create");
      for (int i : act) {
        if (rc) break;
        cudaGraph_t child = nullptr;
        rc = batch_graph<R>(hs[i], sv[i].ws, o.method, sv[i].ell, sv[i].tr, sv[i].batch, nullptr, &child);
        cudaGraphNode_t node;
        if (rc == FDFD_OK) rc = cuda_check(h0, cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, child), "child graph");
      }
      if (rc == FDFD_OK) rc = cuda_check(h0, cudaGraphInstantiate(&pexec, parent, 0), "graph instantiate");
      if (parent) cudaGraphDestroy(parent);
      prev = act;
    }
    if (rc) break;
    // each system's stream → the master stream → the round → back
    for (int i : act) {
      if (rc == FDFD_OK) rc = cuda_check(hs[i], cudaEventRecord(evs[i], hs[i]->stream), "event");
      if (rc == FDFD_OK) rc = cuda_check(h0, cudaStreamWaitEvent(master, evs[i], 0), "wait event");
    }
    if (rc == FDFD_OK) rc = cuda_check(h0, cudaGraphLaunch(pexec, master), "graph launch");
    if (rc == FDFD_OK) rc = cuda_check(h0, cudaEventRecord(evs[nsys], master), "event");
    for (int i : act) {
      if (rc) break;
      rc = cuda_check(hs[i], cudaStreamWaitEvent(hs[i]->stream, evs[nsys], 0), "wait event");
      hs[i]->launches += batch_kernels<R>(sv[i].ws, o.method, sv[i].tr);
      if (rc == FDFD_OK) rc = sv[i].after_batch();
    }
  }
  if (pexec) cudaGraphExecDestroy(pexec);
  cudaStreamSynchronize(master);
  for (auto &e : evs)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(master);
  if (rc) return rc;
  for (int i = 0; i < nsys; ++i) {
    const int r = sv[i].end();
    if (r && first_rc == FDFD_OK) first_rc = r;
  }
  return first_rc;
}

int solve_multi_impl(fdfd_handle *const *hs, int nsys, const double2 *const *b, double2 *const *x,
                     const fdfd_solve_opts *o, fdfd_stats *st) {
  if (o->precision == FDFD_PREC_MIXED) return solve_multi<float>(hs, nsys, b, x, *o, st);
  return solve_multi<double>(hs, nsys, b, x, *o, st);
}

// out = in · V_E (inverse: in / V_E) per DOF, V_E(c) = s∆lₘ[c][g_c] Π_{v≠c} s∆lₑ[v][g_v]
// (the dual volume of the E_c sample; in and out may alias)
__global__ void k_scale_ve(const double2 *__restrict__ coef, int st, int o0, int o1, int o2, int N0, int N1,
                           long long ncell, const double2 *in, double2 *out, int inverse) {
  const int off[3] = {o0, o1, o2};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 3 * ncell;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % 3);
    const long long cell = i / 3;
    const int g[3] = {(int)(cell % N0), (int)((cell / N0) % N1), (int)(cell / ((long long)N0 * N1))};
    double2 v = make_double2(1.0, 0.0);
    for (int ax = 0; ax < 3; ++ax) {
      const double2 f = coef[(ax == c ? 5 : 4) * st + off[ax] + g[ax]];
      v = make_double2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
    }
    if (inverse) {
      const double d = v.x * v.x + v.y * v.y;
      v = make_double2(v.x / d, -v.y / d);
    }
    const double2 a = in[i];
    out[i] = make_double2(a.x * v.x - a.y * v.y, a.x * v.y + a.y * v.x);
  }
}

static int scale_ve(fdfd_handle *h, const double2 *in, double2 *out, bool inverse) {
  k_scale_ve<<<152 * 8, 256, 0, h->stream>>>(h->coef64, h->coef_stride, (int)h->coef_off[0], (int)h->coef_off[1],
                                             (int)h->coef_off[2], h->N[0], h->N[1], h->ncell, in, out,
                                             inverse ? 1 : 0);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_scale_ve");
}

// Aᵀ λ = b through the forward operator: V_E·A is complex symmetric, so
// Aᵀ = V A V⁻¹ and the system is A μ = V⁻¹ b with λ = V μ.  The forward
// solve runs on the fastest operator kernel; its tolerance is on the scaled
// residual, so after each solve the true residual ‖b − Aᵀλ‖ is formed in
// FP64 with the transposed kernel and the forward tolerance tightened (the
// next solve starting from the current μ) until that residual meets tol.
template <typename R>
static int solve_transposed_fwd(fdfd_handle *h, const double2 *b, double2 *x, const fdfd_solve_opts &o,
                                fdfd_stats &st) {
  const int ell = o.method == FDFD_BICGSTABL ? o.ell : 1;
  TRY(ensure_ws(h, sizeof(R) == 4, o.method, ell));
  Workspace *ws = h->ws;
  const long long n = ws->n;
  TRY(alloc(h, (void **)&ws->bt, n * sizeof(double2), "transposed right-hand side"));
  TRY(alloc(h, (void **)&ws->lt, n * sizeof(double2), "transposed solution"));
  TRY(dot<double>(h, b, b, n, ws->scu));
  KScalars tmp;
  TRY(read_scalars(h, ws->scu, &tmp));
  const double bb = tmp.dot1.x;
  st = fdfd_stats{};
  if (!std::isfinite(bb)) {
    st.status = FDFD_ERR_NONFINITE;
    return set_error(h, FDFD_ERR_NONFINITE, "the right-hand side holds a NaN or Inf");
  }
  TRY(scale_ve(h, b, ws->bt, true));
  if (o.x0_given) TRY(scale_ve(h, x, x, true));
  fdfd_solve_opts oi = o;
  oi.transpose = 0;
  double total_ms = 0.0;
  int rc = FDFD_OK;
  double relres = 0.0;
  for (int attempt = 0; attempt < 8; ++attempt) {
    fdfd_stats si{};
    rc = solve_impl<R>(h, ws->bt, x, oi, si);
    st.iterations += si.iterations;
    st.matvecs += si.matvecs;
    st.refinements += si.refinements;
    st.launches += si.launches;
    total_ms += si.time_ms;
    if (rc != FDFD_OK) break;
    // λ = V μ and its true residual in the transposed system
    TRY(scale_ve(h, x, ws->lt, false));
    TRY(launch_apply_fin<double>(h, ws->lt, ws->r64, EPI_RESID, b, FIN_NONE, ws->scu, true));
    TRY(read_scalars(h, ws->scu, &tmp));
    st.matvecs += 1;
    relres = bb > 0.0 ? std::sqrt(tmp.dot0.x / bb) : 0.0;
    if (!(relres > o.tol)) break;
    oi.tol = oi.tol * std::max(0.05, 0.5 * o.tol / relres);
    oi.x0_given = 1;
  }
  // x takes λ = V μ (also when the forward solve stopped early)
  TRY(scale_ve(h, x, x, false));
  TRY(cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync"));
  st.time_ms = total_ms;
  if (rc != FDFD_OK) {
    st.status = rc;
    return rc;
  }
  st.relres = relres;
  st.status = relres <= o.tol ? FDFD_OK : FDFD_ERR_NOT_CONVERGED;
  if (st.status != FDFD_OK)
    return set_error(h, st.status, "the transposed residual did not reach the tolerance");
  return FDFD_OK;
}

int solve_dev_impl(fdfd_handle *h, const double2 *b, double2 *x, const fdfd_solve_opts *o, fdfd_stats *st) {
  fdfd_stats tmp;
  fdfd_stats &s = st ? *st : tmp;
  // transposed systems run through the forward operator unless
  // FDFD_TRANSPOSE_KERNEL=1 asks for the transposed operator kernel
  static const bool tkernel = [] {
    const char *e = std::getenv("FDFD_TRANSPOSE_KERNEL");
    return e != nullptr && e[0] == '1';
  }();
  if (o->transpose && h->ft == FDFD_EE && o->method != FDFD_COCG && !tkernel) {
    if (o->precision == FDFD_PREC_MIXED) return solve_transposed_fwd<float>(h, b, x, *o, s);
    return solve_transposed_fwd<double>(h, b, x, *o, s);
  }
  if (o->precision == FDFD_PREC_MIXED) return solve_impl<float>(h, b, x, *o, s);
  return solve_impl<double>(h, b, x, *o, s);
}

}  // namespace fdfd
