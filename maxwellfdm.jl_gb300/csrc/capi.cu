// C ABI of libfdfd_gb300 (declared in include/fdfd_gb300.h).
//
// The reference's boundary for this path is the assembled operator and
// right-hand side returned by create_linsys / create_A / create_b
// (src/model/model.jl:209-274), consumed by A*x, mul!(y,A,x) and A\b.
// Here the host passes the inputs of that assembly — the stretched ∆l of
// create_stretched_∆ls (:122-139) and the material tensor εarr
// (:51, full.jl:16-70) — once, and every application or solve runs on the
// GPU against device-resident data.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "krylov_fin.cuh"

namespace fdfd {

static thread_local std::string g_last_error;

int set_error(fdfd_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  g_last_error = msg;
  return code;
}

cudaError_t dev_malloc_raw(void **p, size_t bytes) {
  const char *ev = std::getenv("FDFD_FAIL_ALLOC_BYTES");
  if (ev != nullptr) {
    const long long lim = std::atoll(ev);
    if (lim > 0 && bytes >= (size_t)lim) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  return cudaMalloc(p, bytes);
}

int cuda_check(fdfd_handle *h, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return FDFD_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return set_error(h, FDFD_ERR_NOMEM, m);
  return set_error(h, FDFD_ERR_CUDA, m);
}

// Make the handle's device current; an entry point returns the failure.
#define FDFD_SET_DEVICE(h)                                                          \
  do {                                                                              \
    const int _rc_dev = cuda_check((h), cudaSetDevice((h)->dev), "cudaSetDevice"); \
    if (_rc_dev) return _rc_dev;                                                    \
  } while (0)

int check_dev_err(fdfd_handle *h) {
  if (!h->dev_err) return FDFD_OK;
  int v = 0;
  int rc = cuda_check(h, cudaMemcpy(&v, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
  if (rc) return rc;
  if (v == 0) return FDFD_OK;
  cudaMemset(h->dev_err, 0, sizeof(int));
  return set_error(h, FDFD_ERR_TIMEOUT, "a bounded device-side wait gave up (a TMA copy did not complete)");
}

int solve_dev_impl(fdfd_handle *h, const double2 *b, double2 *x, const fdfd_solve_opts *o, fdfd_stats *st);
int solve_multi_impl(fdfd_handle *const *hs, int nsys, const double2 *const *b, double2 *const *x,
                     const fdfd_solve_opts *o, fdfd_stats *st);
int demote(fdfd_handle *, float2 *, const double2 *, long long);
int promote(fdfd_handle *, double2 *, const float2 *, long long);

using cd = std::complex<double>;

// Per-DOF factors of the COCG solver:
//   S = V_E (the symmetriser of A): V_E(c) = s∆lₘ[c][g_c] Π_{v≠c} s∆lₑ[v][g_v];
//   D⁻¹ = 1/diag(A), diag(A)_c = Σ_{v≠c} (1/s∆lₑ[v][g_v])·(1/s∆lₘ[v][g_v] +
//   1/s∆lₘ[v][g_v−1]) − ω² ε_cc, and −ω² ε_cc alone on pinned DOFs.
struct WeightArgs {
  const double2 *coef;
  const double *eps;
  int st, off[3], N[3], bloch[3];
  double2 w2;
};

__global__ void k_weights(WeightArgs a, double2 *w64, float2 *w32, double2 *d64, float2 *d32) {
  const long long ncell = (long long)a.N[0] * a.N[1] * a.N[2];
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < ncell;
       cell += (long long)gridDim.x * blockDim.x) {
    const int g[3] = {(int)(cell % a.N[0]), (int)((cell / a.N[0]) % a.N[1]), (int)(cell / ((long long)a.N[0] * a.N[1]))};
    for (int c = 0; c < 3; ++c) {
      double2 v = make_double2(1.0, 0.0);
      for (int ax = 0; ax < 3; ++ax) {
        const double2 f = a.coef[(ax == c ? 5 : 4) * a.st + a.off[ax] + g[ax]];
        v = make_double2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
      }
      if (w64) w64[3 * cell + c] = v;
      if (w32) w32[3 * cell + c] = make_float2((float)v.x, (float)v.y);
      bool pinned = false;
      double2 d = make_double2(0.0, 0.0);
      for (int ax = 0; ax < 3; ++ax) {
        if (ax == c) continue;
        if (!a.bloch[ax] && g[ax] == 0) pinned = true;
        const int gm = g[ax] > 0 ? g[ax] - 1 : a.N[ax] - 1;
        const double2 ce = a.coef[1 * a.st + a.off[ax] + g[ax]];
        const double2 c0 = a.coef[0 * a.st + a.off[ax] + g[ax]], c1 = a.coef[0 * a.st + a.off[ax] + gm];
        const double2 s = make_double2(c0.x + c1.x, c0.y + c1.y);
        d.x += ce.x * s.x - ce.y * s.y;
        d.y += ce.x * s.y + ce.y * s.x;
      }
      if (pinned) d = make_double2(0.0, 0.0);
      const double e = a.eps[c * ncell + cell];
      d.x -= a.w2.x * e;
      d.y -= a.w2.y * e;
      const double dd = d.x * d.x + d.y * d.y;
      const double2 inv = make_double2(d.x / dd, -d.y / dd);
      if (d64) d64[3 * cell + c] = inv;
      if (d32) d32[3 * cell + c] = make_float2((float)inv.x, (float)inv.y);
    }
  }
}

int build_weights(fdfd_handle *h, double2 *w64, float2 *w32, double2 *d64, float2 *d32) {
  WeightArgs a;
  a.coef = h->coef64;
  a.eps = h->eps64;
  a.st = h->coef_stride;
  for (int w = 0; w < 3; ++w) {
    a.off[w] = (int)h->coef_off[w];
    a.N[w] = h->N[w];
    a.bloch[w] = h->bloch[w];
  }
  a.w2 = make_double2(h->w2[0], h->w2[1]);
  k_weights<<<152 * 4, 256, 0, h->stream>>>(a, w64, w32, d64, d32);
  return cuda_check(h, cudaGetLastError(), "k_weights");
}

// Flag (xy tile, plane k) if any off-diagonal ε that the tile's outputs at
// plane k read is non-zero: corners i ∈ [i0, i0+TX], j ∈ [j0, j0+TY],
// planes k and k+1.
__global__ void k_oflags(const double *eoff, long long ncell, int N0, int N1, int N2, int tiles_x, uint8_t *flag) {
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < ncell;
       cell += (long long)gridDim.x * blockDim.x) {
    if (eoff[cell] == 0.0 && eoff[ncell + cell] == 0.0 && eoff[2 * ncell + cell] == 0.0) continue;
    const int i = (int)(cell % N0), j = (int)((cell / N0) % N1), k = (int)(cell / ((long long)N0 * N1));
    const int tx0 = i / TX, ty0 = j / TY;
    for (int dx = -1; dx <= 0; ++dx) {
      const int tx = tx0 + dx;
      if (tx < 0 || (dx == -1 && i % TX != 0)) continue;
      for (int dy = -1; dy <= 0; ++dy) {
        const int ty = ty0 + dy;
        if (ty < 0 || (dy == -1 && j % TY != 0)) continue;
        const long long tc = tx + (long long)tiles_x * ty;
        flag[tc * N2 + k] = 1;
        if (k > 0) flag[tc * N2 + k - 1] = 1;
      }
    }
  }
}

// Flag (x tile, group of g rows, plane k) if any off-diagonal ε that the
// outputs of those rows at plane k read is non-zero: corners i ∈ [i0, i0+TX],
// rows j ∈ [g·t, g·t+g], planes k and k+1 (the second TMA kernel's warps own
// g rows each).
__global__ void k_oflags_rows(const double *eoff, long long ncell, int N0, int N1, int N2, int tiles_x, int g,
                              uint8_t *flag) {
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < ncell;
       cell += (long long)gridDim.x * blockDim.x) {
    if (eoff[cell] == 0.0 && eoff[ncell + cell] == 0.0 && eoff[2 * ncell + cell] == 0.0) continue;
    const int i = (int)(cell % N0), j = (int)((cell / N0) % N1), k = (int)(cell / ((long long)N0 * N1));
    const int tx0 = i / TX, ty0 = j / g;
    for (int dx = -1; dx <= 0; ++dx) {
      const int tx = tx0 + dx;
      if (tx < 0 || (dx == -1 && i % TX != 0)) continue;
      for (int dy = -1; dy <= 0; ++dy) {
        const int ty = ty0 + dy;
        if (ty < 0 || (dy == -1 && j % g != 0)) continue;
        const long long tc = tx + (long long)tiles_x * ty;
        flag[tc * N2 + k] = 1;
        if (k > 0) flag[tc * N2 + k - 1] = 1;
      }
    }
  }
}

int build_oflags(fdfd_handle *h) {
  if (!h->has_off) return FDFD_OK;
  const int tiles_x = (h->N[0] + TX - 1) / TX, tiles_y = (h->N[1] + TY - 1) / TY;
  const size_t nflag = (size_t)tiles_x * tiles_y * h->N[2];
  if (!h->oflag) {
    if (dev_malloc(&h->oflag, nflag) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(oflag) failed");
    }
  }
  int rc = cuda_check(h, cudaMemsetAsync(h->oflag, 0, nflag, h->stream), "memset oflag");
  if (rc) return rc;
  k_oflags<<<152 * 4, 256, 0, h->stream>>>(h->eoff64, h->ncell, h->N[0], h->N[1], h->N[2], tiles_x, h->oflag);
  if ((rc = cuda_check(h, cudaGetLastError(), "k_oflags"))) return rc;
  // per groups of 1 and 2 rows (the second TMA kernel's warp strips)
  for (int g = 1; g <= 2; ++g) {
    const size_t nf = (size_t)tiles_x * ((h->N[1] + g - 1) / g) * h->N[2];
    uint8_t *&f = h->oflag_rows[g - 1];
    if (!f) {
      if (dev_malloc(&f, nf) != cudaSuccess) {
        cudaGetLastError();
        return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(oflag rows) failed");
      }
    }
    if ((rc = cuda_check(h, cudaMemsetAsync(f, 0, nf, h->stream), "memset oflag rows"))) return rc;
    k_oflags_rows<<<152 * 4, 256, 0, h->stream>>>(h->eoff64, h->ncell, h->N[0], h->N[1], h->N[2], tiles_x, g, f);
    if ((rc = cuda_check(h, cudaGetLastError(), "k_oflags_rows"))) return rc;
  }
  return FDFD_OK;
}

__global__ void k_to_f32(float *dst, const double *src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

static int ensure_eps_buffers(fdfd_handle *h, bool off) {
  const size_t n = 3 * (size_t)h->ncell;
  if (!h->eps64) {
    if (dev_malloc(&h->eps64, n * sizeof(double)) != cudaSuccess ||
        dev_malloc(&h->eps32, n * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(eps) failed");
    }
  }
  if (off && !h->eoff64) {
    if (dev_malloc(&h->eoff64, n * sizeof(double)) != cudaSuccess ||
        dev_malloc(&h->eoff32, n * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(eps off-diagonal) failed");
    }
  }
  return FDFD_OK;
}

// Refresh the FP32 copies from the FP64 masters and rebuild the flags.
int finish_eps(fdfd_handle *h) {
  const long long n = 3 * h->ncell;
  k_to_f32<<<152 * 4, 256, 0, h->stream>>>(h->eps32, h->eps64, n);
  int rc = cuda_check(h, cudaGetLastError(), "k_to_f32");
  if (rc) return rc;
  if (h->has_off) {
    k_to_f32<<<152 * 4, 256, 0, h->stream>>>(h->eoff32, h->eoff64, n);
    rc = cuda_check(h, cudaGetLastError(), "k_to_f32");
    if (rc) return rc;
    rc = build_oflags(h);
    if (rc) return rc;
  }
  rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
  if (rc == FDFD_OK && h->tuned_off >= 0 && h->tuned_off != (h->has_off ? 1 : 0)) {
    // retune the z-chunk for the new operator; captured graphs hold the old
    // launch shapes and possibly a reduction buffer that is about to grow
    drop_graphs(h);
    if ((rc = autotune_kchunk(h))) return rc;
    if ((rc = ensure_red(h, apply_blocks(h)))) return rc;
    rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
  }
  return rc;
}

// eps_diag_aos[c + 3 cell], eps_off_aos[p + 3 cell] (or null) → SoA on device
int upload_eps(fdfd_handle *h, const double *eps_diag_aos, const double *eps_off_aos) {
  const long long nc = h->ncell;
  bool off = false;
  if (eps_off_aos)
    for (long long i = 0; i < 3 * nc && !off; ++i) off = eps_off_aos[i] != 0.0;
  int rc = ensure_eps_buffers(h, off);
  if (rc) return rc;
  std::vector<double> soa(3 * (size_t)nc);
  for (long long cell = 0; cell < nc; ++cell)
    for (int c = 0; c < 3; ++c) soa[c * nc + cell] = eps_diag_aos[c + 3 * cell];
  rc = cuda_check(h, cudaMemcpy(h->eps64, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice),
                  "upload eps");
  if (rc) return rc;
  h->has_off = off;
  h->has_design = false;  // explicit ε replaces any smoothed design region
  if (off) {
    for (long long cell = 0; cell < nc; ++cell)
      for (int p = 0; p < 3; ++p) soa[p * nc + cell] = eps_off_aos[p + 3 * cell];
    rc = cuda_check(h, cudaMemcpy(h->eoff64, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice),
                    "upload eps off");
    if (rc) return rc;
  }
  return finish_eps(h);
}

static int ensure_scratch(fdfd_handle *h, bool c64) {
  const size_t n = 3 * (size_t)h->ncell;
  if (!h->vx64) {
    if (dev_malloc(&h->vx64, n * sizeof(double2)) != cudaSuccess ||
        dev_malloc(&h->vy64, n * sizeof(double2)) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(scratch) failed");
    }
  }
  if (c64 && !h->vx32) {
    if (dev_malloc(&h->vx32, n * sizeof(float2)) != cudaSuccess ||
        dev_malloc(&h->vy32, n * sizeof(float2)) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(scratch c64) failed");
    }
  }
  return FDFD_OK;
}

static bool transpose_ok(const fdfd_handle *h) {
  for (int w = 0; w < 3; ++w)
    if (h->bloch[w] && (h->e_ikl[w][0] != 1.0 || h->e_ikl[w][1] != 0.0)) return false;
  return true;
}

static int matvec_host(fdfd_handle *h, const double *x, double *y, int precision, bool tr) {
  if (!h || !x || !y) return set_error(h, FDFD_ERR_ARG, "null argument");
  if (precision != FDFD_C128 && precision != FDFD_C64) return set_error(h, FDFD_ERR_ARG, "bad precision");
  if (tr && !transpose_ok(h)) return set_error(h, FDFD_ERR_UNSUPPORTED, "transpose with a Bloch phase");
  int rc = ensure_scratch(h, precision == FDFD_C64);
  if (rc) return rc;
  const long long n = 3 * h->ncell;
  const int mask = field_mask(h, h->ft == FDFD_HH);  // the unknown field's components
  if ((rc = h2d_field(h, x, h->vx64, mask))) return rc;
  if (precision == FDFD_C64) {
    if ((rc = demote(h, h->vx32, h->vx64, n))) return rc;
    if ((rc = launch_apply_fin<float>(h, h->vx32, h->vy32, EPI_STORE, nullptr, FIN_NONE, nullptr, tr))) return rc;
    if ((rc = promote(h, h->vy64, h->vy32, n))) return rc;
  } else {
    if ((rc = launch_apply_fin<double>(h, h->vx64, h->vy64, EPI_STORE, nullptr, FIN_NONE, nullptr, tr))) return rc;
  }
  if ((rc = d2h_field(h, h->vy64, y, mask))) return rc;
  rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
  if (rc) return rc;
  return check_dev_err(h);
}

}  // namespace fdfd

using namespace fdfd;

extern "C" {

const char *fdfd_version(void) { return "fdfd_gb300 0.1 (sm_103a)"; }

const char *fdfd_last_error(const fdfd_handle *h) {
  if (h) return h->err.c_str();
  return g_last_error.c_str();
}

void fdfd_default_opts(fdfd_solve_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->method = FDFD_BICGSTABL;  // BiCGStab(4): the fewest operator applications on these systems
  o->precision = FDFD_PREC_MIXED;
  o->tol = 1e-6;
  o->maxit = 200000;
  o->delta = 0.1;
  o->x0_given = 0;
  o->check_every = 50;
  o->transpose = 0;
  o->use_graph = 1;
  o->ell = 4;
}

int fdfd_create(const fdfd_desc *d, fdfd_handle **out) {
  if (!d || !out) return set_error(nullptr, FDFD_ERR_ARG, "null argument");
  *out = nullptr;
  for (int w = 0; w < 3; ++w) {
    if (d->N[w] < 1) return set_error(nullptr, FDFD_ERR_ARG, "N must be >= 1 on every axis");
    if (!d->sdl_e[w] || !d->sdl_m[w]) return set_error(nullptr, FDFD_ERR_ARG, "null s∆l array");
    if (d->boundft[w] != FDFD_EE) return set_error(nullptr, FDFD_ERR_UNSUPPORTED, "boundft = HH is not supported");
    if (d->isbloch[w] != 0 && d->isbloch[w] != 1) return set_error(nullptr, FDFD_ERR_ARG, "isbloch must be 0 or 1");
    if (!d->isbloch[w] && d->N[w] < 2) return set_error(nullptr, FDFD_ERR_ARG, "N must be >= 2 on a symmetry axis");
  }
  if (d->order_cmpfirst != 1) return set_error(nullptr, FDFD_ERR_UNSUPPORTED, "order_cmpfirst = false");
  if (d->slice2d != FDFD_SLICE_NONE) {
    if (d->slice2d != FDFD_SLICE_TE && d->slice2d != FDFD_SLICE_TM) return set_error(nullptr, FDFD_ERR_ARG, "bad slice2d");
    if (d->N[2] != 1 || d->isbloch[2] != 1 || d->e_ikl[2][0] != 1.0 || d->e_ikl[2][1] != 0.0)
      return set_error(nullptr, FDFD_ERR_ARG, "a 2D slice needs N[2] = 1, isbloch[2] = 1 and e_ikl[2] = 1");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(nullptr, FDFD_ERR_NO_DEVICE, "no CUDA device");
  }
  if (d->device < 0 || d->device >= ndev) return set_error(nullptr, FDFD_ERR_ARG, "bad device ordinal");
  if (d->device >= MAX_DEVICES) return set_error(nullptr, FDFD_ERR_UNSUPPORTED, "device ordinal above 63");
  fdfd_handle *h = new fdfd_handle();
  h->dev = d->device;
  int rc;
  if ((rc = cuda_check(h, cudaSetDevice(h->dev), "cudaSetDevice"))) { delete h; return rc; }
  if ((rc = cuda_check(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream"))) {
    delete h;
    return rc;
  }
  cudaEventCreate(&h->ev0);
  cudaEventCreate(&h->ev1);
  for (int w = 0; w < 3; ++w) {
    h->N[w] = d->N[w];
    h->bloch[w] = d->isbloch[w];
    h->slice2d = d->slice2d;
    h->e_ikl[w][0] = d->e_ikl[w][0];
    h->e_ikl[w][1] = d->e_ikl[w][1];
    if (!h->bloch[w]) { h->e_ikl[w][0] = 1.0; h->e_ikl[w][1] = 0.0; }
  }
  h->ncell = (long long)h->N[0] * h->N[1] * h->N[2];
  h->omega[0] = d->omega[0];
  h->omega[1] = d->omega[1];
  const cd om(d->omega[0], d->omega[1]);
  const cd w2 = om * om;
  h->w2[0] = w2.real();
  h->w2[1] = w2.imag();
  // per-axis coefficients, 6 kinds: cm, ce, wm, wp, s∆lₑ, s∆lₘ
  const int st = h->N[0] + h->N[1] + h->N[2];
  h->coef_stride = st;
  h->coef_off[0] = 0;
  h->coef_off[1] = h->N[0];
  h->coef_off[2] = h->N[0] + h->N[1];
  std::vector<double2> c64(6 * (size_t)st);
  std::vector<float2> c32(6 * (size_t)st);
  for (int w = 0; w < 3; ++w) {
    const int N = h->N[w];
    for (int i = 0; i < N; ++i) {
      const cd se(d->sdl_e[w][2 * i], d->sdl_e[w][2 * i + 1]);
      const cd sm(d->sdl_m[w][2 * i], d->sdl_m[w][2 * i + 1]);
      if (std::abs(se) == 0.0 || std::abs(sm) == 0.0 || !std::isfinite(std::abs(se)) || !std::isfinite(std::abs(sm))) {
        fdfd_destroy(h);
        return set_error(nullptr, FDFD_ERR_ARG, "s∆l entries must be finite and non-zero");
      }
      const int jm = i > 0 ? i - 1 : (h->bloch[w] ? N - 1 : 0);
      const cd smm(d->sdl_m[w][2 * jm], d->sdl_m[w][2 * jm + 1]);
      const cd vals[6] = {1.0 / sm, 1.0 / se, smm / (2.0 * se), sm / (2.0 * se), se, sm};
      for (int kd = 0; kd < 6; ++kd) {
        const size_t idx = (size_t)kd * st + h->coef_off[w] + i;
        c64[idx] = make_double2(vals[kd].real(), vals[kd].imag());
        c32[idx] = make_float2((float)vals[kd].real(), (float)vals[kd].imag());
      }
    }
  }
  // the contiguous index range (outside the PML) where the curl and averaging
  // coefficients are real: operator tiles inside it take a real-arithmetic path
  for (int w = 0; w < 3; ++w) {
    const int N = h->N[w];
    auto is_real = [&](int i) {
      for (int kd = 0; kd < 4; ++kd)
        if (c64[(size_t)kd * st + h->coef_off[w] + i].y != 0.0) return false;
      return true;
    };
    int lo = 0;
    while (lo < N && !is_real(lo)) ++lo;
    int hi = lo;
    while (hi + 1 < N && is_real(hi + 1)) ++hi;
    h->rlo[w] = lo < N ? lo : 1;
    h->rhi[w] = lo < N ? hi : 0;
  }
  if (dev_malloc(&h->coef64, c64.size() * sizeof(double2)) != cudaSuccess ||
      dev_malloc(&h->coef32, c32.size() * sizeof(float2)) != cudaSuccess) {
    cudaGetLastError();
    fdfd_destroy(h);
    return set_error(nullptr, FDFD_ERR_NOMEM, "cudaMalloc(coefficients) failed");
  }
  cudaMemcpy(h->coef64, c64.data(), c64.size() * sizeof(double2), cudaMemcpyHostToDevice);
  cudaMemcpy(h->coef32, c32.data(), c32.size() * sizeof(float2), cudaMemcpyHostToDevice);
  // ε = 1 (vacuum) until set
  if ((rc = ensure_eps_buffers(h, false))) { fdfd_destroy(h); return rc; }
  {
    std::vector<double> ones(3 * (size_t)h->ncell, 1.0);
    cudaMemcpy(h->eps64, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  if ((rc = finish_eps(h))) { fdfd_destroy(h); return rc; }
  if (dev_malloc(&h->util_sc, sizeof(KScalars)) != cudaSuccess) {
    cudaGetLastError();
    fdfd_destroy(h);
    return set_error(nullptr, FDFD_ERR_NOMEM, "cudaMalloc(scalars) failed");
  }
  cudaMemsetAsync(h->util_sc, 0, sizeof(KScalars), h->stream);
  if (dev_malloc(&h->dev_err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    fdfd_destroy(h);
    return set_error(nullptr, FDFD_ERR_NOMEM, "cudaMalloc(error flag) failed");
  }
  cudaMemsetAsync(h->dev_err, 0, sizeof(int), h->stream);
  {
    const char *ev = std::getenv("FDFD_DISABLE_TMA");
    h->tma_disabled = ev != nullptr && ev[0] != '\0' && ev[0] != '0';
    // programmatic dependent launch measured slower on the 96³ solve (the
    // early-resident dependants take SM slots); opt in with FDFD_PDL=1
    const char *pd = std::getenv("FDFD_PDL");
    h->pdl = pd != nullptr && pd[0] != '\0' && pd[0] != '0';
    const char *kc = std::getenv("FDFD_KCHUNK");
    if (kc != nullptr) h->kc_force = std::max(1, std::min(std::atoi(kc), h->N[2]));
    const char *ov = std::getenv("FDFD_OPERATOR_V2");
    if (ov != nullptr) h->op_variant = std::atoi(ov);
    const char *wl = std::getenv("FDFD_WAIT_LIMIT_CLOCKS");
    if (wl != nullptr) h->wait_limit = std::max(0ll, std::min(std::atoll(wl), h->wait_limit));
  }
  if ((rc = autotune_kchunk(h))) { fdfd_destroy(h); return rc; }
  if ((rc = ensure_red(h, apply_blocks(h)))) { fdfd_destroy(h); return rc; }
  if ((rc = cuda_check(h, cudaStreamSynchronize(h->stream), "create sync"))) { fdfd_destroy(h); return rc; }
  *out = h;
  return FDFD_OK;
}

void fdfd_destroy(fdfd_handle *h) {
  if (!h) return;
  cudaSetDevice(h->dev);  // best effort: a destructor has no status to return
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_workspace(h);
  if (!h->shares_operator) {
    cudaFree(h->coef64);
    cudaFree(h->coef32);
    cudaFree(h->eps64);
    cudaFree(h->eps32);
    cudaFree(h->eoff64);
    cudaFree(h->eoff32);
    cudaFree(h->oflag);
    cudaFree(h->oflag_rows[0]);
    cudaFree(h->oflag_rows[1]);
    cudaFree(h->smask);
    cudaFree(h->work[0]);
    cudaFree(h->work[1]);
  }
  cudaFree(h->vx64);
  cudaFree(h->vy64);
  cudaFree(h->ve64);
  cudaFree(h->stage64);
  cudaFree(h->vx32);
  cudaFree(h->vy32);
  cudaFree(h->red.part);
  cudaFree(h->red.count);
  cudaFree(h->util_sc);
  cudaFree(h->dev_err);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

void *fdfd_stream(fdfd_handle *h) { return h ? (void *)h->stream : nullptr; }

int fdfd_sync(fdfd_handle *h) {
  if (!h) return set_error(nullptr, FDFD_ERR_ARG, "null handle");
  int rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
  if (rc) return rc;
  return check_dev_err(h);
}

int fdfd_set_eps(fdfd_handle *h, const double *eps_diag, const double *eps_off) {
  if (!h || !eps_diag) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  return upload_eps(h, eps_diag, eps_off);
}

int fdfd_set_eps_tensor(fdfd_handle *h, const double *epsarr) {
  if (!h || !epsarr) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  const long long nc = h->ncell;
  // column-major (Nx,Ny,Nz,3,3): element (cell, r, c) at cell + nc*(r + 3c)
  auto at = [&](long long cell, int r, int c, int part) { return epsarr[2 * (cell + nc * (r + 3 * c)) + part]; };
  std::vector<double> diag(3 * (size_t)nc), off(3 * (size_t)nc);
  const int pr[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  for (long long cell = 0; cell < nc; ++cell) {
    for (int c = 0; c < 3; ++c) {
      if (at(cell, c, c, 1) != 0.0) return set_error(h, FDFD_ERR_UNSUPPORTED, "complex ε (lossy material)");
      diag[c + 3 * cell] = at(cell, c, c, 0);
    }
    for (int p = 0; p < 3; ++p) {
      const double a = at(cell, pr[p][0], pr[p][1], 0), b = at(cell, pr[p][1], pr[p][0], 0);
      if (at(cell, pr[p][0], pr[p][1], 1) != 0.0 || at(cell, pr[p][1], pr[p][0], 1) != 0.0)
        return set_error(h, FDFD_ERR_UNSUPPORTED, "complex off-diagonal ε");
      if (a != b) return set_error(h, FDFD_ERR_UNSUPPORTED, "non-symmetric ε tensor");
      off[p + 3 * cell] = a;
    }
  }
  return upload_eps(h, diag.data(), off.data());
}

int fdfd_smooth_objects(fdfd_handle *h, const double *const lprim[3], const fdfd_object *objs, int32_t nobj,
                        double eps_bg, const fdfd_design *design) {
  if (!h || !lprim || (nobj > 0 && !objs) || nobj < 0) return set_error(h, FDFD_ERR_ARG, "bad argument");
  for (int w = 0; w < 3; ++w)
    if (!lprim[w]) return set_error(h, FDFD_ERR_ARG, "null lprim");
  FDFD_SET_DEVICE(h);
  return smooth_objects_impl(h, lprim, objs, nobj, eps_bg, design);
}

int fdfd_get_eps(fdfd_handle *h, double *eps_diag, double *eps_off, uint8_t *smask) {
  if (!h) return set_error(nullptr, FDFD_ERR_ARG, "null handle");
  FDFD_SET_DEVICE(h);
  const long long nc = h->ncell;
  std::vector<double> soa(3 * (size_t)nc);
  int rc;
  if (eps_diag) {
    if ((rc = cuda_check(h, cudaMemcpy(soa.data(), h->eps64, soa.size() * sizeof(double), cudaMemcpyDeviceToHost),
                         "D2H eps")))
      return rc;
    for (long long cell = 0; cell < nc; ++cell)
      for (int c = 0; c < 3; ++c) eps_diag[c + 3 * cell] = soa[c * nc + cell];
  }
  if (eps_off) {
    if (h->has_off) {
      if ((rc = cuda_check(h, cudaMemcpy(soa.data(), h->eoff64, soa.size() * sizeof(double),
                                         cudaMemcpyDeviceToHost), "D2H eoff")))
        return rc;
      for (long long cell = 0; cell < nc; ++cell)
        for (int p = 0; p < 3; ++p) eps_off[p + 3 * cell] = soa[p * nc + cell];
    } else {
      std::memset(eps_off, 0, 3 * (size_t)nc * sizeof(double));
    }
  }
  if (smask) {
    if (h->smask) {
      if ((rc = cuda_check(h, cudaMemcpy(smask, h->smask, 4 * (size_t)nc, cudaMemcpyDeviceToHost), "D2H smask")))
        return rc;
    } else {
      std::memset(smask, 0, 4 * (size_t)nc);
    }
  }
  return FDFD_OK;
}

int fdfd_matvec(fdfd_handle *h, const double *x, double *y, int32_t precision) {
  if (!h) return set_error(nullptr, FDFD_ERR_ARG, "null handle");
  FDFD_SET_DEVICE(h);
  return matvec_host(h, x, y, precision, false);
}

int fdfd_matvec_transpose(fdfd_handle *h, const double *x, double *y, int32_t precision) {
  if (!h) return set_error(nullptr, FDFD_ERR_ARG, "null handle");
  FDFD_SET_DEVICE(h);
  return matvec_host(h, x, y, precision, true);
}

int fdfd_matvec_dev(fdfd_handle *h, const void *x, void *y, int32_t precision) {
  if (!h || !x || !y) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  if (precision == FDFD_C64)
    return launch_apply_fin<float>(h, (const float2 *)x, (float2 *)y, EPI_STORE, nullptr, FIN_NONE, nullptr, false);
  if (precision == FDFD_C128)
    return launch_apply_fin<double>(h, (const double2 *)x, (double2 *)y, EPI_STORE, nullptr, FIN_NONE, nullptr,
                                    false);
  return set_error(h, FDFD_ERR_ARG, "bad precision");
}

int fdfd_residual_dev(fdfd_handle *h, const void *x, const void *b, void *r, double *rnorm2) {
  if (!h || !x || !b || !r || !rnorm2) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  int rc = ensure_red(h, apply_blocks(h));
  if (rc) return rc;
  rc = launch_apply_fin<double>(h, (const double2 *)x, (double2 *)r, EPI_RESID, (const double2 *)b, FIN_NONE,
                                h->util_sc, false);
  if (rc) return rc;
  KScalars hs;
  rc = cuda_check(h, cudaMemcpyAsync(&hs, h->util_sc, sizeof(KScalars), cudaMemcpyDeviceToHost, h->stream),
                  "D2H residual");
  if (rc) return rc;
  rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
  if (rc) return rc;
  *rnorm2 = hs.dot0.x;
  return FDFD_OK;
}

static int check_opts(fdfd_handle *h, const fdfd_solve_opts *o) {
  if (!o) return set_error(h, FDFD_ERR_ARG, "null options");
  if (o->precision != FDFD_PREC_FP64 && o->precision != FDFD_PREC_MIXED)
    return set_error(h, FDFD_ERR_ARG, "bad precision");
  if (o->method != FDFD_BICGSTAB && o->method != FDFD_COCG && o->method != FDFD_BICGSTABL)
    return set_error(h, FDFD_ERR_ARG, "bad method");
  if (o->method == FDFD_BICGSTABL && (o->ell < 1 || o->ell > 4))
    return set_error(h, FDFD_ERR_ARG, "BiCGStab(l) needs 1 <= ell <= 4");
  if (!(o->tol > 0.0) || o->maxit < 1) return set_error(h, FDFD_ERR_ARG, "bad tol/maxit");
  if (o->precision == FDFD_PREC_MIXED && !(o->delta > 0.0 && o->delta < 1.0))
    return set_error(h, FDFD_ERR_ARG, "delta must be in (0, 1)");
  if (o->transpose && !transpose_ok(h)) return set_error(h, FDFD_ERR_UNSUPPORTED, "transpose with a Bloch phase");
  if (h->ft == FDFD_HH && (o->transpose || o->method == FDFD_COCG))
    return set_error(h, FDFD_ERR_UNSUPPORTED, "the H formulation solves the forward system with BiCGSTAB");
  if (o->method == FDFD_COCG && o->precision == FDFD_PREC_MIXED)
    return set_error(h, FDFD_ERR_UNSUPPORTED, "COCG runs in FP64 only (its complex64 recurrence does not converge)");
  if (o->method == FDFD_COCG && o->transpose)
    return set_error(h, FDFD_ERR_UNSUPPORTED, "COCG solves the forward system only (use BiCGSTAB for Aᵀ)");
  if (o->method == FDFD_COCG && !transpose_ok(h))
    return set_error(h, FDFD_ERR_UNSUPPORTED, "COCG needs a complex-symmetric operator (no Bloch phase)");
  return FDFD_OK;
}

int fdfd_solve_dev(fdfd_handle *h, const void *b, void *x, const fdfd_solve_opts *opts, fdfd_stats *stats) {
  if (!h || !b || !x) return set_error(h, FDFD_ERR_ARG, "null argument");
  int rc = check_opts(h, opts);
  if (rc) return rc;
  FDFD_SET_DEVICE(h);
  return solve_dev_impl(h, (const double2 *)b, (double2 *)x, opts, stats);
}

int fdfd_solve(fdfd_handle *h, const double *b, double *x, int32_t nrhs, const fdfd_solve_opts *opts,
               fdfd_stats *stats) {
  if (!h || !b || !x || nrhs < 1) return set_error(h, FDFD_ERR_ARG, "bad argument");
  int rc = check_opts(h, opts);
  if (rc) return rc;
  FDFD_SET_DEVICE(h);
  if ((rc = ensure_scratch(h, false))) return rc;
  const int mask = field_mask(h, h->ft == FDFD_HH);  // the unknown field's components
  const long long n = __builtin_popcount(mask) * h->ncell;  // complex entries per host vector
  int first_err = FDFD_OK;
  std::string first_msg;
  for (int q = 0; q < nrhs; ++q) {
    const double *bq = b + 2 * n * q;
    double *xq = x + 2 * n * q;
    if ((rc = h2d_field(h, bq, h->vx64, mask))) return rc;
    if (opts->x0_given && (rc = h2d_field(h, xq, h->vy64, mask))) return rc;
    rc = solve_dev_impl(h, h->vx64, h->vy64, opts, stats ? stats + q : nullptr);
    if (rc && rc != FDFD_ERR_NOT_CONVERGED && rc != FDFD_ERR_BREAKDOWN) return rc;
    if (rc && first_err == FDFD_OK) {
      first_err = rc;
      first_msg = h->err;
    }
    int rc2 = d2h_field(h, h->vy64, xq, mask);
    if (rc2) return rc2;
    if ((rc2 = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync"))) return rc2;
  }
  if (first_err) return set_error(h, first_err, first_msg);
  return FDFD_OK;
}

// A worker for concurrent solves: the parent's operator data (read-only
// during a solve) with its own stream, events, reduction buffer, scalars,
// workspace and scratch.
static fdfd_handle *make_worker(fdfd_handle *p, int *rc) {
  fdfd_handle *w = new fdfd_handle();
  w->dev = p->dev;
  for (int a = 0; a < 3; ++a) {
    w->N[a] = p->N[a];
    w->bloch[a] = p->bloch[a];
    w->coef_off[a] = p->coef_off[a];
    w->rlo[a] = p->rlo[a];
    w->rhi[a] = p->rhi[a];
    w->e_ikl[a][0] = p->e_ikl[a][0];
    w->e_ikl[a][1] = p->e_ikl[a][1];
  }
  w->ncell = p->ncell;
  w->omega[0] = p->omega[0];
  w->omega[1] = p->omega[1];
  w->w2[0] = p->w2[0];
  w->w2[1] = p->w2[1];
  w->coef64 = p->coef64;
  w->coef32 = p->coef32;
  w->coef_stride = p->coef_stride;
  w->eps64 = p->eps64;
  w->eps32 = p->eps32;
  w->eoff64 = p->eoff64;
  w->eoff32 = p->eoff32;
  w->oflag = p->oflag;
  w->oflag_rows[0] = p->oflag_rows[0];
  w->oflag_rows[1] = p->oflag_rows[1];
  w->has_off = p->has_off;
  w->smask = p->smask;
  w->slice2d = p->slice2d;
  w->ft = p->ft;
  w->tma_disabled = p->tma_disabled;
  w->pdl = p->pdl;
  w->kc[0] = p->kc[0];
  w->kc[1] = p->kc[1];
  for (int q = 0; q < 2; ++q) {
    w->work[q] = p->work[q];
    w->nwork[q] = p->nwork[q];
  }
  w->kc_force = p->kc_force;
  w->wait_limit = p->wait_limit;
  w->op_variant = p->op_variant;
  w->tuned_off = p->tuned_off;
  w->shares_operator = true;
  *rc = FDFD_OK;
  if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&w->ev0) != cudaSuccess || cudaEventCreate(&w->ev1) != cudaSuccess ||
      dev_malloc(&w->util_sc, sizeof(KScalars)) != cudaSuccess || dev_malloc(&w->dev_err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    *rc = set_error(p, FDFD_ERR_NOMEM, "creating a batch worker failed");
    return w;
  }
  cudaMemsetAsync(w->util_sc, 0, sizeof(KScalars), w->stream);
  cudaMemsetAsync(w->dev_err, 0, sizeof(int), w->stream);
  if ((*rc = ensure_red(w, apply_blocks(w)))) set_error(p, *rc, w->err);
  return w;
}

int fdfd_solve_batch(fdfd_handle *h, const double *b, double *x, int32_t nrhs, int32_t nworkers,
                     const fdfd_solve_opts *opts, fdfd_stats *stats) {
  if (!h || !b || !x || nrhs < 1 || nworkers < 1) return set_error(h, FDFD_ERR_ARG, "bad argument");
  int rc = check_opts(h, opts);
  if (rc) return rc;
  if (nworkers > nrhs) nworkers = nrhs;
  if (nworkers == 1) return fdfd_solve(h, b, x, nrhs, opts, stats);
  FDFD_SET_DEVICE(h);
  if ((rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync"))) return rc;
  std::vector<fdfd_handle *> ws(nworkers, nullptr);
  for (int t = 0; t < nworkers && rc == FDFD_OK; ++t) ws[t] = make_worker(h, &rc);
  const int mask = field_mask(h, h->ft == FDFD_HH);
  const long long n = __builtin_popcount(mask) * h->ncell;
  std::vector<int> rcs(nworkers, FDFD_OK);
  std::vector<std::string> msgs(nworkers);
  if (rc == FDFD_OK) {
    std::vector<std::thread> th;
    for (int t = 0; t < nworkers; ++t) {
      th.emplace_back([&, t]() {
        fdfd_handle *w = ws[t];
        int r = cuda_check(w, cudaSetDevice(w->dev), "cudaSetDevice");
        if (r == FDFD_OK) r = ensure_scratch(w, false);
        for (int q = t; q < nrhs && r == FDFD_OK; q += nworkers) {
          if ((r = h2d_field(w, b + 2 * n * q, w->vx64, mask))) break;
          if (opts->x0_given && (r = h2d_field(w, x + 2 * n * q, w->vy64, mask))) break;
          int rs = solve_dev_impl(w, w->vx64, w->vy64, opts, stats ? stats + q : nullptr);
          if (rs && rs != FDFD_ERR_NOT_CONVERGED && rs != FDFD_ERR_BREAKDOWN) { r = rs; break; }
          if ((r = d2h_field(w, w->vy64, x + 2 * n * q, mask))) break;
          if ((r = cuda_check(w, cudaStreamSynchronize(w->stream), "stream sync"))) break;
          if (rs && rcs[t] == FDFD_OK) {
            rcs[t] = rs;
            msgs[t] = w->err;
          }
        }
        if (r) {
          rcs[t] = r;
          msgs[t] = w->err;
        }
      });
    }
    for (auto &t : th) t.join();
  }
  for (auto *w : ws)
    if (w) fdfd_destroy(w);
  if (rc) return rc;
  for (int t = 0; t < nworkers; ++t)
    if (rcs[t]) return set_error(h, rcs[t], msgs[t]);
  return FDFD_OK;
}

int fdfd_solve_multi(fdfd_handle *const *hs, int32_t n, const void *const *b, void *const *x,
                     const fdfd_solve_opts *opts, fdfd_stats *stats) {
  if (!hs || !b || !x || n < 1) return set_error(nullptr, FDFD_ERR_ARG, "bad argument");
  for (int i = 0; i < n; ++i) {
    if (!hs[i] || !b[i] || !x[i]) return set_error(hs[i], FDFD_ERR_ARG, "null entry");
    if (hs[i]->dev != hs[0]->dev) return set_error(hs[0], FDFD_ERR_UNSUPPORTED, "systems on different devices");
    const int rc = check_opts(hs[i], opts);
    if (rc) return rc;
  }
  FDFD_SET_DEVICE(hs[0]);
  for (int i = 0; i < n; ++i) {
    const int rc = cuda_check(hs[i], cudaStreamSynchronize(hs[i]->stream), "stream sync");
    if (rc) return rc;
  }
  // one worker per entry: its own stream, scalars and Krylov workspace over
  // the shared operator data (entries may name the same handle)
  int rc = FDFD_OK;
  std::vector<fdfd_handle *> ws(n, nullptr);
  for (int i = 0; i < n && rc == FDFD_OK; ++i) ws[i] = make_worker(hs[i], &rc);
  std::vector<fdfd_stats> tmp(n);
  std::string msg;
  if (rc == FDFD_OK) {
    rc = solve_multi_impl(ws.data(), n, reinterpret_cast<const double2 *const *>(b),
                          reinterpret_cast<double2 *const *>(x), opts, stats ? stats : tmp.data());
    if (rc)
      for (auto *w : ws)
        if (w && !w->err.empty()) {
          msg = w->err;
          break;
        }
  }
  for (auto *w : ws)
    if (w) fdfd_destroy(w);
  if (rc) return set_error(hs[0], rc, msg.empty() ? std::string("multi-system solve failed") : msg);
  return FDFD_OK;
}

int fdfd_eps_grad_dev(fdfd_handle *h, const void *e, const void *g, void *lam, double *grad,
                      const fdfd_solve_opts *opts, fdfd_stats *stats) {
  if (!h || !e || !g || !lam || !grad) return set_error(h, FDFD_ERR_ARG, "null argument");
  int rc = check_opts(h, opts);
  if (rc) return rc;
  if (opts->method == FDFD_COCG) return set_error(h, FDFD_ERR_UNSUPPORTED, "the adjoint solve uses BiCGSTAB or BiCGStab(l)");
  if (h->ft != FDFD_EE) return set_error(h, FDFD_ERR_UNSUPPORTED, "the ε gradient is for the E formulation");
  if (!transpose_ok(h)) return set_error(h, FDFD_ERR_UNSUPPORTED, "adjoint with a Bloch phase");
  FDFD_SET_DEVICE(h);
  rc = eps_grad_dev_impl(h, (const double2 *)e, (const double2 *)g, (double2 *)lam, grad, opts, stats);
  if (rc) return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

int fdfd_eps_grad(fdfd_handle *h, const double *e, const double *g, double *grad, const fdfd_solve_opts *opts,
                  fdfd_stats *stats) {
  if (!h || !e || !g || !grad) return set_error(h, FDFD_ERR_ARG, "null argument");
  int rc = check_opts(h, opts);
  if (rc) return rc;
  if (opts->method == FDFD_COCG) return set_error(h, FDFD_ERR_UNSUPPORTED, "the adjoint solve uses BiCGSTAB or BiCGStab(l)");
  if (h->ft != FDFD_EE) return set_error(h, FDFD_ERR_UNSUPPORTED, "the ε gradient is for the E formulation");
  if (!transpose_ok(h)) return set_error(h, FDFD_ERR_UNSUPPORTED, "adjoint with a Bloch phase");
  FDFD_SET_DEVICE(h);
  if ((rc = ensure_scratch(h, false))) return rc;
  const long long n = 3 * h->ncell;
  if (!h->ve64 && dev_malloc(&h->ve64, n * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    h->ve64 = nullptr;
    return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(adjoint scratch) failed");
  }
  const int mask = field_mask(h, false);
  if ((rc = h2d_field(h, e, h->ve64, mask))) return rc;
  if ((rc = h2d_field(h, g, h->vx64, mask))) return rc;
  // λ → vy64; the gradient overwrites g's buffer (g is consumed by the solve)
  double *dgrad = reinterpret_cast<double *>(h->vx64);
  rc = eps_grad_dev_impl(h, h->ve64, h->vx64, h->vy64, dgrad, opts, stats);
  if (rc) return rc;
  if ((rc = d2h_real(h, dgrad, grad, mask))) return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

static int ensure_ve(fdfd_handle *h) {
  if (h->ve64) return FDFD_OK;
  if (dev_malloc(&h->ve64, 3 * (size_t)h->ncell * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    h->ve64 = nullptr;
    return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(field scratch) failed");
  }
  return FDFD_OK;
}

int fdfd_h_from_e_dev(fdfd_handle *h, const void *e, const void *jm, void *hout) {
  if (!h || !e || !hout) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  return h_from_e_dev_impl(h, (const double2 *)e, (const double2 *)jm, (double2 *)hout);
}

int fdfd_h_from_e(fdfd_handle *h, const double *e, const double *jm, double *hout) {
  if (!h || !e || !hout) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  int rc = ensure_scratch(h, false);
  if (!rc && jm) rc = ensure_ve(h);
  if (rc) return rc;
  if ((rc = h2d_field(h, e, h->vx64, field_mask(h, false)))) return rc;
  if (jm && (rc = h2d_field(h, jm, h->ve64, field_mask(h, true)))) return rc;
  if ((rc = h_from_e_dev_impl(h, h->vx64, jm ? h->ve64 : nullptr, h->vy64))) return rc;
  if ((rc = d2h_field(h, h->vy64, hout, field_mask(h, true)))) return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

int fdfd_e_from_h_dev(fdfd_handle *h, const void *hin, const void *je, void *eout) {
  if (!h || !hin || !eout) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  return e_from_h_dev_impl(h, (const double2 *)hin, (const double2 *)je, (double2 *)eout);
}

int fdfd_e_from_h(fdfd_handle *h, const double *hin, const double *je, double *eout) {
  if (!h || !hin || !eout) return set_error(h, FDFD_ERR_ARG, "null argument");
  if (h->has_off)
    return set_error(h, FDFD_ERR_UNSUPPORTED, "e_from_h needs a diagonal ε (Pε \\ …), as in the reference");
  FDFD_SET_DEVICE(h);
  int rc = ensure_scratch(h, false);
  if (!rc && je) rc = ensure_ve(h);
  if (rc) return rc;
  if ((rc = h2d_field(h, hin, h->vx64, field_mask(h, true)))) return rc;
  if (je && (rc = h2d_field(h, je, h->ve64, field_mask(h, false)))) return rc;
  if ((rc = e_from_h_dev_impl(h, h->vx64, je ? h->ve64 : nullptr, h->vy64))) return rc;
  if ((rc = d2h_field(h, h->vy64, eout, field_mask(h, false)))) return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

int fdfd_corner_mean_dev(fdfd_handle *h, int32_t field, const void *in, void *out) {
  if (!h || !in || !out) return set_error(h, FDFD_ERR_ARG, "null argument");
  if (field != FDFD_EE && field != FDFD_HH) return set_error(h, FDFD_ERR_ARG, "field must be FDFD_EE or FDFD_HH");
  FDFD_SET_DEVICE(h);
  return corner_mean_dev_impl(h, field == FDFD_HH, (const double2 *)in, (double2 *)out);
}

int fdfd_corner_mean(fdfd_handle *h, int32_t field, const double *in, double *out) {
  if (!h || !in || !out) return set_error(h, FDFD_ERR_ARG, "null argument");
  if (field != FDFD_EE && field != FDFD_HH) return set_error(h, FDFD_ERR_ARG, "field must be FDFD_EE or FDFD_HH");
  FDFD_SET_DEVICE(h);
  int rc = ensure_scratch(h, false);
  if (rc) return rc;
  const int mask = field_mask(h, field == FDFD_HH);
  if ((rc = h2d_field(h, in, h->vx64, mask))) return rc;
  if ((rc = corner_mean_dev_impl(h, field == FDFD_HH, h->vx64, h->vy64))) return rc;
  if ((rc = d2h_field(h, h->vy64, out, mask))) return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

int fdfd_set_field_type(fdfd_handle *h, int32_t ft) {
  if (!h) return set_error(h, FDFD_ERR_ARG, "null handle");
  if (ft != FDFD_EE && ft != FDFD_HH) return set_error(h, FDFD_ERR_ARG, "field type must be FDFD_EE or FDFD_HH");
  if (ft == FDFD_HH && h->has_off)
    return set_error(h, FDFD_ERR_UNSUPPORTED, "the H formulation needs a diagonal ε (Pε \\ Cₘ)");
  h->ft = ft;
  fdfd::drop_graphs(h);
  return FDFD_OK;
}

int fdfd_design_grad_dev(fdfd_handle *h, const double *grad, double *dgrad) {
  if (!h || !grad || !dgrad) return set_error(h, FDFD_ERR_ARG, "null argument");
  FDFD_SET_DEVICE(h);
  int rc = design_grad_dev_impl(h, grad, dgrad);
  if (rc) return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

int fdfd_design_grad(fdfd_handle *h, const double *grad, double *dgrad) {
  if (!h || !grad || !dgrad) return set_error(h, FDFD_ERR_ARG, "null argument");
  if (!h->has_design) return set_error(h, FDFD_ERR_ARG, "no design region (set one with fdfd_smooth_objects)");
  FDFD_SET_DEVICE(h);
  int rc = ensure_scratch(h, false);
  if (rc) return rc;
  const long long n = 3 * h->ncell;
  long long ne = 1;
  for (int a = 0; a < 3; ++a) ne *= h->design_hi[a] - h->design_lo[a];
  double *dg = reinterpret_cast<double *>(h->vx64);
  double *dout = reinterpret_cast<double *>(h->vy64);
  if ((rc = cuda_check(h, cudaMemcpyAsync(dg, grad, n * sizeof(double), cudaMemcpyHostToDevice, h->stream),
                       "H2D grad")))
    return rc;
  if ((rc = design_grad_dev_impl(h, dg, dout))) return rc;
  if ((rc = cuda_check(h, cudaMemcpyAsync(dgrad, dout, ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
                       "D2H design grad")))
    return rc;
  return cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
}

}  // extern "C"
