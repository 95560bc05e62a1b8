// On-device material assignment and Kottke subpixel smoothing.
//
// Replaces calc_matparams! (src/model/full.jl:16-70): assign_param! finds
// the object index (oind) at every sample point, smooth_param! re-computes
// ε on voxels whose corners see more than one object.  The dual-voxel trick
// of the reference is kept: the voxel around an E_w sample has its corners
// on H_w sample points, so ε_ww smoothing reads the object indices sampled at
// H_w positions (full.jl:58-60, 64); the voxel around an E-voxel corner (where
// the off-diagonal ε lives) has its corners at cell centres (full.jl:61, 65).
//
// Rules (shared with the CPU oracle):
//   * objects are applied in add_obj! order with atomicMax on the index, so
//     the last-added object wins; index 0 is the background;
//   * ghost samples: Bloch axes copy the periodic image, a symmetry (PEC)
//     axis copies dual index 0 into the dual ghost and evaluates the primal
//     ghost on the boundary plane;
//   * a voxel with exactly two objects gets ε̃ = ⟨ε⁻¹⟩⁻¹ P + ⟨ε⟩ (I − P),
//     P = n nᵀ, with n the outward normal of the higher-priority object at
//     its point nearest the voxel centre and the fill fraction the exact
//     volume of the voxel behind that tangent plane; more than two objects:
//     mean of the corner ε (off-diagonal 0);
//   * a design region (per-cell ε) overrides: ε_ww = mean of the 4 cells
//     around the E_w edge, off-diagonals 0 at corners touching the region.
// This file is compiled with --fmad=false: every product and sum rounds
// exactly as in the oracle, so object indices and masks are bit-identical.
#include <algorithm>
#include <vector>

#include "fdfd_internal.cuh"

namespace fdfd {

int finish_eps(fdfd_handle *h);

struct DevObj {
  int kind;
  double eps;
  double p[6];
};

struct Axes {
  const double *pos[3];  // (N+1) sample positions per axis for this sample set
  int n[3];              // extents of the array being indexed
};

__device__ __forceinline__ bool inside(const DevObj &o, double x, double y, double z) {
  if (o.kind == FDFD_SHAPE_SPHERE) {
    const double dx = __dsub_rn(x, o.p[0]), dy = __dsub_rn(y, o.p[1]), dz = __dsub_rn(z, o.p[2]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return d2 <= __dmul_rn(o.p[3], o.p[3]);
  }
  if (o.kind == FDFD_SHAPE_CYLZ) {
    const double dx = __dsub_rn(x, o.p[0]), dy = __dsub_rn(y, o.p[1]);
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) <= __dmul_rn(o.p[2], o.p[2]);
  }
  return x >= o.p[0] && x <= o.p[3] && y >= o.p[1] && y <= o.p[4] && z >= o.p[2] && z <= o.p[5];
}

// oind over index boxes: blockIdx.y = object, threads stride over its box
__global__ void k_assign(int *oind, Axes ax, const DevObj *objs, const int *boxes) {
  const int q = blockIdx.y;
  const DevObj o = objs[q];
  const int *b = boxes + 6 * q;  // lo0, lo1, lo2, hi0, hi1, hi2 (inclusive lo, exclusive hi)
  const int e0 = b[3] - b[0], e1 = b[4] - b[1], e2 = b[5] - b[2];
  if (e0 <= 0 || e1 <= 0 || e2 <= 0) return;
  const long long vol = (long long)e0 * e1 * e2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < vol;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = b[0] + (int)(t % e0), j = b[1] + (int)((t / e0) % e1), k = b[2] + (int)(t / ((long long)e0 * e1));
    if (inside(o, ax.pos[0][i], ax.pos[1][j], ax.pos[2][k])) {
      atomicMax(&oind[i + (long long)ax.n[0] * (j + (long long)ax.n[1] * k)], q + 1);
    }
  }
}

// copy plane src → dst along axis w of an (n0,n1,n2) int array
__global__ void k_copy_plane(int *a, int n0, int n1, int n2, int w, int dst, int src) {
  const int m0 = (w == 0) ? n1 : n0, m1 = (w == 2) ? n1 : n2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)m0 * m1;
       t += (long long)gridDim.x * blockDim.x) {
    const int u = (int)(t % m0), v = (int)(t / m0);
    int id[3], is[3];
    if (w == 0) { id[0] = dst; is[0] = src; id[1] = is[1] = u; id[2] = is[2] = v; }
    else if (w == 1) { id[1] = dst; is[1] = src; id[0] = is[0] = u; id[2] = is[2] = v; }
    else { id[2] = dst; is[2] = src; id[0] = is[0] = u; id[1] = is[1] = v; }
    a[id[0] + (long long)n0 * (id[1] + (long long)n1 * id[2])] = a[is[0] + (long long)n0 * (is[1] + (long long)n1 * is[2])];
  }
}

// ------------------------------------------------------------ Kottke
__device__ double sz_volume(double m1, double m2, double m3, double a) {
  const double m12 = m1 + m2;
  if (a < m1) {
    const double t = a / m1;
    return ((t * a) * a) / ((6.0 * m2) * m3);
  }
  if (a < m2) return (a * (a - m1)) / ((2.0 * m2) * m3) + (m1 * m1) / ((6.0 * m2) * m3);
  if (a < fmin(m12, m3)) {
    const double q = a - m2;
    const double base = ((((3.0 * a) * a) - ((3.0 * a) * m1)) + (m1 * m1)) / ((6.0 * m2) * m3);
    return base - ((((q / m1) * q) * q) / ((6.0 * m2) * m3));
  }
  if (m3 < m12) {
    const double q2 = a - m2, q3 = a - m3;
    const double base = ((((3.0 * a) * a) - ((3.0 * a) * m1)) + (m1 * m1)) / ((6.0 * m2) * m3);
    return base - (((((q2 / m1) * q2) * q2) + (((q3 / m1) * q3) * q3)) / ((6.0 * m2) * m3));
  }
  return ((2.0 * a) - m12) / (2.0 * m3);
}

__device__ double volfrac_plane(const double lo[3], const double hi[3], const double n[3], const double r0[3]) {
  double m[3];
  double d = 0.0;
  for (int a = 0; a < 3; ++a) {
    const double side = hi[a] - lo[a];
    double ma = n[a] * side;
    d += n[a] * (r0[a] - lo[a]);
    if (ma < 0.0) {
      d -= ma;
      ma = -ma;
    }
    m[a] = ma;
  }
  const double s = (m[0] + m[1]) + m[2];
  if (s <= 0.0) return 0.5;
  double alpha = d / s;
  if (alpha <= 0.0) return 0.0;
  if (alpha >= 1.0) return 1.0;
  double v0 = m[0] / s, v1 = m[1] / s, v2 = m[2] / s;
  // ascending sort of three
  if (v0 > v1) { double t = v0; v0 = v1; v1 = t; }
  if (v1 > v2) { double t = v1; v1 = v2; v2 = t; }
  if (v0 > v1) { double t = v0; v0 = v1; v1 = t; }
  const double tiny = 1e-12;
  if (v0 < tiny * v2) v0 = 0.0;
  if (v1 < tiny * v2) v1 = 0.0;
  const bool flip = alpha > 0.5;
  if (flip) alpha = 1.0 - alpha;
  const double v = sz_volume(v0, v1, v2, alpha);
  return flip ? 1.0 - v : v;
}

__device__ void normal_point(const DevObj &o, const double xc[3], double n[3], double r0[3]) {
  if (o.kind == FDFD_SHAPE_SPHERE) {
    const double v0 = xc[0] - o.p[0], v1 = xc[1] - o.p[1], v2 = xc[2] - o.p[2];
    const double nr = sqrt((v0 * v0 + v1 * v1) + v2 * v2);
    if (nr == 0.0) { n[0] = 1.0; n[1] = 0.0; n[2] = 0.0; }
    else { n[0] = v0 / nr; n[1] = v1 / nr; n[2] = v2 / nr; }
    for (int a = 0; a < 3; ++a) r0[a] = o.p[a] + o.p[3] * n[a];
    return;
  }
  if (o.kind == FDFD_SHAPE_CYLZ) {
    // radial in the xy-plane (the disk's normal); z follows the point
    const double v0 = xc[0] - o.p[0], v1 = xc[1] - o.p[1], v2 = 0.0;
    const double nr = sqrt((v0 * v0 + v1 * v1) + v2 * v2);
    if (nr == 0.0) { n[0] = 1.0; n[1] = 0.0; n[2] = 0.0; }
    else { n[0] = v0 / nr; n[1] = v1 / nr; n[2] = 0.0; }
    r0[0] = o.p[0] + o.p[2] * n[0];
    r0[1] = o.p[1] + o.p[2] * n[1];
    r0[2] = xc[2];
    return;
  }
  double best = -INFINITY;
  for (int a = 0; a < 3; ++a) {
    for (int side = 0; side < 2; ++side) {
      const double dist = side == 0 ? (o.p[a] - xc[a]) : (xc[a] - o.p[3 + a]);
      if (dist > best) {
        best = dist;
        for (int b = 0; b < 3; ++b) { n[b] = 0.0; r0[b] = xc[b]; }
        n[a] = side == 0 ? -1.0 : 1.0;
        r0[a] = side == 0 ? o.p[a] : o.p[3 + a];
      }
    }
  }
}

__device__ __forceinline__ double obj_eps(const DevObj *objs, double eps_bg, int q) {
  return q == 0 ? eps_bg : objs[q - 1].eps;
}

// Kottke tensor of a voxel [lo, hi] whose 8 corner indices are c[]; returns
// the number of distinct objects (1, 2 or more) and fills T (row-major 3×3).
__device__ int smoothed_tensor(const int c[8], const DevObj *objs, double eps_bg, const double lo[3],
                               const double hi[3], double T[9]) {
  int qmin = c[0], qmax = c[0];
  for (int t = 1; t < 8; ++t) { qmin = min(qmin, c[t]); qmax = max(qmax, c[t]); }
  int ndist = 1;
  {
    int seen[8];
    int ns = 0;
    for (int t = 0; t < 8; ++t) {
      bool f = false;
      for (int u = 0; u < ns; ++u) f = f || (seen[u] == c[t]);
      if (!f) seen[ns++] = c[t];
    }
    ndist = ns;
  }
  for (int t = 0; t < 9; ++t) T[t] = 0.0;
  if (ndist == 2) {
    const double efg = obj_eps(objs, eps_bg, qmax), ebg = obj_eps(objs, eps_bg, qmin);
    double xc[3], n[3], r0[3];
    for (int a = 0; a < 3; ++a) xc[a] = 0.5 * (lo[a] + hi[a]);
    normal_point(objs[qmax - 1], xc, n, r0);
    const double f = volfrac_plane(lo, hi, n, r0);
    const double em = f * efg + (1.0 - f) * ebg;
    const double eh = 1.0 / (f / efg + (1.0 - f) / ebg);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) T[3 * a + b] = (a == b ? em : 0.0) + (eh - em) * (n[a] * n[b]);
  } else if (ndist > 2) {
    double s = 0.0;
    for (int t = 0; t < 8; ++t) s += obj_eps(objs, eps_bg, c[t]);
    const double mean = s / 8.0;
    T[0] = T[4] = T[8] = mean;
  }
  return ndist;
}

// corner order matches the oracle's ravel of o[i:i+2, j:j+2, k:k+2]
__device__ __forceinline__ void corners8(const int *o, int n0, int n1, int i, int j, int k, int c[8]) {
  int t = 0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) c[t++] = o[(i + a) + (long long)n0 * ((j + b) + (long long)n1 * (k + d))];
}

// ε_ww at E_w samples
__global__ void k_smooth_diag(int w, int N0, int N1, int N2, const int *oe, const int *oh, Axes hax,
                              const DevObj *objs, double eps_bg, double *eps, uint8_t *smask) {
  const long long nc = (long long)N0 * N1 * N2;
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(cell % N0), j = (int)((cell / N0) % N1), k = (int)(cell / ((long long)N0 * N1));
    int c[8];
    corners8(oh, N0 + 1, N1 + 1, i, j, k, c);
    bool same = true;
    for (int t = 1; t < 8; ++t) same = same && (c[t] == c[0]);
    if (same) {
      eps[w * nc + cell] = obj_eps(objs, eps_bg, oe[cell]);
      smask[4 * cell + w] = 0;
      continue;
    }
    const double lo[3] = {hax.pos[0][i], hax.pos[1][j], hax.pos[2][k]};
    const double hi[3] = {hax.pos[0][i + 1], hax.pos[1][j + 1], hax.pos[2][k + 1]};
    double T[9];
    smoothed_tensor(c, objs, eps_bg, lo, hi, T);
    eps[w * nc + cell] = T[4 * w];
    smask[4 * cell + w] = 1;
  }
}

// off-diagonal ε at E-voxel corners (voxel corners at cell centres)
__global__ void k_smooth_off(int N0, int N1, int N2, const int *oc, Axes cax, const DevObj *objs, double eps_bg,
                             double *eoff, uint8_t *smask, unsigned int *nnz) {
  const long long nc = (long long)N0 * N1 * N2;
  unsigned int cnt = 0;
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(cell % N0), j = (int)((cell / N0) % N1), k = (int)(cell / ((long long)N0 * N1));
    int c[8];
    corners8(oc, N0 + 1, N1 + 1, i, j, k, c);
    bool same = true;
    for (int t = 1; t < 8; ++t) same = same && (c[t] == c[0]);
    if (same) {
      eoff[cell] = eoff[nc + cell] = eoff[2 * nc + cell] = 0.0;
      smask[4 * cell + 3] = 0;
      continue;
    }
    const double lo[3] = {cax.pos[0][i], cax.pos[1][j], cax.pos[2][k]};
    const double hi[3] = {cax.pos[0][i + 1], cax.pos[1][j + 1], cax.pos[2][k + 1]};
    double T[9];
    smoothed_tensor(c, objs, eps_bg, lo, hi, T);
    eoff[cell] = T[1];
    eoff[nc + cell] = T[5];
    eoff[2 * nc + cell] = T[6];
    smask[4 * cell + 3] = 1;
    cnt += (T[1] != 0.0 || T[5] != 0.0 || T[6] != 0.0);
  }
  if (cnt) atomicAdd(nnz, cnt);
}

__device__ __forceinline__ int wrap_or_clamp(int t, int N, int bloch) {
  if (t < 0) return bloch ? t + N : 0;
  if (t >= N) return bloch ? t - N : N - 1;
  return t;
}

struct DesignDev {
  int lo[3], hi[3];
  const double *eps;  // x fastest over the region
  int bloch[3];
};

__device__ __forceinline__ bool in_region(const DesignDev &d, int i, int j, int k) {
  return i >= d.lo[0] && i < d.hi[0] && j >= d.lo[1] && j < d.hi[1] && k >= d.lo[2] && k < d.hi[2];
}

__device__ __forceinline__ double cell_value(const DesignDev &d, const int *oc, int N0, int N1, const DevObj *objs,
                                             double eps_bg, int i, int j, int k) {
  if (in_region(d, i, j, k)) {
    const int e0 = d.hi[0] - d.lo[0], e1 = d.hi[1] - d.lo[1];
    return d.eps[(i - d.lo[0]) + (long long)e0 * ((j - d.lo[1]) + (long long)e1 * (k - d.lo[2]))];
  }
  // cell centre = dual ext index + 1 on every axis
  return obj_eps(objs, eps_bg, oc[(i + 1) + (long long)(N0 + 1) * ((j + 1) + (long long)(N1 + 1) * (k + 1))]);
}

__global__ void k_design_diag(int w, int N0, int N1, int N2, DesignDev d, const int *oc, const DevObj *objs,
                              double eps_bg, double *eps, uint8_t *smask) {
  const long long nc = (long long)N0 * N1 * N2;
  const int N[3] = {N0, N1, N2};
  const int u0 = (w == 0) ? 1 : 0, u1 = (w == 2) ? 1 : 2;
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int g[3] = {(int)(cell % N0), (int)((cell / N0) % N1), (int)(cell / ((long long)N0 * N1))};
    double acc = 0.0;
    bool touch = false;
    for (int s0 = -1; s0 <= 0; ++s0)
      for (int s1 = -1; s1 <= 0; ++s1) {
        int t[3] = {g[0], g[1], g[2]};
        t[u0] = wrap_or_clamp(g[u0] + s0, N[u0], d.bloch[u0]);
        t[u1] = wrap_or_clamp(g[u1] + s1, N[u1], d.bloch[u1]);
        acc += cell_value(d, oc, N0, N1, objs, eps_bg, t[0], t[1], t[2]);
        touch = touch || in_region(d, t[0], t[1], t[2]);
      }
    if (touch) {
      eps[w * nc + cell] = 0.25 * acc;
      smask[4 * cell + w] = 2;
    }
  }
}

__global__ void k_design_off(int N0, int N1, int N2, DesignDev d, double *eoff, uint8_t *smask) {
  const long long nc = (long long)N0 * N1 * N2;
  const int N[3] = {N0, N1, N2};
  for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < nc;
       cell += (long long)gridDim.x * blockDim.x) {
    const int g[3] = {(int)(cell % N0), (int)((cell / N0) % N1), (int)(cell / ((long long)N0 * N1))};
    bool touch = false;
    for (int s = 0; s < 8; ++s) {
      int t[3];
      for (int a = 0; a < 3; ++a) t[a] = wrap_or_clamp(g[a] - ((s >> (2 - a)) & 1), N[a], d.bloch[a]);
      touch = touch || in_region(d, t[0], t[1], t[2]);
    }
    if (touch) {
      eoff[cell] = eoff[nc + cell] = eoff[2 * nc + cell] = 0.0;
      smask[4 * cell + 3] = 2;
    }
  }
}

// ------------------------------------------------------------ host
namespace {
struct DevBuf {
  std::vector<void *> ptrs;
  ~DevBuf() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <typename T> T *get(fdfd_handle *h, size_t n, int *rc) {
    void *p = nullptr;
    if (dev_malloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      *rc = set_error(h, FDFD_ERR_NOMEM, "cudaMalloc in fdfd_smooth_objects failed");
      return nullptr;
    }
    ptrs.push_back(p);
    return (T *)p;
  }
};

// index range [first, last] of sorted positions within [a - tiny, b + tiny]
void index_range(const std::vector<double> &pos, double a, double b, int *lo, int *hi) {
  const double pad = 1e-9 * (1.0 + std::fabs(a) + std::fabs(b));
  *lo = (int)(std::lower_bound(pos.begin(), pos.end(), a - pad) - pos.begin());
  *hi = (int)(std::upper_bound(pos.begin(), pos.end(), b + pad) - pos.begin());
}
}  // namespace

int smooth_objects_impl(fdfd_handle *h, const double *const lprim[3], const fdfd_object *objs, int nobj,
                        double eps_bg, const fdfd_design *design) {
  const int N0 = h->N[0], N1 = h->N[1], N2 = h->N[2];
  const long long nc = h->ncell;
  const long long next = (long long)(N0 + 1) * (N1 + 1) * (N2 + 1);
  int rc = FDFD_OK;
  // per-axis positions: primal with +end ghost (N+1), dual with −end ghost (N+1)
  std::vector<double> prim[3], dual[3];
  for (int w = 0; w < 3; ++w) {
    const int N = h->N[w];
    prim[w].assign(lprim[w], lprim[w] + N + 1);
    for (int i = 0; i < N; ++i)
      if (!(prim[w][i + 1] > prim[w][i])) return set_error(h, FDFD_ERR_ARG, "lprim must be strictly increasing");
    const double L = prim[w][N] - prim[w][0];
    std::vector<double> mid(N);
    for (int i = 0; i < N; ++i) mid[i] = 0.5 * (prim[w][i] + prim[w][i + 1]);
    const double g = h->bloch[w] ? mid[N - 1] - L : 2.0 * prim[w][0] - mid[0];
    dual[w].resize(N + 1);
    dual[w][0] = g;
    for (int i = 0; i < N; ++i) dual[w][i + 1] = mid[i];
  }
  for (int q = 0; q < nobj; ++q) {
    if (objs[q].kind != FDFD_SHAPE_SPHERE && objs[q].kind != FDFD_SHAPE_BOX && objs[q].kind != FDFD_SHAPE_CYLZ)
      return set_error(h, FDFD_ERR_ARG, "unknown shape kind");
    if (!(objs[q].eps > 0.0)) return set_error(h, FDFD_ERR_UNSUPPORTED, "object ε must be real and positive");
  }
  if (!(eps_bg > 0.0)) return set_error(h, FDFD_ERR_UNSUPPORTED, "background ε must be real and positive");
  if (design) {
    for (int a = 0; a < 3; ++a)
      if (design->lo[a] < 0 || design->hi[a] > h->N[a] || design->lo[a] >= design->hi[a] || !design->eps_cells)
        return set_error(h, FDFD_ERR_ARG, "bad design region");
  }
  DevBuf buf;
  double *dprim[3], *ddual[3];
  for (int w = 0; w < 3; ++w) {
    dprim[w] = buf.get<double>(h, prim[w].size(), &rc);
    ddual[w] = buf.get<double>(h, dual[w].size(), &rc);
    if (rc) return rc;
    cudaMemcpy(dprim[w], prim[w].data(), prim[w].size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(ddual[w], dual[w].data(), dual[w].size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  std::vector<DevObj> hob(std::max(1, nobj));
  for (int q = 0; q < nobj; ++q) {
    hob[q].kind = objs[q].kind;
    hob[q].eps = objs[q].eps;
    for (int t = 0; t < 6; ++t) hob[q].p[t] = objs[q].p[t];
  }
  DevObj *dobj = buf.get<DevObj>(h, hob.size(), &rc);
  int *dbox = buf.get<int>(h, 6 * hob.size(), &rc);
  // oind arrays: H_w (3, ext), cell centres (ext), E_w (3, N³ sample positions)
  int *oh[3], *oe[3];
  for (int w = 0; w < 3; ++w) {
    oh[w] = buf.get<int>(h, next, &rc);
    oe[w] = buf.get<int>(h, nc, &rc);
  }
  int *oc = buf.get<int>(h, next, &rc);
  unsigned int *dnnz = buf.get<unsigned int>(h, 1, &rc);
  if (!h->smask) {
    if (dev_malloc(&h->smask, 4 * (size_t)nc) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(smask) failed");
    }
  }
  if (!h->eoff64) {
    if (dev_malloc(&h->eoff64, 3 * nc * sizeof(double)) != cudaSuccess ||
        dev_malloc(&h->eoff32, 3 * nc * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(eps off-diagonal) failed");
    }
  }
  if (rc) return rc;
  cudaMemcpy(dobj, hob.data(), hob.size() * sizeof(DevObj), cudaMemcpyHostToDevice);
  cudaStream_t st = h->stream;

  // Assign one sample set: types[w] = 0 primal (positions prim), 1 dual (dual);
  // ext = true: (N+1)³ with ghosts; false: the N³ E sample positions, which
  // are the ext positions offset by one along the dual axes.
  auto assign = [&](int *o, const int types[3], bool ext) -> int {
    Axes ax;
    std::vector<const std::vector<double> *> hpos(3);
    for (int w = 0; w < 3; ++w) {
      const bool du = types[w] == 1;
      const double *base = du ? ddual[w] : dprim[w];
      ax.pos[w] = (!ext && du) ? base + 1 : base;
      ax.n[w] = ext ? h->N[w] + 1 : h->N[w];
      hpos[w] = du ? &dual[w] : &prim[w];
    }
    const long long total = (long long)ax.n[0] * ax.n[1] * ax.n[2];
    cudaMemsetAsync(o, 0, total * sizeof(int), st);
    if (nobj > 0) {
      std::vector<int> boxes(6 * nobj);
      for (int q = 0; q < nobj; ++q) {
        double a[3], b[3];
        if (objs[q].kind == FDFD_SHAPE_SPHERE)
          for (int w = 0; w < 3; ++w) { a[w] = objs[q].p[w] - objs[q].p[3]; b[w] = objs[q].p[w] + objs[q].p[3]; }
        else if (objs[q].kind == FDFD_SHAPE_CYLZ) {
          for (int w = 0; w < 2; ++w) { a[w] = objs[q].p[w] - objs[q].p[2]; b[w] = objs[q].p[w] + objs[q].p[2]; }
          a[2] = -HUGE_VAL;
          b[2] = HUGE_VAL;
        } else
          for (int w = 0; w < 3; ++w) { a[w] = objs[q].p[w]; b[w] = objs[q].p[3 + w]; }
        for (int w = 0; w < 3; ++w) {
          std::vector<double> pw(hpos[w]->begin() + ((!ext && types[w] == 1) ? 1 : 0),
                                 hpos[w]->begin() + ((!ext && types[w] == 1) ? 1 : 0) + ax.n[w]);
          int lo, hi;
          index_range(pw, a[w], b[w], &lo, &hi);
          boxes[6 * q + w] = lo;
          boxes[6 * q + 3 + w] = hi;
        }
      }
      cudaMemcpyAsync(dbox, boxes.data(), boxes.size() * sizeof(int), cudaMemcpyHostToDevice, st);
      cudaStreamSynchronize(st);
      dim3 grid(64, nobj);
      k_assign<<<grid, 256, 0, st>>>(o, ax, dobj, dbox);
      int e = cuda_check(h, cudaGetLastError(), "k_assign");
      if (e) return e;
    }
    if (ext) {
      for (int w = 0; w < 3; ++w) {
        const int N = h->N[w];
        if (types[w] == 0) {
          if (h->bloch[w]) k_copy_plane<<<152, 256, 0, st>>>(o, N0 + 1, N1 + 1, N2 + 1, w, N, 0);
        } else {
          k_copy_plane<<<152, 256, 0, st>>>(o, N0 + 1, N1 + 1, N2 + 1, w, 0, h->bloch[w] ? N : 1);
        }
      }
    }
    return cuda_check(h, cudaGetLastError(), "k_copy_plane");
  };

  for (int w = 0; w < 3; ++w) {
    int te[3], th[3];
    for (int a = 0; a < 3; ++a) {
      te[a] = (a == w) ? 1 : 0;
      th[a] = (a == w) ? 0 : 1;
    }
    if ((rc = assign(oe[w], te, false))) return rc;
    if ((rc = assign(oh[w], th, true))) return rc;
  }
  {
    const int tc[3] = {1, 1, 1};
    if ((rc = assign(oc, tc, true))) return rc;
  }
  cudaMemsetAsync(dnnz, 0, sizeof(unsigned int), st);
  for (int w = 0; w < 3; ++w) {
    Axes hax;
    for (int a = 0; a < 3; ++a) {
      hax.pos[a] = (a == w) ? dprim[a] : ddual[a];
      hax.n[a] = h->N[a] + 1;
    }
    k_smooth_diag<<<152 * 8, 256, 0, st>>>(w, N0, N1, N2, oe[w], oh[w], hax, dobj, eps_bg, h->eps64, h->smask);
  }
  {
    Axes cax;
    for (int a = 0; a < 3; ++a) {
      cax.pos[a] = ddual[a];
      cax.n[a] = h->N[a] + 1;
    }
    k_smooth_off<<<152 * 8, 256, 0, st>>>(N0, N1, N2, oc, cax, dobj, eps_bg, h->eoff64, h->smask, dnnz);
  }
  if ((rc = cuda_check(h, cudaGetLastError(), "smoothing kernels"))) return rc;
  h->has_design = design != nullptr;
  if (design) {
    for (int a = 0; a < 3; ++a) {
      h->design_lo[a] = design->lo[a];
      h->design_hi[a] = design->hi[a];
    }
    DesignDev dd;
    const long long ne = (long long)(design->hi[0] - design->lo[0]) * (design->hi[1] - design->lo[1]) *
                         (design->hi[2] - design->lo[2]);
    double *deps = buf.get<double>(h, ne, &rc);
    if (rc) return rc;
    cudaMemcpy(deps, design->eps_cells, ne * sizeof(double), cudaMemcpyHostToDevice);
    for (int a = 0; a < 3; ++a) {
      dd.lo[a] = design->lo[a];
      dd.hi[a] = design->hi[a];
      dd.bloch[a] = h->bloch[a];
    }
    dd.eps = deps;
    for (int w = 0; w < 3; ++w)
      k_design_diag<<<152 * 8, 256, 0, st>>>(w, N0, N1, N2, dd, oc, dobj, eps_bg, h->eps64, h->smask);
    k_design_off<<<152 * 8, 256, 0, st>>>(N0, N1, N2, dd, h->eoff64, h->smask);
    if ((rc = cuda_check(h, cudaGetLastError(), "design kernels"))) return rc;
  }
  unsigned int nnz = 0;
  cudaMemcpyAsync(&nnz, dnnz, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
  if ((rc = cuda_check(h, cudaStreamSynchronize(st), "smoothing sync"))) return rc;
  // design zeroing can only remove off-diagonals; keep the flag conservative
  h->has_off = nnz > 0;
  return finish_eps(h);
}

}  // namespace fdfd
