// Matrix-free application of the FDFD operator
//     y = A x,  A = Cₘ·Cₑ − ω²·Pε   (μ = 1)
// which the reference assembles as a sparse matrix (create_A,
// src/model/model.jl:238-259) from create_curls (:173-188) and
// create_paramops (:154-171).
//
// Kernel design (sm_103a, HBM-bound):
//   * a CTA owns a 32×8 (x,y) tile and marches along z over a chunk of
//     planes; a 3-slot ring of E planes (with a one-cell halo) lives in
//     shared memory, so every E value is read from HBM about once;
//   * H = Cₑ E is computed once per plane for the tile plus its low halo
//     and kept for two planes (H(k-1), H(k)) in shared memory;
//   * the output y(k) = Cₘ H − ω² Pε E is formed from shared memory with
//     the per-axis 1/s∆l PML factors, the ε diagonal and — only where the
//     (tile, plane) flag says so — the corner-averaged off-diagonal ε terms;
//   * optional fused epilogues produce the dot products a Krylov step needs
//     (block partials in FP64, last-block finalisation, krylov_fin.cuh);
//   * TRANSPOSE applies Aᵀ = S·A·S⁻¹ with S = V_E (the dual volume of each
//     E sample), which holds because S·A is complex symmetric.
#include "krylov_fin.cuh"

namespace fdfd {

constexpr int EX = TX + 2, EY = TY + 2;  // E tile with halo: −1 … T
constexpr int HX = TX + 1, HY = TY + 1;  // H tile: −1 … T−1

template <typename R>
struct StencilSmem {
  using C = typename CT<R>::C;
  C e[3][3][EY][EX];  // [slot][component][jj+1][ii+1]
  C hx[2][HY][HX];
  C hy[2][HY][HX];
  C hz[HY][HX];
};

template <typename R>
struct Extra {
  using C = typename CT<R>::C;
  const C *sdle[3];   // s∆lₑ per axis (TRANSPOSE scaling)
  const C *sdlm[3];   // s∆lₘ per axis
  C ph[3], phinv[3];  // Bloch e^{-ikL} and its inverse
  int kchunk;
};

template <typename R>
__device__ __forceinline__ typename CT<R>::C vol_e(const Extra<R> &ex, int c, int g0, int g1, int g2) {
  // V_E(c) = s∆lₘ[c][g_c] · Π_{v≠c} s∆lₑ[v][g_v]
  using C = typename CT<R>::C;
  const int g[3] = {g0, g1, g2};
  C v = (c == 0) ? ex.sdlm[0][g[0]] : ex.sdle[0][g[0]];
  v = cmul(v, (c == 1) ? ex.sdlm[1][g[1]] : ex.sdle[1][g[1]]);
  v = cmul(v, (c == 2) ? ex.sdlm[2][g[2]] : ex.sdle[2][g[2]]);
  return v;
}

template <typename C>
__device__ __forceinline__ C cinv(C a) {
  auto d = a.x * a.x + a.y * a.y;
  return mk(a.x / d, -a.y / d);
}

// Value of component c of x at (possibly ghost) cell g, following the
// boundary rules: PEC (non-Bloch) — tangential E is 0 on the primal ghost
// plane N and pinned to 0 on plane 0; the normal component mirrors at −1.
// Bloch — periodic with phase e^{-ikL}.
template <typename R, bool TRANSPOSE>
__device__ __forceinline__ typename CT<R>::C load_e(const typename CT<R>::C *__restrict__ x, const OpArgs<R> &a,
                                                    const Extra<R> &ex, int gi, int gj, int gk, int c) {
  using C = typename CT<R>::C;
  int g[3] = {gi, gj, gk};
  C ph = mk(R(1), R(0));
  bool phased = false;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    if (g[v] < 0) {
      if (a.bloch[v]) { g[v] += a.N[v]; ph = cmul(ph, ex.phinv[v]); phased = true; }
      else if (v == c) g[v] = 0;
      else return czero<C>();
    } else if (g[v] >= a.N[v]) {
      if (a.bloch[v]) { g[v] -= a.N[v]; ph = cmul(ph, ex.ph[v]); phased = true; }
      else return czero<C>();
    } else if (g[v] == 0 && v != c && !a.bloch[v]) {
      return czero<C>();
    }
  }
  C val = x[c + 3 * ((long long)g[0] + (long long)a.N[0] * ((long long)g[1] + (long long)a.N[1] * g[2]))];
  if (TRANSPOSE) val = cmul(val, cinv(vol_e<R>(ex, c, g[0], g[1], g[2])));
  if (phased) val = cmul(val, ph);
  return val;
}

template <typename R, bool TRANSPOSE>
__device__ __forceinline__ typename CT<R>::C own_e(const typename CT<R>::C *__restrict__ x, const Extra<R> &ex,
                                                   long long cell, int c, int gi, int gj, int gk) {
  typename CT<R>::C v = x[3 * cell + c];
  if (TRANSPOSE) v = cmul(v, cinv(vol_e<R>(ex, c, gi, gj, gk)));
  return v;
}

template <typename R>
__device__ __forceinline__ int cidx(const OpArgs<R> &a, int v, int g) {
  // coefficient index for a (possibly ghost) H/E position along axis v
  if (g < 0) return a.bloch[v] ? a.N[v] - 1 : 0;
  if (g >= a.N[v]) return a.bloch[v] ? g - a.N[v] : a.N[v] - 1;
  return g;
}

template <typename R, bool TRANSPOSE>
__device__ __forceinline__ void load_plane(StencilSmem<R> &S, const OpArgs<R> &a, const Extra<R> &ex,
                                           const typename CT<R>::C *__restrict__ x, int i0, int j0, int k, int slot,
                                           int tid) {
  for (int p = tid; p < EX * EY; p += NTHR) {
    const int ii = p % EX - 1, jj = p / EX - 1;
    const int gi = i0 + ii, gj = j0 + jj;
#pragma unroll
    for (int c = 0; c < 3; ++c) S.e[slot][c][jj + 1][ii + 1] = load_e<R, TRANSPOSE>(x, a, ex, gi, gj, k, c);
  }
}

// H(k) = Cₑ E over the tile positions −1 … T−1 in x and y.
template <typename R>
__device__ __forceinline__ void compute_h(StencilSmem<R> &S, const OpArgs<R> &a, int i0, int j0, int k, int sk,
                                          int sk1, int hslot, int tid) {
  using C = typename CT<R>::C;
  const C cmz = a.cm[2][cidx(a, 2, k)];
  for (int p = tid; p < HX * HY; p += NTHR) {
    const int ii = p % HX - 1, jj = p / HX - 1;
    const C cmx = a.cm[0][cidx(a, 0, i0 + ii)];
    const C cmy = a.cm[1][cidx(a, 1, j0 + jj)];
    const C ex0 = S.e[sk][0][jj + 1][ii + 1], exy = S.e[sk][0][jj + 2][ii + 1], exz = S.e[sk1][0][jj + 1][ii + 1];
    const C ey0 = S.e[sk][1][jj + 1][ii + 1], eyx = S.e[sk][1][jj + 1][ii + 2], eyz = S.e[sk1][1][jj + 1][ii + 1];
    const C ez0 = S.e[sk][2][jj + 1][ii + 1], ezx = S.e[sk][2][jj + 1][ii + 2], ezy = S.e[sk][2][jj + 2][ii + 1];
    S.hx[hslot][jj + 1][ii + 1] = csub(cmul(cmy, csub(ezy, ez0)), cmul(cmz, csub(eyz, ey0)));
    S.hy[hslot][jj + 1][ii + 1] = csub(cmul(cmz, csub(exz, ex0)), cmul(cmx, csub(ezx, ez0)));
    S.hz[jj + 1][ii + 1] = csub(cmul(cmx, csub(eyx, ey0)), cmul(cmy, csub(exy, ex0)));
  }
}

template <typename R>
__device__ __forceinline__ R ld_eoff(const OpArgs<R> &a, int p, int gi, int gj, int gk) {
  // ε off-diagonal pair p at corner (gi,gj,gk); ghost corners: PEC 0, Bloch periodic
  if (gi >= a.N[0]) { if (!a.bloch[0]) return R(0); gi -= a.N[0]; }
  if (gj >= a.N[1]) { if (!a.bloch[1]) return R(0); gj -= a.N[1]; }
  if (gk >= a.N[2]) { if (!a.bloch[2]) return R(0); gk -= a.N[2]; }
  return a.eoff[(long long)p * a.ncell + gi + (long long)a.N[0] * (gj + (long long)a.N[1] * gk)];
}

template <typename R, int EPI, bool TRANSPOSE>
__global__ void __launch_bounds__(NTHR) k_apply(OpArgs<R> a, Extra<R> ex, const typename CT<R>::C *__restrict__ x,
                                                typename CT<R>::C *__restrict__ y,
                                                const typename CT<R>::C *__restrict__ aux0, RedBuf red, int fin,
                                                KScalars *sc) {
  using C = typename CT<R>::C;
  extern __shared__ __align__(16) unsigned char smraw[];
  StencilSmem<R> &S = *reinterpret_cast<StencilSmem<R> *>(smraw);
  if (sc != nullptr && sc->done) return;

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int k0 = blockIdx.z * ex.kchunk;
  const int k1 = min(k0 + ex.kchunk, a.N[2]);
  const int gi = i0 + tx, gj = j0 + ty;
  const bool active = (gi < a.N[0]) && (gj < a.N[1]);
  const long long plane = (long long)a.N[0] * a.N[1];
  const long long tilecol = blockIdx.x + (long long)gridDim.x * blockIdx.y;

  Acc<R> acc0r, acc0i, acc1r, acc1i;

  // preamble: E(k0−1), E(k0), E(k0+1); H(k0−1)
  load_plane<R, TRANSPOSE>(S, a, ex, x, i0, j0, k0 - 1, (k0 + 2) % 3, tid);
  load_plane<R, TRANSPOSE>(S, a, ex, x, i0, j0, k0, k0 % 3, tid);
  load_plane<R, TRANSPOSE>(S, a, ex, x, i0, j0, k0 + 1, (k0 + 1) % 3, tid);
  __syncthreads();
  compute_h<R>(S, a, i0, j0, k0 - 1, (k0 + 2) % 3, k0 % 3, (k0 + 1) & 1, tid);

  // per-thread constants
  const int cxi = cidx(a, 0, gi), cyj = cidx(a, 1, gj);
  const C cex = a.ce[0][cxi], cey = a.ce[1][cyj];
  const C wmx = a.wm[0][cxi], wpx = a.wp[0][cxi], wmy = a.wm[1][cyj], wpy = a.wp[1][cyj];
  // pinned outputs: E_c at primal index 0 along a non-Bloch axis v ≠ c
  const bool pin_xy = !a.bloch[1] && gj == 0;
  const bool pin_yx = !a.bloch[0] && gi == 0;
  const bool pinz = pin_yx || pin_xy;

  for (int k = k0; k < k1; ++k) {
    const int sm = (k + 2) % 3, s0 = k % 3, s1 = (k + 1) % 3;
    const int hc = k & 1, hp = (k + 1) & 1;
    __syncthreads();  // E(k+1) present, H(k−1) complete
    compute_h<R>(S, a, i0, j0, k, s0, s1, hc, tid);
    __syncthreads();
    if (active) {
      const C cez = a.ce[2][k];
      const C hz00 = S.hz[ty + 1][tx + 1], hzjm = S.hz[ty][tx + 1], hzim = S.hz[ty + 1][tx];
      const C hyk = S.hy[hc][ty + 1][tx + 1], hykm = S.hy[hp][ty + 1][tx + 1], hyim = S.hy[hc][ty + 1][tx];
      const C hxk = S.hx[hc][ty + 1][tx + 1], hxkm = S.hx[hp][ty + 1][tx + 1], hxjm = S.hx[hc][ty][tx + 1];
      C yx = csub(cmul(cey, csub(hz00, hzjm)), cmul(cez, csub(hyk, hykm)));
      C yy = csub(cmul(cez, csub(hxk, hxkm)), cmul(cex, csub(hz00, hzim)));
      C yz = csub(cmul(cex, csub(hyk, hyim)), cmul(cey, csub(hxk, hxjm)));
      const long long cell = gi + (long long)a.N[0] * gj + plane * k;
      const bool pkz = !a.bloch[2] && k == 0;
      const bool pinx = pin_xy || pkz;
      const bool piny = pin_yx || pkz;
      // the cell's own values: shared memory holds 0 for pinned DOFs (they
      // do not enter the curl), but the ε term uses the true value
      C e_x = S.e[s0][0][ty + 1][tx + 1], e_y = S.e[s0][1][ty + 1][tx + 1], e_z = S.e[s0][2][ty + 1][tx + 1];
      if (pinx) e_x = own_e<R, TRANSPOSE>(x, ex, cell, 0, gi, gj, k);
      if (piny) e_y = own_e<R, TRANSPOSE>(x, ex, cell, 1, gi, gj, k);
      if (pinz) e_z = own_e<R, TRANSPOSE>(x, ex, cell, 2, gi, gj, k);
      C dx = cscale(e_x, a.eps[cell]);
      C dy = cscale(e_y, a.eps[a.ncell + cell]);
      C dz = cscale(e_z, a.eps[2 * a.ncell + cell]);
      if (a.eoff != nullptr && (a.oflag == nullptr || a.oflag[tilecol * a.N[2] + k])) {
        const C wmz = a.wm[2][k], wpz = a.wp[2][k];
        // x output: corners (i', j, k), i' ∈ {i, i+1}
        C ox = czero<C>(), oy = czero<C>(), oz = czero<C>();
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const C eym = S.e[s0][1][ty][tx + 1 + s], eyp = S.e[s0][1][ty + 1][tx + 1 + s];
          const C ezm = S.e[sm][2][ty + 1][tx + 1 + s], ezp = S.e[s0][2][ty + 1][tx + 1 + s];
          const R exy = ld_eoff(a, 0, gi + s, gj, k), ezx = ld_eoff(a, 2, gi + s, gj, k);
          ox = cadd(ox, cscale(cadd(cmul(wmy, eym), cmul(wpy, eyp)), exy));
          ox = cadd(ox, cscale(cadd(cmul(wmz, ezm), cmul(wpz, ezp)), ezx));
        }
        // y output: corners (i, j', k), j' ∈ {j, j+1}
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const C exm = S.e[s0][0][ty + 1 + s][tx], exp_ = S.e[s0][0][ty + 1 + s][tx + 1];
          const C ezm = S.e[sm][2][ty + 1 + s][tx + 1], ezp = S.e[s0][2][ty + 1 + s][tx + 1];
          const R exy = ld_eoff(a, 0, gi, gj + s, k), eyz = ld_eoff(a, 1, gi, gj + s, k);
          oy = cadd(oy, cscale(cadd(cmul(wmx, exm), cmul(wpx, exp_)), exy));
          oy = cadd(oy, cscale(cadd(cmul(wmz, ezm), cmul(wpz, ezp)), eyz));
        }
        // z output: corners (i, j, k'), k' ∈ {k, k+1}
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int sl = s ? s1 : s0;
          const C exm = S.e[sl][0][ty + 1][tx], exp_ = S.e[sl][0][ty + 1][tx + 1];
          const C eym = S.e[sl][1][ty][tx + 1], eyp = S.e[sl][1][ty + 1][tx + 1];
          const R ezx = ld_eoff(a, 2, gi, gj, k + s), eyz = ld_eoff(a, 1, gi, gj, k + s);
          oz = cadd(oz, cscale(cadd(cmul(wmx, exm), cmul(wpx, exp_)), ezx));
          oz = cadd(oz, cscale(cadd(cmul(wmy, eym), cmul(wpy, eyp)), eyz));
        }
        if (!pinx) dx = cadd(dx, cscale(ox, R(0.5)));
        if (!piny) dy = cadd(dy, cscale(oy, R(0.5)));
        if (!pinz) dz = cadd(dz, cscale(oz, R(0.5)));
      }
      if (pinx) yx = czero<C>();
      if (piny) yy = czero<C>();
      if (pinz) yz = czero<C>();
      yx = csub(yx, cmul(a.w2, dx));
      yy = csub(yy, cmul(a.w2, dy));
      yz = csub(yz, cmul(a.w2, dz));
      if (TRANSPOSE) {
        yx = cmul(yx, vol_e<R>(ex, 0, gi, gj, k));
        yy = cmul(yy, vol_e<R>(ex, 1, gi, gj, k));
        yz = cmul(yz, vol_e<R>(ex, 2, gi, gj, k));
      }
      C *yo = y + 3 * cell;
      if (EPI == EPI_RESID) {
        const C *bo = aux0 + 3 * cell;
        yx = csub(bo[0], yx);
        yy = csub(bo[1], yy);
        yz = csub(bo[2], yz);
        acc0r.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
      } else if (EPI == EPI_DOT_AUX) {
        const C *ro = aux0 + 3 * cell;
        const C d0 = cdotc(ro[0], yx), d1 = cdotc(ro[1], yy), d2 = cdotc(ro[2], yz);
        acc0r.add(d0.x + d1.x + d2.x);
        acc0i.add(d0.y + d1.y + d2.y);
      } else if (EPI == EPI_DOT_TS) {
        // (t, s) with the unscaled input s (shared memory holds S⁻¹ s for Aᵀ)
        const C sx = TRANSPOSE ? x[3 * cell] : e_x, sy = TRANSPOSE ? x[3 * cell + 1] : e_y,
                sz = TRANSPOSE ? x[3 * cell + 2] : e_z;
        const C d0 = cdotc(yx, sx), d1 = cdotc(yy, sy), d2 = cdotc(yz, sz);
        acc0r.add(d0.x + d1.x + d2.x);
        acc0i.add(d0.y + d1.y + d2.y);
        acc1r.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
      }
      yo[0] = yx;
      yo[1] = yy;
      yo[2] = yz;
    }
    __syncthreads();  // everyone done with E(k−1) and H(k−1)
    if (k + 1 < k1) load_plane<R, TRANSPOSE>(S, a, ex, x, i0, j0, k + 2, sm, tid);
  }
  if (EPI != EPI_STORE) {
    block_reduce_finalise<NTHR>(make_double2(acc0r.get(), acc0i.get()), make_double2(acc1r.get(), acc1i.get()), red,
                                fin, sc);
  }
}

// ------------------------------------------------------------------ host
template <typename R>
OpArgs<R> op_args(const fdfd_handle *h) {
  using C = typename CT<R>::C;
  OpArgs<R> a;
  const C *coef;
  if constexpr (sizeof(R) == 8) {
    coef = reinterpret_cast<const C *>(h->coef64);
    a.eps = reinterpret_cast<const R *>(h->eps64);
    a.eoff = h->has_off ? reinterpret_cast<const R *>(h->eoff64) : nullptr;
  } else {
    coef = reinterpret_cast<const C *>(h->coef32);
    a.eps = reinterpret_cast<const R *>(h->eps32);
    a.eoff = h->has_off ? reinterpret_cast<const R *>(h->eoff32) : nullptr;
  }
  const int st = h->coef_stride;
  for (int w = 0; w < 3; ++w) {
    a.N[w] = h->N[w];
    a.bloch[w] = h->bloch[w];
    a.cm[w] = coef + 0 * st + h->coef_off[w];
    a.ce[w] = coef + 1 * st + h->coef_off[w];
    a.wm[w] = coef + 2 * st + h->coef_off[w];
    a.wp[w] = coef + 3 * st + h->coef_off[w];
  }
  a.ncell = h->ncell;
  a.oflag = h->oflag;
  a.w2 = mk(R(h->w2[0]), R(h->w2[1]));
  return a;
}
template OpArgs<float> op_args<float>(const fdfd_handle *);
template OpArgs<double> op_args<double>(const fdfd_handle *);

static int kchunk_for(const fdfd_handle *h) {
  const int tiles = ((h->N[0] + TX - 1) / TX) * ((h->N[1] + TY - 1) / TY);
  const int target = 152 * 6;  // ~6 CTAs per SM in flight
  int nz = (target + tiles - 1) / tiles;
  if (nz < 1) nz = 1;
  int kc = (h->N[2] + nz - 1) / nz;
  if (kc < 4) kc = 4;
  if (kc > 64) kc = 64;
  return kc;
}

int apply_blocks(const fdfd_handle *h) {
  const int kc = kchunk_for(h);
  return ((h->N[0] + TX - 1) / TX) * ((h->N[1] + TY - 1) / TY) * ((h->N[2] + kc - 1) / kc);
}

template <typename R, int EPI, bool TR>
static int launch_t(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y,
                    const typename CT<R>::C *aux0, int fin, KScalars *sc) {
  using C = typename CT<R>::C;
  static bool attr_set[8] = {false};  // per device ordinal (≤ 8 devices per process)
  const size_t smem = sizeof(StencilSmem<R>);
  const int d = h->dev & 7;
  if (!attr_set[d]) {
    cudaError_t e = cudaFuncSetAttribute(k_apply<R, EPI, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply)");
    attr_set[d] = true;
  }
  const int kc = kchunk_for(h);
  dim3 grid((h->N[0] + TX - 1) / TX, (h->N[1] + TY - 1) / TY, (h->N[2] + kc - 1) / kc);
  dim3 block(TX, TY, 1);
  OpArgs<R> a = op_args<R>(h);
  Extra<R> ex;
  ex.kchunk = kc;
  const C *coef;
  if constexpr (sizeof(R) == 8) coef = reinterpret_cast<const C *>(h->coef64);
  else coef = reinterpret_cast<const C *>(h->coef32);
  const int st = h->coef_stride;
  for (int w = 0; w < 3; ++w) {
    ex.sdle[w] = coef + 4 * st + h->coef_off[w];
    ex.sdlm[w] = coef + 5 * st + h->coef_off[w];
    ex.ph[w] = mk(R(h->e_ikl[w][0]), R(h->e_ikl[w][1]));
    double d2 = h->e_ikl[w][0] * h->e_ikl[w][0] + h->e_ikl[w][1] * h->e_ikl[w][1];
    ex.phinv[w] = mk(R(h->e_ikl[w][0] / d2), R(-h->e_ikl[w][1] / d2));
  }
  if (EPI != EPI_STORE) {
    int rc = ensure_red(h, (int)(grid.x * grid.y * grid.z));
    if (rc) return rc;
  }
  k_apply<R, EPI, TR><<<grid, block, smem, h->stream>>>(a, ex, x, y, aux0, h->red, fin, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_apply launch");
}

// FP64 residual launcher whose block partials, arrival counter and
// finalisation scalars live in caller-provided device memory (used by the
// allocation-free entry point).  Fails if the grid needs more than
// `max_blocks` partial slots.
int launch_residual_ext(fdfd_handle *h, const double2 *x, double2 *r, const double2 *b, RedBuf red, int max_blocks,
                        KScalars *sc) {
  const size_t smem = sizeof(StencilSmem<double>);
  cudaError_t e =
      cudaFuncSetAttribute(k_apply<double, EPI_RESID, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply)");
  const int kc = kchunk_for(h);
  dim3 grid((h->N[0] + TX - 1) / TX, (h->N[1] + TY - 1) / TY, (h->N[2] + kc - 1) / kc);
  if ((long long)grid.x * grid.y * grid.z > max_blocks)
    return set_error(h, FDFD_ERR_ARG, "grid needs more thread blocks than the fixed reduction scratch holds");
  OpArgs<double> a = op_args<double>(h);
  Extra<double> ex;
  ex.kchunk = kc;
  const double2 *coef = h->coef64;
  const int st = h->coef_stride;
  for (int w = 0; w < 3; ++w) {
    ex.sdle[w] = coef + 4 * st + h->coef_off[w];
    ex.sdlm[w] = coef + 5 * st + h->coef_off[w];
    ex.ph[w] = make_double2(h->e_ikl[w][0], h->e_ikl[w][1]);
    const double d2 = h->e_ikl[w][0] * h->e_ikl[w][0] + h->e_ikl[w][1] * h->e_ikl[w][1];
    ex.phinv[w] = make_double2(h->e_ikl[w][0] / d2, -h->e_ikl[w][1] / d2);
  }
  k_apply<double, EPI_RESID, false><<<grid, dim3(TX, TY, 1), smem, h->stream>>>(a, ex, x, r, b, red, FIN_NONE, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_apply launch");
}

// Full-control launcher (epilogue + finalisation mode).
template <typename R>
int launch_apply_fin(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                     const typename CT<R>::C *aux0, int fin, KScalars *sc, bool transpose) {
  if (transpose) {
    switch (epi) {
      case EPI_STORE: return launch_t<R, EPI_STORE, true>(h, x, y, aux0, fin, sc);
      case EPI_RESID: return launch_t<R, EPI_RESID, true>(h, x, y, aux0, fin, sc);
      case EPI_DOT_AUX: return launch_t<R, EPI_DOT_AUX, true>(h, x, y, aux0, fin, sc);
      case EPI_DOT_TS: return launch_t<R, EPI_DOT_TS, true>(h, x, y, aux0, fin, sc);
    }
  } else {
    switch (epi) {
      case EPI_STORE: return launch_t<R, EPI_STORE, false>(h, x, y, aux0, fin, sc);
      case EPI_RESID: return launch_t<R, EPI_RESID, false>(h, x, y, aux0, fin, sc);
      case EPI_DOT_AUX: return launch_t<R, EPI_DOT_AUX, false>(h, x, y, aux0, fin, sc);
      case EPI_DOT_TS: return launch_t<R, EPI_DOT_TS, false>(h, x, y, aux0, fin, sc);
    }
  }
  return set_error(h, FDFD_ERR_ARG, "bad epilogue kind");
}
template int launch_apply_fin<float>(fdfd_handle *, const float2 *, float2 *, int, const float2 *, int, KScalars *,
                                     bool);
template int launch_apply_fin<double>(fdfd_handle *, const double2 *, double2 *, int, const double2 *, int,
                                      KScalars *, bool);

}  // namespace fdfd
