// Matrix-free application of the FDFD operator
//     y = A x,  A = Cₘ·Cₑ − ω²·Pε   (μ = 1)
// which the reference assembles as a sparse matrix (create_A,
// src/model/model.jl:225-246) from create_curls (:160-175) and
// create_paramops (:141-158).
//
// Kernel design (sm_103a, HBM-bound):
//   * a CTA owns a 32×8 (x,y) tile and marches along z over a chunk of
//     planes with a ring of E planes (one-cell halo) in shared memory, so
//     every E value is read from HBM about once;
//   * k_apply_tma (PEC walls, Aᵀ excluded): a 4-slot ring filled by TMA
//     (cp.async.bulk.tensor.3d, one elected thread, mbarrier completion with
//     bounded waits), two planes ahead of the plane being computed; the
//     out-of-bounds zero fill of TMA realises the PEC ghost planes;
//   * k_apply (general: Bloch phases, Aᵀ): a 3-slot ring filled by plain
//     loads that apply the boundary rules element by element;
//   * H = Cₑ E is computed once per plane for the tile plus its low halo and
//     kept for two planes (H(k−1), H(k)) in shared memory;
//   * y(k) = Cₘ H − ω² Pε E is formed from shared memory with the per-axis
//     1/s∆l PML factors, the ε diagonal and — only where the (tile, plane)
//     flag says so — the corner-averaged off-diagonal ε terms;
//   * optional fused epilogues produce the dot products a Krylov step needs
//     (block partials in double-float FP32 for complex64, FP64 for
//     complex128; last-block finalisation, krylov_fin.cuh);
//   * TRANSPOSE applies Aᵀ = S·A·S⁻¹ with S = V_E (the dual volume of each
//     E sample), which holds because S·A is complex symmetric.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <utility>
#include <vector>

#include "krylov_fin.cuh"
#include "operator_common.cuh"
#include "tma_util.cuh"

namespace fdfd {

constexpr int EX = TX + 2, EY = TY + 2;  // E tile with halo: −1 … T
constexpr int HX = TX + 1, HY = TY + 1;  // H tile: −1 … T−1

// H of the current plane over the tile and its low halo (−1 … T−1).  Each
// thread also keeps the H it computed at its own cell in registers, for
// this plane and the previous one, so only the neighbours' values (i−1 and
// j−1) are read back from here.
template <typename R>
struct HTile {
  using C = typename CT<R>::C;
  C hx[HY][HX];
  C hy[HY][HX];
  C hz[HY][HX];
};

// Values a thread carries from the H stage to the output stage of a plane:
// H and E at its own cell.
template <typename R>
struct Own {
  using C = typename CT<R>::C;
  C hx, hy, hz, ex, ey, ez;
};

// Per-tile copies of the x and y coefficient arrays, indexed by position+1
// over −1 … T (ghost entries resolved by cidx).
template <typename R>
struct CoefTile {
  using C = typename CT<R>::C;
  C cmx[TX + 2], cex[TX + 2], wmx[TX + 2], wpx[TX + 2];
  C cmy[TY + 2], cey[TY + 2], wmy[TY + 2], wpy[TY + 2];
};

// Corner terms of the off-diagonal ε operator for one tile-plane, each
// computed once and shared by the two outputs that average it:
//   xc(ii,jj) = ε_xy·⟨E_y⟩ + ε_zx·⟨E_z⟩ at corner (i0+ii, j0+jj, k), ii ∈ [0,T]
//   yc(ii,jj) = ε_xy·⟨E_x⟩ + ε_yz·⟨E_z⟩ at corner (i0+ii, j0+jj, k), jj ∈ [0,T]
//   zc[s](ii,jj) = ε_zx·⟨E_x⟩ + ε_yz·⟨E_y⟩ at corner (i0+ii, j0+jj, k'), s = k'&1
// with ⟨E_v⟩ the s∆l-weighted average of E_v onto the corner.
template <typename R>
struct OffTile {
  using C = typename CT<R>::C;
  C xc[TY][TX + 1];
  C yc[TY + 1][TX];
  C zc[2][TY][TX];
};

// ---- plain-load ring: SoA by component, 3 slots
template <typename R>
struct PlainE {
  using C = typename CT<R>::C;
  C e[3][3][EY][EX];
  __device__ __forceinline__ C get(int s, int c, int jj, int ii) const { return e[s][c][jj + 1][ii + 1]; }
};
template <typename R>
struct PlainSmem {
  PlainE<R> E;
  HTile<R> H;
  CoefTile<R> T;
  OffTile<R> O;
};

// Per-chunk copies of the z coefficient arrays and the off-diagonal flags of
// the tile column, indexed by plane − (k0 − 1) over k0 − 1 … k1 (staged once
// per CTA, so no plane waits on a global load for them).
template <typename R>
struct ZTile {
  using C = typename CT<R>::C;
  C cm[KCMAX + 2], ce[KCMAX + 2], wm[KCMAX + 2], wp[KCMAX + 2];
  unsigned char flag[KCMAX + 2];
};

// ---- TMA ring: the global AoS cell layout, 4 slots.  The box starts XOFF
// cells left of the tile so its x coordinate is 16-byte aligned.
template <typename R>
struct TmaGeom {
  static constexpr int XOFF = sizeof(R) == 4 ? 2 : 1;
  static constexpr int XW = sizeof(R) == 4 ? TX + 4 : TX + 2;
  static constexpr int NSLOT = 4;
  static constexpr int PLANE_BYTES = XW * EY * 3 * 2 * (int)sizeof(R);
  static constexpr int SLOT_BYTES = (PLANE_BYTES + 127) / 128 * 128;
  static constexpr int H_OFF = NSLOT * SLOT_BYTES;
  static constexpr int T_OFF = H_OFF + (int)((sizeof(HTile<R>) + 15) / 16 * 16);
  static constexpr int O_OFF = T_OFF + (int)((sizeof(CoefTile<R>) + 15) / 16 * 16);
  static constexpr int Z_OFF = O_OFF + (int)((sizeof(OffTile<R>) + 15) / 16 * 16);
  // complex64 only: a ring slot per plane for the off-diagonal ε of corners
  // i0 … i0+EOX−1, j0 … j0+TY, laid out [p][jj][ii] (EOX·4 bytes a multiple
  // of 16); complex128 reads them from global memory (shared memory would
  // drop it to one CTA per SM)
  static constexpr int EOX = TX + 4;
  static constexpr int EO_BYTES = sizeof(R) == 4 ? EOX * (TY + 1) * 3 * (int)sizeof(R) : 0;
  static constexpr int EO_SLOT = (EO_BYTES + 127) / 128 * 128;
  // TMA destinations (E slots, ε slots) start on 128-byte boundaries
  static constexpr int EO_OFF = (Z_OFF + (int)sizeof(ZTile<R>) + 127) / 128 * 128;
  static constexpr int BAR_OFF = EO_OFF + NSLOT * EO_SLOT;
  static constexpr int SMEM = BAR_OFF + NSLOT * 8 + 128;  // + alignment slack
  static_assert(SLOT_BYTES % 128 == 0 && EO_OFF % 128 == 0 && EO_SLOT % 128 == 0, "TMA destination alignment");
  static_assert(BAR_OFF % 8 == 0, "mbarrier alignment");
  static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};
template <typename R>
struct TmaE {
  using C = typename CT<R>::C;
  unsigned char *base;
  __device__ __forceinline__ C *ptr(int s, int c, int jj, int ii) const {
    return reinterpret_cast<C *>(base + s * TmaGeom<R>::SLOT_BYTES) +
           ((jj + 1) * TmaGeom<R>::XW + ii + TmaGeom<R>::XOFF) * 3 + c;
  }
  __device__ __forceinline__ C get(int s, int c, int jj, int ii) const { return *ptr(s, c, jj, ii); }
};

template <typename R, bool TRANSPOSE>
__device__ __forceinline__ void load_plane(PlainE<R> &E, const OpArgs<R> &a, const Extra<R> &ex,
                                           const typename CT<R>::C *__restrict__ x, int i0, int j0, int k, int slot,
                                           int tid) {
  for (int p = tid; p < EX * EY; p += NTHR) {
    const int ii = p % EX - 1, jj = p / EX - 1;
    const int gi = i0 + ii, gj = j0 + jj;
#pragma unroll
    for (int c = 0; c < 3; ++c) E.e[slot][c][jj + 1][ii + 1] = load_e<R, TRANSPOSE>(x, a, ex, gi, gj, k, c);
  }
}

template <typename R>
__device__ __forceinline__ void fill_coef(CoefTile<R> &T, const OpArgs<R> &a, int i0, int j0, int tid) {
  if (tid < TX + 2) {
    const int c = cidx(a, 0, i0 + tid - 1);
    T.cmx[tid] = a.cm[0][c];
    T.cex[tid] = a.ce[0][c];
    T.wmx[tid] = a.wm[0][c];
    T.wpx[tid] = a.wp[0][c];
  } else if (tid >= 64 && tid < 64 + TY + 2) {
    const int t = tid - 64;
    const int c = cidx(a, 1, j0 + t - 1);
    T.cmy[t] = a.cm[1][c];
    T.cey[t] = a.ce[1][c];
    T.wmy[t] = a.wm[1][c];
    T.wpy[t] = a.wp[1][c];
  }
}

// H = Cₑ E at tile position (ii, jj) of plane k (E(k), E(k+1) in slots sk,
// sk1); also returns E(k) there.

template <typename R, bool RC, typename ET>
__device__ __forceinline__ void curl_e(const ET &E, const CoefTile<R> &T, typename CT<R>::C cmz, int sk, int sk1,
                                       int ii, int jj, Own<R> &o) {
  using C = typename CT<R>::C;
  const C cmx = T.cmx[ii + 1];
  const C cmy = T.cmy[jj + 1];
  o.ex = E.get(sk, 0, jj, ii);
  o.ey = E.get(sk, 1, jj, ii);
  o.ez = E.get(sk, 2, jj, ii);
  const C exy = E.get(sk, 0, jj + 1, ii), exz = E.get(sk1, 0, jj, ii);
  const C eyx = E.get(sk, 1, jj, ii + 1), eyz = E.get(sk1, 1, jj, ii);
  const C ezx = E.get(sk, 2, jj, ii + 1), ezy = E.get(sk, 2, jj + 1, ii);
  o.hx = csub(mulc<RC>(cmy, csub(ezy, o.ez)), mulc<RC>(cmz, csub(eyz, o.ey)));
  o.hy = csub(mulc<RC>(cmz, csub(exz, o.ex)), mulc<RC>(cmx, csub(ezx, o.ez)));
  o.hz = csub(mulc<RC>(cmx, csub(eyx, o.ey)), mulc<RC>(cmy, csub(exy, o.ex)));
}

constexpr int H_HALO = TX + TY;  // halo positions: column i = −1 (TY), row j = −1 (TX)

// H(k) (cmz: the z coefficient 1/s∆lₘ of plane k): every thread at its own cell (kept in `own` and stored for its
// neighbours), threads 0 … TX+TY−1 also at one low-halo position, storing
// only the components a neighbour reads there (hy, hz on the i = −1
// column; hx, hz on the j = −1 row).
template <typename R, bool RC, typename ET>
__device__ __forceinline__ void compute_h(const ET &E, HTile<R> &H, const CoefTile<R> &T, typename CT<R>::C cmz,
                                          int sk, int sk1, int tx, int ty, int tid, Own<R> &own) {
  using C = typename CT<R>::C;
  curl_e<R, RC>(E, T, cmz, sk, sk1, tx, ty, own);
  H.hx[ty + 1][tx + 1] = own.hx;
  H.hy[ty + 1][tx + 1] = own.hy;
  H.hz[ty + 1][tx + 1] = own.hz;
  if (tid < H_HALO) {
    const int ii = tid < TY ? -1 : tid - TY, jj = tid < TY ? tid : -1;
    Own<R> h;
    curl_e<R, RC>(E, T, cmz, sk, sk1, ii, jj, h);
    if (ii < 0) H.hy[jj + 1][0] = h.hy;
    else H.hx[0][ii + 1] = h.hx;
    H.hz[jj + 1][ii + 1] = h.hz;
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

// Off-diagonal ε of one tile-plane: a TMA-staged shared copy [p][jj][ii]
// (corner (i0+ii, j0+jj); zero beyond the grid, as PEC ghosts are), or —
// s == nullptr — global memory with the ghost rules of ld_eoff.
template <typename R>
struct EoffSrc {
  const R *s;
  __device__ __forceinline__ R get(const OpArgs<R> &a, int p, int i0, int j0, int ii, int jj, int k) const {
    if (s != nullptr) return s[(p * (TY + 1) + jj) * TmaGeom<R>::EOX + ii];
    return ld_eoff(a, p, i0 + ii, j0 + jj, k);
  }
};

// x- and y-directed corner terms of plane k (E(k−1), E(k) in slots sm, s0;
// wmz, wpz: the z averaging weights of plane k).
// A thread owns xc/yc positions t and t + NTHR; all its ε loads are issued
// before any is used, so their latencies overlap.  The positions beyond
// NTHR (8 of xc, 32 of yc) go to warps 2 and 3, clear of the two warps that
// computed the H halo, so no warp does more than one extra round.
constexpr int XC_ROT = 2 * TX;                              // xc extras → warp 2
constexpr int YC_ROT = 3 * TX;                              // yc extras → warp 3
template <typename R, typename ET>
__device__ __forceinline__ void stage_xy(const ET &E, OffTile<R> &O, const CoefTile<R> &T, const OpArgs<R> &a,
                                         const EoffSrc<R> &src, typename CT<R>::C wmz, typename CT<R>::C wpz, int i0,
                                         int j0, int k, int sm, int s0, int tid) {
  using C = typename CT<R>::C;
  constexpr int NXC = TY * (TX + 1), NYC = (TY + 1) * TX;
  const int tx0 = (tid + NTHR - XC_ROT) % NTHR, ty0 = (tid + NTHR - YC_ROT) % NTHR;
  R vx[2][2], vy[2][2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    vx[r][0] = vx[r][1] = vy[r][0] = vy[r][1] = R(0);
    {
      // corners no active output reads (beyond the one-past corner) stay 0
      const int p = tx0 + r * NTHR;
      const int ii = p % (TX + 1), jj = p / (TX + 1);
      if (p < NXC && i0 + ii <= a.N[0] && j0 + jj < a.N[1]) {
        vx[r][0] = src.get(a, 0, i0, j0, ii, jj, k);
        vx[r][1] = src.get(a, 2, i0, j0, ii, jj, k);
      }
    }
    {
      const int p = ty0 + r * NTHR;
      const int ii = p % TX, jj = p / TX;
      if (p < NYC && i0 + ii < a.N[0] && j0 + jj <= a.N[1]) {
        vy[r][0] = src.get(a, 0, i0, j0, ii, jj, k);
        vy[r][1] = src.get(a, 1, i0, j0, ii, jj, k);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int p = tx0 + r * NTHR;
    if (p < NXC) {
      const int ii = p % (TX + 1), jj = p / (TX + 1);
      const C ay = cadd(cmul(T.wmy[jj + 1], E.get(s0, 1, jj - 1, ii)), cmul(T.wpy[jj + 1], E.get(s0, 1, jj, ii)));
      const C az = cadd(cmul(wmz, E.get(sm, 2, jj, ii)), cmul(wpz, E.get(s0, 2, jj, ii)));
      O.xc[jj][ii] = cadd(cscale(ay, vx[r][0]), cscale(az, vx[r][1]));
    }
    const int q = ty0 + r * NTHR;
    if (q < NYC) {
      const int ii = q % TX, jj = q / TX;
      const C ax = cadd(cmul(T.wmx[ii + 1], E.get(s0, 0, jj, ii - 1)), cmul(T.wpx[ii + 1], E.get(s0, 0, jj, ii)));
      const C az = cadd(cmul(wmz, E.get(sm, 2, jj, ii)), cmul(wpz, E.get(s0, 2, jj, ii)));
      O.yc[jj][ii] = cadd(cscale(ax, vy[r][0]), cscale(az, vy[r][1]));
    }
  }
}

// z-directed corner terms of plane kz (E(kz) in slot sz) into zc[kz & 1];
// one position per thread (NTHR = TX·TY).
template <typename R, typename ET>
__device__ __forceinline__ void stage_z(const ET &E, OffTile<R> &O, const CoefTile<R> &T, const OpArgs<R> &a,
                                        const EoffSrc<R> &src, int i0, int j0, int kz, int sz, int tid) {
  using C = typename CT<R>::C;
  const int ii = tid % TX, jj = tid / TX;
  R v0 = R(0), v1 = R(0);
  if (i0 + ii < a.N[0] && j0 + jj < a.N[1]) {
    v0 = src.get(a, 2, i0, j0, ii, jj, kz);
    v1 = src.get(a, 1, i0, j0, ii, jj, kz);
  }
  const C ax = cadd(cmul(T.wmx[ii + 1], E.get(sz, 0, jj, ii - 1)), cmul(T.wpx[ii + 1], E.get(sz, 0, jj, ii)));
  const C ay = cadd(cmul(T.wmy[jj + 1], E.get(sz, 1, jj - 1, ii)), cmul(T.wpy[jj + 1], E.get(sz, 1, jj, ii)));
  O.zc[kz & 1][jj][ii] = cadd(cscale(ax, v0), cscale(ay, v1));
}

template <typename R> struct Accs {
  ShortAcc<R> r0, i0, r1;
};

// Operands of the output stage that come from global memory, loaded at the
// top of a plane iteration so their latency overlaps the H computation: the
// ε diagonal and the epilogue's second operand at the thread's cell.
template <typename R>
struct Pre {
  using C = typename CT<R>::C;
  R e0, e1, e2;
  C a0, a1, a2;
};

template <typename R, int EPI>
__device__ __forceinline__ void prefetch(Pre<R> &pf, const OpArgs<R> &a, const typename CT<R>::C *__restrict__ aux0,
                                         long long cell) {
  pf.e0 = a.eps[cell];
  pf.e1 = a.eps[a.ncell + cell];
  pf.e2 = a.eps[2 * a.ncell + cell];
  if (EPI == EPI_RESID || EPI == EPI_DOT_AUX) {
    pf.a0 = aux0[3 * cell];
    pf.a1 = aux0[3 * cell + 1];
    pf.a2 = aux0[3 * cell + 2];
  }
}

// y(k) at the thread's cell (gi, gj, k) from shared memory (cez: the z
// coefficient 1/s∆lₑ of plane k).
template <typename R, int EPI, bool TRANSPOSE, bool RC>
__device__ __forceinline__ void output_cell(const HTile<R> &H, const CoefTile<R> &T, const OffTile<R> &O,
                                            const OpArgs<R> &a, const Extra<R> &ex, const Pre<R> &pf,
                                            const Own<R> &own, typename CT<R>::C hxkm, typename CT<R>::C hykm,
                                            const typename CT<R>::C *__restrict__ x,
                                            typename CT<R>::C *__restrict__ y, int gi, int gj, int k, int tx, int ty,
                                            bool offd, typename CT<R>::C cez, Accs<R> &acc) {
  using C = typename CT<R>::C;
  const C cex = T.cex[tx + 1], cey = T.cey[ty + 1];
  const C hz00 = own.hz, hzjm = H.hz[ty][tx + 1], hzim = H.hz[ty + 1][tx];
  const C hyk = own.hy, hyim = H.hy[ty + 1][tx];
  const C hxk = own.hx, hxjm = H.hx[ty][tx + 1];
  C yx = csub(mulc<RC>(cey, csub(hz00, hzjm)), mulc<RC>(cez, csub(hyk, hykm)));
  C yy = csub(mulc<RC>(cez, csub(hxk, hxkm)), mulc<RC>(cex, csub(hz00, hzim)));
  C yz = csub(mulc<RC>(cex, csub(hyk, hyim)), mulc<RC>(cey, csub(hxk, hxjm)));
  const long long cell = gi + (long long)a.N[0] * (gj + (long long)a.N[1] * k);
  // pinned outputs: E_c at primal index 0 along a non-Bloch axis v ≠ c
  const bool pin_xy = !a.bloch[1] && gj == 0;
  const bool pin_yx = !a.bloch[0] && gi == 0;
  const bool pkz = !a.bloch[2] && k == 0;
  const bool pinx = pin_xy || pkz;
  const bool piny = pin_yx || pkz;
  const bool pinz = pin_yx || pin_xy;
  // the cell's own values: shared memory holds 0 for pinned DOFs (they do
  // not enter the curl), but the ε term uses the true value
  C e_x = own.ex, e_y = own.ey, e_z = own.ez;
  if (pinx) e_x = own_e<R, TRANSPOSE>(x, ex, cell, 0, gi, gj, k);
  if (piny) e_y = own_e<R, TRANSPOSE>(x, ex, cell, 1, gi, gj, k);
  if (pinz) e_z = own_e<R, TRANSPOSE>(x, ex, cell, 2, gi, gj, k);
  C dx = cscale(e_x, pf.e0);
  C dy = cscale(e_y, pf.e1);
  C dz = cscale(e_z, pf.e2);
  if (offd) {
    // each output averages the two staged corner terms around it (weight ½)
    const C ox = cadd(O.xc[ty][tx], O.xc[ty][tx + 1]);
    const C oy = cadd(O.yc[ty][tx], O.yc[ty + 1][tx]);
    const C oz = cadd(O.zc[k & 1][ty][tx], O.zc[(k + 1) & 1][ty][tx]);
    if (!pinx) dx = cadd(dx, cscale(ox, R(0.5)));
    if (!piny) dy = cadd(dy, cscale(oy, R(0.5)));
    if (!pinz) dz = cadd(dz, cscale(oz, R(0.5)));
  }
  if (pinx) yx = czero<C>();
  if (piny) yy = czero<C>();
  if (pinz) yz = czero<C>();
  if (a.w2.y == R(0)) {  // real ω²
    yx = csub(yx, cscale(dx, a.w2.x));
    yy = csub(yy, cscale(dy, a.w2.x));
    yz = csub(yz, cscale(dz, a.w2.x));
  } else {
    yx = csub(yx, cmul(a.w2, dx));
    yy = csub(yy, cmul(a.w2, dy));
    yz = csub(yz, cmul(a.w2, dz));
  }
  if (TRANSPOSE) {
    yx = cmul(yx, vol_e<R>(ex, 0, gi, gj, k));
    yy = cmul(yy, vol_e<R>(ex, 1, gi, gj, k));
    yz = cmul(yz, vol_e<R>(ex, 2, gi, gj, k));
  }
  C *yo = y + 3 * cell;
  if (EPI == EPI_RESID) {
    yx = csub(pf.a0, yx);
    yy = csub(pf.a1, yy);
    yz = csub(pf.a2, yz);
    acc.r0.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
  } else if (EPI == EPI_DOT_AUX) {
    const C d0 = cdotc(pf.a0, yx), d1 = cdotc(pf.a1, yy), d2 = cdotc(pf.a2, yz);
    acc.r0.add(d0.x + d1.x + d2.x);
    acc.i0.add(d0.y + d1.y + d2.y);
  } else if (EPI == EPI_DOT_TS) {
    // (t, s) with the unscaled input s (shared memory holds S⁻¹ s for Aᵀ)
    const C sx = TRANSPOSE ? x[3 * cell] : e_x, sy = TRANSPOSE ? x[3 * cell + 1] : e_y,
            sz = TRANSPOSE ? x[3 * cell + 2] : e_z;
    const C d0 = cdotc(yx, sx), d1 = cdotc(yy, sy), d2 = cdotc(yz, sz);
    acc.r0.add(d0.x + d1.x + d2.x);
    acc.i0.add(d0.y + d1.y + d2.y);
    acc.r1.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
  } else if (EPI == EPI_DOT_SHD) {
    const C d0 = cdotc(shadow<R>(3 * cell), yx), d1 = cdotc(shadow<R>(3 * cell + 1), yy),
            d2 = cdotc(shadow<R>(3 * cell + 2), yz);
    acc.r0.add(d0.x + d1.x + d2.x);
    acc.i0.add(d0.y + d1.y + d2.y);
  } else if (EPI == EPI_DOT_SU) {
    // Σ V_E·x·y over the cell (COCG's S-weighted bilinear form)
    const C d0 = cmul(cmul(vol_e<R>(ex, 0, gi, gj, k), e_x), yx);
    const C d1 = cmul(cmul(vol_e<R>(ex, 1, gi, gj, k), e_y), yy);
    const C d2 = cmul(cmul(vol_e<R>(ex, 2, gi, gj, k), e_z), yz);
    acc.r0.add(d0.x + d1.x + d2.x);
    acc.i0.add(d0.y + d1.y + d2.y);
  }
  yo[0] = yx;
  yo[1] = yy;
  yo[2] = yz;
}

__device__ __forceinline__ bool offd_on(const OpArgs<float> &a, long long tilecol, int k) {
  return a.eoff != nullptr && (a.oflag == nullptr || a.oflag[tilecol * a.N[2] + k]);
}
__device__ __forceinline__ bool offd_on(const OpArgs<double> &a, long long tilecol, int k) {
  return a.eoff != nullptr && (a.oflag == nullptr || a.oflag[tilecol * a.N[2] + k]);
}

// ------------------------------------------------------------------ plain kernel
template <typename R, int EPI, bool TRANSPOSE>
__global__ void __launch_bounds__(NTHR, sizeof(R) == 4 ? 3 : 2) k_apply(OpArgs<R> a, Extra<R> ex, const typename CT<R>::C *__restrict__ x,
                                                typename CT<R>::C *__restrict__ y,
                                                const typename CT<R>::C *__restrict__ aux0, RedBuf red, int fin,
                                                KScalars *sc) {
  extern __shared__ __align__(16) unsigned char smraw[];
  PlainSmem<R> &S = *reinterpret_cast<PlainSmem<R> *>(smraw);
  pdl_trigger();

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int k0 = blockIdx.z * ex.kchunk;
  const int k1 = min(k0 + ex.kchunk, a.N[2]);
  const int gi = i0 + tx, gj = j0 + ty;
  const bool active = (gi < a.N[0]) && (gj < a.N[1]);
  const long long tilecol = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  // the tile's x/y coefficient tables (−1 … T) lie outside the PML
  const bool rxy = i0 - 1 >= a.rlo[0] && i0 + TX <= a.rhi[0] && j0 - 1 >= a.rlo[1] && j0 + TY <= a.rhi[1];
  Accs<R> acc;

  // preamble: coefficient tables (static data, before the dependency wait);
  // E(k0−1), E(k0), E(k0+1); H(k0−1)
  fill_coef<R>(S.T, a, i0, j0, tid);
  pdl_wait();
  if (sc != nullptr && sc->done) return;
  load_plane<R, TRANSPOSE>(S.E, a, ex, x, i0, j0, k0 - 1, (k0 + 2) % 3, tid);
  load_plane<R, TRANSPOSE>(S.E, a, ex, x, i0, j0, k0, k0 % 3, tid);
  load_plane<R, TRANSPOSE>(S.E, a, ex, x, i0, j0, k0 + 1, (k0 + 1) % 3, tid);
  __syncthreads();
  // H(k0−1) at the thread's own cell (the output of plane k0 reads no
  // neighbour of it)
  typename CT<R>::C hxp, hyp;
  {
    Own<R> o;
    curl_e<R, false>(S.E, S.T, a.cm[2][cidx(a, 2, k0 - 1)], (k0 + 2) % 3, k0 % 3, tx, ty, o);
    hxp = o.hx;
    hyp = o.hy;
  }
  bool zvalid = false;  // zc[k & 1] already holds plane k's z-directed corners

  for (int k = k0; k < k1; ++k) {
    const int sm = (k + 2) % 3, s0 = k % 3, s1 = (k + 1) % 3;
    Pre<R> pf;
    if (active) prefetch<R, EPI>(pf, a, aux0, gi + (long long)a.N[0] * (gj + (long long)a.N[1] * k));
    __syncthreads();  // E(k+1) present; the previous plane's reads of H are done
    Own<R> own;
    const bool rc = rxy && k >= a.rlo[2] && k <= a.rhi[2];
    const typename CT<R>::C cmz = a.cm[2][cidx(a, 2, k)];
    if (rc) compute_h<R, true>(S.E, S.H, S.T, cmz, s0, s1, tx, ty, tid, own);
    else compute_h<R, false>(S.E, S.H, S.T, cmz, s0, s1, tx, ty, tid, own);
    const bool offd = offd_on(a, tilecol, k);
    if (offd) {
      const EoffSrc<R> g{nullptr};
      stage_xy<R>(S.E, S.O, S.T, a, g, a.wm[2][k], a.wp[2][k], i0, j0, k, sm, s0, tid);
      if (!zvalid) stage_z<R>(S.E, S.O, S.T, a, g, i0, j0, k, s0, tid);
      stage_z<R>(S.E, S.O, S.T, a, g, i0, j0, k + 1, s1, tid);
    }
    zvalid = offd;
    __syncthreads();  // H(k), staged corners complete; nobody reads E(k−1) any more
    if (active) {
      const typename CT<R>::C cez = a.ce[2][k];
      if (rc) output_cell<R, EPI, TRANSPOSE, true>(S.H, S.T, S.O, a, ex, pf, own, hxp, hyp, x, y, gi, gj, k, tx, ty, offd, cez, acc);
      else output_cell<R, EPI, TRANSPOSE, false>(S.H, S.T, S.O, a, ex, pf, own, hxp, hyp, x, y, gi, gj, k, tx, ty, offd, cez, acc);
    }
    hxp = own.hx;
    hyp = own.hy;
    // E(k−1)'s slot takes E(k+2); the next iteration's first barrier orders
    // it (and this plane's reads of H and the corners) before their reuse
    if (k + 1 < k1) load_plane<R, TRANSPOSE>(S.E, a, ex, x, i0, j0, k + 2, sm, tid);
  }
  if (EPI != EPI_STORE) {
    sum_finalise<NTHR>(acc.r0, acc.i0, acc.r1, red, fin, sc);
  }
}

// ------------------------------------------------------------------ TMA kernel
// Zero the pinned DOFs of a freshly landed plane (their Cₑ columns are 0):
// E_y, E_z on x = 0; E_x, E_z on y = 0; E_x, E_y on z = 0 (PEC walls).
// Run by the warp that waited for the plane (lane, 32 lanes), so the block
// barrier that follows the wait orders it for every thread.
template <typename R>
__device__ __forceinline__ void pin_fixup(const TmaE<R> &E, int slot, int i0, int j0, int q, int lane) {
  using C = typename CT<R>::C;
  using G = TmaGeom<R>;
  constexpr int NL = 32;
  const C z = czero<C>();
  if (q == 0) {
    for (int p = lane; p < G::XW * EY; p += NL) {
      const int ii = p % G::XW - G::XOFF, jj = p / G::XW - 1;
      *E.ptr(slot, 0, jj, ii) = z;
      *E.ptr(slot, 1, jj, ii) = z;
    }
  }
  if (i0 == 0) {
    for (int jj = lane - 1; jj <= TY; jj += NL) {
      *E.ptr(slot, 1, jj, 0) = z;
      *E.ptr(slot, 2, jj, 0) = z;
    }
  }
  if (j0 == 0) {
    for (int p = lane; p < G::XW; p += NL) {
      const int ii = p - G::XOFF;
      *E.ptr(slot, 0, 0, ii) = z;
      *E.ptr(slot, 2, 0, ii) = z;
    }
  }
}

// Issue the copies of plane q into ring slot `slot` (one thread): the E
// tile and, when the TMA kernel stages the off-diagonal ε and plane q or
// q−1 is flagged (the z-directed corners of q serve both), the ε tile too —
// both completing on the slot's mbarrier.
template <typename R>
__device__ __forceinline__ void issue_plane(unsigned char *smraw, uint64_t *bars, const CUtensorMap *tmap,
                                            const CUtensorMap *emap, const Extra<R> &ex, const ZTile<R> &Z,
                                            int cx, int cy, int i0, int j0, int k0, int q, int slot) {
  using G = TmaGeom<R>;
  bool eo = false;
  // flags of planes q and q − 1 (table index q − (k0 − 1) and one less)
  if (G::EO_SLOT > 0 && ex.eoff_tma && q >= k0) eo = Z.flag[q - k0 + 1] || Z.flag[q - k0];
  const uint32_t bar = smem_u32(&bars[slot]);
  mbar_expect(bar, (uint32_t)(G::PLANE_BYTES + (eo ? G::EO_BYTES : 0)));
  tma_copy3d(smem_u32(smraw + slot * G::SLOT_BYTES), tmap, cx, cy, q, bar);
  if (eo) tma_copy4d(smem_u32(smraw + G::EO_OFF + slot * G::EO_SLOT), emap, i0, j0, q, 0, bar);
}

template <typename R, int EPI>
__global__ void __launch_bounds__(NTHR, sizeof(R) == 4 ? 3 : 2)
    k_apply_tma(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap emap, OpArgs<R> a,
                Extra<R> ex, const typename CT<R>::C *__restrict__ x,
                                                    typename CT<R>::C *__restrict__ y,
                                                    const typename CT<R>::C *__restrict__ aux0, RedBuf red, int fin,
                                                    KScalars *sc, int *errflag) {
  using G = TmaGeom<R>;
  extern __shared__ __align__(128) unsigned char smdyn[];
  // TMA destinations must be 128-byte aligned
  unsigned char *smraw = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smdyn) + 127) & ~uintptr_t(127));
  TmaE<R> E{smraw};
  HTile<R> &H = *reinterpret_cast<HTile<R> *>(smraw + G::H_OFF);
  CoefTile<R> &T = *reinterpret_cast<CoefTile<R> *>(smraw + G::T_OFF);
  OffTile<R> &O = *reinterpret_cast<OffTile<R> *>(smraw + G::O_OFF);
  ZTile<R> &Z = *reinterpret_cast<ZTile<R> *>(smraw + G::Z_OFF);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smraw + G::BAR_OFF);
  pdl_trigger();

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int k0 = blockIdx.z * ex.kchunk;
  const int k1 = min(k0 + ex.kchunk, a.N[2]);
  const int gi = i0 + tx, gj = j0 + ty;
  const bool active = (gi < a.N[0]) && (gj < a.N[1]);
  const long long tilecol = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  const int kfirst = k0 - 1;  // planes kfirst … k1 are needed
  const int cx = 6 * (i0 - G::XOFF), cy = j0 - 1;
  // the tile's x/y coefficient tables (−1 … T) lie outside the PML
  const bool rxy = i0 - 1 >= a.rlo[0] && i0 + TX <= a.rhi[0] && j0 - 1 >= a.rlo[1] && j0 + TY <= a.rhi[1];
  Accs<R> acc;
  bool ok = true;

  // prologue on static data, overlapping the previous kernel's tail
  if (tid == 0) {
    for (int s = 0; s < G::NSLOT; ++s) mbar_init(smem_u32(&bars[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
    if (ex.eoff_tma) asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&emap)) : "memory");
  }
  fill_coef<R>(T, a, i0, j0, tid);
  {
    // z tables over kfirst … k1 (k1 − kfirst ≤ KCMAX + 1); flags are 0
    // outside the grid
    const int t = tid - 128;  // warps 4 … 6, clear of fill_coef's threads
    const int q = kfirst + t;
    if (t >= 0 && q <= k1) {
      Z.cm[t] = a.cm[2][cidx(a, 2, q)];
      if (q >= 0 && q < a.N[2]) {
        Z.ce[t] = a.ce[2][q];
        Z.wm[t] = a.wm[2][q];
        Z.wp[t] = a.wp[2][q];
      }
      Z.flag[t] = (q >= 0 && q < a.N[2] && offd_on(a, tilecol, q)) ? 1 : 0;
    }
  }
  pdl_wait();
  if (sc != nullptr && sc->done) return;
  __syncthreads();
  if (tid == 0) {
    for (int p = 0; p < G::NSLOT; ++p) {
      const int q = kfirst + p;
      if (q <= k1) issue_plane<R>(smraw, bars, &tmap, &emap, ex, Z, cx, cy, i0, j0, k0, q, p);
    }
  }
  // Only warp 0 polls the mbarriers; the block then joins at bar.sync, which
  // orders the landed tile for every thread (polling from all warps would
  // burn issue slots the computing warps need).  Pinned-DOF fix-ups run only
  // in CTAs that touch the low walls, by warp 0 right after its wait (tid is
  // its lane), before that barrier.
  // A wait that gives up stops the whole block at the next barrier
  // (__syncthreads_and), so no further copy is issued into a slot whose
  // previous copy may still be in flight; the block then drains what it
  // issued (below) and reports FDFD_ERR_TIMEOUT through errflag.
  const bool warp0 = tid < 32;
  const bool wall = (i0 == 0) || (j0 == 0);
  if (warp0) {
    ok = mbar_wait(smem_u32(&bars[0]), 0, ex.wait_limit);
    ok = ok && mbar_wait(smem_u32(&bars[1]), 0, ex.wait_limit);
    // planes kfirst = k0 − 1 and k0: the z = 0 wall plane is among them when k0 ≤ 1
    if (ok && (wall || k0 <= 1)) {
      pin_fixup<R>(E, 0, i0, j0, kfirst, tid);
      pin_fixup<R>(E, 1, i0, j0, k0, tid);
    }
  }
  int kstop = k0;  // planes up to kstop + 2 have been issued
  bool run = __syncthreads_and(ok) != 0;
  // H(k0−1) at the thread's own cell (the output of plane k0 reads no
  // neighbour of it)
  typename CT<R>::C hxp, hyp;
  {
    Own<R> o;
    curl_e<R, false>(E, T, Z.cm[0], 0, 1, tx, ty, o);
    hxp = o.hx;
    hyp = o.hy;
  }
  bool zvalid = false;  // zc[k & 1] already holds plane k's z-directed corners

  for (int k = k0; run && k < k1; ++k) {
    const int pm = k - 1 - kfirst, p0 = k - kfirst, p1 = k + 1 - kfirst;
    const int sm = pm % G::NSLOT, s0 = p0 % G::NSLOT, s1 = p1 % G::NSLOT;
    Pre<R> pf;
    if (active) prefetch<R, EPI>(pf, a, aux0, gi + (long long)a.N[0] * (gj + (long long)a.N[1] * k));
    if (warp0) {
      ok = mbar_wait(smem_u32(&bars[s1]), (p1 / G::NSLOT) & 1, ex.wait_limit);
      if (ok && wall) pin_fixup<R>(E, s1, i0, j0, k + 1, tid);
    }
    // E(k+1) present and fixed up; the previous plane's reads of H are done
    if (!__syncthreads_and(ok)) {
      run = false;
      kstop = k;
      break;
    }
    Own<R> own;
    const bool rc = rxy && k >= a.rlo[2] && k <= a.rhi[2];
    // corner staging first, then H: the values H leaves in registers for the
    // output stage are then not live across the staging
    const int zt = k - kfirst;
    const bool offd = Z.flag[zt] != 0;
    if (offd) {
      const bool eo = G::EO_SLOT > 0 && ex.eoff_tma;
      const EoffSrc<R> e0{eo ? reinterpret_cast<const R *>(smraw + G::EO_OFF + s0 * G::EO_SLOT) : nullptr};
      const EoffSrc<R> e1{eo ? reinterpret_cast<const R *>(smraw + G::EO_OFF + s1 * G::EO_SLOT) : nullptr};
      stage_xy<R>(E, O, T, a, e0, Z.wm[zt], Z.wp[zt], i0, j0, k, sm, s0, tid);
      if (!zvalid) stage_z<R>(E, O, T, a, e0, i0, j0, k, s0, tid);
      stage_z<R>(E, O, T, a, e1, i0, j0, k + 1, s1, tid);
    }
    zvalid = offd;
    if (rc) compute_h<R, true>(E, H, T, Z.cm[zt], s0, s1, tx, ty, tid, own);
    else compute_h<R, false>(E, H, T, Z.cm[zt], s0, s1, tx, ty, tid, own);
    __syncthreads();  // H(k), staged corners complete; nobody reads E(k−1) any more
    // refill E(k−1)'s slot (and its ε slot) right away: the output stage reads
    // only E(k), H and the staged corners, and the next iteration's first
    // barrier orders this plane's reads of H/corners before they are rewritten
    if (tid == 0) {
      const int q = k + G::NSLOT - 1;  // the plane this freed slot takes
      if (q <= k1) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_plane<R>(smraw, bars, &tmap, &emap, ex, Z, cx, cy, i0, j0, k0, q, sm);
      }
    }
    if (active) {
      if (rc) output_cell<R, EPI, false, true>(H, T, O, a, ex, pf, own, hxp, hyp, x, y, gi, gj, k, tx, ty, offd, Z.ce[zt], acc);
      else output_cell<R, EPI, false, false>(H, T, O, a, ex, pf, own, hxp, hyp, x, y, gi, gj, k, tx, ty, offd, Z.ce[zt], acc);
    }
    hxp = own.hx;
    hyp = own.hy;
  }
  if (!run) {
    // a bounded wait gave up: report it and wait (with the full limit) for
    // the last copy issued into each slot — planes kfirst … min(k1, kstop+2),
    // plane q in slot (q − kfirst) mod NSLOT as phase (q − kfirst) / NSLOT —
    // so no copy lands in this block's shared memory after it exits
    if (tid == 0) {
      atomicExch(errflag, 1);
      const int qlast = min(k1, kstop + 2);
      for (int q = max(kfirst, qlast - G::NSLOT + 1); q <= qlast; ++q)
        mbar_wait(smem_u32(&bars[(q - kfirst) % G::NSLOT]), ((q - kfirst) / G::NSLOT) & 1);
    }
  }
  __syncthreads();  // no thread leaves while tid 0 may still drain copies into this block's memory
  if (EPI != EPI_STORE) {
    sum_finalise<NTHR>(acc.r0, acc.i0, acc.r1, red, fin, sc);
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
  for (int w = 0; w < 3; ++w) {
    a.rlo[w] = h->rlo[w];
    a.rhi[w] = h->rhi[w];
  }
  a.w2 = mk(R(h->w2[0]), R(h->w2[1]));
  return a;
}
template OpArgs<float> op_args<float>(const fdfd_handle *);
template OpArgs<double> op_args<double>(const fdfd_handle *);

// z-chunk length (planes per CTA).  autotune_kchunk picks it per precision
// at fdfd_create; FDFD_KCHUNK overrides; until then a heuristic aims at
// about three resident CTAs per SM.
static int kchunk_heuristic(const fdfd_handle *h) {
  const int tiles = ((h->N[0] + TX - 1) / TX) * ((h->N[1] + TY - 1) / TY);
  const int target = 152 * 3;
  int nz = (target + tiles - 1) / tiles;
  if (nz < 1) nz = 1;
  int kc = (h->N[2] + nz - 1) / nz;
  if (kc < 4) kc = 4;
  if (kc > 64) kc = 64;
  return kc;
}

static int kchunk_for(const fdfd_handle *h, bool c64) {
  if (h->kc_force > 0) return std::min(h->kc_force, KCMAX);
  const int t = h->kc[c64 ? 1 : 0];
  return t > 0 ? t : kchunk_heuristic(h);
}

static int blocks_for(const fdfd_handle *h, int kc) {
  return ((h->N[0] + TX - 1) / TX) * ((h->N[1] + TY - 1) / TY) * ((h->N[2] + kc - 1) / kc);
}

int apply_blocks(const fdfd_handle *h) {
  const int a = blocks_for(h, kchunk_for(h, true)), b = blocks_for(h, kchunk_for(h, false));
  return std::max(std::max(a, b), std::max(h->nwork[0], h->nwork[1]));
}

template <typename R>
Extra<R> make_extra(const fdfd_handle *h) {
  using C = typename CT<R>::C;
  Extra<R> ex;
  ex.kchunk = kchunk_for(h, sizeof(R) == 4);
  ex.eoff_tma = 0;
  ex.ediag_tma = 0;
  ex.oflag_w = nullptr;
  ex.wait_limit = h->wait_limit;
  ex.work = nullptr;
  const C *coef;
  if constexpr (sizeof(R) == 8) coef = reinterpret_cast<const C *>(h->coef64);
  else coef = reinterpret_cast<const C *>(h->coef32);
  const int st = h->coef_stride;
  for (int w = 0; w < 3; ++w) {
    ex.sdle[w] = coef + 4 * st + h->coef_off[w];
    ex.sdlm[w] = coef + 5 * st + h->coef_off[w];
    ex.ph[w] = mk(R(h->e_ikl[w][0]), R(h->e_ikl[w][1]));
    const double d2 = h->e_ikl[w][0] * h->e_ikl[w][0] + h->e_ikl[w][1] * h->e_ikl[w][1];
    ex.phinv[w] = mk(R(h->e_ikl[w][0] / d2), R(-h->e_ikl[w][1] / d2));
  }
  return ex;
}
template Extra<float> make_extra<float>(const fdfd_handle *);
template Extra<double> make_extra<double>(const fdfd_handle *);

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // resolved once (a function-local static is initialised thread-safely)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    cudaGetLastError();
    return nullptr;
  }();
  return fn;
}
PFN_cuTensorMapEncodeTiled_v12000 tensor_encode_fn() { return encode_fn(); }

// The TMA kernel serves PEC (non-Bloch) walls, the forward operator, 16-byte
// aligned inputs and an x row pitch that is a multiple of 16 bytes.
template <typename R>
static bool tma_ok(const fdfd_handle *h, const void *x, bool transpose) {
  if (transpose || h->tma_disabled) return false;
  if (h->bloch[0] || h->bloch[1] || h->bloch[2]) return false;
  if ((reinterpret_cast<uintptr_t>(x) & 15) != 0) return false;
  if (((long long)h->N[0] * 6 * (long long)sizeof(R)) % 16 != 0) return false;
  return encode_fn() != nullptr;
}

template <typename R>
static int make_map(fdfd_handle *h, const void *x, CUtensorMap *map) {
  using G = TmaGeom<R>;
  const cuuint64_t dims[3] = {(cuuint64_t)6 * h->N[0], (cuuint64_t)h->N[1], (cuuint64_t)h->N[2]};
  const cuuint64_t strides[2] = {(cuuint64_t)6 * h->N[0] * sizeof(R), (cuuint64_t)6 * h->N[0] * h->N[1] * sizeof(R)};
  const cuuint32_t box[3] = {(cuuint32_t)(6 * G::XW), (cuuint32_t)EY, 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = encode_fn()(map, sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                           const_cast<void *>(x), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(h, FDFD_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return FDFD_OK;
}

// Off-diagonal ε (complex64 operator) as a 4D tensor (x, y, z, pair) for the
// shared-memory ring; needs an x pitch that is a multiple of 16 bytes.
static bool emap_ok(const fdfd_handle *h) {
  return h->has_off && h->eoff32 != nullptr && (h->N[0] % 4) == 0 &&
         (reinterpret_cast<uintptr_t>(h->eoff32) & 15) == 0;
}
static int make_emap(fdfd_handle *h, CUtensorMap *map) {
  using G = TmaGeom<float>;
  const cuuint64_t dims[4] = {(cuuint64_t)h->N[0], (cuuint64_t)h->N[1], (cuuint64_t)h->N[2], 3};
  const cuuint64_t strides[3] = {(cuuint64_t)h->N[0] * 4, (cuuint64_t)h->N[0] * h->N[1] * 4,
                                 (cuuint64_t)h->ncell * 4};
  const cuuint32_t box[4] = {(cuuint32_t)G::EOX, (cuuint32_t)(TY + 1), 1u, 3u};
  const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
  CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->eoff32, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(h, FDFD_ERR_CUDA, "cuTensorMapEncodeTiled(eps off-diagonal) failed");
  return FDFD_OK;
}

template <typename R, int EPI, bool TR>
static int launch_t(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y,
                    const typename CT<R>::C *aux0, int fin, KScalars *sc) {
  Extra<R> ex = make_extra<R>(h);
  dim3 grid((h->N[0] + TX - 1) / TX, (h->N[1] + TY - 1) / TY, (h->N[2] + ex.kchunk - 1) / ex.kchunk);
  dim3 block(TX, TY, 1);
  const OpArgs<R> a = op_args<R>(h);
  if (EPI != EPI_STORE) {
    int rc = ensure_red(h, (int)(grid.x * grid.y * grid.z));
    if (rc) return rc;
  }
  const int d = h->dev;
  if (!TR && EPI != EPI_DOT_SU && tma_ok<R>(h, x, TR)) {
    const int rc2 = launch_apply_v2<R>(h, x, y, EPI, aux0, fin, sc, ex.kchunk);
    if (rc2 != FDFD_ERR_UNSUPPORTED) return rc2;
  }
  if (!TR && tma_ok<R>(h, x, TR)) {
    static DevFlags attr_tma;
    const int smem = TmaGeom<R>::SMEM;
    if (!attr_tma.done(d)) {
      cudaError_t e = cudaFuncSetAttribute(k_apply_tma<R, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply_tma)");
      // shared memory, not L1, limits how many CTAs fit on an SM
      e = cudaFuncSetAttribute(k_apply_tma<R, EPI>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(carveout)");
      attr_tma.set(d);
    }
    CUtensorMap map, emap;
    int rc = make_map<R>(h, x, &map);
    if (rc) return rc;
    emap = map;  // placeholder unless the ε ring is used
    if (sizeof(R) == 4 && emap_ok(h)) {
      if ((rc = make_emap(h, &emap))) return rc;
      ex.eoff_tma = 1;
    }
    const cudaError_t e = launch_k(h, k_apply_tma<R, EPI>, grid, block, (size_t)smem, map, emap, a, ex, x, y, aux0,
                                   h->red, fin, sc, h->dev_err);
    h->launches++;
    return cuda_check(h, e, "k_apply_tma launch");
  }
  static DevFlags attr_set;
  const size_t smem = sizeof(PlainSmem<R>);
  if (!attr_set.done(d)) {
    cudaError_t e = cudaFuncSetAttribute(k_apply<R, EPI, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply)");
    attr_set.set(d);
  }
  const cudaError_t e = launch_k(h, k_apply<R, EPI, TR>, grid, block, smem, a, ex, x, y, aux0, h->red, fin, sc);
  h->launches++;
  return cuda_check(h, e, "k_apply launch");
}

// Reads a buffer larger than L2: evicts the operands of the next launch and,
// unlike a memset, leaves no dirty lines whose write-back would be charged
// to it.  The sink is written only if the running xor meets a value the
// buffer's contents never produce, which keeps the loads.
__global__ void k_read_flush(const uint4 *__restrict__ p, size_t n, unsigned *sink) {
  unsigned acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = p[i];
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (acc == 0x9e3779b9u) *sink = acc;
}

// Seeded values in [−1, 1) (the shadow vector's hash): the tuning input, so
// that no candidate is timed on all-zero data.
template <typename R>
__global__ void k_fill_hash(typename CT<R>::C *x, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = shadow<R>(i);
}

// Rows per warp strip of the second TMA kernel's layout (its tiles are 8
// strips high).
static int v2_rows_per_warp(const fdfd_handle *h, bool c64) {
  if (!c64) return 1;
  return (h->op_variant == 1 || h->op_variant == 3) ? 1 : 2;
}

// Balanced z-chunk schedule of the second TMA kernel for tiles of 8·rw rows.
// In each (x tile, y tile) column a plane costs 1, or 1 + wcorner when a
// warp strip of the tile-plane carries off-diagonal ε terms (every warp then
// waits at the plane's barrier for that strip's corner work).  Each column
// is cut at even cost thresholds into the fewest chunks of at most about
// total/target cost (and at most KCMAX planes), and the chunks are listed
// heaviest first, so that a launch of more than one wave starts them first.
static void build_schedule(const fdfd_handle *h, const std::vector<uint8_t> &strip_flags, int rw, int target,
                           double wcorner, std::vector<int4> &out) {
  const int tyt = 8 * rw;
  const int tx = (h->N[0] + TX - 1) / TX, ty = (h->N[1] + tyt - 1) / tyt, nz = h->N[2];
  const int strips_y = (h->N[1] + rw - 1) / rw;
  std::vector<double> cost((size_t)tx * ty * nz);
  double total = 0;
  for (int by = 0; by < ty; ++by)
    for (int bx = 0; bx < tx; ++bx)
      for (int q = 0; q < nz; ++q) {
        bool f = false;
        for (int st = 0; st < 8 && !strip_flags.empty() && !f; ++st) {
          const int tr = by * 8 + st;
          if (tr < strips_y) f = strip_flags[((size_t)bx + (size_t)tx * tr) * nz + q] != 0;
        }
        const double c = f ? 1.0 + wcorner : 1.0;
        cost[((size_t)by * tx + bx) * nz + q] = c;
        total += c;
      }
  // the per-column chunk counts round up: raise the goal until the total
  // fits the target (a one-wave schedule must not spill into a second wave)
  const int min_per_col = (nz + KCMAX - 1) / KCMAX;
  std::vector<double> colcost((size_t)tx * ty, 0.0);
  for (size_t col = 0; col < colcost.size(); ++col)
    for (int q = 0; q < nz; ++q) colcost[col] += cost[col * nz + q];
  double goal_all = total / std::max(1, target);
  for (int it = 0; it < 200; ++it) {
    long long count = 0;
    for (const double cc : colcost) count += std::max((int)std::ceil(cc / goal_all - 1e-9), min_per_col);
    if (count <= target) break;
    goal_all *= 1.02;
  }
  std::vector<std::pair<double, int4>> chunks;
  for (int by = 0; by < ty; ++by)
    for (int bx = 0; bx < tx; ++bx) {
      const double *c = &cost[((size_t)by * tx + bx) * nz];
      double left_cost = colcost[(size_t)by * tx + bx];
      int left = std::max((int)std::ceil(left_cost / goal_all - 1e-9), min_per_col);
      int q = 0;
      while (q < nz) {
        const double goal = left_cost / std::max(left, 1);
        const int k0 = q;
        double acc = 0;
        while (q < nz && q - k0 < KCMAX) {
          acc += c[q++];
          if (left > 1 && acc >= goal - 1e-9) break;
        }
        chunks.push_back({acc, make_int4(bx, by, k0, q)});
        left_cost -= acc;
        left = std::max(left - 1, 1);
      }
    }
  std::stable_sort(chunks.begin(), chunks.end(),
                   [](const std::pair<double, int4> &a, const std::pair<double, int4> &b) { return a.first > b.first; });
  out.resize(chunks.size());
  for (size_t i = 0; i < chunks.size(); ++i) out[i] = chunks[i].second;
}

// Autotuner for the z-chunk length (and, for complex64, the tile layout of
// the second TMA kernel, and for both its balanced schedules): times y = A x
// for each candidate with CUDA events on the handle's stream — one warm-up,
// then five launches each preceded by an L2 flush (a 192 MiB read, larger
// than the 129 MB L2), the median counting — so the choice holds for inputs
// streamed from HBM, and keeps the fastest, separately for complex64 and
// complex128.  Runs at fdfd_create (vacuum ε) and again whenever new ε data
// switches the off-diagonal tensor on or off, since the corner-term work
// changes the best chunk length.
int autotune_kchunk(fdfd_handle *h) {
  if (h->kc_force > 0) return FDFD_OK;
  for (int p = 0; p < 2; ++p) {  // uniform chunks until a schedule wins again
    cudaFree(h->work[p]);
    h->work[p] = nullptr;
    h->nwork[p] = 0;
  }
  const size_t n = 3 * (size_t)h->ncell;
  const size_t flush_bytes = 192ull << 20;
  void *bx = nullptr, *by = nullptr, *fl = nullptr;
  if (dev_malloc(&bx, n * sizeof(double2)) != cudaSuccess || dev_malloc(&by, n * sizeof(double2)) != cudaSuccess ||
      dev_malloc(&fl, flush_bytes) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(bx);
    cudaFree(by);
    return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(autotune buffers) failed");
  }
  int rc = cuda_check(h, cudaMemsetAsync(fl, 0, flush_bytes, h->stream), "memset");
  const int cand[] = {4, 6, 8, 12, 16, 24, 32, 48, 64};
  const bool verbose = std::getenv("FDFD_VERBOSE") != nullptr;
  // complex64 also picks the tile layout of the second TMA kernel (two rows
  // per warp with a 4-slot ring; one row per warp with 3 or 2 CTAs per SM)
  // unless FDFD_OPERATOR_V2 fixed it; complex128 has one layout
  const bool tune_layout = h->op_variant != 0 && std::getenv("FDFD_OPERATOR_V2") == nullptr;
  const int layouts_c64[] = {4, 1, 3};
  int sms = 152;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->dev) != cudaSuccess) {
    cudaGetLastError();
    sms = 152;
  }
  for (int prec = 0; prec < 2 && rc == FDFD_OK; ++prec) {
    // median of five launches of the current configuration, each after an L2 flush
    auto timed = [&](float *med) -> int {
      auto launch = [&]() {
        return prec == 1 ? launch_apply_fin<float>(h, (const float2 *)bx, (float2 *)by, EPI_STORE, nullptr,
                                                   FIN_NONE, nullptr, false)
                         : launch_apply_fin<double>(h, (const double2 *)bx, (double2 *)by, EPI_STORE, nullptr,
                                                    FIN_NONE, nullptr, false);
      };
      int r2 = launch();
      float ts[5];
      for (int r = 0; r < 5 && r2 == FDFD_OK; ++r) {
        k_read_flush<<<sms * 4, 512, 0, h->stream>>>((const uint4 *)fl, flush_bytes / sizeof(uint4) - 1,
                                                      (unsigned *)fl + flush_bytes / sizeof(unsigned) - 1);
        cudaEventRecord(h->ev0, h->stream);
        r2 = launch();
        cudaEventRecord(h->ev1, h->stream);
        if (r2 || (r2 = cuda_check(h, cudaEventSynchronize(h->ev1), "autotune sync"))) break;
        cudaEventElapsedTime(&ts[r], h->ev0, h->ev1);
      }
      if (r2 == FDFD_OK) {
        std::sort(ts, ts + 5);
        *med = ts[2];
      }
      return r2;
    };
    if (prec == 1) k_fill_hash<float><<<sms * 4, 256, 0, h->stream>>>((float2 *)bx, (long long)n);
    else k_fill_hash<double><<<sms * 4, 256, 0, h->stream>>>((double2 *)bx, (long long)n);
    if ((rc = cuda_check(h, cudaGetLastError(), "k_fill_hash"))) break;
    float best = 1e30f;
    int best_kc = 0, best_layout = h->op_variant;
    std::vector<int4> best_sched;  // empty: uniform chunks
    int4 *dw = nullptr;            // device copy of the schedule being timed
    size_t dw_cap = 0;
    // FDFD_SCHEDULE=w takes the w-wave schedule (weight 1) untimed, 0 none
    const char *fs = std::getenv("FDFD_SCHEDULE");
    const int forced = fs != nullptr ? std::atoi(fs) : -1;
    const int nlay = (prec == 1 && tune_layout) ? 3 : 1;
    for (int li = 0; li < nlay && rc == FDFD_OK; ++li) {
      if (prec == 1 && tune_layout) h->op_variant = layouts_c64[li];
      int last_chunks = -1;
      for (int kc : cand) {
        if (kc > h->N[2] && last_chunks == 1) break;
        const int chunks = (h->N[2] + kc - 1) / kc;
        if (chunks == last_chunks) continue;
        last_chunks = chunks;
        h->kc[prec] = kc;
        float med = 0.f;
        if ((rc = timed(&med))) break;
        if (verbose)
          fprintf(stderr, "fdfd autotune: %s layout %d kchunk %d: %.1f us\n", prec ? "c64" : "c128", h->op_variant,
                  kc, med * 1e3);
        // candidates come in increasing kc (fewer CTAs) and the default
        // layout first: take a later one only if it is clearly faster
        if (med < 0.97f * best && forced <= 0) {
          best = med;
          best_kc = kc;
          best_layout = h->op_variant;
          best_sched.clear();
        }
      }
      // the second TMA kernel can also run a balanced schedule of this
      // layout: columns cut into chunks of equal estimated cost (planes with
      // off-diagonal terms weigh more), for one to four waves of blocks
      if (rc != FDFD_OK || h->op_variant == 0 || forced == 0) continue;
      const int rw = v2_rows_per_warp(h, prec == 1);
      std::vector<uint8_t> flags;
      if (h->has_off && h->oflag_rows[rw - 1] != nullptr) {
        flags.resize((size_t)((h->N[0] + TX - 1) / TX) * ((h->N[1] + rw - 1) / rw) * h->N[2]);
        rc = cuda_check(h, cudaMemcpyAsync(flags.data(), h->oflag_rows[rw - 1], flags.size(), cudaMemcpyDeviceToHost,
                                           h->stream), "copy strip flags");
        if (rc == FDFD_OK) rc = cuda_check(h, cudaStreamSynchronize(h->stream), "stream sync");
      }
      const int slots = sms * ((prec == 1 && h->op_variant == 1) ? 3 : 2);
      const int tyt = 8 * rw;
      const int ncol = ((h->N[0] + TX - 1) / TX) * ((h->N[1] + tyt - 1) / tyt);
      // corner-plane weights 0.25 … 1 for one and two waves, 1 beyond
      for (int waves = 1; waves <= 4 && rc == FDFD_OK; ++waves)
        for (const double wc : {0.25, 0.5, 1.0}) {
          if (rc != FDFD_OK) break;
          if (!h->has_off && wc != 1.0) continue;  // no corner terms: one weight is enough
          if (waves > 2 && wc != 1.0) continue;
          if (forced > 0 && (waves != forced || wc != 1.0)) continue;
          std::vector<int4> sc;
          build_schedule(h, flags, rw, waves * slots, h->has_off ? wc : 0.0, sc);
          // every column's planes once, in chunks of 1 … KCMAX planes, or
          // the schedule is not used
          long long planes = 0;
          bool bad = sc.empty();
          for (const int4 &e : sc) {
            bad = bad || e.w <= e.z || e.w - e.z > KCMAX || e.z < 0 || e.w > h->N[2];
            planes += e.w - e.z;
          }
          if (bad || planes != (long long)ncol * h->N[2]) {
            if (verbose) fprintf(stderr, "fdfd autotune: schedule dropped (bad chunks)\n");
            continue;
          }
          if (sc.size() > dw_cap) {
            cudaFree(dw);
            dw = nullptr;
            dw_cap = 0;
            if (dev_malloc(&dw, sc.size() * sizeof(int4)) != cudaSuccess) {
              cudaGetLastError();
              rc = set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(schedule) failed");
              break;
            }
            dw_cap = sc.size();
          }
          if ((rc = cuda_check(h, cudaMemcpyAsync(dw, sc.data(), sc.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                                  h->stream), "upload schedule")))
            break;
          h->work[prec] = dw;
          h->nwork[prec] = (int)sc.size();
          float med = 0.f;
          rc = timed(&med);
          h->work[prec] = nullptr;
          h->nwork[prec] = 0;
          if (rc) break;
          if (verbose)
            fprintf(stderr, "fdfd autotune: %s layout %d schedule %d waves, weight %.2f (%zu blocks): %.1f us\n",
                    prec ? "c64" : "c128", h->op_variant, waves, h->has_off ? wc : 0.0, sc.size(), med * 1e3);
          if (med < 0.97f * best || (forced > 0 && best_sched.empty())) {
            best = med;
            best_kc = h->kc[prec] > 0 ? h->kc[prec] : 4;
            best_layout = h->op_variant;
            best_sched = sc;
          }
        }
    }
    cudaFree(dw);
    h->kc[prec] = best_kc;
    if (prec == 1 && tune_layout) h->op_variant = best_layout;
    if (rc == FDFD_OK && !best_sched.empty()) {
      int4 *w = nullptr;
      if (dev_malloc(&w, best_sched.size() * sizeof(int4)) != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(schedule) failed");
      } else {
        rc = cuda_check(h, cudaMemcpyAsync(w, best_sched.data(), best_sched.size() * sizeof(int4),
                                           cudaMemcpyHostToDevice, h->stream), "upload schedule");
        h->work[prec] = w;
        h->nwork[prec] = (int)best_sched.size();
      }
    }
  }
  cudaFree(bx);
  cudaFree(by);
  cudaFree(fl);
  h->launches = 0;
  if (rc == FDFD_OK) rc = check_dev_err(h);
  if (rc == FDFD_OK) h->tuned_off = h->has_off ? 1 : 0;
  return rc;
}

// FP64 residual launcher whose block partials, arrival counter and
// finalisation scalars live in caller-provided device memory (used by the
// allocation-free entry point).  The plain-load kernel takes any z-chunk
// length, so when the tuned chunk would need more than `max_blocks` partial
// slots the chunk is lengthened (up to the whole z extent) until the grid
// fits; only an (x, y) tiling larger than `max_blocks` is rejected.
int launch_residual_ext(fdfd_handle *h, const double2 *x, double2 *r, const double2 *b, RedBuf red, int max_blocks,
                        KScalars *sc) {
  const size_t smem = sizeof(PlainSmem<double>);
  cudaError_t e =
      cudaFuncSetAttribute(k_apply<double, EPI_RESID, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply)");
  Extra<double> ex = make_extra<double>(h);
  const long long tiles = (long long)((h->N[0] + TX - 1) / TX) * ((h->N[1] + TY - 1) / TY);
  if (tiles > max_blocks)
    return set_error(h, FDFD_ERR_ARG, "the grid's x-y tiling needs more thread blocks than the fixed reduction "
                                      "scratch holds");
  // smallest chunk length at or above the tuned one whose grid fits
  const long long zmax = max_blocks / tiles;  // ≥ 1
  const int kmin = (int)((h->N[2] + zmax - 1) / zmax);
  if (ex.kchunk < kmin) ex.kchunk = kmin;
  dim3 grid((h->N[0] + TX - 1) / TX, (h->N[1] + TY - 1) / TY, (h->N[2] + ex.kchunk - 1) / ex.kchunk);
  if ((long long)grid.x * grid.y * grid.z > max_blocks)
    return set_error(h, FDFD_ERR_ARG, "grid needs more thread blocks than the fixed reduction scratch holds");
  const OpArgs<double> a = op_args<double>(h);
  k_apply<double, EPI_RESID, false><<<grid, dim3(TX, TY, 1), smem, h->stream>>>(a, ex, x, r, b, red, FIN_NONE, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_apply launch");
}

// Full-control launcher (epilogue + finalisation mode).
template <typename R>
int launch_apply_fin(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                     const typename CT<R>::C *aux0, int fin, KScalars *sc, bool transpose) {
  if (h->ft == FDFD_HH) {
    if (transpose) return set_error(h, FDFD_ERR_UNSUPPORTED, "transpose of the H formulation");
    return launch_apply_hh<R>(h, x, y, epi, aux0, fin, sc);
  }
  if (transpose) {
    switch (epi) {
      case EPI_STORE: return launch_t<R, EPI_STORE, true>(h, x, y, aux0, fin, sc);
      case EPI_RESID: return launch_t<R, EPI_RESID, true>(h, x, y, aux0, fin, sc);
      case EPI_DOT_AUX: return launch_t<R, EPI_DOT_AUX, true>(h, x, y, aux0, fin, sc);
      case EPI_DOT_TS: return launch_t<R, EPI_DOT_TS, true>(h, x, y, aux0, fin, sc);
      case EPI_DOT_SHD: return launch_t<R, EPI_DOT_SHD, true>(h, x, y, aux0, fin, sc);
    }
  } else {
    switch (epi) {
      case EPI_STORE: return launch_t<R, EPI_STORE, false>(h, x, y, aux0, fin, sc);
      case EPI_RESID: return launch_t<R, EPI_RESID, false>(h, x, y, aux0, fin, sc);
      case EPI_DOT_AUX: return launch_t<R, EPI_DOT_AUX, false>(h, x, y, aux0, fin, sc);
      case EPI_DOT_TS: return launch_t<R, EPI_DOT_TS, false>(h, x, y, aux0, fin, sc);
      case EPI_DOT_SU: return launch_t<R, EPI_DOT_SU, false>(h, x, y, aux0, fin, sc);
      case EPI_DOT_SHD: return launch_t<R, EPI_DOT_SHD, false>(h, x, y, aux0, fin, sc);
    }
  }
  return set_error(h, FDFD_ERR_ARG, "bad epilogue kind");
}
template int launch_apply_fin<float>(fdfd_handle *, const float2 *, float2 *, int, const float2 *, int, KScalars *,
                                     bool);
template int launch_apply_fin<double>(fdfd_handle *, const double2 *, double2 *, int, const double2 *, int,
                                      KScalars *, bool);

}  // namespace fdfd
