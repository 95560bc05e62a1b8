// Device helpers shared by the operator kernels (stencil.cu) and the field
// post-processing kernels (fields.cu): boundary rules for reading E at a
// possibly-ghost cell, the E dual volume, coefficient indexing.
#pragma once

#include "fdfd_internal.cuh"

namespace fdfd {

constexpr int KCMAX = 64;  // longest z-chunk of the operator kernels (the autotuner's range)

template <typename R>
struct Extra {
  using C = typename CT<R>::C;
  const C *sdle[3];   // s∆lₑ per axis (TRANSPOSE scaling)
  const C *sdlm[3];   // s∆lₘ per axis
  C ph[3], phinv[3];  // Bloch e^{-ikL} and its inverse
  int kchunk;
  int eoff_tma;       // TMA kernel: off-diagonal ε staged through the shared-memory ring
  int ediag_tma;      // second TMA kernel: ε diagonal staged through the ring
  const uint8_t *oflag_w;  // second TMA kernel: off-diagonal flags per x tile, warp strip and plane
  long long wait_limit;  // TMA kernel: SM clocks a pipeline wait may take before it gives up
  const int4 *work;      // second TMA kernel: (x tile, y tile, k0, k1) per block, or null (uniform chunks)
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

// c·v for a coefficient c that is real when RC (tiles outside the PML)
template <bool RC, typename C>
__device__ __forceinline__ C mulc(C c, C v) {
  if constexpr (RC) return cscale(v, c.x);
  else return cmul(c, v);
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

// per-launch extras (s∆l arrays, Bloch phases, z-chunk) of the handle
template <typename R> Extra<R> make_extra(const fdfd_handle *h);

}  // namespace fdfd
