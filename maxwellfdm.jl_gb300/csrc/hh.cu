// The H-field formulation (ft = HH in create_A / create_b,
// src/model/model.jl:238-240, 266-268):
//     y = A_H h,   A_H = Cₑ·(Pε \ Cₘ) − ω²·Pμ     (Pμ = I here)
// applied matrix-free on the same Yee grid and boundaries as the E operator:
// E' = ε⁻¹ ⊙ (Cₘ h) by backward differences of H (ghost H(−1) mirrors H(0)
// on a symmetry wall, Bloch axes wrap with the phase), then the forward
// differences of Cₑ back onto the H samples, with E' = 0 on the pinned
// tangential samples of the low walls and on the PEC ghost plane N.  Like
// the reference (whose Pε \ Cₘ needs a diagonal Pε), this path takes a
// diagonal ε only.
//
// Kernel: a CTA owns a 32×8 (x, y) tile and marches along z with a 3-slot
// ring of H planes (one-cell halo) and a 2-slot ring of E' planes over the
// tile plus its high halo (0 … T), so each plane's E' is computed once and
// used for planes k and k−1.  The same fused epilogues as the E operator
// provide the dot products of a BiCGSTAB step.
#include <cuda_runtime.h>

#include "krylov_fin.cuh"
#include "operator_common.cuh"

namespace fdfd {

namespace {

constexpr int HEX = TX + 2, HEY = TY + 2;  // H tile −1 … T
constexpr int PEX = TX + 1, PEY = TY + 1;  // E' tile 0 … T

template <typename R>
struct HHSmem {
  using C = typename CT<R>::C;
  C h[3][3][HEY][HEX];  // [slot][component][jj+1][ii+1]
  C e[2][3][PEY][PEX];  // [slot][component][jj][ii]
  C cex[TX + 2], cey[TY + 2], cmx[TX + 2], cmy[TY + 2];
};

// H component c at (possibly ghost) cell g: symmetry wall → the mirror at
// −1 (H(−1) = H(0)); past the high end the value is never used on a
// symmetry axis (E' there is 0), read as 0; Bloch → periodic with phase.
template <typename R>
__device__ __forceinline__ typename CT<R>::C load_h(const typename CT<R>::C *__restrict__ x, const OpArgs<R> &a,
                                                    const Extra<R> &ex, int gi, int gj, int gk, int c) {
  using C = typename CT<R>::C;
  int g[3] = {gi, gj, gk};
  C ph = mk(R(1), R(0));
  bool phased = false;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    if (g[v] < 0) {
      if (a.bloch[v]) { g[v] += a.N[v]; ph = cmul(ph, ex.phinv[v]); phased = true; }
      else g[v] = 0;
    } else if (g[v] >= a.N[v]) {
      if (a.bloch[v]) { g[v] -= a.N[v]; ph = cmul(ph, ex.ph[v]); phased = true; }
      else return czero<C>();
    }
  }
  C val = x[c + 3 * ((long long)g[0] + (long long)a.N[0] * ((long long)g[1] + (long long)a.N[1] * g[2]))];
  if (phased) val = cmul(val, ph);
  return val;
}

template <typename R>
__device__ __forceinline__ void load_hplane(HHSmem<R> &S, const OpArgs<R> &a, const Extra<R> &ex,
                                            const typename CT<R>::C *__restrict__ x, int i0, int j0, int k, int slot,
                                            int tid) {
  for (int p = tid; p < HEX * HEY; p += NTHR) {
    const int ii = p % HEX - 1, jj = p / HEX - 1;
#pragma unroll
    for (int c = 0; c < 3; ++c) S.h[slot][c][jj + 1][ii + 1] = load_h<R>(x, a, ex, i0 + ii, j0 + jj, k, c);
  }
}

// E'(q) = ε⁻¹ ⊙ Cₘ h over the tile plus its high halo, from H(q) (slot sq)
// and H(q−1) (slot sqm), into E' slot `eslot`.
template <typename R>
__device__ __forceinline__ void compute_ep(HHSmem<R> &S, const OpArgs<R> &a, int i0, int j0, int q, int sq, int sqm,
                                           int eslot, int tid) {
  using C = typename CT<R>::C;
  // plane q past the high end of a symmetry axis, or pinned on the low wall
  const bool zghost = !a.bloch[2] && q >= a.N[2];
  const bool zpin = !a.bloch[2] && q == 0;
  const int qz = q >= a.N[2] ? q - a.N[2] : q;
  const C cez = a.ce[2][cidx(a, 2, q)];
  for (int p = tid; p < PEX * PEY; p += NTHR) {
    const int ii = p % PEX, jj = p / PEX;
    int gi = i0 + ii, gj = j0 + jj;
    const bool ghost = zghost || (!a.bloch[0] && gi >= a.N[0]) || (!a.bloch[1] && gj >= a.N[1]);
    C ex_ = czero<C>(), ey_ = czero<C>(), ez_ = czero<C>();
    if (!ghost) {
      const C hx = S.h[sq][0][jj + 1][ii + 1], hy = S.h[sq][1][jj + 1][ii + 1], hz = S.h[sq][2][jj + 1][ii + 1];
      const C hxj = S.h[sq][0][jj][ii + 1], hzj = S.h[sq][2][jj][ii + 1];    // j − 1
      const C hyi = S.h[sq][1][jj + 1][ii], hzi = S.h[sq][2][jj + 1][ii];    // i − 1
      const C hxk = S.h[sqm][0][jj + 1][ii + 1], hyk = S.h[sqm][1][jj + 1][ii + 1];  // k − 1
      const C cex = S.cex[ii + 1], cey = S.cey[jj + 1];
      if (gi >= a.N[0]) gi -= a.N[0];  // Bloch wrap (ghost otherwise)
      if (gj >= a.N[1]) gj -= a.N[1];
      const long long cell = gi + (long long)a.N[0] * (gj + (long long)a.N[1] * qz);
      const bool pi = !a.bloch[0] && gi == 0, pj = !a.bloch[1] && gj == 0;
      if (!(pj || zpin))
        ex_ = cscale(csub(cmul(cey, csub(hz, hzj)), cmul(cez, csub(hy, hyk))), R(1) / a.eps[cell]);
      if (!(pi || zpin))
        ey_ = cscale(csub(cmul(cez, csub(hx, hxk)), cmul(cex, csub(hz, hzi))), R(1) / a.eps[a.ncell + cell]);
      if (!(pi || pj))
        ez_ = cscale(csub(cmul(cex, csub(hy, hyi)), cmul(cey, csub(hx, hxj))), R(1) / a.eps[2 * a.ncell + cell]);
    }
    S.e[eslot][0][jj][ii] = ex_;
    S.e[eslot][1][jj][ii] = ey_;
    S.e[eslot][2][jj][ii] = ez_;
  }
}

}  // namespace

template <typename R, int EPI>
__global__ void __launch_bounds__(NTHR, 2) k_apply_hh(OpArgs<R> a, Extra<R> ex, const typename CT<R>::C *__restrict__ x,
                                                      typename CT<R>::C *__restrict__ y,
                                                      const typename CT<R>::C *__restrict__ aux0, RedBuf red, int fin,
                                                      KScalars *sc) {
  using C = typename CT<R>::C;
  extern __shared__ __align__(16) unsigned char smraw[];
  HHSmem<R> &S = *reinterpret_cast<HHSmem<R> *>(smraw);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int k0 = blockIdx.z * ex.kchunk;
  const int k1 = min(k0 + ex.kchunk, a.N[2]);
  const int gi = i0 + tx, gj = j0 + ty;
  const bool active = gi < a.N[0] && gj < a.N[1];
  ShortAcc<R> r0, i0acc, r1;

  if (tid < TX + 2) {
    const int c = cidx(a, 0, i0 + tid - 1);
    S.cex[tid] = a.ce[0][c];
    S.cmx[tid] = a.cm[0][c];
  } else if (tid >= 64 && tid < 64 + TY + 2) {
    const int t = tid - 64;
    const int c = cidx(a, 1, j0 + t - 1);
    S.cey[t] = a.ce[1][c];
    S.cmy[t] = a.cm[1][c];
  }
  if (sc != nullptr && sc->done) return;
  // H(k0−1), H(k0), H(k0+1); E'(k0)
  load_hplane<R>(S, a, ex, x, i0, j0, k0 - 1, (k0 + 2) % 3, tid);
  load_hplane<R>(S, a, ex, x, i0, j0, k0, k0 % 3, tid);
  load_hplane<R>(S, a, ex, x, i0, j0, k0 + 1, (k0 + 1) % 3, tid);
  __syncthreads();
  compute_ep<R>(S, a, i0, j0, k0, k0 % 3, (k0 + 2) % 3, k0 & 1, tid);

  for (int k = k0; k < k1; ++k) {
    const int sm = (k + 2) % 3, s0 = k % 3, s1 = (k + 1) % 3;
    const int e0 = k & 1, e1 = (k + 1) & 1;
    __syncthreads();  // H(k+1) loaded, E'(k) complete, the previous outputs are done with E'(k−1)
    compute_ep<R>(S, a, i0, j0, k + 1, s1, s0, e1, tid);
    __syncthreads();
    if (active) {
      const long long cell = gi + (long long)a.N[0] * (gj + (long long)a.N[1] * k);
      const C cmx = S.cmx[tx + 1], cmy = S.cmy[ty + 1], cmz = a.cm[2][k];
      const C ex0 = S.e[e0][0][ty][tx], ey0 = S.e[e0][1][ty][tx], ez0 = S.e[e0][2][ty][tx];
      const C exj = S.e[e0][0][ty + 1][tx], ezj = S.e[e0][2][ty + 1][tx];   // j + 1
      const C eyi = S.e[e0][1][ty][tx + 1], ezi = S.e[e0][2][ty][tx + 1];   // i + 1
      const C exk = S.e[e1][0][ty][tx], eyk = S.e[e1][1][ty][tx];           // k + 1
      C yx = csub(cmul(cmy, csub(ezj, ez0)), cmul(cmz, csub(eyk, ey0)));
      C yy = csub(cmul(cmz, csub(exk, ex0)), cmul(cmx, csub(ezi, ez0)));
      C yz = csub(cmul(cmx, csub(eyi, ey0)), cmul(cmy, csub(exj, ex0)));
      const C hx = S.h[s0][0][ty + 1][tx + 1], hy = S.h[s0][1][ty + 1][tx + 1], hz = S.h[s0][2][ty + 1][tx + 1];
      yx = csub(yx, cmul(a.w2, hx));
      yy = csub(yy, cmul(a.w2, hy));
      yz = csub(yz, cmul(a.w2, hz));
      if (EPI == EPI_RESID) {
        yx = csub(aux0[3 * cell], yx);
        yy = csub(aux0[3 * cell + 1], yy);
        yz = csub(aux0[3 * cell + 2], yz);
        r0.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
      } else if (EPI == EPI_DOT_AUX) {
        const C d0 = cdotc(aux0[3 * cell], yx), d1 = cdotc(aux0[3 * cell + 1], yy), d2 = cdotc(aux0[3 * cell + 2], yz);
        r0.add(d0.x + d1.x + d2.x);
        i0acc.add(d0.y + d1.y + d2.y);
      } else if (EPI == EPI_DOT_SHD) {
        const C d0 = cdotc(shadow<R>(3 * cell), yx), d1 = cdotc(shadow<R>(3 * cell + 1), yy),
                d2 = cdotc(shadow<R>(3 * cell + 2), yz);
        r0.add(d0.x + d1.x + d2.x);
        i0acc.add(d0.y + d1.y + d2.y);
      } else if (EPI == EPI_DOT_TS) {
        const C d0 = cdotc(yx, hx), d1 = cdotc(yy, hy), d2 = cdotc(yz, hz);
        r0.add(d0.x + d1.x + d2.x);
        i0acc.add(d0.y + d1.y + d2.y);
        r1.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
      }
      y[3 * cell] = yx;
      y[3 * cell + 1] = yy;
      y[3 * cell + 2] = yz;
    }
    // H(k−1)'s slot takes H(k+2): E'(k+1) (done) was its last reader; the
    // next iteration's first barrier orders the load before its use
    if (k + 1 < k1) load_hplane<R>(S, a, ex, x, i0, j0, k + 2, sm, tid);
  }
  if (EPI != EPI_STORE) {
    sum_finalise<NTHR>(r0, i0acc, r1, red, fin, sc);
  }
}

template <typename R, int EPI>
static int launch_hh_t(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y,
                       const typename CT<R>::C *aux0, int fin, KScalars *sc) {
  const Extra<R> ex = make_extra<R>(h);
  dim3 grid((h->N[0] + TX - 1) / TX, (h->N[1] + TY - 1) / TY, (h->N[2] + ex.kchunk - 1) / ex.kchunk);
  if (EPI != EPI_STORE) {
    int rc = ensure_red(h, (int)(grid.x * grid.y * grid.z));
    if (rc) return rc;
  }
  const size_t smem = sizeof(HHSmem<R>);
  static DevFlags attr;
  if (!attr.done(h->dev)) {
    cudaError_t e = cudaFuncSetAttribute(k_apply_hh<R, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply_hh)");
    attr.set(h->dev);
  }
  const OpArgs<R> a = op_args<R>(h);
  k_apply_hh<R, EPI><<<grid, dim3(TX, TY, 1), smem, h->stream>>>(a, ex, x, y, aux0, h->red, fin, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_apply_hh launch");
}

template <typename R>
int launch_apply_hh(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                    const typename CT<R>::C *aux0, int fin, KScalars *sc) {
  if (h->has_off) return set_error(h, FDFD_ERR_UNSUPPORTED, "the H formulation needs a diagonal ε (Pε \\ Cₘ)");
  switch (epi) {
    case EPI_STORE: return launch_hh_t<R, EPI_STORE>(h, x, y, aux0, fin, sc);
    case EPI_RESID: return launch_hh_t<R, EPI_RESID>(h, x, y, aux0, fin, sc);
    case EPI_DOT_AUX: return launch_hh_t<R, EPI_DOT_AUX>(h, x, y, aux0, fin, sc);
    case EPI_DOT_TS: return launch_hh_t<R, EPI_DOT_TS>(h, x, y, aux0, fin, sc);
    case EPI_DOT_SHD: return launch_hh_t<R, EPI_DOT_SHD>(h, x, y, aux0, fin, sc);
  }
  return set_error(h, FDFD_ERR_UNSUPPORTED, "this reduction is not available for the H formulation");
}
template int launch_apply_hh<float>(fdfd_handle *, const float2 *, float2 *, int, const float2 *, int, KScalars *);
template int launch_apply_hh<double>(fdfd_handle *, const double2 *, double2 *, int, const double2 *, int, KScalars *);

}  // namespace fdfd
