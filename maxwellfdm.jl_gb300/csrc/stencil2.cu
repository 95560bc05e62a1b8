// Matrix-free y = A x, A = Cₘ·Cₑ − ω²·Pε (create_A, src/model/model.jl:225-246,
// from create_curls :160-175 and create_paramops :141-158): the second TMA
// kernel, laid out for the instruction budget of a stencil that has to
// stream 60 B per cell (complex64) at HBM speed.
//
//   * a CTA owns a 32 × TYT (x, y) tile (TYT = 8·RW): warp w owns RW rows,
//     lane = x.  It marches along z over a chunk of planes; one elected
//     thread keeps a ring of NS E planes (one-cell halo, 16-byte aligned x
//     box) filled by cp.async.bulk.tensor, completing on one mbarrier per
//     slot; every thread waits on the mbarrier itself (bounded);
//   * each thread keeps its cells' E(k) and the FP32/FP64 diagonal term
//     ε·E(k) in registers and loads E(k+1) once per plane, so the curls read
//     only the i+1 neighbour (and, for a warp's last row, the j+1 one) from
//     shared memory;
//   * H(k) stays in registers; H(i−1) comes from the neighbouring lane by a
//     warp shuffle, H(j−1) from the row below in registers or — for a
//     warp's first row — from the warp below through a small exchange
//     buffer (double-buffered by plane parity), H(k−1) from the previous
//     plane's registers;
//   * the few values no thread of the tile owns are computed once per
//     plane by different warps: the tile row j0−1 (warp 0), the column
//     i0−1 (warp 1), and on planes carrying off-diagonal ε the corner terms
//     of column i0+32 (warp 2) and row j0+TYT (warp 3);
//   * one __syncthreads per plane (the exchange); the ring slot of plane
//     k−1 is refilled right after it, by the last warp (warp 0 already
//     carries a halo job);
//   * pinned DOFs (tangential E on the low PEC walls, kept in the vector
//     but outside Cₑ) are zeroed as they are loaded, so no fix-up pass
//     touches the ring; the diagonal ε term uses their true values;
//   * off-diagonal ε (only where the 32×8 tile-plane flag is set): each
//     thread forms the corner terms at its own corner from registers and
//     shuffles and averages the two corners around each output.
// It serves the forward operator on PEC walls with 16-byte aligned inputs;
// the first TMA kernel (stencil.cu) keeps the S-weighted COCG epilogue and
// the plain-load kernel Bloch phases and Aᵀ.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "krylov_fin.cuh"
#include "operator_common.cuh"
#include "tma_util.cuh"

namespace fdfd {

PFN_cuTensorMapEncodeTiled_v12000 tensor_encode_fn();

template <typename R, int RW, int NS, bool EDR = true>
struct V2 {
  using C = typename CT<R>::C;
  static constexpr int NW = 8;          // warps per CTA, RW rows each
  static constexpr int NT = NW * 32;
  static constexpr int TYT = NW * RW;   // tile rows
  static constexpr int XOFF = sizeof(R) == 4 ? 2 : 1;
  static constexpr int XW = sizeof(R) == 4 ? TX + 4 : TX + 2;
  static constexpr int BY = TYT + 2;    // box rows j0−1 … j0+TYT
  static constexpr int PLANE_BYTES = XW * BY * 3 * (int)sizeof(C);
  static constexpr int SLOT = (PLANE_BYTES + 127) / 128 * 128;
  static constexpr int KC2 = KCMAX + 2;
  // exchange, per plane parity: H_x, H_z of the row below each warp ([0]:
  // tile row j0−1, [w+1]: warp w's last row), y-directed corner terms of each
  // warp's first row ([w]) and of row j0+TYT ([NW]), H at column i0−1 and the
  // x-directed corner terms at column i0+32 per tile row
  struct Exch {
    C hx[NW + 1][TX];
    C hz[NW + 1][TX];
    C yc[NW + 1][TX];
    C hyh[TYT], hzh[TYT];
    C xce[TYT];
  };
  // complex64: a ring slot per plane for the off-diagonal ε of corners
  // i0 … i0+EOX−1, j0 … j0+TYT, laid out [pair][jj][ii] (EOX·4 bytes a
  // multiple of 16); complex128 reads them from global memory
  static constexpr int EOX = TX + 4, EOY = TYT + 1;
  static constexpr int EO_BYTES = sizeof(R) == 4 ? EOX * EOY * 3 * (int)sizeof(R) : 0;
  static constexpr int EO_SLOT = (EO_BYTES + 127) / 128 * 128;
  static constexpr int EO_OFF = NS * SLOT;
  // complex64: a ring slot per plane for the ε diagonal of the tile's cells,
  // laid out [c][jj][ii]; complex128 loads it from global memory
  static constexpr int ED_BYTES = (EDR && sizeof(R) == 4) ? TX * TYT * 3 * (int)sizeof(R) : 0;
  static constexpr int ED_SLOT = (ED_BYTES + 127) / 128 * 128;
  static constexpr int ED_OFF = EO_OFF + NS * EO_SLOT;
  static constexpr int EXCH_OFF = ED_OFF + NS * ED_SLOT;
  static constexpr int XT_OFF = EXCH_OFF + 2 * (int)sizeof(Exch);
  static constexpr int XT_N = TX + 2;   // x coefficients of columns i0−1 … i0+32
  static constexpr int YT_OFF = XT_OFF + 4 * XT_N * (int)sizeof(C);
  static constexpr int ZT_OFF = YT_OFF + 4 * (TYT + 2) * (int)sizeof(C);
  static constexpr int ZF_OFF = ZT_OFF + 4 * KC2 * (int)sizeof(C);
  static constexpr int ZA_OFF = ZF_OFF + KC2 * NW;  // per plane: any strip flagged
  static constexpr int BAR_OFF = (ZA_OFF + KC2 + 15) / 16 * 16;
  static constexpr int SMEM = BAR_OFF + NS * 8;
  static_assert(SLOT % 128 == 0 && EXCH_OFF % 128 == 0, "TMA destination alignment");
  static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
  static_assert(XW * 6 <= 256, "TMA box inner extent");
};

template <typename R, int RW, int NS>
__device__ __forceinline__ typename CT<R>::C ev2(const unsigned char *sm, int s, int c, int jj, int ii) {
  using G = V2<R, RW, NS>;
  return reinterpret_cast<const typename CT<R>::C *>(sm + s * G::SLOT)[((jj + 1) * G::XW + ii + G::XOFF) * 3 + c];
}

template <typename C>
__device__ __forceinline__ C zif(bool z, C v) {
  return z ? czero<C>() : v;
}

template <typename C>
__device__ __forceinline__ C shfl_up1(C v) {
  return mk(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
}
template <typename C>
__device__ __forceinline__ C shfl_down1(C v) {
  return mk(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
}


// Complex64 arithmetic of the curls and the diagonal term on the paired FP32
// instructions of sm_100 and later (__fadd2_rn, __fmul2_rn, __ffma2_rn:
// both lanes rounded to nearest, as the scalar forms are), half the
// instructions of the scalar forms; complex128 keeps the scalar forms.
__device__ __forceinline__ float2 f2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ double2 psub(double2 a, double2 b) { return csub(a, b); }
// a·s + b for real s
__device__ __forceinline__ float2 pfma(float2 a, float s, float2 b) { return __ffma2_rn(a, f2(s), b); }
__device__ __forceinline__ double2 pfma(double2 a, double s, double2 b) { return cadd(cscale(a, s), b); }
// a·u − b·v for coefficients a, b that are real when RC
template <bool RC>
__device__ __forceinline__ float2 pdiff(float2 a, float2 u, float2 b, float2 v) {
  if constexpr (RC) {
    return __ffma2_rn(f2(a.x), u, __fmul2_rn(f2(-b.x), v));
  } else {
    float2 t = __fmul2_rn(make_float2(b.y, -b.y), make_float2(v.y, v.x));  // −b·v
    t = __ffma2_rn(f2(-b.x), v, t);
    t = __ffma2_rn(make_float2(-a.y, a.y), make_float2(u.y, u.x), t);     // + a·u
    return __ffma2_rn(f2(a.x), u, t);
  }
}
template <bool RC>
__device__ __forceinline__ double2 pdiff(double2 a, double2 u, double2 b, double2 v) {
  return csub(mulc<RC>(a, u), mulc<RC>(b, v));
}
// conj(a0)·b0 + conj(a1)·b1 + conj(a2)·b2
__device__ __forceinline__ float2 pdot3(float2 a0, float2 b0, float2 a1, float2 b1, float2 a2, float2 b2) {
  float2 t = __fmul2_rn(f2(a0.x), b0);
  t = __ffma2_rn(make_float2(a0.y, -a0.y), make_float2(b0.y, b0.x), t);
  t = __ffma2_rn(f2(a1.x), b1, t);
  t = __ffma2_rn(make_float2(a1.y, -a1.y), make_float2(b1.y, b1.x), t);
  t = __ffma2_rn(f2(a2.x), b2, t);
  return __ffma2_rn(make_float2(a2.y, -a2.y), make_float2(b2.y, b2.x), t);
}
__device__ __forceinline__ double2 pdot3(double2 a0, double2 b0, double2 a1, double2 b1, double2 a2, double2 b2) {
  return cadd(cadd(cdotc(a0, b0), cdotc(a1, b1)), cdotc(a2, b2));
}
// a·u + b·v for coefficients a, b that are real when RC (corner averaging)
template <bool RC>
__device__ __forceinline__ float2 wsum(float2 a, float2 u, float2 b, float2 v) {
  return cadd(mulc<RC>(a, u), mulc<RC>(b, v));
}
template <bool RC>
__device__ __forceinline__ double2 wsum(double2 a, double2 u, double2 b, double2 v) {
  return cadd(mulc<RC>(a, u), mulc<RC>(b, v));
}
// u·s + v·t for real s, t
__device__ __forceinline__ float2 pmix(float2 u, float s, float2 v, float t) {
  return __ffma2_rn(u, f2(s), __fmul2_rn(v, f2(t)));
}
__device__ __forceinline__ double2 pmix(double2 u, double s, double2 v, double t) {
  return cadd(cscale(u, s), cscale(v, t));
}
// (u + v)·s for real s
__device__ __forceinline__ float2 psums(float2 u, float2 v, float s) { return __fmul2_rn(__fadd2_rn(u, v), f2(s)); }
__device__ __forceinline__ double2 psums(double2 u, double2 v, double s) { return cscale(cadd(u, v), s); }

template <typename R>
struct Accs2 {
  ShortAcc<R> r0, i0, r1;
};

template <typename R>
__device__ __forceinline__ R eoff_at(const OpArgs<R> &a, int p, int gi, int gj, int gk) {
  // off-diagonal pair p at corner (gi, gj, gk); PEC ghost corners (index N) are 0
  if (gi >= a.N[0] || gj >= a.N[1] || gk >= a.N[2]) return R(0);
  return __ldg(&a.eoff[(long long)p * a.ncell + gi + (long long)a.N[0] * (gj + (long long)a.N[1] * gk)]);
}

template <typename R, int EPI, int RW, int NS, int MB, bool EDR>
__global__ void __launch_bounds__(V2<R, RW, NS, EDR>::NT, MB)
    k_apply_v2(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap emap,
               const __grid_constant__ CUtensorMap dmap, OpArgs<R> a,
               Extra<R> ex, const typename CT<R>::C *__restrict__ x, typename CT<R>::C *__restrict__ y,
               const typename CT<R>::C *__restrict__ aux0, RedBuf red, int fin, KScalars *sc, int *errflag) {
  using G = V2<R, RW, NS, EDR>;
  using C = typename CT<R>::C;
  using X = typename G::Exch;
  constexpr int NW = G::NW, TYT = G::TYT, KC2 = G::KC2;
  // indexed directly (not through a realigned generic pointer) so that every
  // access compiles to a shared-memory load with a 32-bit address
  extern __shared__ __align__(128) unsigned char sm[];
  X *xch = reinterpret_cast<X *>(sm + G::EXCH_OFF);
  C *xt = reinterpret_cast<C *>(sm + G::XT_OFF);
  C *yt = reinterpret_cast<C *>(sm + G::YT_OFF);
  C *zt = reinterpret_cast<C *>(sm + G::ZT_OFF);
  unsigned char *zf = sm + G::ZF_OFF;
  unsigned char *za = sm + G::ZA_OFF;
  uint64_t *bars = reinterpret_cast<uint64_t *>(sm + G::BAR_OFF);
  pdl_trigger();

  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  // the block's column (x tile, y tile) and planes [k0, k1): uniform
  // chunks of ex.kchunk planes, or an entry of the balanced schedule
  int bx = blockIdx.x, by = blockIdx.y, k0 = blockIdx.z * ex.kchunk, k1;
  if (ex.work != nullptr) {
    const int4 wk = ex.work[blockIdx.x];
    bx = wk.x;
    by = wk.y;
    k0 = wk.z;
    k1 = wk.w;
  } else {
    k1 = min(k0 + ex.kchunk, a.N[2]);
  }
  const int tiles_x = (a.N[0] + TX - 1) / TX;
  const int i0 = bx * TX, j0 = by * TYT;
  const int kfirst = k0 - 1;
  const int gi = i0 + lane;
  const int cx = 6 * (i0 - G::XOFF), cy = j0 - 1;
  const int jw = RW * w;  // the warp's first tile row
  const int tiles_yr = (a.N[1] + RW - 1) / RW;
  const bool ering = G::EO_SLOT > 0 && ex.eoff_tma != 0;
  const bool edr = G::ED_SLOT > 0 && ex.ediag_tma != 0;

  // TMA destinations need 128-byte alignment; the declared alignment gives
  // it, checked here once (every thread returns together, before any copy)
  if ((smem_u32(sm) & 127u) != 0u) {
    if (tid == 0) atomicExch(errflag, 2);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(smem_u32(&bars[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
    if (ering) asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&emap)) : "memory");
    if (edr) asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&dmap)) : "memory");
  }
  pdl_wait();
  if (sc != nullptr && sc->done) return;  // every thread, before any copy is issued
  // the first planes' E tiles go out now, so their latency overlaps the
  // coefficient tables below; each slot's single arrival (and its ε tiles,
  // which need the off-diagonal flags) follows once the tables are in place
  if (tid == 0) {
    for (int p = 0; p < NS; ++p) {
      const int q = kfirst + p;
      if (q <= k1) {
        const uint32_t bar = smem_u32(&bars[p]);
        mbar_expect_only(bar, (uint32_t)G::PLANE_BYTES);
        tma_copy3d(smem_u32(sm + p * G::SLOT), &tmap, cx, cy, q, bar);
      }
    }
  }
  if (tid >= 160 && tid < 160 + TX + 2) {  // x coefficients, columns −1 … TX
    const int t = tid - 160;
    const int c = cidx(a, 0, i0 + t - 1);
    xt[t] = a.cm[0][c];
    xt[(TX + 2) + t] = a.ce[0][c];
    xt[2 * (TX + 2) + t] = a.wm[0][c];
    xt[3 * (TX + 2) + t] = a.wp[0][c];
  }
  if (tid < TYT + 2) {  // y coefficients, tile rows −1 … TYT
    const int c = cidx(a, 1, j0 + tid - 1);
    yt[tid] = a.cm[1][c];
    yt[(TYT + 2) + tid] = a.ce[1][c];
    yt[2 * (TYT + 2) + tid] = a.wm[1][c];
    yt[3 * (TYT + 2) + tid] = a.wp[1][c];
  }
  {  // z coefficients and off-diagonal flags over planes kfirst … k1 (k1 − kfirst ≤ KCMAX + 1)
    const int t = tid - 64;
    const int q = kfirst + t;
    if (t >= 0 && t < KC2 && q <= k1) {
      const int c = cidx(a, 2, q);
      zt[t] = a.cm[2][c];
      zt[KC2 + t] = a.ce[2][c];
      zt[2 * KC2 + t] = a.wm[2][c];
      zt[3 * KC2 + t] = a.wp[2][c];
      // one flag per warp strip (RW rows): its outputs at plane q read a
      // non-zero off-diagonal ε (the 32×8 tile flags stand in when the
      // strip flags are absent)
      unsigned char any = 0;
#pragma unroll
      for (int s = 0; s < NW; ++s) {
        const int tr = j0 / RW + s;
        unsigned char f = 0;
        if (a.eoff != nullptr && q >= 0 && q < a.N[2] && tr < tiles_yr) {
          if (ex.oflag_w != nullptr) f = ex.oflag_w[(bx + (long long)tiles_x * tr) * a.N[2] + q];
          else if (a.oflag != nullptr) f = a.oflag[(bx + (long long)tiles_x * ((tr * RW) / 8)) * a.N[2] + q];
          else f = 1;
        }
        zf[t * NW + s] = f;
        any |= f;
      }
      za[t] = any;
    }
  }
  const int cxi = cidx(a, 0, gi);
  const C cmx = a.cm[0][cxi], cex = a.ce[0][cxi];
  // real coefficient ranges for this warp: columns i0−1 … i0+32, rows jw−1 … jw+RW
  const bool rx = i0 - 1 >= a.rlo[0] && i0 + TX <= a.rhi[0];
  const bool ry = j0 + jw - 1 >= a.rlo[1] && j0 + jw + RW <= a.rhi[1];

  __syncthreads();
  // the copies of plane q into ring slot s: the E tile, and the off-diagonal
  // ε of the tile when plane q or q−1 carries off-diagonal terms (the
  // z-directed corners of q serve both); with_e = false completes a slot
  // whose E tile is already on its way
  auto issue = [&](int q, int s, bool with_e) {
    bool eo = false;
    if (ering) {
      const int t = q - kfirst;
      eo = za[t] != 0 || (t > 0 && za[t - 1] != 0);
    }
    const uint32_t bar = smem_u32(&bars[s]);
    const uint32_t bytes = (with_e ? G::PLANE_BYTES : 0) + (eo ? G::EO_BYTES : 0) + (edr ? G::ED_BYTES : 0);
    if (bytes) mbar_expect_only(bar, bytes);
    if (with_e) tma_copy3d(smem_u32(sm + s * G::SLOT), &tmap, cx, cy, q, bar);
    if (eo) tma_copy4d(smem_u32(sm + G::EO_OFF + s * G::EO_SLOT), &emap, i0, j0, q, 0, bar);
    if (edr) tma_copy4d(smem_u32(sm + G::ED_OFF + s * G::ED_SLOT), &dmap, i0, j0, q, 0, bar);
    mbar_arrive(bar);
  };
  if (tid == 0) {
    for (int p = 0; p < NS; ++p) {
      const int q = kfirst + p;
      if (q <= k1) issue(q, p, false);
    }
  }
  // off-diagonal pair p at tile corner (ii, jj) of the plane in slot s
  // (plane gk): the ε ring, or global memory
  auto eps_off = [&](int s, int p, int jj, int ii, int gk) -> R {
    if (ering) return reinterpret_cast<const R *>(sm + G::EO_OFF + s * G::EO_SLOT)[(p * G::EOY + jj) * G::EOX + ii];
    return eoff_at(a, p, i0 + ii, j0 + jj, gk);
  };

  Accs2<R> acc;
  int kstop = k0;
  bool run = true;
  const int plane = a.N[0] * a.N[1];  // 3·Ncell < 2³¹ (checked at launch)
  const int nc = (int)a.ncell;

  // The march over the chunk.  WALL: the CTA touches a low PEC wall (i0 or j0
  // = 0, or planes from k0 − 1 ≤ 0) and may meet pinned DOFs; the other CTAs
  // run without the pin selects.
  auto march = [&](auto wall_tag) {
    constexpr bool WALL = decltype(wall_tag)::value;
    bool ok = mbar_wait_sleep(smem_u32(&bars[0]), 0, ex.wait_limit, 100000u);
    ok = ok && mbar_wait_sleep(smem_u32(&bars[1]), 0, ex.wait_limit, 100000u);
    const bool pin_i = WALL && gi == 0;  // PEC x wall: E_y, E_z at i = 0 are pinned
    C eo[RW][3];         // E(k), pinned DOFs zeroed
    C od[RW][3];         // off-diagonal ε terms of plane k (½ of each corner around an output)
    C hxp[RW], hyp[RW];  // H_x, H_y at k−1
    C ezp[RW];           // E_z(k−1), pinned zeroed
    C zcn[RW];           // z-directed corner term at plane k (valid when zvalid)
    bool zvalid = false;
    bool pin_j[RW], act[RW];
    int cell[RW];  // cell index at plane k
#pragma unroll
    for (int r = 0; r < RW; ++r) {
      const int gj = j0 + jw + r;
      pin_j[r] = WALL && gj == 0;
      act[r] = gi < a.N[0] && gj < a.N[1];
      cell[r] = gi + a.N[0] * gj + plane * k0;
      zcn[r] = czero<C>();
    }
    {
      const bool zpin0 = WALL && k0 == 0, zpinm = WALL && kfirst == 0;
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const int jj = jw + r;
        const C v0 = ev2<R, RW, NS>(sm, 1, 0, jj, lane), v1 = ev2<R, RW, NS>(sm, 1, 1, jj, lane),
                v2 = ev2<R, RW, NS>(sm, 1, 2, jj, lane);
        eo[r][0] = zif(pin_j[r] || zpin0, v0);
        eo[r][1] = zif(pin_i || zpin0, v1);
        eo[r][2] = zif(pin_i || pin_j[r], v2);
      }
      const C cmzm = zt[0];
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const int jj = jw + r;
        const C cmy = yt[jj + 1];
        const C mx = zif(pin_j[r] || zpinm, ev2<R, RW, NS>(sm, 0, 0, jj, lane));
        const C my = zif(pin_i || zpinm, ev2<R, RW, NS>(sm, 0, 1, jj, lane));
        const C mz = zif(pin_i || pin_j[r], ev2<R, RW, NS>(sm, 0, 2, jj, lane));
        const C mzi = zif(pin_j[r], ev2<R, RW, NS>(sm, 0, 2, jj, lane + 1));
        const C mzj = zif(pin_i, ev2<R, RW, NS>(sm, 0, 2, jj + 1, lane));
        hxp[r] = csub(cmul(cmy, csub(mzj, mz)), cmul(cmzm, csub(eo[r][1], my)));
        hyp[r] = csub(cmul(cmzm, csub(eo[r][0], mx)), cmul(cmx, csub(mzi, mz)));
        ezp[r] = mz;
      }
    }
    run = !__syncthreads_or(!ok);

    // ring slots of planes k−1, k, k+1 and the phase parity expected next in
    // each slot, advanced without divisions
    int sm1 = 0, s0 = 1, s1 = 2 % NS;
    unsigned phase = 0x3u;  // slots 0 and 1 have completed phase 0
    for (int k = k0; run && k < k1; ++k) {
      const int p0 = k - kfirst;
      X &xc_ = xch[k & 1];
      const bool z0 = WALL && k == 0;
      // diagonal ε (when it does not come through the ring) and the epilogue
      // operand at plane k: their latency overlaps this plane's curls
      R epk[RW][3];
      C aux[RW][3];
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        epk[r][0] = epk[r][1] = epk[r][2] = R(0);
        if (!edr && act[r]) {
          epk[r][0] = a.eps[cell[r]];
          epk[r][1] = a.eps[nc + cell[r]];
          epk[r][2] = a.eps[2 * nc + cell[r]];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) od[r][c] = czero<C>();
        if (EPI == EPI_RESID || EPI == EPI_DOT_AUX) {
          if (act[r]) {
            aux[r][0] = aux0[3 * cell[r]];
            aux[r][1] = aux0[3 * cell[r] + 1];
            aux[r][2] = aux0[3 * cell[r] + 2];
          }
        }
      }
      ok = mbar_wait_sleep(smem_u32(&bars[s1]), (phase >> s1) & 1u, ex.wait_limit, 100000u);
      phase ^= 1u << s1;
      const C cmz = zt[p0], cez = zt[KC2 + p0];
      const bool rc = rx && ry && k >= a.rlo[2] && k <= a.rhi[2];
      // E(k+1) at the thread's cells (true values; the curls take the pinned
      // entries as 0)
      C en[RW][3];
#pragma unroll
      for (int r = 0; r < RW; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) en[r][c] = ev2<R, RW, NS>(sm, s1, c, jw + r, lane);
      }
      // ---- H(k) at the thread's cells
      C hx[RW], hy[RW], hz[RW];
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const int jj = jw + r;
        const C cmy = yt[jj + 1];
        const C eyi = zif(z0, ev2<R, RW, NS>(sm, s0, 1, jj, lane + 1));
        const C ezi = zif(pin_j[r], ev2<R, RW, NS>(sm, s0, 2, jj, lane + 1));
        C exj, ezj;
        if (r + 1 < RW) {
          exj = eo[r + 1][0];
          ezj = eo[r + 1][2];
        } else {
          exj = zif(z0, ev2<R, RW, NS>(sm, s0, 0, jj + 1, lane));
          ezj = zif(pin_i, ev2<R, RW, NS>(sm, s0, 2, jj + 1, lane));
        }
        const C eny = zif(pin_i, en[r][1]), enx = zif(pin_j[r], en[r][0]);
        if (rc) {
          hx[r] = pdiff<true>(cmy, psub(ezj, eo[r][2]), cmz, psub(eny, eo[r][1]));
          hy[r] = pdiff<true>(cmz, psub(enx, eo[r][0]), cmx, psub(ezi, eo[r][2]));
          hz[r] = pdiff<true>(cmx, psub(eyi, eo[r][1]), cmy, psub(exj, eo[r][0]));
        } else {
          hx[r] = pdiff<false>(cmy, psub(ezj, eo[r][2]), cmz, psub(eny, eo[r][1]));
          hy[r] = pdiff<false>(cmz, psub(enx, eo[r][0]), cmx, psub(ezi, eo[r][2]));
          hz[r] = pdiff<false>(cmx, psub(eyi, eo[r][1]), cmy, psub(exj, eo[r][0]));
        }
      }
      // last row's H_x, H_z for the warp above
      xc_.hx[w + 1][lane] = hx[RW - 1];
      xc_.hz[w + 1][lane] = hz[RW - 1];
      if (w == 0) {
        // tile row j0−1 (its values reach only outputs of pinned DOFs when j0 = 0)
        const C cmy = yt[0];
        const C mx = zif(z0, ev2<R, RW, NS>(sm, s0, 0, -1, lane));
        const C my = zif(pin_i || z0, ev2<R, RW, NS>(sm, s0, 1, -1, lane));
        const C mz = zif(pin_i, ev2<R, RW, NS>(sm, s0, 2, -1, lane));
        const C myk = zif(pin_i, ev2<R, RW, NS>(sm, s1, 1, -1, lane));
        const C myi = zif(z0, ev2<R, RW, NS>(sm, s0, 1, -1, lane + 1));
        xc_.hx[0][lane] = csub(cmul(cmy, csub(eo[0][2], mz)), cmul(cmz, csub(myk, my)));
        xc_.hz[0][lane] = csub(cmul(cmx, csub(myi, my)), cmul(cmy, csub(eo[0][0], mx)));
      } else if (w == 1 && lane < TYT) {
        // column i0−1, tile row `lane` (reaches only pinned outputs when i0 = 0)
        const int jj = lane;
        const bool pj = WALL && j0 + jj == 0, pi0 = WALL && i0 == 0;
        const C cmy = yt[jj + 1], cmh = xt[0];
        const C ex_k = zif(pj || z0, ev2<R, RW, NS>(sm, s0, 0, jj, -1));
        const C ex_k1 = zif(pj, ev2<R, RW, NS>(sm, s1, 0, jj, -1));
        const C ey_ = zif(z0, ev2<R, RW, NS>(sm, s0, 1, jj, -1));
        const C ez_ = zif(pj, ev2<R, RW, NS>(sm, s0, 2, jj, -1));
        const C exj = zif(z0, ev2<R, RW, NS>(sm, s0, 0, jj + 1, -1));
        const C ey0 = zif(pi0 || z0, ev2<R, RW, NS>(sm, s0, 1, jj, 0));
        const C ez0 = zif(pi0 || pj, ev2<R, RW, NS>(sm, s0, 2, jj, 0));
        xc_.hyh[jj] = csub(cmul(cmz, csub(ex_k1, ex_k)), cmul(cmh, csub(ez0, ez_)));
        xc_.hzh[jj] = csub(cmul(cmh, csub(ey0, ey_)), cmul(cmy, csub(exj, ex_k)));
      }
      // ---- off-diagonal ε: corner terms of this warp's cells, folded into the
      // diagonal term (½ of each of the two corners around an output; pinned
      // outputs take none); lane 31's column i0+32 and the last row's row
      // above arrive through the exchange after the barrier
      const bool offd = zf[p0 * NW + w] != 0;
      // corner terms with real averaging weights outside the PML
      auto corners = [&](auto rc_tag) {
        constexpr bool RCW = decltype(rc_tag)::value;
        const C wmx = xt[2 * (TX + 2) + lane + 1], wpx = xt[3 * (TX + 2) + lane + 1];
        const C wmz = zt[2 * KC2 + p0], wpz = zt[3 * KC2 + p0];
#pragma unroll
        for (int r = 0; r < RW; ++r) {
          const int jj = jw + r;
          const C wmy = yt[2 * (TYT + 2) + jj + 1], wpy = yt[3 * (TYT + 2) + jj + 1];
          const C enx = zif(pin_j[r], en[r][0]), eny = zif(pin_i, en[r][1]);
          // E_x(i−1) at k and k+1
          C exm = shfl_up1(eo[r][0]), exm1 = shfl_up1(enx);
          if (lane == 0) {
            exm = zif(pin_j[r] || z0, ev2<R, RW, NS>(sm, s0, 0, jj, -1));
            exm1 = zif(pin_j[r], ev2<R, RW, NS>(sm, s1, 0, jj, -1));
          }
          // E_y(j−1) at k and k+1
          C eym, eym1;
          if (r > 0) {
            eym = eo[r - 1][1];
            eym1 = zif(pin_i, en[r - 1][1]);
          } else {
            eym = zif(pin_i || z0, ev2<R, RW, NS>(sm, s0, 1, jj - 1, lane));
            eym1 = zif(pin_i, ev2<R, RW, NS>(sm, s1, 1, jj - 1, lane));
          }
          const R exy = eps_off(s0, 0, jj, lane, k), eyz = eps_off(s0, 1, jj, lane, k),
                  ezx = eps_off(s0, 2, jj, lane, k);
          const R eyz1 = eps_off(s1, 1, jj, lane, k + 1), ezx1 = eps_off(s1, 2, jj, lane, k + 1);
          const C ax = wsum<RCW>(wmx, exm, wpx, eo[r][0]);
          const C ay = wsum<RCW>(wmy, eym, wpy, eo[r][1]);
          const C az = wsum<RCW>(wmz, ezp[r], wpz, eo[r][2]);
          const C xcv = cadd(cscale(ay, exy), cscale(az, ezx));
          const C ycv = cadd(cscale(ax, exy), cscale(az, eyz));
          const C zc0 = zvalid ? zcn[r] : cadd(cscale(ax, ezx), cscale(ay, eyz));
          const C ax1 = wsum<RCW>(wmx, exm1, wpx, enx);
          const C ay1 = wsum<RCW>(wmy, eym1, wpy, eny);
          const C zc1 = cadd(cscale(ax1, ezx1), cscale(ay1, eyz1));
          zcn[r] = zc1;
          C xn = shfl_down1(xcv);
          if (lane == TX - 1) xn = czero<C>();
          const bool px = pin_j[r] || z0, py = pin_i || z0, pz = pin_i || pin_j[r];
          if (!px) od[r][0] = cscale(cadd(xcv, xn), R(0.5));
          if (!pz) od[r][2] = cscale(cadd(zc0, zc1), R(0.5));
          if (!py) od[r][1] = cscale(ycv, R(0.5));
          if (r > 0) {
            if (!py) od[r - 1][1] = cadd(od[r - 1][1], cscale(ycv, R(0.5)));
          } else {
            xc_.yc[w][lane] = ycv;
          }
        }
      };
      if (offd) {
        if (rc) corners(std::true_type{});
        else corners(std::false_type{});
      } else {
        // a warp without off-diagonal terms leaves zeros for its neighbours
        xc_.yc[w][lane] = czero<C>();
      }
      zvalid = offd;
      if (w == 2 && lane < TYT && zf[p0 * NW + lane / RW]) {
        // x-directed corner terms at column i0+32, tile row `lane`
        const int jj = lane;
        const bool pj = WALL && j0 + jj == 0;
        const C wmy = yt[2 * (TYT + 2) + jj + 1], wpy = yt[3 * (TYT + 2) + jj + 1];
        const C eym = zif(z0, ev2<R, RW, NS>(sm, s0, 1, jj - 1, TX));
        const C ey0 = zif(z0, ev2<R, RW, NS>(sm, s0, 1, jj, TX));
        const C ezm = zif(pj, ev2<R, RW, NS>(sm, sm1, 2, jj, TX));
        const C ez0 = zif(pj, ev2<R, RW, NS>(sm, s0, 2, jj, TX));
        const C ay = wsum<false>(wmy, eym, wpy, ey0);
        const C az = wsum<false>(zt[2 * KC2 + p0], ezm, zt[3 * KC2 + p0], ez0);
        xc_.xce[jj] = cadd(cscale(ay, eps_off(s0, 0, jj, TX, k)), cscale(az, eps_off(s0, 2, jj, TX, k)));
      } else if (w == 3 && zf[p0 * NW + NW - 1]) {
        // y-directed corner terms at row j0+TYT
        const int jj = TYT;
        const C exm = zif(z0, ev2<R, RW, NS>(sm, s0, 0, jj, lane - 1));
        const C ex0 = zif(z0, ev2<R, RW, NS>(sm, s0, 0, jj, lane));
        const C ezm = zif(pin_i, ev2<R, RW, NS>(sm, sm1, 2, jj, lane));
        const C ez0 = zif(pin_i, ev2<R, RW, NS>(sm, s0, 2, jj, lane));
        const C ax = wsum<false>(xt[2 * (TX + 2) + lane + 1], exm, xt[3 * (TX + 2) + lane + 1], ex0);
        const C az = wsum<false>(zt[2 * KC2 + p0], ezm, zt[3 * KC2 + p0], ez0);
        xc_.yc[NW][lane] = cadd(cscale(ax, eps_off(s0, 0, jj, lane, k)), cscale(az, eps_off(s0, 1, jj, lane, k)));
      }
      // ---- all H(k) and corner terms written; planes k and k+1 no longer
      // read after this plane, plane k−1 not at all
      if (__syncthreads_or(!ok)) {
        run = false;
        kstop = k;
        break;
      }
      // the refill goes out from the last warp, which has no halo job
      if (tid == G::NT - 32) {
        const int q = k - 1 + NS;  // the plane that takes plane k−1's slot
        if (q <= k1) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(q, sm1, true);
        }
      }
      // ---- outputs y(k)
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const int jj = jw + r;
        const C cey = yt[(TYT + 2) + jj + 1];
        const C hzjm = r > 0 ? hz[r - 1] : xc_.hz[w][lane];
        const C hxjm = r > 0 ? hx[r - 1] : xc_.hx[w][lane];
        C hzim = shfl_up1(hz[r]), hyim = shfl_up1(hy[r]);
        if (lane == 0) {
          hzim = xc_.hzh[jj];
          hyim = xc_.hyh[jj];
        }
        C yx, yy, yz;
        if (rc) {
          yx = pdiff<true>(cey, psub(hz[r], hzjm), cez, psub(hy[r], hyp[r]));
          yy = pdiff<true>(cez, psub(hx[r], hxp[r]), cex, psub(hz[r], hzim));
          yz = pdiff<true>(cex, psub(hy[r], hyim), cey, psub(hx[r], hxjm));
        } else {
          yx = pdiff<false>(cey, psub(hz[r], hzjm), cez, psub(hy[r], hyp[r]));
          yy = pdiff<false>(cez, psub(hx[r], hxp[r]), cex, psub(hz[r], hzim));
          yz = pdiff<false>(cex, psub(hy[r], hyim), cey, psub(hx[r], hxjm));
        }
        const bool px = pin_j[r] || z0, py = pin_i || z0, pz = pin_i || pin_j[r];
        // Pε E at the cell: the diagonal with the true E (the ring slot of
        // plane k still holds it where eo has a pinned 0) plus the corner terms
        R e0, e1, e2;
        if (edr) {
          const R *edk = reinterpret_cast<const R *>(sm + G::ED_OFF + s0 * G::ED_SLOT);
          e0 = edk[jj * TX + lane];
          e1 = edk[(TYT + jj) * TX + lane];
          e2 = edk[(2 * TYT + jj) * TX + lane];
        } else {
          e0 = epk[r][0];
          e1 = epk[r][1];
          e2 = epk[r][2];
        }
        C t0 = eo[r][0], t1 = eo[r][1], t2 = eo[r][2];
        if (WALL) {
          if (px) t0 = ev2<R, RW, NS>(sm, s0, 0, jj, lane);
          if (py) t1 = ev2<R, RW, NS>(sm, s0, 1, jj, lane);
          if (pz) t2 = ev2<R, RW, NS>(sm, s0, 2, jj, lane);
        }
        C d0 = pfma(t0, e0, od[r][0]), d1 = pfma(t1, e1, od[r][1]), d2 = pfma(t2, e2, od[r][2]);
        if (offd) {
          if (lane == TX - 1 && !px) d0 = pfma(xc_.xce[jj], R(0.5), d0);
          if (r == RW - 1 && !py) d1 = pfma(xc_.yc[w + 1][lane], R(0.5), d1);
        }
        if (WALL) {
          if (px) yx = czero<C>();
          if (py) yy = czero<C>();
          if (pz) yz = czero<C>();
        }
        if (a.w2.y == R(0)) {
          yx = pfma(d0, -a.w2.x, yx);
          yy = pfma(d1, -a.w2.x, yy);
          yz = pfma(d2, -a.w2.x, yz);
        } else {
          yx = csub(yx, cmul(a.w2, d0));
          yy = csub(yy, cmul(a.w2, d1));
          yz = csub(yz, cmul(a.w2, d2));
        }
        if (act[r]) {
          const int ce = cell[r];
          if (EPI == EPI_RESID) {
            yx = csub(aux[r][0], yx);
            yy = csub(aux[r][1], yy);
            yz = csub(aux[r][2], yz);
            acc.r0.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
          } else if (EPI == EPI_DOT_AUX) {
            const C q0 = cdotc(aux[r][0], yx), q1 = cdotc(aux[r][1], yy), q2 = cdotc(aux[r][2], yz);
            acc.r0.add(q0.x + q1.x + q2.x);
            acc.i0.add(q0.y + q1.y + q2.y);
          } else if (EPI == EPI_DOT_TS) {
            // (t, s) with the true input s (its pinned entries are not in eo)
            const C sx = t0, sy = t1, sz = t2;
            const C q0 = cdotc(yx, sx), q1 = cdotc(yy, sy), q2 = cdotc(yz, sz);
            acc.r0.add(q0.x + q1.x + q2.x);
            acc.i0.add(q0.y + q1.y + q2.y);
            acc.r1.add(yx.x * yx.x + yx.y * yx.y + yy.x * yy.x + yy.y * yy.y + yz.x * yz.x + yz.y * yz.y);
          } else if (EPI == EPI_DOT_SHD) {
            const C q = pdot3(shadow<R>(3ll * ce), yx, shadow<R>(3ll * ce + 1), yy, shadow<R>(3ll * ce + 2), yz);
            acc.r0.add(q.x);
            acc.i0.add(q.y);
          }
          C *yo = y + 3 * ce;
          yo[0] = yx;
          yo[1] = yy;
          yo[2] = yz;
        }
      }
      // ---- advance to plane k+1
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        hxp[r] = hx[r];
        hyp[r] = hy[r];
        ezp[r] = eo[r][2];
        eo[r][0] = zif(pin_j[r], en[r][0]);
        eo[r][1] = zif(pin_i, en[r][1]);
        eo[r][2] = zif(pin_i || pin_j[r], en[r][2]);
        cell[r] += plane;
      }
      sm1 = s0;
      s0 = s1;
      s1 = s1 + 1 == NS ? 0 : s1 + 1;
    }
  };
  // a chunk starting at plane 1 reads the z = 0 wall plane as its plane k−1
  if (i0 == 0 || j0 == 0 || k0 <= 1) march(std::true_type{});
  else march(std::false_type{});

  if (!run) {
    // a bounded wait gave up: report it and wait (with the full limit) for
    // the last copy issued into each slot — planes up to min(k1, kstop+NS−2),
    // plane q in slot (q − kfirst) mod NS as phase (q − kfirst) / NS — so no
    // copy lands in this block's shared memory after it exits
    if (tid == 0) {
      atomicExch(errflag, 1);
      const int qlast = min(k1, kstop + NS - 2);
      for (int q = max(kfirst, qlast - NS + 1); q <= qlast; ++q)
        mbar_wait(smem_u32(&bars[(q - kfirst) % NS]), ((q - kfirst) / NS) & 1);
    }
  }
  __syncthreads();
  if (EPI != EPI_STORE) sum_finalise<G::NT>(acc.r0, acc.i0, acc.r1, red, fin, sc);
}

// ------------------------------------------------------------------ host
template <typename R, int RW, int NS>
static int make_map_v2(fdfd_handle *h, const void *x, CUtensorMap *map) {
  using G = V2<R, RW, NS>;
  const cuuint64_t dims[3] = {(cuuint64_t)6 * h->N[0], (cuuint64_t)h->N[1], (cuuint64_t)h->N[2]};
  const cuuint64_t strides[2] = {(cuuint64_t)6 * h->N[0] * sizeof(R), (cuuint64_t)6 * h->N[0] * h->N[1] * sizeof(R)};
  const cuuint32_t box[3] = {(cuuint32_t)(6 * G::XW), (cuuint32_t)G::BY, 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = tensor_encode_fn()(map, sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                                  3, const_cast<void *>(x), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(h, FDFD_ERR_CUDA, "cuTensorMapEncodeTiled (second TMA kernel) failed");
  return FDFD_OK;
}

// Off-diagonal ε (complex64) as a 4D tensor (x, y, z, pair) for the ring;
// needs an x pitch that is a multiple of 16 bytes.
template <typename R, int RW, int NS>
static bool emap_v2(fdfd_handle *h, CUtensorMap *map) {
  using G = V2<R, RW, NS>;
  if (G::EO_SLOT == 0 || !h->has_off || h->eoff32 == nullptr || (h->N[0] % 4) != 0 ||
      (reinterpret_cast<uintptr_t>(h->eoff32) & 15) != 0)
    return false;
  const cuuint64_t dims[4] = {(cuuint64_t)h->N[0], (cuuint64_t)h->N[1], (cuuint64_t)h->N[2], 3};
  const cuuint64_t strides[3] = {(cuuint64_t)h->N[0] * 4, (cuuint64_t)h->N[0] * h->N[1] * 4,
                                 (cuuint64_t)h->ncell * 4};
  const cuuint32_t box[4] = {(cuuint32_t)G::EOX, (cuuint32_t)G::EOY, 1u, 3u};
  const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
  return tensor_encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->eoff32, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ε diagonal (complex64) as a 4D tensor (x, y, z, component) for the ring.
template <typename R, int RW, int NS, bool EDR>
static bool dmap_v2(fdfd_handle *h, CUtensorMap *map) {
  using G = V2<R, RW, NS, EDR>;
  if (G::ED_SLOT == 0 || h->eps32 == nullptr || (h->N[0] % 4) != 0 ||
      (reinterpret_cast<uintptr_t>(h->eps32) & 15) != 0)
    return false;
  const cuuint64_t dims[4] = {(cuuint64_t)h->N[0], (cuuint64_t)h->N[1], (cuuint64_t)h->N[2], 3};
  const cuuint64_t strides[3] = {(cuuint64_t)h->N[0] * 4, (cuuint64_t)h->N[0] * h->N[1] * 4,
                                 (cuuint64_t)h->ncell * 4};
  const cuuint32_t box[4] = {(cuuint32_t)TX, (cuuint32_t)G::TYT, 1u, 3u};
  const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
  return tensor_encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->eps32, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename R, int EPI, int RW, int NS, int MB, bool EDR = true>
static int launch_v2_t(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y,
                       const typename CT<R>::C *aux0, int fin, KScalars *sc, int kc) {
  using G = V2<R, RW, NS, EDR>;
  Extra<R> ex = make_extra<R>(h);
  ex.kchunk = kc;
  dim3 grid((h->N[0] + TX - 1) / TX, (h->N[1] + G::TYT - 1) / G::TYT, (h->N[2] + kc - 1) / kc);
  const int p = sizeof(R) == 4 ? 1 : 0;
  if (h->nwork[p] > 0) {  // the balanced schedule (built for this layout's tile rows)
    ex.work = h->work[p];
    grid = dim3((unsigned)h->nwork[p], 1, 1);
  }
  if (EPI != EPI_STORE) {
    int rc = ensure_red(h, (int)(grid.x * grid.y * grid.z));
    if (rc) return rc;
  }
  static DevFlags attr;
  if (!attr.done(h->dev)) {
    cudaError_t e = cudaFuncSetAttribute(k_apply_v2<R, EPI, RW, NS, MB, EDR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         G::SMEM);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(k_apply_v2)");
    e = cudaFuncSetAttribute(k_apply_v2<R, EPI, RW, NS, MB, EDR>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaFuncSetAttribute(carveout)");
    attr.set(h->dev);
  }
  CUtensorMap map, emap, dmap;
  int rc = make_map_v2<R, RW, NS>(h, x, &map);
  if (rc) return rc;
  emap = map;  // placeholders unless the ε rings are used
  dmap = map;
  ex.eoff_tma = emap_v2<R, RW, NS>(h, &emap) ? 1 : 0;
  ex.ediag_tma = dmap_v2<R, RW, NS, EDR>(h, &dmap) ? 1 : 0;
  ex.oflag_w = h->has_off ? h->oflag_rows[RW - 1] : nullptr;
  const OpArgs<R> a = op_args<R>(h);
  const cudaError_t e = launch_k(h, k_apply_v2<R, EPI, RW, NS, MB, EDR>, grid, dim3(G::NT, 1, 1), (size_t)G::SMEM, map, emap,
                                 dmap, a, ex, x, y, aux0, h->red, fin, sc, h->dev_err);
  h->launches++;
  return cuda_check(h, e, "k_apply_v2 launch");
}

template <typename R, int EPI>
static int launch_v2_e(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y,
                       const typename CT<R>::C *aux0, int fin, KScalars *sc, int kc) {
  if constexpr (sizeof(R) == 8) {
    return launch_v2_t<R, EPI, 1, 4, 2>(h, x, y, aux0, fin, sc, kc);
  } else {
    switch (h->op_variant) {
      case 1: return launch_v2_t<R, EPI, 1, 4, 3>(h, x, y, aux0, fin, sc, kc);
      case 2: return launch_v2_t<R, EPI, 2, 3, 2>(h, x, y, aux0, fin, sc, kc);
      case 3: return launch_v2_t<R, EPI, 1, 4, 2>(h, x, y, aux0, fin, sc, kc);
      default: return launch_v2_t<R, EPI, 2, 4, 2, false>(h, x, y, aux0, fin, sc, kc);
    }
  }
}

// Launch through the second TMA kernel when it serves the call; returns
// FDFD_ERR_UNSUPPORTED (without touching the error string) when it does not.
template <typename R>
int launch_apply_v2(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                    const typename CT<R>::C *aux0, int fin, KScalars *sc, int kc) {
  // cell offsets are 32-bit in the kernel
  if (h->op_variant == 0 || 3 * h->ncell >= (1ll << 31)) return FDFD_ERR_UNSUPPORTED;
  switch (epi) {
    case EPI_STORE: return launch_v2_e<R, EPI_STORE>(h, x, y, aux0, fin, sc, kc);
    case EPI_RESID: return launch_v2_e<R, EPI_RESID>(h, x, y, aux0, fin, sc, kc);
    case EPI_DOT_AUX: return launch_v2_e<R, EPI_DOT_AUX>(h, x, y, aux0, fin, sc, kc);
    case EPI_DOT_TS: return launch_v2_e<R, EPI_DOT_TS>(h, x, y, aux0, fin, sc, kc);
    case EPI_DOT_SHD: return launch_v2_e<R, EPI_DOT_SHD>(h, x, y, aux0, fin, sc, kc);
  }
  return FDFD_ERR_UNSUPPORTED;
}
template int launch_apply_v2<float>(fdfd_handle *, const float2 *, float2 *, int, const float2 *, int, KScalars *, int);
template int launch_apply_v2<double>(fdfd_handle *, const double2 *, double2 *, int, const double2 *, int, KScalars *,
                                     int);

}  // namespace fdfd
