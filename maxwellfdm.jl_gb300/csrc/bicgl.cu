// BiCGStab(ℓ) (Sleijpen & Fokkema, ETNA 1, 1993), ℓ ≤ 4, for the same
// systems as BiCGSTAB: ℓ BiCG steps followed by a minimal-residual
// polynomial of degree ℓ.  On the FDFD operator, whose spectrum has large
// imaginary parts, the degree-1 polynomial of BiCGSTAB stalls where the
// degree-ℓ one does not; it needs markedly fewer operator applications in
// both precisions, for about 1.3× the vector traffic per application.
//
// One cycle = 4ℓ + 3 kernels, all reading their scalars from device memory
// (so a batch of cycles replays as one CUDA graph):
//   for j = 0 … ℓ−1:
//     u_i = r_i − β u_i (i ≤ j)                      k_bl_u (+ the deferred
//                                                    updates of step j−1)
//     u_{j+1} = A u_j, γ = (r̂, u_{j+1}), α = ρ/γ     operator, EPI_DOT_SHD + FIN_ALPHA
//     r_j −= α u_{j+1}; the other r_i and x are      k_bl_r
//     updated by the next k_bl_u (last step: by
//     k_bl_gram and k_bl_fin, on the fly)
//     r_{j+1} = A r_j [, ρ₁ = (r̂, r_{j+1}), β]       operator, EPI_DOT_SHD + FIN_BL_RHO
// r̂ is the generated shadow vector (shadow() in krylov_fin.cuh): no
// memory traffic for it.
//   Gram matrix of r_0 … r_ℓ                                  k_bl_gram
//   minimal-residual coefficients (modified Gram–Schmidt
//   carried out on the Gram matrix, one thread)               k_bl_mr
//   x, r_0, u_0 closing update, (r̂, r_0), ‖r_0‖², stop tests  k_bl_fin + FIN_BL_CYCLE
// The last BiCG step's updates r_i −= α u_{i+1} (i < ℓ−1) and x += α u_0
// are never stored: k_bl_gram and k_bl_fin read r_i and u_{i+1} anyway and
// apply them in registers (only r_0, u_0 and x outlive the cycle), which
// saves nine vector passes per cycle.
// Vectors and products are in the solve's inner precision; every sum
// across threads and blocks is double-float FP32 (complex64) or FP64
// (complex128), in a fixed order.
// The grid-stride vector kernels run one full wave (SM count × the
// kernel's resident blocks per SM), so none ends on a partial wave.
#include <mutex>
#include <unordered_map>

#include "krylov_fin.cuh"

namespace fdfd {

namespace {

constexpr int VB = 256;
constexpr int RED_BLOCKS = 152 * 4;
constexpr int LMAX = 4;

template <typename C>
struct VSet {
  C *v[LMAX + 1];
};

__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 addd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 subd(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 scd(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

template <typename R>
__device__ __forceinline__ long long vstride() { return (long long)gridDim.x * VB; }

// Two consecutive complex elements per access (16-byte loads for complex64).
template <typename C> struct Pair { C a, b; };
__device__ __forceinline__ Pair<float2> ldp(const float2 *__restrict__ p, long long q) {
  const float4 v = reinterpret_cast<const float4 *>(p)[q];
  return {make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ Pair<double2> ldp(const double2 *__restrict__ p, long long q) {
  return {p[2 * q], p[2 * q + 1]};
}
__device__ __forceinline__ void stp(float2 *p, long long q, Pair<float2> v) {
  reinterpret_cast<float4 *>(p)[q] = make_float4(v.a.x, v.a.y, v.b.x, v.b.y);
}
__device__ __forceinline__ void stp(double2 *p, long long q, Pair<double2> v) {
  p[2 * q] = v.a;
  p[2 * q + 1] = v.b;
}

// Grid-stride visit of element pairs (n is even: 3·Ncell with Ncell ≥ 2 …
// an odd tail element is still handled, by block 0 thread 0).
template <typename F2, typename F1>
__device__ __forceinline__ void pairs(long long n, F2 f2, F1 f1) {
  const long long np = n >> 1;
  for (long long q = blockIdx.x * (long long)VB + threadIdx.x; q < np; q += (long long)gridDim.x * VB) f2(q);
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) f1(n - 1);
}

// BiCG step J of a cycle, first half: u_i = r_i − β u_i for i = 0 … J.
// For J ≥ 1 it first completes the previous step's updates that the
// operator did not need (step J−1 updated only r_{J−1}):
//   r_i −= α u_{i+1} (i < J−1) and x += α u_0, with α of step J−1 —
// one pass over those vectors instead of two.
template <typename R, int J>
__global__ void __launch_bounds__(VB) k_bl_u(VSet<typename CT<R>::C> r, VSet<typename CT<R>::C> u,
                                             typename CT<R>::C *x, long long n, const KScalars *sc) {
  using C = typename CT<R>::C;
  if (sc->done) return;
  C ba[2];
  scalars<R>([&](int i) { return i == 0 ? sc->beta : sc->alpha; }, ba);
  const C be = ba[0], al = ba[1];
  pairs(
      n,
      [&](long long q) {
        Pair<C> rv[J + 1], uv[J + 1];
#pragma unroll
        for (int i = 0; i <= J; ++i) {
          rv[i] = ldp(r.v[i], q);
          uv[i] = ldp(u.v[i], q);
        }
        if (J >= 1) {
#pragma unroll
          for (int i = 0; i + 1 < J; ++i) {
            rv[i] = Pair<C>{csub(rv[i].a, cmul(al, uv[i + 1].a)), csub(rv[i].b, cmul(al, uv[i + 1].b))};
            stp(r.v[i], q, rv[i]);
          }
          const Pair<C> xv = ldp(x, q);
          stp(x, q, Pair<C>{cadd(xv.a, cmul(al, uv[0].a)), cadd(xv.b, cmul(al, uv[0].b))});
        }
#pragma unroll
        for (int i = 0; i <= J; ++i)
          stp(u.v[i], q, Pair<C>{csub(rv[i].a, cmul(be, uv[i].a)), csub(rv[i].b, cmul(be, uv[i].b))});
      },
      [&](long long e) {
        C rv[J + 1], uv[J + 1];
#pragma unroll
        for (int i = 0; i <= J; ++i) {
          rv[i] = r.v[i][e];
          uv[i] = u.v[i][e];
        }
        if (J >= 1) {
#pragma unroll
          for (int i = 0; i + 1 < J; ++i) {
            rv[i] = csub(rv[i], cmul(al, uv[i + 1]));
            r.v[i][e] = rv[i];
          }
          x[e] = cadd(x[e], cmul(al, uv[0]));
        }
#pragma unroll
        for (int i = 0; i <= J; ++i) u.v[i][e] = csub(rv[i], cmul(be, uv[i]));
      });
}

// BiCG step J, second half: r_J −= α u_{J+1} (the operator's next input).
template <typename R, int J>
__global__ void __launch_bounds__(VB) k_bl_r(VSet<typename CT<R>::C> r, VSet<typename CT<R>::C> u, long long n,
                                             const KScalars *sc) {
  using C = typename CT<R>::C;
  if (sc->done) return;
  C a1[1];
  scalars<R>([&](int) { return sc->alpha; }, a1);
  const C al = a1[0];
  pairs(
      n,
      [&](long long q) {
        const Pair<C> rv = ldp(r.v[J], q), uv = ldp(u.v[J + 1], q);
        stp(r.v[J], q, Pair<C>{csub(rv.a, cmul(al, uv.a)), csub(rv.b, cmul(al, uv.b))});
      },
      [&](long long e) { r.v[J][e] = csub(r.v[J][e], cmul(al, u.v[J + 1][e])); });
}

constexpr int pow2_at_least(int k) { return k <= 1 ? 1 : 2 * pow2_at_least((k + 1) / 2); }

// Sum NV complex FP64 values over the block (complex128 kernels), write the
// block's partials, and return true in the block that arrives last (which
// then holds the grid sums, in block order, in `tot`).
template <int NV>
__device__ bool block_sums_last(double2 (&v)[NV], RedBuf red, double2 (&tot)[NV]) {
  __shared__ double2 wred[VB / 32][NV];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v[q].x += __shfl_xor_sync(0xffffffffu, v[q].x, o);
      v[q].y += __shfl_xor_sync(0xffffffffu, v[q].y, o);
    }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) wred[wid][q] = v[q];
  __syncthreads();
  if (tid < NV) {
    double2 s = make_double2(0, 0);
    for (int w = 0; w < VB / 32; ++w) s = addd(s, wred[w][tid]);
    red.part[(long long)NV * blockIdx.x + tid] = s;
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(red.count, 1u);
    last = prev == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // every thread sums a fixed subset of the blocks, then a fixed tree:
  // deterministic for a given launch shape
  double2 s[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) s[q] = make_double2(0, 0);
  for (unsigned b = tid; b < gridDim.x; b += VB)
#pragma unroll
    for (int q = 0; q < NV; ++q) s[q] = addd(s[q], __ldcg(&red.part[(long long)NV * b + q]));
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s[q].x += __shfl_xor_sync(0xffffffffu, s[q].x, o);
      s[q].y += __shfl_xor_sync(0xffffffffu, s[q].y, o);
    }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) wred[wid][q] = s[q];
  __syncthreads();
  if (tid < NV) {
    double2 t = make_double2(0, 0);
    for (int w = 0; w < VB / 32; ++w) t = addd(t, wred[w][tid]);
    tot[tid] = t;  // tot lives in shared memory of the caller
  }
  __syncthreads();
  if (tid == 0) *red.count = 0u;
  return true;
}

// Gram matrix of r_0 … r_L — (r_i, r_j) for 1 ≤ i ≤ j ≤ L, then (r_i, r_0)
// for 1 ≤ i ≤ L — into sc->gram (last block).  The stored r_i (i < L−1)
// still lack the last BiCG step's −α u_{i+1}; it is applied in registers.
template <typename R, int L>
__global__ void __launch_bounds__(VB, 2) k_bl_gram(VSet<typename CT<R>::C> r, VSet<typename CT<R>::C> u, long long n,
                                                   RedBuf red, KScalars *sc) {
  using C = typename CT<R>::C;
  constexpr int NV = L * (L + 1) / 2 + L;
  constexpr int ND = L > 1 ? L - 1 : 1;  // deferred corrections (L − 1 of them)
  if (sc->done) return;
  C a1[1];
  scalars<R>([&](int) { return sc->alpha; }, a1);
  const C al = a1[0];
  R ar[NV], ai[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) ar[q] = ai[q] = R(0);
  auto one = [&](const C (&v)[L + 1]) {
    int q = 0;
#pragma unroll
    for (int j = 1; j <= L; ++j)
#pragma unroll
      for (int i = 1; i <= j; ++i, ++q) {
        const C d = cdotc(v[i], v[j]);
        ar[q] += d.x;
        ai[q] += d.y;
      }
#pragma unroll
    for (int i = 1; i <= L; ++i, ++q) {
      const C d = cdotc(v[i], v[0]);
      ar[q] += d.x;
      ai[q] += d.y;
    }
  };
  pairs(
      n,
      [&](long long q) {
        C va[L + 1], vb[L + 1];
        Pair<C> ud[ND];
#pragma unroll
        for (int i = 0; i <= L; ++i) {
          const Pair<C> p = ldp(r.v[i], q);
          va[i] = p.a;
          vb[i] = p.b;
        }
#pragma unroll
        for (int i = 0; i + 1 < L; ++i) ud[i] = ldp(u.v[i + 1], q);
#pragma unroll
        for (int i = 0; i + 1 < L; ++i) {
          va[i] = csub(va[i], cmul(al, ud[i].a));
          vb[i] = csub(vb[i], cmul(al, ud[i].b));
        }
        one(va);
        one(vb);
      },
      [&](long long e) {
        C v[L + 1];
#pragma unroll
        for (int i = 0; i <= L; ++i) v[i] = r.v[i][e];
#pragma unroll
        for (int i = 0; i + 1 < L; ++i) v[i] = csub(v[i], cmul(al, u.v[i + 1][e]));
        one(v);
      });
  if constexpr (sizeof(R) == 4) {
    constexpr int K = pow2_at_least(2 * NV);
    DF v[K];
#pragma unroll
    for (int q = 0; q < K; ++q) v[q] = DF{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      v[2 * q].hi = ar[q];
      v[2 * q + 1].hi = ai[q];
    }
    __shared__ double tot[2 * NV];
    if (!df_block_sums_last<VB, K, 2 * NV>(v, red, tot)) return;
    if (threadIdx.x < NV) sc->gram[threadIdx.x] = make_double2(tot[2 * threadIdx.x], tot[2 * threadIdx.x + 1]);
  } else {
    double2 acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = make_double2((double)ar[q], (double)ai[q]);
    __shared__ double2 tot[NV];
    if (!block_sums_last<NV>(acc, red, tot)) return;
    if (threadIdx.x < NV) sc->gram[threadIdx.x] = tot[threadIdx.x];
  }
}

// The minimal-residual step of the cycle from the Gram matrix (one thread;
// its own launch so the arrays stay in registers): modified Gram–Schmidt on
// r_1 … r_ℓ carried out on the Gram matrix — r̂_j = Σ_k Lc[j][k] r_k —
// then the closing coefficients in terms of the original r_k.
template <int L>
__global__ void k_bl_mr(KScalars *sc) {
  if (threadIdx.x != 0 || sc->done) return;
  double2 G[L + 1][L + 1], g0[L + 1];
  {
    int q = 0;
#pragma unroll
    for (int j = 1; j <= L; ++j)
#pragma unroll
      for (int i = 1; i <= j; ++i, ++q) {
        G[i][j] = sc->gram[q];
        G[j][i] = conjd(sc->gram[q]);
      }
#pragma unroll
    for (int i = 1; i <= L; ++i, ++q) g0[i] = sc->gram[q];
  }
  double2 Lc[L + 1][L + 1], tau[L + 1][L + 1], gp[L + 1], gam[L + 1], gpp[L + 1];
  double isig[L + 1];
#pragma unroll
  for (int a = 0; a <= L; ++a)
#pragma unroll
    for (int b = 0; b <= L; ++b) Lc[a][b] = tau[a][b] = make_double2(0, 0);
  double2 gr0[L + 1];  // (r̂_i, r_0)
#pragma unroll
  for (int j = 1; j <= L; ++j) {
    Lc[j][j] = make_double2(1, 0);
    double2 dij[L + 1];  // (r̂_i, r_j)
#pragma unroll
    for (int i = 1; i < j; ++i) {
      double2 d = make_double2(0, 0);
#pragma unroll
      for (int k = 1; k <= i; ++k) d = addd(d, dcmul(conjd(Lc[i][k]), G[k][j]));
      dij[i] = d;
      tau[i][j] = scd(d, isig[i]);
#pragma unroll
      for (int k = 1; k <= i; ++k) Lc[j][k] = subd(Lc[j][k], dcmul(tau[i][j], Lc[i][k]));
    }
    // with r̂_j = r_j − Σ_{i<j} τ_ij r̂_i and the r̂_i orthogonal:
    //   (r̂_j, r̂_j) = (r_j, r_j) − Σ_i |(r̂_i, r_j)|²/σ_i
    //   (r̂_j, r_0)  = (r_j, r_0) − Σ_i conj(τ_ij) (r̂_i, r_0)
    double s = G[j][j].x;
    double2 g = g0[j];
#pragma unroll
    for (int i = 1; i < j; ++i) {
      s -= (dij[i].x * dij[i].x + dij[i].y * dij[i].y) * isig[i];
      g = subd(g, dcmul(conjd(tau[i][j]), gr0[i]));
    }
    if (!(s > 0.0) || !isfinite(s)) {
      sc->done = 1;
      sc->reason = isfinite(s) ? 3 : 4;
      return;
    }
    isig[j] = 1.0 / s;
    gr0[j] = g;
    gp[j] = scd(g, isig[j]);
  }
  gam[L] = gp[L];
#pragma unroll
  for (int j = L - 1; j >= 1; --j) {
    double2 t = gp[j];
#pragma unroll
    for (int i = j + 1; i <= L; ++i) t = subd(t, dcmul(tau[j][i], gam[i]));
    gam[j] = t;
  }
#pragma unroll
  for (int j = 1; j < L; ++j) {
    double2 t = gam[j + 1];
#pragma unroll
    for (int i = j + 1; i < L; ++i) t = addd(t, dcmul(tau[j][i], gam[i + 1]));
    gpp[j] = t;
  }
#pragma unroll
  for (int k = 0; k <= LMAX; ++k) sc->cx[k] = sc->cr[k] = sc->cu[k] = make_double2(0, 0);
  sc->cx[0] = gam[1];
#pragma unroll
  for (int k = 1; k <= L; ++k) {
    double2 cx = make_double2(0, 0), cr = make_double2(0, 0);
#pragma unroll
    for (int j = k; j < L; ++j) cx = addd(cx, dcmul(gpp[j], Lc[j][k]));
#pragma unroll
    for (int j = k; j <= L; ++j) cr = subd(cr, dcmul(gp[j], Lc[j][k]));
    sc->cx[k] = cx;
    sc->cr[k] = cr;
    sc->cu[k] = make_double2(-gam[k].x, -gam[k].y);
  }
  sc->omega = gam[L];
}

// x += α u_0 + Σ cx_k r_k ; r_0 += Σ cr_k r_k ; u_0 += Σ cu_k u_k ; then
// (r̂, r_0) and ‖r_0‖² → FIN_BL_CYCLE.  α u_0 and the r_i −= α u_{i+1}
// (i < L−1) are the last BiCG step's deferred updates (α of that step:
// nothing writes sc->alpha between it and this kernel).
template <typename R, int L>
__global__ void __launch_bounds__(VB, sizeof(R) == 4 ? 3 : 2) k_bl_fin(VSet<typename CT<R>::C> r, VSet<typename CT<R>::C> u,
                                                  typename CT<R>::C *x, long long n, RedBuf red, KScalars *sc) {
  using C = typename CT<R>::C;
  if (sc->done) return;
  C cs[3 * (L + 1) + 1];
  scalars<R>(
      [&](int i) {
        return i <= L ? sc->cx[i] : i <= 2 * L + 1 ? sc->cr[i - (L + 1)] : i <= 3 * L + 2 ? sc->cu[i - 2 * (L + 1)] : sc->alpha;
      },
      cs);
  const C *cx = cs, *cr = cs + (L + 1), *cu = cs + 2 * (L + 1);
  const C al = cs[3 * (L + 1)];
  Acc<R> a0r, a0i, a1;
  pairs(
      n,
      [&](long long q) {
        C ra[L + 1], rb[L + 1], ua[L + 1], ub[L + 1];
#pragma unroll
        for (int k = 0; k <= L; ++k) {
          const Pair<C> pr = ldp(r.v[k], q), pu = ldp(u.v[k], q);
          ra[k] = pr.a;
          rb[k] = pr.b;
          ua[k] = pu.a;
          ub[k] = pu.b;
        }
        Pair<C> xv = ldp(x, q);
        const Pair<C> hv{shadow<R>(2 * q), shadow<R>(2 * q + 1)};
#pragma unroll
        for (int k = 0; k + 1 < L; ++k) {
          ra[k] = csub(ra[k], cmul(al, ua[k + 1]));
          rb[k] = csub(rb[k], cmul(al, ub[k + 1]));
        }
        xv.a = cadd(xv.a, cmul(al, ua[0]));
        xv.b = cadd(xv.b, cmul(al, ub[0]));
        C r0a = ra[0], r0b = rb[0], u0a = ua[0], u0b = ub[0];
#pragma unroll
        for (int k = 0; k <= L; ++k) {
          xv.a = cadd(xv.a, cmul(cx[k], ra[k]));
          xv.b = cadd(xv.b, cmul(cx[k], rb[k]));
        }
#pragma unroll
        for (int k = 1; k <= L; ++k) {
          r0a = cadd(r0a, cmul(cr[k], ra[k]));
          r0b = cadd(r0b, cmul(cr[k], rb[k]));
          u0a = cadd(u0a, cmul(cu[k], ua[k]));
          u0b = cadd(u0b, cmul(cu[k], ub[k]));
        }
        stp(x, q, xv);
        stp(r.v[0], q, Pair<C>{r0a, r0b});
        stp(u.v[0], q, Pair<C>{u0a, u0b});
        const C da = cdotc(hv.a, r0a), db = cdotc(hv.b, r0b);
        a0r.add(da.x + db.x);
        a0i.add(da.y + db.y);
        a1.add((r0a.x * r0a.x + r0a.y * r0a.y) + (r0b.x * r0b.x + r0b.y * r0b.y));
      },
      [&](long long e) {
        C rk[L + 1], uk[L + 1];
#pragma unroll
        for (int k = 0; k <= L; ++k) {
          rk[k] = r.v[k][e];
          uk[k] = u.v[k][e];
        }
#pragma unroll
        for (int k = 0; k + 1 < L; ++k) rk[k] = csub(rk[k], cmul(al, uk[k + 1]));
        C xe = cadd(x[e], cmul(al, uk[0])), r0 = rk[0], u0 = uk[0];
#pragma unroll
        for (int k = 0; k <= L; ++k) xe = cadd(xe, cmul(cx[k], rk[k]));
#pragma unroll
        for (int k = 1; k <= L; ++k) {
          r0 = cadd(r0, cmul(cr[k], rk[k]));
          u0 = cadd(u0, cmul(cu[k], uk[k]));
        }
        x[e] = xe;
        r.v[0][e] = r0;
        u.v[0][e] = u0;
        const C d = cdotc(shadow<R>(e), r0);
        a0r.add(d.x);
        a0i.add(d.y);
        a1.add(r0.x * r0.x + r0.y * r0.y);
      });
  sum_finalise<VB>(a0r, a0i, a1, red, FIN_BL_CYCLE, sc);
}

// (r̂, r_0) with the generated shadow vector: FIN_BL_REDO after a replaced
// residual, FIN_NONE (into dot0) for the first ρ of a (re)started solve
template <typename R>
__global__ void __launch_bounds__(VB) k_bl_redo(const typename CT<R>::C *__restrict__ r0, long long n, RedBuf red,
                                                int fin, KScalars *sc) {
  using C = typename CT<R>::C;
  Acc<R> a0r, a0i;
  for (long long e = blockIdx.x * (long long)VB + threadIdx.x; e < n; e += vstride<R>()) {
    const C d = cdotc(shadow<R>(e), r0[e]);
    a0r.add(d.x);
    a0i.add(d.y);
  }
  sum_finalise<VB>(a0r, a0i, red, fin, sc);
}

}  // namespace

template <typename R>
static VSet<typename CT<R>::C> vset(typename CT<R>::C *const *v, int count) {
  VSet<typename CT<R>::C> s{};
  for (int i = 0; i < count && i <= LMAX; ++i) s.v[i] = v[i];
  return s;
}

// Blocks for one full wave of a grid-stride kernel: SM count × its resident
// blocks per SM (cached per kernel and device), at most `cap`.
static int wave_blocks(const void *kern, int cap) {
  static std::mutex mu;
  static std::unordered_map<const void *, int> cache[16];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) {
    cudaGetLastError();
    return std::min(RED_BLOCKS, cap);
  }
  std::lock_guard<std::mutex> lock(mu);
  const auto it = cache[dev].find(kern);
  if (it != cache[dev].end()) return std::min(it->second, cap);
  int sms = 0, per = 0;
  int b = RED_BLOCKS;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, VB, 0) == cudaSuccess && sms * per > 0)
    b = sms * per;
  else
    cudaGetLastError();
  cache[dev].emplace(kern, b);
  return std::min(b, cap);
}

// Launch a grid-stride vector kernel on one full wave.
template <typename... P, typename... A>
static void launch_wave(fdfd_handle *h, void (*kern)(P...), int cap, A... args) {
  kern<<<wave_blocks(reinterpret_cast<const void *>(kern), cap), VB, 0, h->stream>>>(args...);
  h->launches++;
}

template <typename R, int L>
static int bl_cycle_t(fdfd_handle *h, typename CT<R>::C *x, typename CT<R>::C *const *r, typename CT<R>::C *const *u,
                      long long n, KScalars *sc, bool tr) {
  const VSet<typename CT<R>::C> rs = vset<R>(r, L + 1), us = vset<R>(u, L + 1);
  constexpr int NOCAP = 1 << 30;
  int rc;
  for (int j = 0; j < L; ++j) {
    switch (j) {
      case 0: launch_wave(h, k_bl_u<R, 0>, NOCAP, rs, us, x, n, (const KScalars *)sc); break;
      case 1: launch_wave(h, k_bl_u<R, 1>, NOCAP, rs, us, x, n, (const KScalars *)sc); break;
      case 2: launch_wave(h, k_bl_u<R, 2>, NOCAP, rs, us, x, n, (const KScalars *)sc); break;
      default: launch_wave(h, k_bl_u<R, 3>, NOCAP, rs, us, x, n, (const KScalars *)sc); break;
    }
    if ((rc = cuda_check(h, cudaGetLastError(), "k_bl_u"))) return rc;
    if ((rc = launch_apply_fin<R>(h, u[j], u[j + 1], EPI_DOT_SHD, nullptr, FIN_ALPHA, sc, tr))) return rc;
    switch (j) {
      case 0: launch_wave(h, k_bl_r<R, 0>, NOCAP, rs, us, n, (const KScalars *)sc); break;
      case 1: launch_wave(h, k_bl_r<R, 1>, NOCAP, rs, us, n, (const KScalars *)sc); break;
      case 2: launch_wave(h, k_bl_r<R, 2>, NOCAP, rs, us, n, (const KScalars *)sc); break;
      default: launch_wave(h, k_bl_r<R, 3>, NOCAP, rs, us, n, (const KScalars *)sc); break;
    }
    if ((rc = cuda_check(h, cudaGetLastError(), "k_bl_r"))) return rc;
    if (j + 1 < L) rc = launch_apply_fin<R>(h, r[j], r[j + 1], EPI_DOT_SHD, nullptr, FIN_BL_RHO, sc, tr);
    else rc = launch_apply_fin<R>(h, r[j], r[j + 1], EPI_STORE, nullptr, FIN_NONE, sc, tr);
    if (rc) return rc;
  }
  // the reducing kernels keep ≤ RED_BLOCKS blocks: 8·RED_BLOCKS partial
  // slots hold the Gram matrix's L(L+1)/2 + L ≤ 14 values per block
  if ((rc = ensure_red(h, 8 * RED_BLOCKS))) return rc;
  launch_wave(h, k_bl_gram<R, L>, RED_BLOCKS, rs, us, n, h->red, sc);
  if ((rc = cuda_check(h, cudaGetLastError(), "k_bl_gram"))) return rc;
  k_bl_mr<L><<<1, 32, 0, h->stream>>>(sc);
  h->launches++;
  if ((rc = cuda_check(h, cudaGetLastError(), "k_bl_mr"))) return rc;
  launch_wave(h, k_bl_fin<R, L>, RED_BLOCKS, rs, us, x, n, h->red, sc);
  return cuda_check(h, cudaGetLastError(), "k_bl_fin");
}

// One BiCGStab(ℓ) cycle (2ℓ operator applications).
template <typename R>
int bl_cycle(fdfd_handle *h, typename CT<R>::C *x, typename CT<R>::C *const *r, typename CT<R>::C *const *u,
             long long n, int ell, KScalars *sc, bool tr) {
  switch (ell) {
    case 1: return bl_cycle_t<R, 1>(h, x, r, u, n, sc, tr);
    case 2: return bl_cycle_t<R, 2>(h, x, r, u, n, sc, tr);
    case 3: return bl_cycle_t<R, 3>(h, x, r, u, n, sc, tr);
    case 4: return bl_cycle_t<R, 4>(h, x, r, u, n, sc, tr);
  }
  return set_error(h, FDFD_ERR_ARG, "BiCGStab(l) needs 1 <= l <= 4");
}

template <typename R>
int bl_redo(fdfd_handle *h, const typename CT<R>::C *r0, long long n, int fin, KScalars *sc) {
  int rc = ensure_red(h, RED_BLOCKS);
  if (rc) return rc;
  k_bl_redo<R><<<RED_BLOCKS, VB, 0, h->stream>>>(r0, n, h->red, fin, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_bl_redo");
}

template int bl_cycle<float>(fdfd_handle *, float2 *, float2 *const *, float2 *const *, long long, int, KScalars *,
                             bool);
template int bl_cycle<double>(fdfd_handle *, double2 *, double2 *const *, double2 *const *, long long, int,
                              KScalars *, bool);
template int bl_redo<float>(fdfd_handle *, const float2 *, long long, int, KScalars *);
template int bl_redo<double>(fdfd_handle *, const double2 *, long long, int, KScalars *);

}  // namespace fdfd
