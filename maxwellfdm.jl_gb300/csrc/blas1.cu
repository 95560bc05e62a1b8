// Vector kernels of the Krylov solvers: the BiCGSTAB / COCG updates with
// their dot products fused in, precision conversions for the mixed
// (complex64 + FP64 refinement) solver, and the reduction buffer.
//
// All reducing kernels use a fixed grid (RED_BLOCKS × 256 threads) and a
// grid-stride loop, so the per-block partials and therefore the reduced
// values are deterministic for a given problem size.
#include "krylov_fin.cuh"

namespace fdfd {

constexpr int VB = 256;          // threads per block
constexpr int RED_BLOCKS = 152 * 4;

int ensure_red(fdfd_handle *h, int blocks) {
  if (blocks < RED_BLOCKS) blocks = RED_BLOCKS;
  if (h->red.part != nullptr && h->red_blocks >= blocks) return FDFD_OK;
  if (h->red.part) cudaFree(h->red.part);
  if (h->red.count) cudaFree(h->red.count);
  h->red.part = nullptr;
  h->red.count = nullptr;
  cudaError_t e = dev_malloc(&h->red.part, sizeof(double2) * 2 * (size_t)blocks);
  if (e != cudaSuccess) return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(reduction partials) failed");
  e = dev_malloc(&h->red.count, sizeof(unsigned int));
  if (e != cudaSuccess) return set_error(h, FDFD_ERR_NOMEM, "cudaMalloc(reduction counter) failed");
  e = cudaMemsetAsync(h->red.count, 0, sizeof(unsigned int), h->stream);
  if (e != cudaSuccess) return cuda_check(h, e, "cudaMemsetAsync(counter)");
  h->red_blocks = blocks;
  return FDFD_OK;
}

template <typename C> __device__ __forceinline__ C ld(const C *p, long long i) { return p[i]; }

// Two consecutive complex elements (2q, 2q+1) per access: one 16-byte
// float4 for complex64, two 16-byte double2 for complex128.
__device__ __forceinline__ void ld2(const float2 *__restrict__ a, long long q, float2 &e0, float2 &e1) {
  const float4 v = reinterpret_cast<const float4 *>(a)[q];
  e0 = make_float2(v.x, v.y);
  e1 = make_float2(v.z, v.w);
}
__device__ __forceinline__ void ld2(const double2 *__restrict__ a, long long q, double2 &e0, double2 &e1) {
  e0 = a[2 * q];
  e1 = a[2 * q + 1];
}
__device__ __forceinline__ void st2(float2 *a, long long q, float2 e0, float2 e1) {
  reinterpret_cast<float4 *>(a)[q] = make_float4(e0.x, e0.y, e1.x, e1.y);
}
__device__ __forceinline__ void st2(double2 *a, long long q, double2 e0, double2 e1) {
  a[2 * q] = e0;
  a[2 * q + 1] = e1;
}

// Visit element pairs with a grid-stride loop; an odd last element is
// handled by one thread.
template <typename F2, typename F1>
__device__ __forceinline__ void pair_loop(long long n, F2 f2, F1 f1) {
  const long long np = n >> 1;
  for (long long q = blockIdx.x * (long long)VB + threadIdx.x; q < np; q += (long long)gridDim.x * VB) f2(q);
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) f1(n - 1);
}

// p = r + β (p − ω v)
template <typename R>
__global__ void __launch_bounds__(VB) k_bicg_p(const typename CT<R>::C *__restrict__ r, typename CT<R>::C *p,
                                               const typename CT<R>::C *__restrict__ v, long long n,
                                               const KScalars *sc) {
  using C = typename CT<R>::C;
  pdl_trigger();
  pdl_wait();
  if (sc->done) return;
  C bo[2];
  scalars<R>([&](int i) { return i == 0 ? sc->beta : sc->omega; }, bo);
  const C be = bo[0], om = bo[1];
  auto one = [&](C ri, C pi, C vi) { return cadd(ri, cmul(be, csub(pi, cmul(om, vi)))); };
  pair_loop(
      n,
      [&](long long q) {
        C r0, r1, p0, p1, v0, v1;
        ld2(r, q, r0, r1);
        ld2(p, q, p0, p1);
        ld2(v, q, v0, v1);
        st2(p, q, one(r0, p0, v0), one(r1, p1, v1));
      },
      [&](long long i) { p[i] = one(r[i], p[i], v[i]); });
}

// s = r − α v
template <typename R>
__global__ void __launch_bounds__(VB) k_bicg_s(const typename CT<R>::C *__restrict__ r,
                                               const typename CT<R>::C *__restrict__ v, typename CT<R>::C *s,
                                               long long n, const KScalars *sc) {
  using C = typename CT<R>::C;
  pdl_trigger();
  pdl_wait();
  if (sc->done) return;
  C a1[1];
  scalars<R>([&](int) { return sc->alpha; }, a1);
  const C al = a1[0];
  pair_loop(
      n,
      [&](long long q) {
        C r0, r1, v0, v1;
        ld2(r, q, r0, r1);
        ld2(v, q, v0, v1);
        st2(s, q, csub(r0, cmul(al, v0)), csub(r1, cmul(al, v1)));
      },
      [&](long long i) { s[i] = csub(r[i], cmul(al, v[i])); });
}

// x += α p + ω s;  r = s − ω t;  (r̂, r), ‖r‖²  → FIN_XR
template <typename R>
__global__ void __launch_bounds__(VB) k_bicg_xr(typename CT<R>::C *x, const typename CT<R>::C *__restrict__ p,
                                                const typename CT<R>::C *__restrict__ s,
                                                const typename CT<R>::C *__restrict__ t, typename CT<R>::C *r,
                                                const typename CT<R>::C *__restrict__ rh, long long n, RedBuf red,
                                                KScalars *sc) {
  using C = typename CT<R>::C;
  pdl_trigger();
  pdl_wait();
  if (sc->done) return;
  C ao[2];
  scalars<R>([&](int i) { return i == 0 ? sc->alpha : sc->omega; }, ao);
  const C al = ao[0], om = ao[1];
  Acc<R> a0r, a0i, a1;
  auto acc = [&](C rhi, C ri) {
    const C d = cdotc(rhi, ri);
    a0r.add(d.x);
    a0i.add(d.y);
    a1.add(ri.x * ri.x + ri.y * ri.y);
  };
  pair_loop(
      n,
      [&](long long q) {
        C x0, x1, p0, p1, s0, s1, t0, t1, h0, h1;
        ld2(s, q, s0, s1);
        ld2(t, q, t0, t1);
        ld2(x, q, x0, x1);
        ld2(p, q, p0, p1);
        ld2(rh, q, h0, h1);
        st2(x, q, cadd(x0, cadd(cmul(al, p0), cmul(om, s0))), cadd(x1, cadd(cmul(al, p1), cmul(om, s1))));
        const C r0 = csub(s0, cmul(om, t0)), r1 = csub(s1, cmul(om, t1));
        st2(r, q, r0, r1);
        acc(h0, r0);
        acc(h1, r1);
      },
      [&](long long i) {
        const C si = s[i];
        x[i] = cadd(x[i], cadd(cmul(al, p[i]), cmul(om, si)));
        const C ri = csub(si, cmul(om, t[i]));
        r[i] = ri;
        acc(rh[i], ri);
      });
  sum_finalise<VB>(a0r, a0i, a1, red, FIN_XR, sc);
}

// Jacobi-preconditioned COCG on the S-symmetric operator (S = V_E, so S·A
// is complex symmetric; z = D⁻¹ r with D = diag(A)):
//   x += α p ; r −= α q ; ρ' = rᵀ S z and ‖r‖²  → FIN_COCG_R
template <typename R>
__global__ void __launch_bounds__(VB) k_cocg_xr(typename CT<R>::C *x, const typename CT<R>::C *__restrict__ p,
                                                const typename CT<R>::C *__restrict__ q, typename CT<R>::C *r,
                                                const typename CT<R>::C *__restrict__ wgt,
                                                const typename CT<R>::C *__restrict__ dinv, long long n, RedBuf red,
                                                KScalars *sc) {
  using C = typename CT<R>::C;
  if (sc->done) return;
  C as[1];
  scalars<R>([&](int) { return sc->alpha; }, as);
  const C al = as[0];
  Acc<R> a0r, a0i, a1;
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    x[i] = cadd(x[i], cmul(al, p[i]));
    const C ri = csub(r[i], cmul(al, q[i]));
    r[i] = ri;
    const C zi = cmul(dinv[i], ri);
    const C d = cmul(cmul(wgt[i], ri), zi);  // rᵀ S z (unconjugated)
    a0r.add(d.x);
    a0i.add(d.y);
    a1.add(ri.x * ri.x + ri.y * ri.y);
  }
  sum_finalise<VB>(a0r, a0i, a1, red, FIN_COCG_R, sc);
}

// COCG direction: p = D⁻¹ r + β p
template <typename R>
__global__ void __launch_bounds__(VB) k_cocg_p(const typename CT<R>::C *__restrict__ r,
                                               const typename CT<R>::C *__restrict__ dinv, typename CT<R>::C *p,
                                               long long n, const KScalars *sc) {
  using C = typename CT<R>::C;
  if (sc->done) return;
  C bs[1];
  scalars<R>([&](int) { return sc->beta; }, bs);
  const C be = bs[0];
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB)
    p[i] = cadd(cmul(dinv[i], r[i]), cmul(be, p[i]));
}

// y = a ∘ b (elementwise complex product)
template <typename R>
__global__ void __launch_bounds__(VB) k_vmul(typename CT<R>::C *y, const typename CT<R>::C *__restrict__ a,
                                             const typename CT<R>::C *__restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB)
    y[i] = cmul(a[i], b[i]);
}

// Generic reductions: mode 0: (a, b) Hermitian and ‖a‖²;  mode 1: aᵀ S a
template <typename R>
__global__ void __launch_bounds__(VB) k_dot(const typename CT<R>::C *__restrict__ a,
                                            const typename CT<R>::C *__restrict__ b, long long n, RedBuf red,
                                            KScalars *sc) {
  using C = typename CT<R>::C;
  Acc<R> a0r, a0i, a1;
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const C ai = a[i];
    const C d = cdotc(ai, b[i]);
    a0r.add(d.x);
    a0i.add(d.y);
    a1.add(ai.x * ai.x + ai.y * ai.y);
  }
  sum_finalise<VB>(a0r, a0i, a1, red, FIN_NONE, sc);
}

// pᵀ (S q) (unconjugated, weighted) → FIN_COCG_A
template <typename R>
__global__ void __launch_bounds__(VB) k_dot_u(const typename CT<R>::C *__restrict__ a,
                                              const typename CT<R>::C *__restrict__ b,
                                              const typename CT<R>::C *__restrict__ wgt, long long n, RedBuf red,
                                              int fin, KScalars *sc) {
  using C = typename CT<R>::C;
  if (fin != FIN_NONE && sc->done) return;
  Acc<R> a0r, a0i;
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const C d = cmul(a[i], cmul(wgt[i], b[i]));
    a0r.add(d.x);
    a0i.add(d.y);
  }
  sum_finalise<VB>(a0r, a0i, red, fin, sc);
}

// ---------------------------------------------------------------- mixed precision
// x64 += x32; x32 = 0
__global__ void __launch_bounds__(VB) k_accum(double2 *x64, float2 *x32, long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const float2 v = x32[i];
    double2 a = x64[i];
    a.x += (double)v.x;
    a.y += (double)v.y;
    x64[i] = a;
    x32[i] = make_float2(0.f, 0.f);
  }
}
// x64 += x (double) ; x = 0
__global__ void __launch_bounds__(VB) k_accum64(double2 *x64, double2 *x, long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const double2 v = x[i];
    double2 a = x64[i];
    a.x += v.x;
    a.y += v.y;
    x64[i] = a;
    x[i] = make_double2(0.0, 0.0);
  }
}
__global__ void __launch_bounds__(VB) k_demote(float2 *y, const double2 *__restrict__ x, long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const double2 v = x[i];
    y[i] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void __launch_bounds__(VB) k_promote(double2 *y, const float2 *__restrict__ x, long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const float2 v = x[i];
    y[i] = make_double2((double)v.x, (double)v.y);
  }
}
template <typename R>
__global__ void __launch_bounds__(VB) k_copy(typename CT<R>::C *y, const typename CT<R>::C *__restrict__ x,
                                             long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) y[i] = x[i];
}
template <typename R>
__global__ void __launch_bounds__(VB) k_conj_copy(typename CT<R>::C *y, const typename CT<R>::C *__restrict__ x,
                                                  long long n) {
  for (long long i = blockIdx.x * (long long)VB + threadIdx.x; i < n; i += (long long)gridDim.x * VB) {
    const auto v = x[i];
    y[i] = mk(v.x, -v.y);
  }
}

static inline int vgrid(long long n) {
  long long b = (n + VB - 1) / VB;
  if (b > RED_BLOCKS) b = RED_BLOCKS;
  if (b < 1) b = 1;
  return (int)b;
}

// ------------------------------------------------------------------ launchers
template <typename R>
int bicg_p(fdfd_handle *h, const typename CT<R>::C *r, typename CT<R>::C *p, const typename CT<R>::C *v, long long n,
           const KScalars *sc) {
  const cudaError_t e = launch_k(h, k_bicg_p<R>, dim3(vgrid(n)), dim3(VB), 0, r, p, v, n, sc);
  h->launches++;
  return cuda_check(h, e, "k_bicg_p");
}
template <typename R>
int bicg_s(fdfd_handle *h, const typename CT<R>::C *r, const typename CT<R>::C *v, typename CT<R>::C *s, long long n,
           const KScalars *sc) {
  const cudaError_t e = launch_k(h, k_bicg_s<R>, dim3(vgrid(n)), dim3(VB), 0, r, v, s, n, sc);
  h->launches++;
  return cuda_check(h, e, "k_bicg_s");
}
template <typename R>
int bicg_xr(fdfd_handle *h, typename CT<R>::C *x, const typename CT<R>::C *p, const typename CT<R>::C *s,
            const typename CT<R>::C *t, typename CT<R>::C *r, const typename CT<R>::C *rh, long long n, KScalars *sc) {
  int rc = ensure_red(h, RED_BLOCKS);
  if (rc) return rc;
  const cudaError_t e = launch_k(h, k_bicg_xr<R>, dim3(vgrid(n)), dim3(VB), 0, x, p, s, t, r, rh, n, h->red, sc);
  h->launches++;
  return cuda_check(h, e, "k_bicg_xr");
}
template <typename R>
int cocg_xr(fdfd_handle *h, typename CT<R>::C *x, const typename CT<R>::C *p, const typename CT<R>::C *q,
            typename CT<R>::C *r, const typename CT<R>::C *w, const typename CT<R>::C *dinv, long long n,
            KScalars *sc) {
  int rc = ensure_red(h, RED_BLOCKS);
  if (rc) return rc;
  k_cocg_xr<R><<<vgrid(n), VB, 0, h->stream>>>(x, p, q, r, w, dinv, n, h->red, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_cocg_xr");
}
template <typename R>
int cocg_p(fdfd_handle *h, const typename CT<R>::C *r, const typename CT<R>::C *dinv, typename CT<R>::C *p,
           long long n, const KScalars *sc) {
  k_cocg_p<R><<<vgrid(n), VB, 0, h->stream>>>(r, dinv, p, n, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_cocg_p");
}
template <typename R>
int vmul(fdfd_handle *h, typename CT<R>::C *y, const typename CT<R>::C *a, const typename CT<R>::C *b, long long n) {
  k_vmul<R><<<vgrid(n), VB, 0, h->stream>>>(y, a, b, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_vmul");
}
template <typename R>
int dot(fdfd_handle *h, const typename CT<R>::C *a, const typename CT<R>::C *b, long long n, KScalars *sc) {
  int rc = ensure_red(h, RED_BLOCKS);
  if (rc) return rc;
  k_dot<R><<<vgrid(n), VB, 0, h->stream>>>(a, b, n, h->red, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_dot");
}
template <typename R>
int dot_u(fdfd_handle *h, const typename CT<R>::C *a, const typename CT<R>::C *b, const typename CT<R>::C *w,
          long long n, int fin, KScalars *sc) {
  int rc = ensure_red(h, RED_BLOCKS);
  if (rc) return rc;
  k_dot_u<R><<<vgrid(n), VB, 0, h->stream>>>(a, b, w, n, h->red, fin, sc);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_dot_u");
}
int accum(fdfd_handle *h, double2 *x64, float2 *x32, long long n) {
  k_accum<<<vgrid(n), VB, 0, h->stream>>>(x64, x32, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_accum");
}
int accum64(fdfd_handle *h, double2 *x64, double2 *x, long long n) {
  k_accum64<<<vgrid(n), VB, 0, h->stream>>>(x64, x, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_accum64");
}
int demote(fdfd_handle *h, float2 *y, const double2 *x, long long n) {
  k_demote<<<vgrid(n), VB, 0, h->stream>>>(y, x, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_demote");
}
int promote(fdfd_handle *h, double2 *y, const float2 *x, long long n) {
  k_promote<<<vgrid(n), VB, 0, h->stream>>>(y, x, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_promote");
}
template <typename R>
int copy(fdfd_handle *h, typename CT<R>::C *y, const typename CT<R>::C *x, long long n) {
  k_copy<R><<<vgrid(n), VB, 0, h->stream>>>(y, x, n);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "k_copy");
}

#define INST(R)                                                                                                      \
  template int bicg_p<R>(fdfd_handle *, const CT<R>::C *, CT<R>::C *, const CT<R>::C *, long long, const KScalars *); \
  template int bicg_s<R>(fdfd_handle *, const CT<R>::C *, const CT<R>::C *, CT<R>::C *, long long, const KScalars *); \
  template int bicg_xr<R>(fdfd_handle *, CT<R>::C *, const CT<R>::C *, const CT<R>::C *, const CT<R>::C *,          \
                          CT<R>::C *, const CT<R>::C *, long long, KScalars *);                                       \
  template int cocg_xr<R>(fdfd_handle *, CT<R>::C *, const CT<R>::C *, const CT<R>::C *, CT<R>::C *,                 \
                          const CT<R>::C *, const CT<R>::C *, long long, KScalars *);                                 \
  template int cocg_p<R>(fdfd_handle *, const CT<R>::C *, const CT<R>::C *, CT<R>::C *, long long,                  \
                         const KScalars *);                                                                           \
  template int vmul<R>(fdfd_handle *, CT<R>::C *, const CT<R>::C *, const CT<R>::C *, long long);                   \
  template int dot<R>(fdfd_handle *, const CT<R>::C *, const CT<R>::C *, long long, KScalars *);                     \
  template int dot_u<R>(fdfd_handle *, const CT<R>::C *, const CT<R>::C *, const CT<R>::C *, long long, int,        \
                        KScalars *);                                                                                  \
  template int copy<R>(fdfd_handle *, CT<R>::C *, const CT<R>::C *, long long);
INST(float)
INST(double)
#undef INST

}  // namespace fdfd
