// Grid-wide reductions and the scalar recurrences of the Krylov solvers.
//
// Every reducing kernel writes its partial sums per block; the last block
// to arrive (atomic counter) sums them in block order — so the result is
// deterministic — and runs the scalar update of the solver step
// (finalise).  No block ever waits on another: the counter is only read by
// the block that incremented it last.  complex128 kernels sum in FP64;
// complex64 kernels sum in double-float FP32 arithmetic (DF below) up to
// the single value per sum that is widened for finalise.
#pragma once

#include "fdfd_internal.cuh"

namespace fdfd {

enum FinMode : int {
  FIN_NONE = 0,    // store the sums in sc->dot0 / sc->dot1
  FIN_ALPHA = 1,   // BiCGSTAB: α = ρ / (r̂, v)
  FIN_OMEGA = 2,   // BiCGSTAB: ω = (t, s) / (t, t)
  FIN_XR = 3,      // BiCGSTAB: ρ' = (r̂, r), β = ρ'/ρ · α/ω, ‖r‖², stop tests
  FIN_RESID = 4,   // ‖b − A x‖² into dot0.x (reliable update / final check)
  FIN_COCG_A = 5,  // COCG: α = ρ / (pᵀ q)
  FIN_COCG_R = 6,  // COCG: ρ' = rᵀ r, β = ρ'/ρ, ‖r‖², stop tests
  FIN_BL_RHO = 7,    // BiCGStab(ℓ) inside a cycle: ρ₁ = (r̂, r_j), β = α ρ₁/ρ₀, ρ₀ = ρ₁
  FIN_BL_CYCLE = 8,  // BiCGStab(ℓ) cycle end: ρ₀ = −ω ρ₀, then as FIN_BL_RHO; ‖r₀‖², stop tests
  FIN_BL_REDO = 9,   // after a replaced residual: ρ₁ = (r̂, r₀) against the stored −ω ρ₀
};

__device__ __forceinline__ double2 dcdiv(double2 a, double2 b) {
  double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 dcmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ bool dfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }

__device__ __forceinline__ void stop_tests(KScalars *sc, double rr) {
  sc->rr = rr;
  sc->iter += 1;
  if (rr > sc->rr_max) sc->rr_max = rr;
  if (!isfinite(rr)) { sc->done = 1; sc->reason = 4; return; }
  if (rr <= sc->stop2) { sc->done = 1; sc->reason = 1; return; }
  if (rr <= sc->upd2 * sc->rr_max) { sc->done = 1; sc->reason = 2; return; }
}

__device__ inline void finalise(int mode, KScalars *sc, double2 d0, double2 d1) {
  sc->dot0 = d0;
  sc->dot1 = d1;
  switch (mode) {
    case FIN_ALPHA: {
      if (!dfinite(d0)) { sc->done = 1; sc->reason = 4; break; }
      if (d0.x == 0.0 && d0.y == 0.0) { sc->done = 1; sc->reason = 3; break; }
      sc->alpha = dcdiv(sc->rho, d0);
      break;
    }
    case FIN_OMEGA: {
      if (!dfinite(d0) || !isfinite(d1.x)) { sc->done = 1; sc->reason = 4; break; }
      sc->omega = d1.x > 0.0 ? make_double2(d0.x / d1.x, d0.y / d1.x) : make_double2(0.0, 0.0);
      break;
    }
    case FIN_XR: {
      double2 rho_new = d0;
      double2 om = sc->omega;
      if (om.x == 0.0 && om.y == 0.0) { stop_tests(sc, d1.x); if (!sc->done) { sc->done = 1; sc->reason = 3; } break; }
      if (rho_new.x == 0.0 && rho_new.y == 0.0) { stop_tests(sc, d1.x); if (!sc->done) { sc->done = 1; sc->reason = 3; } break; }
      sc->beta = dcmul(dcdiv(rho_new, sc->rho), dcdiv(sc->alpha, om));
      sc->rho = rho_new;
      stop_tests(sc, d1.x);
      break;
    }
    case FIN_COCG_A: {
      if (!dfinite(d0)) { sc->done = 1; sc->reason = 4; break; }
      if (d0.x == 0.0 && d0.y == 0.0) { sc->done = 1; sc->reason = 3; break; }
      sc->alpha = dcdiv(sc->rho, d0);
      break;
    }
    case FIN_BL_RHO:
    case FIN_BL_REDO:
    case FIN_BL_CYCLE: {
      if (mode == FIN_BL_CYCLE) sc->rho_pre = make_double2(-(sc->omega.x * sc->rho.x - sc->omega.y * sc->rho.y),
                                                          -(sc->omega.x * sc->rho.y + sc->omega.y * sc->rho.x));
      const double2 rho0 = mode == FIN_BL_RHO ? sc->rho : sc->rho_pre;
      if (!dfinite(d0)) { sc->done = 1; sc->reason = 4; break; }
      if (rho0.x == 0.0 && rho0.y == 0.0) {
        if (mode == FIN_BL_CYCLE) stop_tests(sc, d1.x);
        if (!sc->done) { sc->done = 1; sc->reason = 3; }
        break;
      }
      sc->beta = dcmul(sc->alpha, dcdiv(d0, rho0));
      sc->rho = d0;
      if (mode == FIN_BL_CYCLE) stop_tests(sc, d1.x);
      break;
    }
    case FIN_COCG_R: {
      double2 rho_new = d0;
      if (sc->rho.x == 0.0 && sc->rho.y == 0.0) { sc->done = 1; sc->reason = 3; break; }
      sc->beta = dcdiv(rho_new, sc->rho);
      sc->rho = rho_new;
      stop_tests(sc, d1.x);
      break;
    }
    default:
      break;
  }
}

// The BiCGStab(ℓ) shadow vector r̂, generated from the DOF index instead of
// stored: r̂_i = (a + i·b)/32768 with a, b the two 16-bit halves (as signed
// integers) of a 32-bit integer hash of i — Chris Wellons' "lowbias32"
// mixing function (xor-shift / multiply rounds).  Any fixed r̂ is a valid
// shadow vector; a random one converged at least as fast as r̂ = r₀ on
// these systems, and generating it saves a vector read in every operator
// application with a dot product.  The values are exact in FP32, so both
// precisions use the same r̂.
__host__ __device__ __forceinline__ uint32_t shadow_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
template <typename R>
__device__ __forceinline__ typename CT<R>::C shadow(long long dof) {
  const uint32_t hsh = shadow_hash((uint32_t)dof);
  if constexpr (sizeof(R) == 4) {
    // the same values without integer→float conversions: a half h, read as
    // signed, is (h ^ 0x8000) − 32768; the float with bits 0x4B000000 | v is
    // 2²³ + v exactly, and (2²³ + v)·2⁻¹⁵ − (2⁸ + 1) = (v − 32768)/32768
    // is exact in one fused multiply-add per lane
    const float2 b = make_float2(__uint_as_float(0x4B000000u | ((hsh & 0xffffu) ^ 0x8000u)),
                                 __uint_as_float(0x4B000000u | ((hsh >> 16) ^ 0x8000u)));
    return __ffma2_rn(b, make_float2(1.0f / 32768.0f, 1.0f / 32768.0f), make_float2(-257.0f, -257.0f));
  } else {
    const int re = (int)(int16_t)(hsh & 0xffffu), im = (int)(int16_t)(hsh >> 16);
    return mk(R(re) * R(1.0 / 32768.0), R(im) * R(1.0 / 32768.0));
  }
}

template <typename R>
__device__ __forceinline__ typename CT<R>::C tocr(double2 v) {
  return mk(R(v.x), R(v.y));
}

// Complex scalars of the recurrence in the kernel's precision (at(i) gives
// the i-th as double2).  complex64 kernels convert each one once per block
// into shared memory: an FP64 → FP32 conversion runs on the narrow FP64
// pipe, and done by every thread it held back the first vector loads by
// microseconds.  Every thread of the block must call it.
template <typename R, int NS, typename F>
__device__ __forceinline__ void scalars(F at, typename CT<R>::C (&out)[NS]) {
  using C = typename CT<R>::C;
  if constexpr (sizeof(R) == 8) {
#pragma unroll
    for (int i = 0; i < NS; ++i) out[i] = at(i);
  } else {
    __shared__ C s[NS];
    if (threadIdx.x < NS) s[threadIdx.x] = tocr<R>(at(threadIdx.x));
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NS; ++i) out[i] = s[i];
  }
}

// Error-free FP32 addition (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Double-float value hi + lo: about 48 significant bits carried in FP32
// arithmetic.  The GPU's FP64 pipe (conversions included) is a small
// fraction of its FP32 pipe, so the complex64 kernels keep every
// cross-thread and cross-block sum in this form.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s, e;
  two_sum_f(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  DF r;
  two_sum_f(s, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ DF df_shfl_xor(DF v, int o) {
  return DF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ double df_widen(DF v) { return (double)v.hi + (double)v.lo; }

// Warp reduce-scatter of K double-float values per lane (K a power of two,
// ≤ 32): butterfly levels 16, 8, … each halve the values a lane keeps
// (lanes with the level's bit set keep the upper half), then plain
// butterfly levels once one value is left — K−1+(5−log2 K) additions per
// lane instead of 5K.  Lane l ends with the warp sum of value
// l >> (5 − log2 K) in v[0]; the order of additions is fixed.
template <int M, int O>
struct DfScatter {
  static __device__ __forceinline__ void run(DF *v, int lane) {
    if constexpr (M > 1) {
      const bool up = (lane & O) != 0;
#pragma unroll
      for (int i = 0; i < M / 2; ++i) {
        const DF keep = up ? v[M / 2 + i] : v[i];
        const DF send = up ? v[i] : v[M / 2 + i];
        v[i] = df_add(keep, df_shfl_xor(send, O));
      }
      DfScatter<M / 2, O / 2>::run(v, lane);
    } else {
      v[0] = df_add(v[0], df_shfl_xor(v[0], O));
      DfScatter<1, O / 2>::run(v, lane);
    }
  }
};
template <int M>
struct DfScatter<M, 0> {
  static __device__ __forceinline__ void run(DF *, int) {}
};
template <int K>
constexpr int df_shift() {
  return K >= 32 ? 0 : K >= 16 ? 1 : K >= 8 ? 2 : K >= 4 ? 3 : K >= 2 ? 4 : 5;
}

// Block and grid sums of KR double-float values per thread (v holds K ≥ KR
// slots, K a power of two, the slots from KR on zero).  Writes the block's
// KR partials (float2 each, KR/2 double2 slots of red.part per block) and
// returns true in the block that arrives last, which then holds the grid
// sums, widened to FP64, in tot (shared, KR entries).  Every thread of the
// block must call it.
template <int NT, int K, int KR>
__device__ bool df_block_sums_last(DF (&v)[K], RedBuf red, double *tot) {
  static_assert((K & (K - 1)) == 0 && K <= 32 && KR <= K && (KR % 2) == 0, "DF block sums");
  constexpr int NW = NT / 32;
  __shared__ DF wred[NW][K];
  __shared__ bool last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, wid = tid >> 5;
  DfScatter<K, 16>::run(v, lane);
  if ((lane & ((1 << df_shift<K>()) - 1)) == 0) wred[wid][lane >> df_shift<K>()] = v[0];
  __syncthreads();
  const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
  const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  float2 *part = reinterpret_cast<float2 *>(red.part);
  if (tid < KR) {
    DF s = wred[0][tid];
#pragma unroll
    for (int w = 1; w < NW; ++w) s = df_add(s, wred[w][tid]);
    part[(long long)KR * bid + tid] = make_float2(s.hi, s.lo);
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) last = atomicAdd(red.count, 1u) == nblk - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // value q is summed by warp q mod NW: lanes over the blocks in a fixed
  // order, then a fixed butterfly
  for (int q = wid; q < KR; q += NW) {
    DF s{0.f, 0.f};
    for (unsigned b = lane; b < nblk; b += 32) {
      const float2 p = __ldcg(&part[(long long)KR * b + q]);
      s = df_add(s, DF{p.x, p.y});
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_xor(s, o));
    if (lane == 0) tot[q] = df_widen(s);
  }
  __syncthreads();
  if (tid == 0) *red.count = 0u;
  return true;
}

// complex64 kernels: grid sums of the complex a0 and a1 (as four
// double-float reals), then finalise in the last block.
template <int NT>
__device__ inline void block_reduce_finalise_df(DF a0r, DF a0i, DF a1r, DF a1i, RedBuf red, int mode, KScalars *sc) {
  __shared__ double tot[4];
  DF v[4] = {a0r, a0i, a1r, a1i};
  if (!df_block_sums_last<NT, 4, 4>(v, red, tot)) return;
  if (threadIdx.x + threadIdx.y + threadIdx.z == 0 && sc)
    finalise(mode, sc, make_double2(tot[0], tot[1]), make_double2(tot[2], tot[3]));
}

// Block-level reduction of two complex FP64 values (complex128 kernels),
// then the grid-level last-block finalisation.  Must be called by every
// thread of the block.
template <int NT>
__device__ inline void block_reduce_finalise(double2 a0, double2 a1, RedBuf red, int mode, KScalars *sc) {
  __shared__ double2 wred[NT / 32][2];
  __shared__ bool last;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0.x += __shfl_xor_sync(0xffffffffu, a0.x, o);
    a0.y += __shfl_xor_sync(0xffffffffu, a0.y, o);
    a1.x += __shfl_xor_sync(0xffffffffu, a1.x, o);
    a1.y += __shfl_xor_sync(0xffffffffu, a1.y, o);
  }
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, wid = tid >> 5;
  if (lane == 0) { wred[wid][0] = a0; wred[wid][1] = a1; }
  __syncthreads();
  const unsigned nblk = gridDim.x * gridDim.y * gridDim.z;
  const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (tid == 0) {
    double2 s0 = make_double2(0, 0), s1 = make_double2(0, 0);
    for (int w = 0; w < NT / 32; ++w) {
      s0.x += wred[w][0].x; s0.y += wred[w][0].y;
      s1.x += wred[w][1].x; s1.y += wred[w][1].y;
    }
    red.part[2 * bid] = s0;
    red.part[2 * bid + 1] = s1;
    __threadfence();
    unsigned prev = atomicAdd(red.count, 1u);
    last = (prev == nblk - 1);
  }
  __syncthreads();
  if (!last) return;
  // last block: deterministic sum of all partials in block order
  __threadfence();
  double2 s0 = make_double2(0, 0), s1 = make_double2(0, 0);
  for (unsigned b = tid; b < nblk; b += NT) {
    double2 p0 = __ldcg(&red.part[2 * b]);
    double2 p1 = __ldcg(&red.part[2 * b + 1]);
    s0.x += p0.x; s0.y += p0.y;
    s1.x += p1.x; s1.y += p1.y;
  }
  // fixed-order tree over the block (deterministic for a fixed launch shape)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0.x += __shfl_xor_sync(0xffffffffu, s0.x, o);
    s0.y += __shfl_xor_sync(0xffffffffu, s0.y, o);
    s1.x += __shfl_xor_sync(0xffffffffu, s1.x, o);
    s1.y += __shfl_xor_sync(0xffffffffu, s1.y, o);
  }
  __syncthreads();
  if (lane == 0) { wred[wid][0] = s0; wred[wid][1] = s1; }
  __syncthreads();
  if (tid == 0) {
    double2 t0 = make_double2(0, 0), t1 = make_double2(0, 0);
    for (int w = 0; w < NT / 32; ++w) {
      t0.x += wred[w][0].x; t0.y += wred[w][0].y;
      t1.x += wred[w][1].x; t1.y += wred[w][1].y;
    }
    *red.count = 0u;
    if (sc) finalise(mode, sc, t0, t1);
  }
}

// Per-thread accumulator: FP64 for double kernels; for float kernels a
// compensated (Neumaier) FP32 sum, handed to the block reduction as a
// double-float — products and per-thread sums in FP32, every cross-thread
// and cross-block addition in double-float (float kernels) or FP64.
template <typename R> struct Acc;
template <> struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double get() const { return s; }
};
template <> struct Acc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float t = s + v;
    c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
    s = t;
  }
  __device__ __forceinline__ DF df() const {
    DF r;
    two_sum_f(s, c, r.hi, r.lo);
    return r;
  }
};

// Short per-thread sum (the operator kernel's epilogue adds at most
// 3 × z-chunk terms per thread): plain FP32 for float kernels.
template <typename R> struct ShortAcc;
template <> struct ShortAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double get() const { return s; }
};
template <> struct ShortAcc<float> {
  float s = 0.f;
  __device__ __forceinline__ void add(float v) { s += v; }
  __device__ __forceinline__ DF df() const { return DF{s, 0.f}; }
};

// Grid sums a0 = a0r + i·a0i and a1 (real) of a reducing kernel, then the
// solver's scalar step `mode` in the last block (the accumulators'
// precision picks the FP64 or the double-float path).
template <int NT, typename A, typename B>
__device__ inline void sum_finalise(const A &a0r, const A &a0i, const B &a1, RedBuf red, int mode, KScalars *sc) {
  if constexpr (sizeof(a0r.s) == 4)
    block_reduce_finalise_df<NT>(a0r.df(), a0i.df(), a1.df(), DF{0.f, 0.f}, red, mode, sc);
  else
    block_reduce_finalise<NT>(make_double2(a0r.get(), a0i.get()), make_double2(a1.get(), 0.0), red, mode, sc);
}
template <int NT, typename A>
__device__ inline void sum_finalise(const A &a0r, const A &a0i, RedBuf red, int mode, KScalars *sc) {
  if constexpr (sizeof(a0r.s) == 4)
    block_reduce_finalise_df<NT>(a0r.df(), a0i.df(), DF{0.f, 0.f}, DF{0.f, 0.f}, red, mode, sc);
  else
    block_reduce_finalise<NT>(make_double2(a0r.get(), a0i.get()), make_double2(0.0, 0.0), red, mode, sc);
}

// Programmatic dependent launch: a kernel lets the next one in the stream
// start its prologue early (launch_dependents) and waits for the previous
// kernel's results to be complete and visible (wait) before reading them.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch with programmatic stream serialisation (when h->pdl): the kernel
// may begin while its predecessor in the stream is finishing; the kernel's
// own pdl_wait() orders its reads.  Recorded as programmatic edges when the
// stream is being captured into a CUDA graph.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(const fdfd_handle *h, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                            Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = h->pdl ? at : nullptr;
  cfg.numAttrs = h->pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace fdfd
