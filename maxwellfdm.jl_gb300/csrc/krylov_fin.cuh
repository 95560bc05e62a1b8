// Grid-wide reductions and the scalar recurrences of the Krylov solvers.
//
// Every reducing kernel writes two FP64 complex partials per block; the
// last block to arrive (atomic counter) sums them in block order — so the
// result is deterministic — and runs the scalar update of the solver step
// (finalise).  No block ever waits on another: the counter is only read by
// the block that incremented it last.
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
  const int re = (int)(int16_t)(hsh & 0xffffu), im = (int)(int16_t)(hsh >> 16);
  return mk(R(re) * R(1.0 / 32768.0), R(im) * R(1.0 / 32768.0));
}

// Error-free FP32 addition (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Warp sum of a value that carries at most about 48 significant bits (an
// FP32 sum, or a compensated FP32 sum widened to FP64): split into FP32
// (hi, lo), add along an FP32 TwoSum tree, widen once.  The GPU's FP64 pipe
// is a small fraction of its FP32 pipe, so the warp trees of the complex64
// kernels avoid FP64 additions altogether.
__device__ __forceinline__ double warp_sum_split(double x) {
  float hi = (float)x, lo = (float)(x - (double)hi);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
    float s, e;
    two_sum_f(hi, oh, s, e);
    hi = s;
    lo = lo + ol + e;
  }
  return (double)hi + (double)lo;
}

// Block-level reduction of two complex FP64 values, then the grid-level
// last-block finalisation.  Must be called by every thread of the block.
// F32 (complex64 kernels): the warp trees run in FP32 TwoSum arithmetic.
template <int NT, bool F32 = false>
__device__ inline void block_reduce_finalise(double2 a0, double2 a1, RedBuf red, int mode, KScalars *sc) {
  __shared__ double2 wred[NT / 32][2];
  __shared__ bool last;
  if (F32) {
    a0.x = warp_sum_split(a0.x);
    a0.y = warp_sum_split(a0.y);
    a1.x = warp_sum_split(a1.x);
    a1.y = warp_sum_split(a1.y);
  } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0.x += __shfl_xor_sync(0xffffffffu, a0.x, o);
      a0.y += __shfl_xor_sync(0xffffffffu, a0.y, o);
      a1.x += __shfl_xor_sync(0xffffffffu, a1.x, o);
      a1.y += __shfl_xor_sync(0xffffffffu, a1.y, o);
    }
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
// compensated (Neumaier) FP32 sum, widened to FP64 before the block
// reduction — products and the short per-thread sums stay in FP32, every
// cross-thread and cross-block addition is FP64.
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
  __device__ __forceinline__ double get() const { return (double)s + (double)c; }
};

// Short per-thread sum (the operator kernel's epilogue adds at most
// 3 × z-chunk terms per thread): plain FP32, widened before the FP64
// block and grid sums.
template <typename R> struct ShortAcc;
template <> struct ShortAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double get() const { return s; }
};
template <> struct ShortAcc<float> {
  float s = 0.f;
  __device__ __forceinline__ void add(float v) { s += v; }
  __device__ __forceinline__ double get() const { return (double)s; }
};

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
