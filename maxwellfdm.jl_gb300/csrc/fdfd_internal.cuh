// Internal declarations shared by the translation units of libfdfd_gb300.
//
// Data layout in HBM (per handle):
//   field vectors   AoS complex, component fastest: v[c + 3*cell],
//                   cell = i + Nx*(j + Ny*k)  (the reference's order_cmpfirst
//                   DOF order, model.jl:72, 75-81) — float2 or double2.
//   eps diagonal    SoA real: eps[c*Ncell + cell] = ε_cc at the E_c sample.
//   eps off-diag    SoA real: eoff[p*Ncell + cell], p = xy, yz, zx, at the
//                   E-voxel corner (primal³ point) of the cell.
//   per-axis coefs  complex, length N[w]:  cm = 1/s∆lₘ (curl E→H), ce = 1/s∆lₑ
//                   (curl H→E), wm/wp = corner-averaging weights
//                   s∆lₘ[j-1]/(2 s∆lₑ[j]), s∆lₘ[j]/(2 s∆lₑ[j]).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/fdfd_gb300.h"

namespace fdfd {

// ---------------------------------------------------------------- complex
template <typename R> struct CT;
template <> struct CT<float> { using C = float2; };
template <> struct CT<double> { using C = double2; };

__host__ __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return mk(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return mk(a.x - b.x, a.y - b.y); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) { return mk(a.x * s, a.y * s); }
// conj(a) * b
template <typename C> __host__ __device__ __forceinline__ C cdotc(C a, C b) {
  return mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename C> __host__ __device__ __forceinline__ C czero() { return mk(decltype(C{}.x)(0), decltype(C{}.x)(0)); }

// Device ordinals a handle may use (fdfd_create rejects larger ones).
constexpr int MAX_DEVICES = 64;

// One flag per device for a one-time, per-device set-up step (e.g. a
// kernel's launch attributes).  Atomic: handles on different host threads
// may reach the step together; the step itself is idempotent.
struct DevFlags {
  std::atomic<bool> f[MAX_DEVICES];
  bool done(int dev) const { return f[dev].load(std::memory_order_acquire); }
  void set(int dev) { f[dev].store(true, std::memory_order_release); }
};

// ---------------------------------------------------------------- tiling
constexpr int TX = 32;   // tile width (x), one warp
constexpr int TY = 8;    // tile height (y)
constexpr int NTHR = TX * TY;

// ---------------------------------------------------------------- operator
template <typename R>
struct OpArgs {
  using C = typename CT<R>::C;
  int N[3];
  int bloch[3];
  long long ncell;
  const C *cm[3], *ce[3], *wm[3], *wp[3];
  const R *eps;      // 3*ncell (SoA)
  const R *eoff;     // 3*ncell (SoA) or nullptr
  const uint8_t *oflag;  // per (tile, z-plane) flag: off-diagonal present; nullptr = everywhere
  C w2;              // ω²
  int rlo[3], rhi[3];  // per axis: index range whose cm, ce, wm, wp are all real (outside the PML)
};

// Epilogue of the stencil: what to do with y = A x at each cell.
enum EpiKind : int {
  EPI_STORE = 0,        // y = A x
  EPI_RESID = 1,        // y = b - A x, accumulate ‖y‖²       (aux0 = b)
  EPI_DOT_AUX = 2,      // y = A x, accumulate conj(aux0)·y     (aux0 = r̂)
  EPI_DOT_TS = 3,       // y = A x, accumulate conj(y)·x, ‖y‖²  (t = A s)
  EPI_DOT_SU = 4,       // y = A x, accumulate Σ V_E·x·y (unconjugated, COCG's pᵀ S q)
  EPI_DOT_SHD = 5,      // y = A x, accumulate conj(r̂)·y with the generated shadow vector r̂
};

// Reduction slots used by the fused kernels: each kernel accumulates up to
// two complex partial sums per block into part[blk*2 + {0,1}] (FP64).
struct RedBuf {
  double2 *part;         // >= 2 * max blocks
  unsigned int *count;   // arrival counter for the last-block finalisation
};

// Scalars of a Krylov iteration, resident in device memory so that whole
// batches of iterations run (and replay as a CUDA graph) without host sync.
struct KScalars {
  double2 rho, alpha, omega, beta;
  double2 dot0, dot1;    // raw finalised reductions of the last kernel
  double rr;             // recursive ‖r‖² (inner precision)
  double rr_max;         // largest ‖r‖² since the last reliable update
  double bb;             // ‖b‖²
  double stop2;          // recursive-residual stop threshold (‖r‖²)
  double upd2;           // δ²: reliable update when rr < upd2 * rr_max
  int done;              // 1: later kernels of the batch are no-ops
  int reason;            // 1 recursive converged, 2 reliable update due, 3 breakdown, 4 nonfinite
  long long iter;
  // BiCGStab(ℓ), ℓ ≤ 4: −ω·ρ of the last cycle end, and the coefficients of
  // the cycle's closing update x += Σ cx_k r_k, r₀ += Σ cr_k r_k, u₀ += Σ cu_k u_k
  double2 rho_pre;
  double2 cx[5], cr[5], cu[5];
  double2 gram[14];  // (r_i, r_j), 1 ≤ i ≤ j ≤ ℓ, then (r_i, r_0)
};

struct Workspace;  // solver vectors (solver.cu)

}  // namespace fdfd

struct fdfd_handle {
  int dev = 0;
  cudaStream_t stream = nullptr;
  int N[3] = {0, 0, 0};
  int bloch[3] = {0, 0, 0};
  long long ncell = 0;
  double omega[2] = {0, 0};
  double w2[2] = {0, 0};
  double e_ikl[3][2];
  // per-axis coefficients: [kind(4)][axis(3)] contiguous, kind = cm, ce, wm, wp
  double2 *coef64 = nullptr;
  float2 *coef32 = nullptr;
  long long coef_off[3] = {0, 0, 0};
  int coef_stride = 0;  // = N[0]+N[1]+N[2]
  int rlo[3] = {1, 1, 1}, rhi[3] = {0, 0, 0};  // real-coefficient index range per axis (empty: lo > hi)
  double *eps64 = nullptr;
  float *eps32 = nullptr;
  double *eoff64 = nullptr;
  float *eoff32 = nullptr;
  uint8_t *oflag = nullptr;
  uint8_t *oflag_rows[2] = {nullptr, nullptr};  // the same per x tile, group of 1 / 2 rows and plane
  bool has_off = false;
  uint8_t *smask = nullptr;  // 4*ncell smoothing mask (from fdfd_smooth_objects)
  bool has_design = false;   // a design region was applied by fdfd_smooth_objects
  int design_lo[3] = {0, 0, 0}, design_hi[3] = {0, 0, 0};
  // scratch for host-pointer entry points
  double2 *vx64 = nullptr, *vy64 = nullptr;
  double2 *ve64 = nullptr;  // adjoint entry point: the forward field
  double2 *stage64 = nullptr;  // 2D slices: compact host-layout staging
  int slice2d = 0;             // FDFD_SLICE_NONE / _TE / _TM
  int ft = 0;                  // field solved for: FDFD_EE (A = CₘCₑ − ω²Pε) or FDFD_HH (A = CₑPε⁻¹Cₘ − ω²)
  bool shares_operator = false;  // a batch worker: coefficients, ε and flags belong to its parent
  float2 *vx32 = nullptr, *vy32 = nullptr;
  fdfd::RedBuf red{nullptr, nullptr};
  int red_blocks = 0;
  fdfd::Workspace *ws = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  long long launches = 0;  // kernels launched by this handle (graph replays included)
  fdfd::KScalars *util_sc = nullptr;  // finalisation target of one-off reductions
  int *dev_err = nullptr;             // set by a kernel whose bounded wait gave up
  bool tma_disabled = false;          // FDFD_DISABLE_TMA=1: plain-load operator kernel only
  bool pdl = false;                   // programmatic dependent launch (FDFD_PDL=1 enables)
  int kc[2] = {0, 0};                 // tuned z-chunk length: [complex128, complex64]
  // second TMA kernel: a balanced schedule per precision (same order) of
  // (x tile, y tile, k0, k1) per thread block, heaviest first, when the
  // tuner found it faster than uniform chunks (nwork 0: uniform)
  int4 *work[2] = {nullptr, nullptr};
  int nwork[2] = {0, 0};
  int kc_force = 0;                   // FDFD_KCHUNK: fixed z-chunk length (no tuning)
  // SM clocks a pipeline wait of the TMA operator kernel may take before it
  // gives up (≈1 s); FDFD_WAIT_LIMIT_CLOCKS lowers it, so that a test can
  // make a wait run out and see FDFD_ERR_TIMEOUT without hanging anything
  long long wait_limit = 1ll << 31;
  // layout of the second TMA operator kernel (stencil2.cu): picked by the
  // autotuner among 4, 1 and 3 for complex64, or fixed by FDFD_OPERATOR_V2
  // at create: 0 = first TMA kernel only; 4 (default) = two
  // rows per warp, 4-slot ring, ε diagonal from global memory, 2 CTAs per SM;
  // 1 = one row per warp, 4 slots, 3 CTAs; 2 = two rows, 3 slots, ε diagonal
  // through the ring; 3 = as 1 with 2 CTAs.  Measured at 320³ with 400
  // spheres: 4: 439 µs, 2: 496 µs, 3: 494 µs, 1: 556 µs, first kernel 525 µs.
  int op_variant = 4;
  int tuned_off = -1;                 // has_off at the last tuning (−1: not tuned yet)
  std::string err;
};

namespace fdfd {

int set_error(fdfd_handle *h, int code, const std::string &msg);
// cudaMalloc with a host-side failure hook: while the environment variable
// FDFD_FAIL_ALLOC_BYTES holds a positive number, every request of at least
// that many bytes fails with cudaErrorMemoryAllocation without calling the
// runtime — the way tests exercise FDFD_ERR_NOMEM without exhausting a GPU.
cudaError_t dev_malloc_raw(void **p, size_t bytes);
template <typename T> inline cudaError_t dev_malloc(T **p, size_t bytes) {
  return dev_malloc_raw(reinterpret_cast<void **>(p), bytes);
}
int cuda_check(fdfd_handle *h, cudaError_t e, const char *what);
// FDFD_ERR_TIMEOUT (and clears the flag) if a kernel reported a bounded
// wait that gave up; call after the stream has been synchronised.
int check_dev_err(fdfd_handle *h);

template <typename R> OpArgs<R> op_args(const fdfd_handle *h);

// Launch y = A x (or Aᵀ x), with the fused epilogue `epi` and, for reducing
// epilogues, the finalisation `fin` into `sc` (which also gates the launch:
// sc->done != 0 turns it into a no-op).  On the handle's stream.
template <typename R>
int launch_apply_fin(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                     const typename CT<R>::C *aux0, int fin, KScalars *sc, bool transpose);
// the second TMA operator kernel (stencil2.cu); FDFD_ERR_UNSUPPORTED when it
// does not serve the call (the caller then uses the first one)
template <typename R>
int launch_apply_v2(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                    const typename CT<R>::C *aux0, int fin, KScalars *sc, int kc);
// number of blocks launch_apply uses (reduction buffer sizing)
int apply_blocks(const fdfd_handle *h);
// pick the z-chunk length per precision by timing (stencil.cu)
int autotune_kchunk(fdfd_handle *h);

// Finalise per-block partials; defined in blas1.cu
int ensure_red(fdfd_handle *h, int blocks);

void free_workspace(fdfd_handle *h);
// destroy the captured solver graphs (launch shapes or buffers changed)
void drop_graphs(fdfd_handle *h);
int smooth_objects_impl(fdfd_handle *h, const double *const lprim[3], const fdfd_object *objs, int nobj,
                        double eps_bg, const fdfd_design *design);
int upload_eps(fdfd_handle *h, const double *eps_diag_aos, const double *eps_off_aos);
// adjoint.cu
int eps_grad_dev_impl(fdfd_handle *h, const double2 *e, const double2 *g, double2 *lam, double *grad,
                      const fdfd_solve_opts *opts, fdfd_stats *stats);
int design_grad_dev_impl(fdfd_handle *h, const double *grad, double *out);
// fields.cu
int h_from_e_dev_impl(fdfd_handle *h, const double2 *e, const double2 *jm, double2 *hout);
int e_from_h_dev_impl(fdfd_handle *h, const double2 *hin, const double2 *je, double2 *eout);
int corner_mean_dev_impl(fdfd_handle *h, int hfield, const double2 *in, double2 *out);
// host vectors of a 2D slice carry only some components (fields.cu)
int field_mask(const fdfd_handle *h, bool hfield);
int h2d_field(fdfd_handle *h, const double *src, double2 *dst, int mask);
int d2h_field(fdfd_handle *h, const double2 *src, double *dst, int mask);
int d2h_real(fdfd_handle *h, const double *src, double *dst, int mask);
// the H formulation's operator (hh.cu)
template <typename R>
int launch_apply_hh(fdfd_handle *h, const typename CT<R>::C *x, typename CT<R>::C *y, int epi,
                    const typename CT<R>::C *aux0, int fin, KScalars *sc);
int build_oflags(fdfd_handle *h);

}  // namespace fdfd
