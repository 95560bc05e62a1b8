/*
 * fdfd_gb300.h — C ABI of the GB300 FDFD operator and solver.
 *
 * A drop-in for the hot path of MaxwellFDFD.jl: the sparse operator
 *     A = Cₘ·(Pμ \ Cₑ) − ω²·Pε          (src/model/model.jl:235-237)
 * that the reference assembles as a SparseMatrixCSC{ComplexF64} and the
 * caller then applies (A*x, mul!(y,A,x)) or solves (A\b).  Here A is never
 * assembled: it is applied matrix-free by sm_103a kernels.
 *
 * Conventions shared with the reference:
 *   - complex numbers cross the boundary as interleaved (re, im) doubles
 *     (Julia ComplexF64 memory layout);
 *   - field vectors are component-fastest, DOF index c + 3·(i + Nx·(j + Ny·k))
 *     (order_cmpfirst = true, model.jl:72, 75-81);
 *   - the stretched ∆l arrays are the outputs of create_stretched_∆ls
 *     (model.jl:122-139);
 *   - the material tensor is the reference's εarr, an (Nx,Ny,Nz,3,3)
 *     column-major ComplexF64 array (model.jl:51; full.jl:16-70).
 *
 * Every call returns an int status (FDFD_OK = 0); none aborts or traps.
 * fdfd_last_error() returns the message of the last failure on a handle.
 * A handle owns one CUDA stream and its device buffers; it must not be used
 * from two threads at once.  Separate handles are independent.
 */
#ifndef FDFD_GB300_H
#define FDFD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  FDFD_OK = 0,
  FDFD_ERR_ARG = 1,           /* invalid argument: NULL pointer, bad size or enum   */
  FDFD_ERR_UNSUPPORTED = 2,   /* valid model feature this library does not implement */
  FDFD_ERR_CUDA = 3,          /* CUDA runtime error                                  */
  FDFD_ERR_NOMEM = 4,         /* device or pinned-host allocation failed             */
  FDFD_ERR_NOT_CONVERGED = 5, /* solver reached maxit before tol                      */
  FDFD_ERR_BREAKDOWN = 6,     /* Krylov breakdown (a recurrence scalar vanished)     */
  FDFD_ERR_NO_DEVICE = 7,     /* no CUDA device                                       */
  FDFD_ERR_NONFINITE = 8,     /* NaN/Inf met in the iteration                        */
  FDFD_ERR_TIMEOUT = 9        /* a bounded device-side wait gave up                  */
};

/* arithmetic of an operator application */
enum { FDFD_C128 = 0, FDFD_C64 = 1 };
/* boundary field type (MaxwellBase EE / HH) */
enum { FDFD_EE = 0, FDFD_HH = 1 };
/* solver precision */
enum { FDFD_PREC_FP64 = 0, FDFD_PREC_MIXED = 1 };
/* Krylov method: BiCGSTAB; Jacobi-preconditioned COCG on the symmetrised
 * operator (FP64 only); BiCGStab(ℓ) (Sleijpen–Fokkema), ℓ = opts.ell ≤ 4 */
enum { FDFD_BICGSTAB = 0, FDFD_COCG = 1, FDFD_BICGSTABL = 2 };

typedef struct fdfd_handle fdfd_handle;

/* 2D models (ModelTE, src/model/te.jl: E = (Ex, Ey), H = Hz; ModelTM,
 * src/model/tm.jl: E = Ez, H = (Hx, Hy)) run as the z-invariant slice of the
 * 3D operator: N[2] = 1, isbloch[2] = 1, e_ikl[2] = 1, where ∂z vanishes and
 * the operator splits exactly into the TE and TM blocks.  Host field
 * vectors then carry only the slice's components, component fastest
 * (TE: E 2·Ncell and H Ncell complex values; TM: E Ncell and H 2·Ncell) —
 * the reference's 2D DOF order.  Device-buffer entry points and the ε
 * arrays keep the 3-component layout. */
enum { FDFD_SLICE_NONE = 0, FDFD_SLICE_TE = 1, FDFD_SLICE_TM = 2 };

/* Model description.  Replaces the inputs the reference feeds to
 * create_curls / create_paramops (model.jl:154-188): grid size, boundary,
 * Bloch phase, ω and the stretched ∆l arrays. */
typedef struct {
  int32_t N[3];             /* cells per axis                                          */
  int32_t isbloch[3];       /* 1 = Bloch, 0 = symmetry boundary (PEC for boundft EE)   */
  int32_t boundft[3];       /* FDFD_EE on every axis (HH staggering: unsupported)   */
  int32_t order_cmpfirst;   /* must be 1                                               */
  int32_t device;           /* CUDA device ordinal                                     */
  int32_t slice2d;          /* FDFD_SLICE_NONE (3D), FDFD_SLICE_TE or FDFD_SLICE_TM      */
  double omega[2];          /* ω (re, im)                                              */
  double e_ikl[3][2];       /* e^{-i kbloch L} per axis (used on Bloch axes)           */
  const double *sdl_e[3];   /* s∆lₑ: N[w] complex values at E-voxel-corner planes      */
  const double *sdl_m[3];   /* s∆lₘ: N[w] complex values at H-voxel-corner planes      */
} fdfd_desc;

/* Shapes for the on-device assignment + subpixel smoothing of ε
 * (replaces add_obj! + calc_matparams!, model.jl:107-120, full.jl:16-70). */
enum { FDFD_SHAPE_SPHERE = 0, FDFD_SHAPE_BOX = 1, FDFD_SHAPE_CYLZ = 2 };
typedef struct {
  int32_t kind;     /* FDFD_SHAPE_*                                  */
  int32_t pad;
  double eps;       /* isotropic real ε of the object's material    */
  double p[6];      /* sphere: cx, cy, cz, r; box: lox, loy, loz, hix, hiy, hiz;
                       cylz (infinite along z, the 2D disk): cx, cy, r        */
} fdfd_object;

/* Optional per-cell ε design region over cells [lo, hi) (inverse design). */
typedef struct {
  int32_t lo[3];
  int32_t hi[3];
  const double *eps_cells;  /* (hi-lo) cells, x fastest                        */
} fdfd_design;

typedef struct {
  int32_t method;           /* FDFD_BICGSTABL (default), FDFD_BICGSTAB or FDFD_COCG    */
  int32_t precision;        /* FDFD_PREC_FP64 or FDFD_PREC_MIXED                       */
  double tol;               /* target true relative residual ‖b − A x‖/‖b‖ (FP64)      */
  int64_t maxit;            /* iteration cap                                           */
  double delta;             /* mixed: reliable-update trigger (residual drop factor)   */
  int32_t x0_given;         /* 1: x holds the initial guess                            */
  int32_t check_every;      /* iterations per launched batch between host checks       */
  int32_t transpose;        /* 1: solve Aᵀ x = b (adjoint)                             */
  int32_t use_graph;        /* 1: replay each batch as a CUDA graph                     */
  int32_t ell;              /* FDFD_BICGSTABL: degree ℓ of the minimal-residual part (1–4) */
} fdfd_solve_opts;

typedef struct {
  int64_t iterations;       /* Krylov iterations                                       */
  int64_t matvecs;          /* operator applications (all precisions)                  */
  int32_t refinements;      /* FP64 residual replacements (mixed)                      */
  int32_t status;           /* FDFD_* status of the solve                              */
  double relres;            /* final true FP64 relative residual                        */
  double time_ms;           /* device time of the solve (CUDA events on the stream)    */
  int64_t launches;         /* kernels launched for this solve (graph replays counted) */
} fdfd_stats;

/* ---- lifetime ------------------------------------------------------------
 * fdfd_create replaces create_linsys(EE, ω, create_paramops, create_curls, …)
 * (model.jl:209-220) as the point where the operator comes into being. */
int fdfd_create(const fdfd_desc *desc, fdfd_handle **out);
void fdfd_destroy(fdfd_handle *h);
const char *fdfd_last_error(const fdfd_handle *h);   /* h may be NULL        */
const char *fdfd_version(void);
void *fdfd_stream(fdfd_handle *h);                   /* the handle's cudaStream_t */
int fdfd_sync(fdfd_handle *h);

/* ---- material ------------------------------------------------------------
 * Pε of create_paramops (model.jl:141-158).  εarr is the reference's
 * (Nx,Ny,Nz,3,3) column-major ComplexF64 array: diagonal entries at the E_w
 * samples, off-diagonal entries at E-voxel corners.  This library requires a
 * real, symmetric tensor (lossless dielectric); other input returns
 * FDFD_ERR_UNSUPPORTED. */
int fdfd_set_eps_tensor(fdfd_handle *h, const double *epsarr);
/* Compact form: eps_diag[c + 3·cell] = ε_cc at E_c; eps_off[p + 3·cell] =
 * ε_xy, ε_yz, ε_zx at the corner of cell (NULL = no off-diagonal). */
int fdfd_set_eps(fdfd_handle *h, const double *eps_diag, const double *eps_off);
/* On-device assign + Kottke smoothing.  lprim[w] holds the N[w]+1 primal
 * plane locations (both domain ends); objects are in add_obj! order (last
 * wins); design may be NULL. */
int fdfd_smooth_objects(fdfd_handle *h, const double *const lprim[3],
                        const fdfd_object *objs, int32_t nobj, double eps_bg,
                        const fdfd_design *design);
/* Read back ε (compact form, doubles) and the smoothing mask
 * smask[s + 4·cell] (s = Exx, Eyy, Ezz, corner; 0 assigned, 1 Kottke,
 * 2 design).  Any pointer may be NULL. */
int fdfd_get_eps(fdfd_handle *h, double *eps_diag, double *eps_off, uint8_t *smask);

/* Field solved for (create_linsys's ft, model.jl:238-240, 266-268):
 * FDFD_EE (default) — A = Cₘ Cₑ − ω² Pε on E; FDFD_HH — A = Cₑ (Pε \ Cₘ) − ω² Pμ
 * on H (Pμ = I), for which ε must be diagonal as in the reference.  Under
 * FDFD_HH the matvec and solve entry points take H vectors (same DOF
 * order); transpose, COCG, the ε gradient and the allocation-free residual
 * are E-formulation only (FDFD_ERR_UNSUPPORTED). */
int fdfd_set_field_type(fdfd_handle *h, int32_t ft);

/* ---- operator application --------------------------------------------------
 * y = A x (mul!(y, A, x) on the reference's assembled A, model.jl:225-246).
 * Host buffers: 2·3·Ncell doubles (ComplexF64).  precision = FDFD_C64
 * computes in complex64 (x rounded, y widened). */
int fdfd_matvec(fdfd_handle *h, const double *x, double *y, int32_t precision);
/* Device buffers on the handle's stream (asynchronous): double2 for
 * FDFD_C128, float2 for FDFD_C64. */
int fdfd_matvec_dev(fdfd_handle *h, const void *x, void *y, int32_t precision);
/* y = Aᵀ x (transpose(A)*x; used by the adjoint). */
int fdfd_matvec_transpose(fdfd_handle *h, const double *x, double *y, int32_t precision);
/* r = b − A x and rnorm2 = ‖r‖₂², all complex128 device buffers (double2,
 * 3·Ncell each), computed in FP64 by the operator kernel with a fused
 * reduction (the true residual of create_linsys's system, model.jl:209-220,
 * that a caller checks a solution against).  Returns once rnorm2 is on the
 * host.  Uses the handle's reduction buffer. */
int fdfd_residual_dev(fdfd_handle *h, const void *x, const void *b, void *r, double *rnorm2);
/* The residual of fdfd_residual_dev (E formulation only; FDFD_ERR_UNSUPPORTED
 * under FDFD_HH), for callers that cannot allocate device memory — e.g. a
 * Julia or Python program whose GPU memory is reserved by its framework's
 * caching pool, or a pipelined caller that must not incur the implicit
 * device synchronisation a cudaMalloc/cudaFree can cause.  It has no
 * counterpart in the reference (which never touches a GPU).  The call
 * allocates nothing: its reduction scratch (block partials, arrival counter,
 * result) is a fixed 512 KiB static device array that every GPU loading the
 * library holds until process exit.  It is synchronous — it returns once
 * rnorm2 is on the host — so it cannot be captured into a CUDA graph.  Limits: the scratch holds 16384 thread-block
 * partials; the z-chunk is lengthened as needed, so only grids whose x-y
 * tiling ⌈Nx/32⌉·⌈Ny/8⌉ exceeds 16384 (more than about 2048×2048 cells per
 * z-plane) are rejected with FDFD_ERR_ARG.  The first call on a device looks
 * up the array's device address (make it while no other stream of the
 * process is capturing).  All
 * calls share the array: calls that overlap on the GPU race, so serialise
 * them. */
int fdfd_residual_dev_noalloc(fdfd_handle *h, const void *x, const void *b, void *r, double *rnorm2);

/* ---- solve -----------------------------------------------------------------
 * x = A \ b to a true relative residual opts->tol (the reference leaves this
 * to Julia's A\b).  Host buffers, nrhs right-hand sides stored one after the
 * other (each 2·3·Ncell doubles).  stats may be NULL or an array of nrhs. */
int fdfd_solve(fdfd_handle *h, const double *b, double *x, int32_t nrhs,
               const fdfd_solve_opts *opts, fdfd_stats *stats);
/* As fdfd_solve, with up to nworkers right-hand sides solved at the same
 * time, each on its own CUDA stream and host thread (workers share the
 * handle's operator data and own their Krylov workspace): small grids, whose
 * kernels fill a fraction of the GPU, overlap.  Independent of the
 * reference (which solves right-hand sides one by one). */
int fdfd_solve_batch(fdfd_handle *h, const double *b, double *x, int32_t nrhs, int32_t nworkers,
                     const fdfd_solve_opts *opts, fdfd_stats *stats);
/* Several independent systems solved together — e.g. the instances of a
 * batch of uneven grids, frequencies and sources, one entry per right-hand
 * side: entry i solves hs[i]'s system (A of its grid, ω and ε) for the
 * complex128 device buffers b[i] → x[i] (3·Ncell of that handle each).  An
 * entry gets its own stream and Krylov workspace over the handle's operator
 * data, so entries may name the same handle.  Every round replays the
 * captured iteration batch (opts.check_every iterations) of each system
 * still iterating as one parent CUDA graph of child graphs, which the GPU
 * runs concurrently — small grids fill the machine together — then each
 * system does its own refinement and stop tests.  All handles on one
 * device; opts as for fdfd_solve_dev; stats (NULL or n entries) per entry.
 * Independent of the reference (which solves systems one by one). */
int fdfd_solve_multi(fdfd_handle *const *hs, int32_t n, const void *const *b, void *const *x,
                     const fdfd_solve_opts *opts, fdfd_stats *stats);
/* Device buffers (double2, 3·Ncell each) on the handle's stream; returns
 * after the solve completes. */
int fdfd_solve_dev(fdfd_handle *h, const void *b, void *x,
                   const fdfd_solve_opts *opts, fdfd_stats *stats);
/* Defaults: BiCGStab(4), mixed precision, tol 1e-6, maxit 200000, δ 0.1,
 * check_every 50, CUDA graphs on. */
void fdfd_default_opts(fdfd_solve_opts *opts);

/* ---- field post-processing -------------------------------------------------
 * H = (i/ω)·(Cₑ e + jₘ): h_from_e (model.jl:276-279) with Pμ = I.  jm may be
 * NULL (jₘ = 0).  e, jm, hout: complex, 2·3·Ncell doubles, H_w at the H_w
 * sample of each cell.  Host buffers; the _dev form takes double2 device
 * buffers and runs asynchronously on the handle's stream. */
int fdfd_h_from_e(fdfd_handle *h, const double *e, const double *jm, double *hout);
int fdfd_h_from_e_dev(fdfd_handle *h, const void *e, const void *jm, void *hout);
/* E = (−i/ω)·Pε⁻¹·(Cₘ h − jₑ): e_from_h (model.jl:281-284) — the E field of
 * an H-formulation solution.  Pε must be diagonal (the reference's Pε \ …
 * divides by it); with off-diagonal ε the call returns FDFD_ERR_UNSUPPORTED.
 * je may be NULL (jₑ = 0).  hin: complex, 2·3·Ncell doubles (H_w at the H_w
 * sample); je, eout: the same for E (2D slices: each field's components).
 * Host buffers; the _dev form takes double2 device buffers (3·Ncell) and
 * runs asynchronously on the handle's stream. */
int fdfd_e_from_h(fdfd_handle *h, const double *hin, const double *je, double *eout);
int fdfd_e_from_h_dev(fdfd_handle *h, const void *hin, const void *je, void *eout);
/* Corner interpolation of create_Mcs (model.jl:287-306): field = FDFD_EE
 * applies Mcₑ (E_w averaged backward along w onto the primal voxel corner,
 * weights s∆lₘ / (2 s∆lₑ)); FDFD_HH applies Mcₘ (H_w averaged forward along w
 * onto the dual corner, weights s∆lₑ / (2 s∆lₘ)).  in, out: complex,
 * 2·3·Ncell doubles. */
int fdfd_corner_mean(fdfd_handle *h, int32_t field, const double *in, double *out);
int fdfd_corner_mean_dev(fdfd_handle *h, int32_t field, const void *in, void *out);

/* ---- adjoint gradient --------------------------------------------------------
 * No counterpart in the reference, which only assembles A (create_A,
 * model.jl:225-246) and leaves differentiation to its users.  For A e = b and
 * a real objective L(e), pass g = ∂L/∂e, the Wirtinger derivative
 * ½(∂L/∂Re e − i·∂L/∂Im e) (so that dL = 2·Re(gᵀ de)); e.g. for
 * L = |Fᴴe|², g = conj(Fᴴe)·conj(F).  The call solves Aᵀ λ = g with
 * opts->method (BiCGStab(ℓ) or BiCGSTAB; COCG is rejected) and opts' tol,
 * precision and maxit (opts->transpose is ignored), and returns
 *     grad[c + 3·cell] = dL/dε_cc = 2·Re(ω²·λ_c·e_c)
 * at every E_c sample (∂A/∂ε_cc = −ω²).  e, g: complex (2·3·Ncell doubles);
 * grad: 3·Ncell doubles.  Host buffers. */
int fdfd_eps_grad(fdfd_handle *h, const double *e, const double *g, double *grad,
                  const fdfd_solve_opts *opts, fdfd_stats *stats);
/* Device-buffer form: e, g, lam are double2[3·Ncell] (lam receives λ),
 * grad double[3·Ncell]; returns after the handle's stream has finished. */
int fdfd_eps_grad_dev(fdfd_handle *h, const void *e, const void *g, void *lam, double *grad,
                      const fdfd_solve_opts *opts, fdfd_stats *stats);
/* Chain dL/dε_ww (grad as returned above) to the cells of the design region
 * that the last fdfd_smooth_objects call applied: the sample value there is
 * the mean of the 4 cells around the E_w edge, so dgrad[cell] collects ¼ of
 * every sample gradient whose mean includes the cell.  dgrad holds
 * (hi−lo) cells, x fastest.  FDFD_ERR_ARG without a design region. */
int fdfd_design_grad(fdfd_handle *h, const double *grad, double *dgrad);
int fdfd_design_grad_dev(fdfd_handle *h, const double *grad, double *dgrad);

#ifdef __cplusplus
}
#endif
#endif /* FDFD_GB300_H */
