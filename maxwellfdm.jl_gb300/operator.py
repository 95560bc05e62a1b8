"""GPU FDFD operator: the drop-in for the reference's assembled A.

The reference returns ``A = Cₘ·(Pμ \\ Cₑ) − ω²·Pε`` as a
``SparseMatrixCSC{ComplexF64}`` (create_A, src/model/model.jl:225-246) and
the caller applies ``A*x`` / ``mul!(y, A, x)`` or solves ``A\\b``.
``FDFDOperator`` exposes the same operations — ``A @ x``, ``A.T @ x``,
``A.solve(b)`` — executed matrix-free by libfdfd_gb300 on one GPU.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr


class FDFDOperator:
    """Matrix-free A on the GPU (complex128 semantics, DOF order c + 3·cell)."""

    def __init__(self, N, omega, sdl_e, sdl_m, isbloch=(False, False, False), e_ikl=(1, 1, 1), device=0,
                 slice2d=0):
        """slice2d: 0 (3D), 1 (TE) or 2 (TM) — a 2D model as the z-invariant
        slice (N[2] = 1, Bloch z); host field vectors then carry only the
        slice's components (TE: E = (Ex, Ey), H = Hz; TM: E = Ez, H = (Hx, Hy))."""
        lib = _lib.load()
        self.N = tuple(int(n) for n in N)
        self.ncell = self.N[0] * self.N[1] * self.N[2]
        self.slice2d = int(slice2d)
        self.ncomp_e, self.ncomp_h = {0: (3, 3), 1: (2, 1), 2: (1, 2)}[self.slice2d]
        self.n = self.ncomp_e * self.ncell
        self.omega = complex(omega)
        d = _lib.fdfd_desc()
        self._keep = []
        for w in range(3):
            d.N[w] = self.N[w]
            d.isbloch[w] = int(bool(isbloch[w]))
            d.boundft[w] = _lib.FDFD_EE
            ph = complex(e_ikl[w])
            d.e_ikl[w][0], d.e_ikl[w][1] = ph.real, ph.imag
            se = np.ascontiguousarray(sdl_e[w], dtype=np.complex128)
            sm = np.ascontiguousarray(sdl_m[w], dtype=np.complex128)
            if se.shape != (self.N[w],) or sm.shape != (self.N[w],):
                raise ValueError("s∆l arrays must have N[w] entries")
            self._keep += [se, sm]
            d.sdl_e[w] = dptr(se)
            d.sdl_m[w] = dptr(sm)
        d.order_cmpfirst = 1
        d.device = int(device)
        d.slice2d = self.slice2d
        d.omega[0], d.omega[1] = self.omega.real, self.omega.imag
        h = C.c_void_p()
        check(lib.fdfd_create(C.byref(d), C.byref(h)))
        self._h = h
        self._lib = lib
        self._keep = None

    # ---------------------------------------------------------------- basics
    @property
    def shape(self):
        return (self.n, self.n)

    dtype = np.complex128

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fdfd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        check(rc, self._h)

    @property
    def stream(self):
        return self._lib.fdfd_stream(self._h)

    def sync(self):
        self._check(self._lib.fdfd_sync(self._h))

    # ---------------------------------------------------------------- material
    _design_shape = None
    ft = "E"

    def set_field_type(self, ft):
        """Solve for E (A = CₘCₑ − ω²Pε) or H (A = Cₑ(Pε \\ Cₘ) − ω², diagonal ε
        only) — create_linsys's ft (model.jl:238-240)."""
        if ft not in ("E", "H"):
            raise ValueError("ft must be 'E' or 'H'")
        self._check(self._lib.fdfd_set_field_type(self._h, _lib.FDFD_EE if ft == "E" else _lib.FDFD_HH))
        self.ft = ft
        self.n = (self.ncomp_e if ft == "E" else self.ncomp_h) * self.ncell

    def set_eps(self, eps_diag, eps_off=None):
        """eps_diag, eps_off: (Nx,Ny,Nz,3) real arrays (ε_cc at E_c; ε_xy, ε_yz,
        ε_zx at the cell's corner)."""
        ed = _cell_aos(eps_diag, self.N, np.float64)
        eo = None if eps_off is None else _cell_aos(eps_off, self.N, np.float64)
        self._check(self._lib.fdfd_set_eps(self._h, dptr(ed), None if eo is None else dptr(eo)))

    def set_eps_tensor(self, epsarr):
        """epsarr: the reference's εarr, (Nx,Ny,Nz,3,3) complex indexed
        [i,j,k,r,c] (stored here in Julia's column-major order)."""
        e = np.asarray(epsarr, dtype=np.complex128)
        if e.shape != self.N + (3, 3):
            raise ValueError(f"εarr must have shape {self.N + (3, 3)}")
        jl = np.ascontiguousarray(np.transpose(e, (4, 3, 2, 1, 0)))  # column-major bytes
        self._check(self._lib.fdfd_set_eps_tensor(self._h, dptr(jl)))

    def smooth_objects(self, lprim, objects, eps_bg=1.0, design=None):
        """On-device assignment + Kottke smoothing of sphere/box objects."""
        arrs = [np.ascontiguousarray(l, dtype=np.float64) for l in lprim]
        lp = (_lib._dp * 3)(*[dptr(a) for a in arrs])
        objs = (_lib.fdfd_object * max(1, len(objects)))()
        for q, o in enumerate(objects):
            objs[q] = o.to_c()
        dptr_ = None
        keep = None
        if design is not None:
            dd = _lib.fdfd_design()
            for a in range(3):
                dd.lo[a], dd.hi[a] = design.lo[a], design.hi[a]
            keep = np.ascontiguousarray(np.transpose(np.asarray(design.eps, np.float64), (2, 1, 0)))
            dd.eps_cells = dptr(keep)
            dptr_ = C.pointer(dd)
        self._check(self._lib.fdfd_smooth_objects(self._h, lp, objs, len(objects), float(eps_bg), dptr_))
        self._design_shape = None if design is None else tuple(design.hi[a] - design.lo[a] for a in range(3))

    def get_eps(self):
        """Returns (eps_diag, eps_off, smask) as (Nx,Ny,Nz,3|4) arrays."""
        ed = np.zeros(3 * self.ncell)    # ε keeps the 3-component layout in every mode
        eo = np.zeros(3 * self.ncell)
        sm = np.zeros(4 * self.ncell, dtype=np.uint8)
        self._check(self._lib.fdfd_get_eps(self._h, dptr(ed), dptr(eo), sm.ctypes.data_as(C.POINTER(C.c_uint8))))
        return (_aos_cell(ed, self.N, 3), _aos_cell(eo, self.N, 3), _aos_cell(sm, self.N, 4))

    # ---------------------------------------------------------------- apply
    def matvec(self, x, precision="c128"):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        if x.size != self.n:
            raise ValueError("x has the wrong length")
        y = np.empty_like(x)
        self._check(self._lib.fdfd_matvec(self._h, dptr(x), dptr(y), _prec(precision)))
        return y

    def rmatvec_transpose(self, x, precision="c128"):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        if x.size != self.n:
            raise ValueError("x has the wrong length")
        y = np.empty_like(x)
        self._check(self._lib.fdfd_matvec_transpose(self._h, dptr(x), dptr(y), _prec(precision)))
        return y

    def __matmul__(self, x):
        return self.matvec(x)

    @property
    def T(self):
        return _Transposed(self)

    def matvec_dev(self, x_ptr, y_ptr, precision="c64"):
        """y = A x on device pointers (float2 for c64, double2 for c128), asynchronous on the handle's stream."""
        self._check(self._lib.fdfd_matvec_dev(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), _prec(precision)))

    def residual_dev(self, x_ptr, b_ptr, r_ptr):
        """r = b − A x on complex128 device buffers; returns ‖r‖₂² (FP64)."""
        out = C.c_double()
        self._check(self._lib.fdfd_residual_dev(self._h, C.c_void_p(x_ptr), C.c_void_p(b_ptr), C.c_void_p(r_ptr),
                                                C.byref(out)))
        return out.value

    # ---------------------------------------------------------------- solve
    def solve(self, b, tol=1e-6, precision="mixed", method="bicgstabl", maxit=200000, x0=None, delta=0.1,
              check_every=50, transpose=False, use_graph=True, ell=4, workers=1):
        """x = A \\ b to a true relative residual ``tol``.  b may hold several
        right-hand sides as rows of a 2D array; ``workers`` > 1 solves up to
        that many of them at the same time on separate streams.  method:
        "bicgstab", "bicgstabl" (BiCGStab(ℓ), ℓ = ell) or "cocg".  Returns
        (x, [stats])."""
        b = np.ascontiguousarray(b, dtype=np.complex128)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        b2 = b.reshape(nrhs, -1)
        if b2.shape[1] != self.n:
            raise ValueError("b has the wrong length")
        x = np.zeros_like(b2) if x0 is None else np.ascontiguousarray(x0, np.complex128).reshape(nrhs, -1).copy()
        o = self._opts(tol, precision, method, maxit, x0 is not None, delta, check_every, transpose, use_graph, ell)
        st = (_lib.fdfd_stats * nrhs)()
        if workers > 1 and nrhs > 1:
            rc = self._lib.fdfd_solve_batch(self._h, dptr(b2), dptr(x), nrhs, int(workers), C.byref(o), st)
        else:
            rc = self._lib.fdfd_solve(self._h, dptr(b2), dptr(x), nrhs, C.byref(o), st)
        stats = [s.as_dict() for s in st]
        if rc != _lib.FDFD_OK:
            err = _lib.FDFDError(rc, (self._lib.fdfd_last_error(self._h) or b"").decode())
            err.stats = stats
            err.x = x.reshape(b.shape)
            raise err
        return x.reshape(b.shape), stats

    def solve_dev(self, b_ptr, x_ptr, **kw):
        """Solve with complex128 device buffers (already resident in HBM)."""
        o = self._opts(kw.get("tol", 1e-6), kw.get("precision", "mixed"), kw.get("method", "bicgstabl"),
                       kw.get("maxit", 200000), kw.get("x0_given", False), kw.get("delta", 0.1),
                       kw.get("check_every", 50), kw.get("transpose", False), kw.get("use_graph", True),
                       kw.get("ell", 4))
        st = _lib.fdfd_stats()
        rc = self._lib.fdfd_solve_dev(self._h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(o), C.byref(st))
        if rc != _lib.FDFD_OK:
            err = _lib.FDFDError(rc, (self._lib.fdfd_last_error(self._h) or b"").decode())
            err.stats = st.as_dict()   # iterations, applications and the final true residual so far
            raise err
        return st.as_dict()

    # ---------------------------------------------------------------- fields
    def h_from_e(self, e, jm=None):
        """H = (i/ω)·(Cₑ e + jₘ) (h_from_e, model.jl:276-279), as a DOF vector."""
        e = np.ascontiguousarray(e, dtype=np.complex128).reshape(-1)
        if e.size != self.n:
            raise ValueError("e has the wrong length")
        jmv = None if jm is None else np.ascontiguousarray(jm, dtype=np.complex128).reshape(-1)
        if jmv is not None and jmv.size != self.ncomp_h * self.ncell:
            raise ValueError("jm has the wrong length")
        out = np.empty(self.ncomp_h * self.ncell, dtype=np.complex128)
        self._check(self._lib.fdfd_h_from_e(self._h, dptr(e), None if jmv is None else dptr(jmv), dptr(out)))
        return out

    def e_from_h(self, h, je=None):
        """E = (−i/ω)·Pε⁻¹·(Cₘ h − jₑ) (e_from_h, model.jl:281-284; diagonal ε
        only, as the reference's Pε \\ requires), as a DOF vector."""
        h = np.ascontiguousarray(h, dtype=np.complex128).reshape(-1)
        if h.size != self.ncomp_h * self.ncell:
            raise ValueError("h has the wrong length")
        jev = None if je is None else np.ascontiguousarray(je, dtype=np.complex128).reshape(-1)
        if jev is not None and jev.size != self.ncomp_e * self.ncell:
            raise ValueError("je has the wrong length")
        out = np.empty(self.ncomp_e * self.ncell, dtype=np.complex128)
        self._check(self._lib.fdfd_e_from_h(self._h, dptr(h), None if jev is None else dptr(jev), dptr(out)))
        return out

    def corner_mean(self, v, field="E"):
        """create_Mcs corner interpolation (model.jl:287-306): field "E" → Mcₑ v
        (primal corners), "H" → Mcₘ v (dual corners)."""
        v = np.ascontiguousarray(v, dtype=np.complex128).reshape(-1)
        if v.size != (self.ncomp_e if field == "E" else self.ncomp_h) * self.ncell:
            raise ValueError("field vector has the wrong length")
        f = {"E": _lib.FDFD_EE, "H": _lib.FDFD_HH}[field]
        out = np.empty_like(v)
        self._check(self._lib.fdfd_corner_mean(self._h, f, dptr(v), dptr(out)))
        return out

    # ---------------------------------------------------------------- adjoint
    def eps_grad(self, e, g, tol=1e-8, precision="fp64", maxit=200000, delta=0.1, check_every=50, use_graph=True,
                 method="bicgstabl", ell=4):
        """dL/dε_cc at every E_c sample for A e = b and g = ∂L/∂e (Wirtinger
        derivative, dL = 2·Re(gᵀ de)): solves Aᵀ λ = g on the GPU and returns
        2·Re(ω²·λ·e) as an (Nx,Ny,Nz,3) array, with the solve's stats."""
        e = np.ascontiguousarray(e, dtype=np.complex128).reshape(-1)
        g = np.ascontiguousarray(g, dtype=np.complex128).reshape(-1)
        if e.size != self.n or g.size != self.n:
            raise ValueError("e and g need 3·Ncell entries")
        grad = np.empty(self.n)
        o = self._opts(tol, precision, method, maxit, False, delta, check_every, True, use_graph, ell)
        st = _lib.fdfd_stats()
        self._check(self._lib.fdfd_eps_grad(self._h, dptr(e), dptr(g), dptr(grad), C.byref(o), C.byref(st)))
        return _aos_cell(grad, self.N, self.ncomp_e), st.as_dict()

    def design_grad(self, grad):
        """Chain dL/dε_ww ((Nx,Ny,Nz,3), as eps_grad returns it) to the cells
        of the design region applied by smooth_objects → (hi−lo) array."""
        if self._design_shape is None:
            raise ValueError("no design region was applied")
        if self.slice2d:
            raise ValueError("design regions are 3D only")
        gv = _cell_aos(grad, self.N, np.float64)
        ds = self._design_shape
        out = np.empty(ds[0] * ds[1] * ds[2])
        self._check(self._lib.fdfd_design_grad(self._h, dptr(gv), dptr(out)))
        return np.transpose(out.reshape(ds[2], ds[1], ds[0]), (2, 1, 0))

    def _opts(self, tol, precision, method, maxit, x0_given, delta, check_every, transpose, use_graph, ell=4):
        methods = {"bicgstab": _lib.FDFD_BICGSTAB, "cocg": _lib.FDFD_COCG, "bicgstabl": _lib.FDFD_BICGSTABL}
        if method not in methods:
            raise ValueError(f"unknown method {method}")
        return _lib.default_opts(ell=int(ell),
            tol=float(tol), precision=_lib.FDFD_PREC_MIXED if precision == "mixed" else _lib.FDFD_PREC_FP64,
            method=methods[method], maxit=int(maxit),
            x0_given=int(bool(x0_given)), delta=float(delta), check_every=int(check_every),
            transpose=int(bool(transpose)), use_graph=int(bool(use_graph)))


def solve_multi(entries, tol=1e-6, precision="mixed", method="bicgstabl", maxit=200000, delta=0.1,
                check_every=50, use_graph=True, ell=4):
    """Solve several independent systems together (fdfd_solve_multi):
    ``entries`` is a list of (FDFDOperator, b_ptr, x_ptr) with complex128
    device buffers; entries may share an operator (one per right-hand side).
    Each round replays every unfinished system's iteration batch as one
    parent CUDA graph.  Returns the per-entry stats."""
    if not entries:
        return []
    lib = _lib.load()
    n = len(entries)
    hs = (C.c_void_p * n)(*[e[0]._h.value for e in entries])
    bs = (C.c_void_p * n)(*[int(e[1]) for e in entries])
    xs = (C.c_void_p * n)(*[int(e[2]) for e in entries])
    o = entries[0][0]._opts(tol, precision, method, maxit, False, delta, check_every, False, use_graph, ell)
    st = (_lib.fdfd_stats * n)()
    rc = lib.fdfd_solve_multi(hs, n, bs, xs, C.byref(o), C.cast(st, C.c_void_p))
    stats = [s.as_dict() for s in st]
    if rc != _lib.FDFD_OK:
        err = _lib.FDFDError(rc, (lib.fdfd_last_error(entries[0][0]._h) or b"").decode())
        err.stats = stats
        raise err
    return stats


class _Transposed:
    def __init__(self, A):
        self.A = A

    def __matmul__(self, x):
        return self.A.rmatvec_transpose(x)


def _prec(p):
    if p in ("c128", "fp64", _lib.FDFD_C128):
        return _lib.FDFD_C128
    if p in ("c64", "fp32", _lib.FDFD_C64):
        return _lib.FDFD_C64
    raise ValueError(f"bad precision {p}")


def _cell_aos(a, N, dtype):
    """(Nx,Ny,Nz,m) → flat [c + m·(i + Nx(j + Ny k))]."""
    a = np.asarray(a, dtype=dtype)
    return np.ascontiguousarray(np.transpose(a, (2, 1, 0, 3))).reshape(-1)


def _aos_cell(v, N, m):
    return np.transpose(v.reshape(N[2], N[1], N[0], m), (2, 1, 0, 3))
