"""Host-side mirror of MaxwellFDFD's ``Model`` API for the 3D (ModelFull) path.

The reference's user flow (src/model/model.jl, full.jl):

    mdl = ModelFull(grid)                       full.jl:7-13
    set_ωpml!(mdl, ω); set_Npml!(mdl, Npml)     model.jl:86-89
    add_obj!(mdl, "Si", shapes...; ε=12.25)     model.jl:107-120
    add_srce!(mdl, PointSrc(...))               model.jl:184-191
    A, b = create_linsys(EE, ω, create_paramops(mdl), create_curls(mdl), create_srcs(mdl))
    e = A \\ b

becomes

    mdl = ModelFull(grid)
    set_ωpml(mdl, ω); set_Npml(mdl, Npml)
    add_obj(mdl, "Si", Sphere(...), ε=12.25)
    add_srce(mdl, PointSrc(...))
    A, b = create_linsys(mdl, ω)          # A: FDFDOperator on the GPU
    e, stats = A.solve(b)

Material assignment and smoothing run on the GPU (fdfd_smooth_objects);
sources and the per-axis PML arrays are assembled on the host.
"""
import numpy as np

from . import _lib
from .grid import PRIM, PMLParam, create_stretched_dl
from .operator import FDFDOperator

EE, HH = 0, 1


class Sphere:
    def __init__(self, c, r):
        self.c = np.asarray(c, dtype=np.float64)
        self.r = float(r)

    def to_c(self, eps):
        o = _lib.fdfd_object()
        o.kind = _lib.FDFD_SHAPE_SPHERE
        o.eps = float(eps)
        o.p[0], o.p[1], o.p[2], o.p[3] = self.c[0], self.c[1], self.c[2], self.r
        return o


class Box:
    def __init__(self, lo, hi):
        self.lo = np.asarray(lo, dtype=np.float64)
        self.hi = np.asarray(hi, dtype=np.float64)

    def to_c(self, eps):
        o = _lib.fdfd_object()
        o.kind = _lib.FDFD_SHAPE_BOX
        o.eps = float(eps)
        for a in range(3):
            o.p[a] = self.lo[a]
            o.p[3 + a] = self.hi[a]
        return o


class Disk:
    """A disk of the 2D models (the z-invariant cylinder of the slice)."""

    def __init__(self, c, r):
        self.c = np.asarray(c, dtype=np.float64)[:2]
        self.r = float(r)

    def to_c(self, eps):
        o = _lib.fdfd_object()
        o.kind = _lib.FDFD_SHAPE_CYLZ
        o.eps = float(eps)
        o.p[0], o.p[1], o.p[2] = self.c[0], self.c[1], self.r
        return o


class Rect:
    """An axis-aligned rectangle of the 2D models (a box unbounded in z)."""

    def __init__(self, lo, hi):
        self.lo = np.asarray(lo, dtype=np.float64)[:2]
        self.hi = np.asarray(hi, dtype=np.float64)[:2]

    def to_c(self, eps):
        return Box((self.lo[0], self.lo[1], -1e300), (self.hi[0], self.hi[1], 1e300)).to_c(eps)


class _Obj:
    def __init__(self, name, shape, eps):
        self.name = name
        self.shape = shape
        self.eps = float(eps)

    def to_c(self):
        return self.shape.to_c(self.eps)


class DesignRegion:
    """Per-cell ε over cells [lo, hi) (inverse design)."""

    def __init__(self, lo, hi, eps):
        self.lo = tuple(int(v) for v in lo)
        self.hi = tuple(int(v) for v in hi)
        self.eps = np.asarray(eps, dtype=np.float64)
        if self.eps.shape != tuple(h - l for l, h in zip(self.lo, self.hi)):
            raise ValueError("design ε has the wrong shape")


class ModelFull:
    """3D full-vector model (Model{3,3,3,…}, model.jl:45-86)."""

    def __init__(self, grid):
        self.grid = grid
        self.ωpml = 0.0
        self.boundft = (EE, EE, EE)
        self.Npml = ((0, 0, 0), (0, 0, 0))
        self.kbloch = (0.0, 0.0, 0.0)
        self.objects = []
        self.eps_bg = 1.0
        self.design = None
        self.pml = PMLParam()
        self.je = np.zeros(tuple(grid.N) + (3,), dtype=np.complex128)
        self.order_cmpfirst = True


class Model2D(ModelFull):
    """Common part of ModelTE / ModelTM: a 2D grid held as the z-invariant
    slice of a 3D grid (one cell along z, periodic), where ∂z vanishes and
    the 3D operator splits into the TE and TM blocks."""

    slice2d = 0
    comps = (0, 1, 2)

    def __init__(self, lprim_xy, isbloch_xy=(False, False)):
        from .grid import Grid
        g = Grid((lprim_xy[0], lprim_xy[1], np.array([0.0, 1.0])), (isbloch_xy[0], isbloch_xy[1], True))
        super().__init__(g)


class ModelTE(Model2D):
    """2D TE model: E = (Ex, Ey), H = Hz (ModelTE, src/model/te.jl:1-13)."""

    slice2d = 1
    comps = (0, 1)


class ModelTM(Model2D):
    """2D TM model: E = Ez, H = (Hx, Hy) (ModelTM, src/model/tm.jl)."""

    slice2d = 2
    comps = (2,)


def uniform_lprim2d(N, h=1.0):
    """Primal plane locations of a uniform 2D grid with N = (Nx, Ny) cells."""
    return tuple(np.arange(N[a] + 1, dtype=np.float64) * h for a in range(2))


def set_ωpml(mdl, ωpml):
    mdl.ωpml = ωpml


def set_Npml(mdl, Npml):
    if isinstance(mdl, Model2D) and len(Npml[0]) == 2:
        Npml = (tuple(Npml[0]) + (0,), tuple(Npml[1]) + (0,))
    mdl.Npml = (tuple(int(v) for v in Npml[0]), tuple(int(v) for v in Npml[1]))


def set_boundft(mdl, boundft):
    if any(b != EE for b in boundft):
        raise NotImplementedError("boundft = HH is not implemented on the GPU path")
    mdl.boundft = tuple(boundft)


def set_kbloch(mdl, kbloch):
    mdl.kbloch = tuple(float(k) for k in kbloch)


def add_obj(mdl, matname, *shapes, ε=1.0, μ=1.0):
    if μ != 1.0:
        raise NotImplementedError("μ ≠ 1 is not implemented on the GPU path (Pμ = I)")
    if np.iscomplexobj(ε) and np.imag(ε) != 0:
        raise NotImplementedError("lossy (complex) ε is not implemented on the GPU path")
    for s in shapes:
        mdl.objects.append(_Obj(matname, s, np.real(ε)))


def clear_objs(mdl):
    mdl.objects = []
    mdl.design = None


def set_design(mdl, design):
    mdl.design = design


def add_srce(mdl, src):
    src.add_to(mdl.je, (PRIM, PRIM, PRIM), mdl.grid)


def clear_srcs(mdl):
    mdl.je[...] = 0


def e_ikl(mdl):
    return tuple(np.exp(-1j * mdl.kbloch[w] * mdl.grid.L[w]) for w in range(3))


def create_stretched_dls(mdl):
    return create_stretched_dl(mdl.grid, mdl.ωpml, mdl.Npml, mdl.pml)


def field_arr2vec(F):
    """(Nx,Ny,Nz,3) → component-fastest vector (order_cmpfirst)."""
    return np.ascontiguousarray(np.transpose(F, (2, 1, 0, 3))).reshape(-1)


def vec2field_arr(v, N):
    return np.transpose(np.asarray(v).reshape(N[2], N[1], N[0], 3), (2, 1, 0, 3))


def create_A(mdl, ω, device=0, ft=EE):
    """The GPU operator (create_A, model.jl:225-246) with ε assigned and
    smoothed on the device: ft = EE → A = Cₘ Cₑ − ω² Pε on E; ft = HH →
    A = Cₑ (Pε \\ Cₘ) − ω² on H (diagonal ε only, as in the reference)."""
    sdl_e, sdl_m = create_stretched_dls(mdl)
    A = FDFDOperator(mdl.grid.N, ω, sdl_e, sdl_m, mdl.grid.isbloch, e_ikl(mdl), device,
                     getattr(mdl, "slice2d", 0))
    if mdl.objects or mdl.design is not None or mdl.eps_bg != 1.0:
        A.smooth_objects(mdl.grid.lprim, mdl.objects, mdl.eps_bg, mdl.design)
    if ft == HH:
        A.set_field_type("H")
    return A


def create_b(mdl, ω, ft=EE, A=None):
    """b = −iω jₑ (create_b, model.jl:251-274, jₘ = 0); for a 2D model, the
    slice's components only (component fastest).  ft = HH: b = Cₑ (Pε \\ jₑ),
    formed on the GPU by the operator A of the same model (its ε and its
    curl), as (−iω)·h_from_e(ε⁻¹ jₑ)."""
    if ft == HH:
        if A is None:
            raise ValueError("the H formulation's b needs the model's operator A")
        ed, _, _ = A.get_eps()
        je = mdl.je / ed
        if isinstance(mdl, Model2D):
            x = field_arr2vec_2d(je[:, :, 0, [c for c in (0, 1, 2) if c in mdl.comps]])
        else:
            x = field_arr2vec(je)
        return -1j * ω * A.h_from_e(x)
    if isinstance(mdl, Model2D):
        return -1j * ω * field_arr2vec_2d(mdl.je[:, :, 0, list(mdl.comps)])
    return -1j * ω * field_arr2vec(mdl.je)


def field_arr2vec_2d(F):
    """(Nx,Ny,m) → component-fastest vector of a 2D model."""
    F = np.asarray(F)
    return np.ascontiguousarray(np.transpose(F, (1, 0, 2))).reshape(-1)


def vec2field_arr_2d(v, N, m):
    return np.transpose(np.asarray(v).reshape(N[1], N[0], m), (1, 0, 2))


def create_linsys(mdl, ω, device=0, ft=EE):
    A = create_A(mdl, ω, device, ft)
    return A, create_b(mdl, ω, ft, A)
