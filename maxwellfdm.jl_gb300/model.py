"""Host-side mirror of MaxwellFDFD's ``Model`` API for the 3D (ModelFull) path.

The reference's user flow (src/model/model.jl, full.jl):

    mdl = ModelFull(grid)                       full.jl:7-13
    set_ωpml!(mdl, ω); set_Npml!(mdl, Npml)     model.jl:99-102
    add_obj!(mdl, "Si", shapes...; ε=12.25)     model.jl:120-133
    add_srce!(mdl, PointSrc(...))               model.jl:197-204
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


def set_ωpml(mdl, ωpml):
    mdl.ωpml = ωpml


def set_Npml(mdl, Npml):
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


def create_A(mdl, ω, device=0):
    """The GPU operator A = Cₘ Cₑ − ω² Pε (create_A, model.jl:238-259),
    with ε assigned and smoothed on the device."""
    sdl_e, sdl_m = create_stretched_dls(mdl)
    A = FDFDOperator(mdl.grid.N, ω, sdl_e, sdl_m, mdl.grid.isbloch, e_ikl(mdl), device)
    if mdl.objects or mdl.design is not None or mdl.eps_bg != 1.0:
        A.smooth_objects(mdl.grid.lprim, mdl.objects, mdl.eps_bg, mdl.design)
    return A


def create_b(mdl, ω):
    """b = −iω jₑ (create_b, model.jl:264-287, jₘ = 0)."""
    return -1j * ω * field_arr2vec(mdl.je)


def create_linsys(mdl, ω, device=0):
    return create_A(mdl, ω, device), create_b(mdl, ω)
