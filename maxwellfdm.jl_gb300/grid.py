"""Yee grid and stretched-coordinate PML on the host.

Mirrors the pieces of MaxwellBase that MaxwellFDFD consumes on this path:
``Grid(lprim, isbloch)`` (its ``N``, ``L``, ``bounds``, ``l``, ``∆l`` fields,
as read by ``add_srce!`` at src/model/model.jl:184-191) and
``create_stretched_∆ls`` (model.jl:122-139).  These are per-axis arrays of
length N — tiny next to the 3D fields — so they stay host-side; the 3D work
happens in the CUDA library.

Index conventions (0-based): along each axis the N non-ghost primal planes
are lprim[0..N-1] (lprim[N] is the positive-end ghost); the N dual planes are
the midpoints lprim[i] + lprim[i+1] / 2 with a ghost at the negative end
(periodic image for Bloch, mirror image about lprim[0] otherwise).
"""
import math

import numpy as np

PRIM, DUAL = 0, 1
NEG, POS = 0, 1


class Grid:
    """3D Yee grid built from the primal plane locations of each axis."""

    def __init__(self, lprim, isbloch=(False, False, False)):
        if len(lprim) != 3:
            raise ValueError("grids are 3D here (2D models use ModelTE/ModelTM)")
        self.lprim = tuple(np.array(l, dtype=np.float64) for l in lprim)
        for l in self.lprim:
            if l.ndim != 1 or len(l) < 2 or np.any(np.diff(l) <= 0):
                raise ValueError("each lprim axis must be strictly increasing with >= 2 entries")
        self.isbloch = tuple(bool(b) for b in isbloch)
        self.N = tuple(len(l) - 1 for l in self.lprim)
        self.bounds = (np.array([l[0] for l in self.lprim]), np.array([l[-1] for l in self.lprim]))
        self.L = self.bounds[1] - self.bounds[0]
        lpr, ldu, dpr, ddu, ghost = [], [], [], [], []
        for w, lf in enumerate(self.lprim):
            mid = (lf[1:] + lf[:-1]) / 2
            g = (mid[-1] - self.L[w]) if self.isbloch[w] else (2 * lf[0] - mid[0])
            lpr.append(lf[:-1])
            ldu.append(mid)
            ddu.append(lf[1:] - lf[:-1])
            dpr.append(mid - np.concatenate(([g], mid[:-1])))
            ghost.append(g)
        self.l = (tuple(lpr), tuple(ldu))
        self.dl = (tuple(dpr), tuple(ddu))
        self.ldual_ghost = tuple(ghost)

    @property
    def ncell(self):
        return self.N[0] * self.N[1] * self.N[2]

    def __repr__(self):
        return f"Grid(N={self.N}, bounds={self.bounds[0].tolist()}..{self.bounds[1].tolist()}, isbloch={self.isbloch})"


def uniform_grid(N, h=1.0, isbloch=(False, False, False), origin=(0.0, 0.0, 0.0)):
    return Grid(tuple(origin[w] + h * np.arange(N[w] + 1) for w in range(3)), isbloch)


class PMLParam:
    """Polynomially graded SC-PML: σ(d) = σmax (d/Lpml)^m, σmax = -(m+1) ln R / (2 Lpml)."""

    def __init__(self, m=4.0, R=1e-8):
        self.m = float(m)
        self.R = float(R)


def sfactor(grid, w, gt, omega_pml, Npml, pml=PMLParam()):
    """s = 1 + σ/(iω) at the N primal (gt=PRIM) or dual (gt=DUAL) locations of axis w."""
    lf = grid.lprim[w]
    N = grid.N[w]
    u = grid.l[gt][w]
    sig = np.zeros(N)
    for side, n in ((NEG, int(Npml[NEG][w])), (POS, int(Npml[POS][w]))):
        if n <= 0:
            continue
        if side == NEG:
            inner, outer = lf[n], lf[0]
            depth = inner - u
        else:
            inner, outer = lf[N - n], lf[N]
            depth = u - inner
        Lp = abs(outer - inner)
        smax = -(pml.m + 1.0) * math.log(pml.R) / (2.0 * Lp)
        sig += smax * np.clip(depth / Lp, 0.0, None) ** pml.m
    return 1.0 + sig / (1j * omega_pml)


def create_stretched_dl(grid, omega_pml, Npml, pml=PMLParam()):
    """(s∆lₑ, s∆lₘ) for boundft = EE: stretched ∆l at the E-voxel corners
    (primal planes) and at the H-voxel corners (dual planes), per axis.

    Mirrors create_stretched_∆ls (src/model/model.jl:122-139) with
    gₑ = PRIM, gₘ = DUAL."""
    sdl_e = tuple(grid.dl[PRIM][w] * sfactor(grid, w, PRIM, omega_pml, Npml, pml) for w in range(3))
    sdl_m = tuple(grid.dl[DUAL][w] * sfactor(grid, w, DUAL, omega_pml, Npml, pml) for w in range(3))
    return sdl_e, sdl_m
