"""Current sources: the host-side mirror of src/source/*.jl.

``distweights`` splits a point location over the two nearest grid planes
(src/source/source.jl:208-306); ``PointSrc`` (pointsrc.jl:51-103) and
``PlaneSrc`` (planesrc.jl:14-80) distribute a dipole or a current sheet onto
the J array.  These are O(1)/O(plane) host operations; the right-hand side
b = -iω J then crosses to the GPU with the solve.
"""
import numpy as np

from .grid import DUAL, PRIM


def distweights(c, gt, bounds, l, dl, isbloch):
    """Returns ((i1, i2), (w1, w2)) with 0-based plane indices and weights in
    1/length.  ValueError where the reference throws ArgumentError."""
    lo, hi = float(bounds[0]), float(bounds[1])
    c = float(c)
    if c < lo or c > hi:
        raise ValueError(f"c = {c} must be within bounds = ({lo}, {hi}).")
    n = len(l)
    if n < 2 and not isbloch:
        raise ValueError(f"length(l) = {n} must be > 1 for a symmetry boundary.")
    zeroing = gt == PRIM and not isbloch
    first = 1 if zeroing else 0
    last = n - 1
    interior = l[first] <= c < l[last]
    if interior:
        i1 = int(np.searchsorted(l, c, side="right")) - 1
        i2 = i1 + 1
        frac = (c - l[i1]) / (l[i2] - l[i1])
    else:
        if c < l[first]:
            i1, i2, edge = first, n - 1, lo
        else:
            i1, i2, edge = last, 0, hi
        span = abs(l[i1] - edge) if gt == PRIM else (
            (hi - lo) - abs(l[i1] - l[i2]) if isbloch else 2.0 * abs(l[i1] - edge))
        frac = abs(l[i1] - c) / span
    w1 = 1.0 / dl[i1]
    if interior or isbloch or zeroing:
        w1 *= 1.0 - frac
    if c == l[i1] or (not interior and not isbloch):
        return (i1, i1), (w1, 0.0)
    w2 = 1.0 / dl[i2]
    if interior or isbloch:
        w2 *= frac
    return (i1, i2), (w1, w2)


def _component_gt(nw, gt0):
    return tuple(1 - g if a == nw else g for a, g in enumerate(gt0))


class PointSrc:
    """Point dipole I∆r at location c with polarisation p (normalised)."""

    def __init__(self, c, p, Idr=1.0):
        self.c = np.asarray(c, dtype=np.float64)
        p = np.asarray(p, dtype=np.float64)
        self.p = p / np.linalg.norm(p)
        self.Idr = complex(Idr)

    def add_to(self, j, gt0, grid):
        for nw in range(3):
            if self.p[nw] == 0.0:
                continue
            gtc = _component_gt(nw, gt0)
            idx, wts = [], []
            for a in range(3):
                g = gtc[a]
                ia, wa = distweights(self.c[a], g, (grid.bounds[0][a], grid.bounds[1][a]), grid.l[g][a],
                                     grid.dl[g][a], grid.isbloch[a])
                idx.append(ia)
                wts.append(np.asarray(wa))
            wv = wts[0][:, None, None] * wts[1][None, :, None] * wts[2][None, None, :]
            amp = self.Idr * self.p[nw]
            for a in range(2):
                for b in range(2):
                    for cc in range(2):
                        j[idx[0][a], idx[1][b], idx[2][cc], nw] += amp * wv[a, b, cc]


class PlaneSrc:
    """Current sheet J∆n on the plane x_n = c with polarisation p."""

    def __init__(self, n, c, p, Jdn=1.0):
        n = np.asarray(n, dtype=np.float64)
        if np.count_nonzero(n) != 1:
            raise ValueError(f"n = {n} must be along a Cartesian direction.")
        self.axis = int(np.flatnonzero(n)[0])
        self.c = float(c)
        p = np.asarray(p, dtype=np.float64)
        self.p = p / np.linalg.norm(p)
        self.Jdn = complex(Jdn)

    def add_to(self, j, gt0, grid):
        a = self.axis
        for nw in range(3):
            if self.p[nw] == 0.0:
                continue
            g = _component_gt(nw, gt0)[a]
            (i1, i2), (w1, w2) = distweights(self.c, g, (grid.bounds[0][a], grid.bounds[1][a]), grid.l[g][a],
                                             grid.dl[g][a], grid.isbloch[a])
            amp = self.Jdn * self.p[nw]
            for ii, ww in ((i1, w1), (i2, w2)):
                sl = [slice(None)] * 3
                sl[a] = ii
                j[tuple(sl) + (nw,)] += amp * ww
