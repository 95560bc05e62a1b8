"""CPU FP64 oracle for the MaxwellFDFD.jl FDFD hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module: only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, and only as the checker (or the timed CPU baseline),
never as the thing measured on the GPU path.

What it restates (plain numpy/scipy, complex128):

* the Yee grid with ghost points (MaxwellBase ``Grid``, as used at
  src/model/model.jl:122-139 and test/source.jl:6-15, 130);
* ``distweights`` and the PointSrc / PlaneSrc current assembly
  (src/source/source.jl:208-306, src/source/pointsrc.jl:64-103,
  src/source/planesrc.jl:34-80);
* stretched-coordinate PML ∆l (``create_stretched_∆ls``, model.jl:122-139);
* the curl operators Cₑ, Cₘ (``create_curls``, model.jl:160-175);
* the ε parameter operator with off-diagonal averaging
  (``create_paramops``, model.jl:141-158);
* point-in-object assignment plus Kottke subpixel smoothing with the
  dual-voxel object-index trick (``calc_matparams!``, src/model/full.jl:16-70);
* ``create_A`` / ``create_b`` / ``h_from_e`` (model.jl:225-279);
* an FP64 BiCGSTAB (the reference has no solver; users call ``A\\b``).

Parity status.  The source discretisation (``distweights``, PointSrc,
PlaneSrc) is pinned by the reference's own known-answer and conservation
tests (test/source.jl:5-230, restated as fixtures in tests/golden/).  The
grid/PML/curl/parameter-operator/smoothing arithmetic lives in the external
package MaxwellBase (^0.1.6), which is not vendored with the reference; those
pieces restate the published method under the conventions listed below and
are **parity unpinned** against the real MaxwellBase.

Conventions (each one a choice, recorded here and in the design notes):

A1  boundft = EE on every axis.  A non-Bloch axis is a PEC wall at both ends:
    E tangential to the wall is zero at the primal plane l₀ (those E DOFs are
    kept in the vector but pinned: their Cₑ columns are zero) and at the
    positive-end ghost primal plane.  H ghosts at the negative end mirror
    H at index 0.  This matches the zeroing of primal-plane currents on
    symmetry boundaries in ``distweights`` (source.jl:243-244).
A2  PML: s(u) = 1 + σ(u)/(iω_pml), σ = σmax·(d/Lpml)^m with d the depth from
    the PML inner face, σmax = -(m+1)·ln R/(2·Lpml), m = 4, R = 1e-8,
    evaluated at each primal / dual sample location; s∆l = ∆l·s.
A3  Off-diagonal ε_wv lives at E-voxel corners (primal³).  E_v is averaged
    to a corner with the s∆l-weighted means s∆lₘ[v][j-1]/(2 s∆lₑ[v][j]),
    s∆lₘ[v][j]/(2 s∆lₑ[v][j]) (create_paramop's weights, model.jl:166); the
    corner product is averaged back to E_w with weights 1/2, the choice that
    makes V_E·Pε exactly symmetric (V_E = s∆lₘ[w]·s∆lₑ[u]·s∆lₑ[v], the dual
    volume of E_w).  Pinned DOFs are masked on both sides.
A4  Kottke: ε̃ = ⟨ε⁻¹⟩⁻¹ P + ⟨ε⟩ (I-P), P = n nᵀ, for a voxel whose 8 corner
    object indices hold exactly two objects.  The foreground is the
    higher-priority object; n is its outward normal at the point nearest the
    voxel centre (sphere: radial; box: the face of largest signed distance);
    the fill fraction is the exact volume of the voxel on the inner side of
    the tangent plane (planar approximation, closed form).
A5  Object priority: the last-added object wins (index 0 = background).
A6  Voxels whose corners hold more than two objects: ε̃ = mean of the corner
    objects' ε (diagonal), 0 off-diagonal.
A7  Design region: per-cell ε; ε_ww at an E_w edge touching the region is the
    mean of the 4 cells sharing that edge (cells outside the region take the
    object ε at their centre); off-diagonals are 0 at corners touching it.
A8  b uses ω, not ωpml (model.jl:262-265); callers set ωpml = ω.
A9  μ = 1, so Pμ = I.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

PRIM, DUAL = 0, 1
NEG, POS = 0, 1
EE, HH = 0, 1


# --------------------------------------------------------------------------
# Grid
# --------------------------------------------------------------------------
class Grid:
    """Yee grid from primal plane locations (both domain ends included).

    Restates MaxwellBase ``Grid(lprim, isbloch)`` as it is consumed by
    ``add_srce!`` (model.jl:184-191: ``grid.bounds, grid.l, grid.∆l``) and as
    the reference test constructs it (test/source.jl:130, 145).

    * ``l[PRIM][w]``: the N non-ghost primal planes ``lprim[:-1]``;
      the positive-end plane ``lprim[-1]`` is the primal ghost.
    * ``l[DUAL][w]``: the N midpoints of consecutive primal planes; the
      dual ghost sits at the negative end (periodic image for Bloch, mirror
      image about lprim[0] otherwise).
    * ``dl[PRIM][w][i] = ldual[i] - ldual[i-1]`` (ghost used for i = 0),
      ``dl[DUAL][w][i] = lprim[i+1] - lprim[i]`` (test/source.jl:14-15).
    """

    def __init__(self, lprim, isbloch):
        self.lprim_full = tuple(np.asarray(l, dtype=np.float64) for l in lprim)
        K = len(self.lprim_full)
        self.K = K
        self.isbloch = tuple(bool(b) for b in isbloch)
        self.N = tuple(len(l) - 1 for l in self.lprim_full)
        self.bounds = (np.array([l[0] for l in self.lprim_full]),
                       np.array([l[-1] for l in self.lprim_full]))
        self.L = self.bounds[1] - self.bounds[0]
        lp, ld, dlp, dld, gh = [], [], [], [], []
        for w in range(K):
            lf = self.lprim_full[w]
            ldual = 0.5 * (lf[:-1] + lf[1:])
            g = ldual[-1] - self.L[w] if self.isbloch[w] else 2.0 * lf[0] - ldual[0]
            lp.append(lf[:-1].copy())
            ld.append(ldual)
            dld.append(np.diff(lf))
            dlp.append(np.diff(np.concatenate([[g], ldual])))
            gh.append(g)
        self.l = (tuple(lp), tuple(ld))
        self.dl = (tuple(dlp), tuple(dld))
        self.ldual_ghost = tuple(gh)

    def ldual_ext(self, w):
        """Dual locations with the negative-end ghost first (N+1 entries)."""
        return np.concatenate([[self.ldual_ghost[w]], self.l[DUAL][w]])

    @property
    def ncell(self):
        return int(np.prod(self.N))


def uniform_grid(N, h=1.0, isbloch=(False, False, False), origin=0.0):
    return Grid(tuple(origin + h * np.arange(n + 1) for n in N), isbloch)


# --------------------------------------------------------------------------
# Sources  (src/source/source.jl, pointsrc.jl, planesrc.jl)
# --------------------------------------------------------------------------
def distweights(c, gt, bounds, l, dl, isbloch):
    """Split a point at ``c`` over the two nearest planes of ``l``.

    Restates src/source/source.jl:208-306 line for line in meaning; returns
    0-based indices ``(ind1, ind2)`` and weights ``(wt1, wt2)`` (1/length).
    Raises ValueError where the reference throws ArgumentError (:214, :230).
    """
    c = float(c)
    l = np.asarray(l, dtype=np.float64)
    dl = np.asarray(dl, dtype=np.float64)
    b0, b1 = float(bounds[0]), float(bounds[1])
    if not (b0 <= c <= b1):
        raise ValueError(f"c = {c} must be within bounds = {(b0, b1)}.")
    L = b1 - b0
    N = len(l)
    if not (N > 1 or isbloch):
        raise ValueError(f"length(l) = {N} must be > 1 for symmetry boundary.")
    zeroing_bc = (gt == PRIM) and not isbloch          # source.jl:243
    indn = 1 if zeroing_bc else 0                       # source.jl:244
    indp = N - 1                                        # source.jl:245
    bc_noeff = l[indn] <= c < l[indp]                   # source.jl:250
    if bc_noeff:
        ind1 = int(np.nonzero(l - c <= 0)[0][-1])       # source.jl:252
        ind2 = ind1 + 1
        dc1 = c - l[ind1]
        dlc = l[ind2] - l[ind1]
    else:
        if c < l[indn]:                                 # source.jl:257-260
            ind1, ind2, bnd = indn, N - 1, b0
        else:                                           # source.jl:261-264
            ind1, ind2, bnd = indp, 0, b1
        dc1 = abs(l[ind1] - c)
        if gt == PRIM:
            dlc = abs(l[ind1] - bnd)
        else:
            dlc = (L - abs(l[ind1] - l[ind2])) if isbloch else 2.0 * abs(l[ind1] - bnd)
    r = dc1 / dlc
    wt1 = 1.0 / dl[ind1]
    if bc_noeff or isbloch or zeroing_bc:               # source.jl:283
        wt1 *= 1.0 - r
    if c == l[ind1] or (not bc_noeff and not isbloch):  # source.jl:289
        ind2 = ind1
        wt2 = 0.0
    else:
        wt2 = 1.0 / dl[ind2]
        if bc_noeff or isbloch:                         # source.jl:299
            wt2 *= r
    return (ind1, ind2), (wt1, wt2)


def _gt_w(nw, gt0):
    """Grid type of the w-component location (flip along w)."""
    return tuple((1 - g) if k == nw else g for k, g in enumerate(gt0))


def create_field_array(N, ncmp=3):
    return np.zeros(tuple(N) + (ncmp,), dtype=np.complex128)


def add_pointsrc(j, gt0, grid, c, p, Idr=1.0):
    """PointSrc assembly, src/source/pointsrc.jl:64-103 (3D, field ∥ shape)."""
    p = np.asarray(p, dtype=np.float64)
    p = p / np.linalg.norm(p)
    for nw in range(3):
        gtc = _gt_w(nw, gt0)
        inds, wts = [], []
        for nu in range(3):
            g = gtc[nu]
            ind, wt = distweights(c[nu], g, (grid.bounds[0][nu], grid.bounds[1][nu]),
                                  grid.l[g][nu], grid.dl[g][nu], grid.isbloch[nu])
            inds.append(ind)
            wts.append(wt)
        Iw = Idr * p[nw]
        for a in range(2):
            for b in range(2):
                for cc in range(2):
                    wv = wts[0][a] * wts[1][b] * wts[2][cc]
                    j[inds[0][a], inds[1][b], inds[2][cc], nw] += Iw * wv
    return j


def add_planesrc(j, gt0, grid, n_axis, c, p, Jdn=1.0):
    """PlaneSrc assembly, src/source/planesrc.jl:34-80 (Cartesian normal)."""
    p = np.asarray(p, dtype=np.float64)
    p = p / np.linalg.norm(p)
    nn = int(n_axis)
    for nw in range(3):
        gtc = _gt_w(nw, gt0)
        g = gtc[nn]
        ind, wt = distweights(c, g, (grid.bounds[0][nn], grid.bounds[1][nn]),
                              grid.l[g][nn], grid.dl[g][nn], grid.isbloch[nn])
        for k in range(2):
            sl = [slice(None)] * 3
            sl[nn] = ind[k]
            j[tuple(sl) + (nw,)] += Jdn * p[nw] * wt[k]
    return j


# --------------------------------------------------------------------------
# PML (create_stretched_∆ls, model.jl:122-139)
# --------------------------------------------------------------------------
def pml_sfactors(grid, omega_pml, Npml, m=4.0, R=1e-8):
    """s-factors at the N primal and N dual locations of each axis."""
    lnR = math.log(R)
    s = ([], [])
    for w in range(3):
        lf = grid.lprim_full[w]
        N = grid.N[w]
        nneg, npos = int(Npml[NEG][w]), int(Npml[POS][w])
        for gt in (PRIM, DUAL):
            u = grid.l[gt][w]
            sig = np.zeros_like(u)
            if nneg > 0:
                lin = lf[nneg]
                Lp = lin - lf[0]
                smax = -(m + 1.0) * lnR / (2.0 * Lp)
                d = np.clip((lin - u) / Lp, 0.0, None)
                sig = sig + smax * d ** m
            if npos > 0:
                lin = lf[N - npos]
                Lp = lf[N] - lin
                smax = -(m + 1.0) * lnR / (2.0 * Lp)
                d = np.clip((u - lin) / Lp, 0.0, None)
                sig = sig + smax * d ** m
            s[gt].append(1.0 + sig / (1j * omega_pml))
    return s


def stretched_dl(grid, omega_pml, Npml, m=4.0, R=1e-8):
    """Returns (s∆lₑ, s∆lₘ): stretched ∆l at E-voxel corners (primal for
    boundft = EE) and at H-voxel corners (dual), per axis."""
    s = pml_sfactors(grid, omega_pml, Npml, m, R)
    sdl_e = tuple(grid.dl[PRIM][w] * s[PRIM][w] for w in range(3))
    sdl_m = tuple(grid.dl[DUAL][w] * s[DUAL][w] for w in range(3))
    return sdl_e, sdl_m


# --------------------------------------------------------------------------
# DOF indexing (component-fastest, order_cmpfirst = true, model.jl:72-81)
# --------------------------------------------------------------------------
def field_to_vec(F):
    """(Nx,Ny,Nz,3) field array → vector indexed c + 3(i + Nx(j + Ny k))."""
    return np.ascontiguousarray(np.transpose(F, (2, 1, 0, 3))).reshape(-1)


def vec_to_field(v, N):
    Nx, Ny, Nz = N
    return np.transpose(v.reshape(Nz, Ny, Nx, 3), (2, 1, 0, 3))


def pinned_mask(grid):
    """(Nx,Ny,Nz,3) bool: E_w at primal index 0 along a non-Bloch axis v ≠ w."""
    N = grid.N
    M = np.zeros(tuple(N) + (3,), dtype=bool)
    for w in range(3):
        for v in range(3):
            if v == w or grid.isbloch[v]:
                continue
            sl = [slice(None)] * 3
            sl[v] = 0
            M[tuple(sl) + (w,)] = True
    return M


def _ijk(N):
    return np.meshgrid(np.arange(N[0]), np.arange(N[1]), np.arange(N[2]), indexing="ij")


def _dof(c, i, j, k, N):
    return c + 3 * (i + N[0] * (j + N[1] * k))


class _Coo:
    def __init__(self, n):
        self.n = n
        self.r, self.c, self.v = [], [], []

    def add(self, r, c, v):
        r = np.asarray(r)
        v = np.broadcast_to(np.asarray(v, dtype=np.complex128), r.shape).ravel()
        r = r.ravel()
        c = np.asarray(c).ravel()
        self.r.append(r)
        self.c.append(c)
        self.v.append(v)

    def csr(self):
        r = np.concatenate(self.r) if self.r else np.zeros(0, int)
        c = np.concatenate(self.c) if self.c else np.zeros(0, int)
        v = np.concatenate(self.v) if self.v else np.zeros(0, complex)
        return sp.csr_matrix((v, (r, c)), shape=(self.n, self.n))


def _bloch_phase(grid, kbloch):
    return tuple(np.exp(-1j * kbloch[w] * grid.L[w]) for w in range(3))


def _diff(coo, grid, cout, cin, v, coef, sign, fwd, ph):
    """Add sign·coef[idx_v]·(difference of component cin along v) into rows
    of component cout.  fwd: f[i+1]-f[i] (ghost at N); else g[i]-g[i-1]
    (ghost at -1)."""
    N = grid.N
    I, J, K = _ijk(N)
    idx = (I, J, K)
    rows = _dof(cout, I, J, K, N)
    cf = coef[idx[v]] * sign
    self_cols = _dof(cin, I, J, K, N)
    nb = [I.copy(), J.copy(), K.copy()]
    if fwd:
        coo.add(rows, self_cols, -cf)
        nb[v] = idx[v] + 1
        ghost = nb[v] == N[v]
        fac = np.ones(I.shape, dtype=np.complex128)
        if grid.isbloch[v]:
            nb[v] = np.where(ghost, 0, nb[v])
            fac = np.where(ghost, ph[v], 1.0)
            keep = np.ones(I.shape, bool)
        else:
            keep = ~ghost          # PEC: tangential E at the primal ghost is 0
        cols = _dof(cin, nb[0], nb[1], nb[2], N)
        coo.add(rows[keep], cols[keep], (cf * fac)[keep])
    else:
        coo.add(rows, self_cols, cf)
        nb[v] = idx[v] - 1
        ghost = nb[v] < 0
        fac = np.ones(I.shape, dtype=np.complex128)
        if grid.isbloch[v]:
            nb[v] = np.where(ghost, N[v] - 1, nb[v])
            fac = np.where(ghost, 1.0 / ph[v], 1.0)
        else:
            nb[v] = np.where(ghost, 0, nb[v])   # mirror: H(-1) = H(0)
        cols = _dof(cin, nb[0], nb[1], nb[2], N)
        coo.add(rows, cols, -cf * fac)


def create_curls(grid, sdl_e, sdl_m, kbloch=(0.0, 0.0, 0.0)):
    """Cₑ (E→H, forward differences / s∆lₘ) and Cₘ (H→E, backward
    differences / s∆lₑ); create_curls, model.jl:160-175."""
    n = 3 * grid.ncell
    ph = _bloch_phase(grid, kbloch)
    ce = _Coo(n)
    cm = _Coo(n)
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        # H_a = ∂_b E_c - ∂_c E_b
        _diff(ce, grid, a, c, b, 1.0 / sdl_m[b], +1.0, True, ph)
        _diff(ce, grid, a, b, c, 1.0 / sdl_m[c], -1.0, True, ph)
        # E_a = ∂_b H_c - ∂_c H_b
        _diff(cm, grid, a, c, b, 1.0 / sdl_e[b], +1.0, False, ph)
        _diff(cm, grid, a, b, c, 1.0 / sdl_e[c], -1.0, False, ph)
    Ce = ce.csr()
    Cm = cm.csr()
    keep = (~field_to_vec(pinned_mask(grid))).astype(np.float64)
    Ce = Ce @ sp.diags(keep)
    Ce.sum_duplicates()
    Cm.sum_duplicates()
    return Ce.tocsr(), Cm.tocsr()


_PAIR = {(0, 1): 0, (1, 0): 0, (1, 2): 1, (2, 1): 1, (2, 0): 2, (0, 2): 2}


def create_paramop(grid, eps_diag, eps_off, sdl_e, sdl_m, kbloch=(0.0, 0.0, 0.0)):
    """Pε = diag(ε_ww at E_w) + M·(Σ Mout_w diag(ε_wv at corners) Min_v)·M.

    eps_diag: (Nx,Ny,Nz,3) real/complex, ε_ww at the E_w sample of cell (i,j,k).
    eps_off:  (Nx,Ny,Nz,3) or None, ε_xy, ε_yz, ε_zx at corner (i,j,k).
    Follows create_paramops, model.jl:141-158 (isfwd_in = boundft .!= EE:
    backward averaging of the input to the corners)."""
    n = 3 * grid.ncell
    N = grid.N
    P = sp.diags(field_to_vec(np.asarray(eps_diag, dtype=np.complex128)))
    if eps_off is None or not np.any(eps_off):
        return P.tocsr()
    ph = _bloch_phase(grid, kbloch)
    I, J, K = _ijk(N)
    idx = (I, J, K)
    coo = _Coo(n)
    for w in range(3):
        for v in range(3):
            if v == w:
                continue
            pe = eps_off[..., _PAIR[(w, v)]]
            rows = _dof(w, I, J, K, N)
            for sw in (0, 1):          # corner at primal w-index i + sw
                cw = idx[w] + sw
                ghost_w = cw == N[w]
                if grid.isbloch[w]:
                    cw_r = np.where(ghost_w, 0, cw)
                    facw = np.where(ghost_w, ph[w], 1.0)
                    keepw = np.ones(I.shape, bool)
                else:
                    cw_r = np.where(ghost_w, 0, cw)
                    facw = np.ones(I.shape, dtype=np.complex128)
                    keepw = ~ghost_w
                wout = 0.5
                corner = [I.copy(), J.copy(), K.copy()]
                corner[w] = cw_r
                eps_c = pe[corner[0], corner[1], corner[2]]
                for sv in (0, 1):      # E_v at dual v-index (corner_v - 1 + sv)
                    cv = corner[v]
                    ev = cv - 1 + sv
                    sdl_m_ext = sdl_m[v][np.where(ev < 0, (N[v] - 1) if grid.isbloch[v] else 0, ev)]
                    win = sdl_m_ext / (2.0 * sdl_e[v][cv])
                    gv = ev < 0
                    if grid.isbloch[v]:
                        ev_r = np.where(gv, N[v] - 1, ev)
                        facv = np.where(gv, 1.0 / ph[v], 1.0)
                    else:
                        ev_r = np.where(gv, 0, ev)
                        facv = np.ones(I.shape, dtype=np.complex128)
                    src = list(corner)
                    src[v] = ev_r
                    cols = _dof(v, src[0], src[1], src[2], N)
                    val = wout * eps_c * win * facw * facv
                    coo.add(rows[keepw], cols[keepw], val[keepw])
    Poff = coo.csr()
    m = sp.diags((~field_to_vec(pinned_mask(grid))).astype(np.float64))
    return (P + m @ Poff @ m).tocsr()


def create_A(omega, Peps, Ce, Cm):
    """A = Cₘ·(Pμ \\ Cₑ) - ω²·Pε with Pμ = I (model.jl:235-237, A9)."""
    A = Cm @ Ce
    if omega != 0:
        A = A - (omega ** 2) * Peps
    return A.tocsr()


def create_A_hh(omega, eps_diag_vec, Ce, Cm):
    """H formulation: A = Cₑ·(Pε \\ Cₘ) − ω²·Pμ with Pμ = I and a diagonal
    Pε (model.jl:238-240; the reference divides by Pε only when it is
    diagonal).  eps_diag_vec: ε at every E sample (DOF order)."""
    A = Ce @ sp.diags(1.0 / np.asarray(eps_diag_vec, dtype=np.complex128)) @ Cm
    if omega != 0:
        A = A - (omega ** 2) * sp.identity(Ce.shape[0], dtype=np.complex128, format="csr")
    return A.tocsr()


def create_b_hh(omega, eps_diag_vec, Ce, je_vec, jm_vec=None):
    """b = Cₑ (Pε \\ jₑ) − iω jₘ (model.jl:266-268)."""
    b = Ce @ (np.asarray(je_vec, dtype=np.complex128) / np.asarray(eps_diag_vec, dtype=np.complex128))
    if jm_vec is not None and omega != 0:
        b = b - (1j * omega) * jm_vec
    return b


def create_b(omega, je_vec, jm_vec=None, Cm=None):
    """b = -Cₘ(Pμ⁻¹ jₘ) - iω jₑ (model.jl:262-265)."""
    b = np.zeros_like(je_vec, dtype=np.complex128)
    if jm_vec is not None and Cm is not None:
        b = -(Cm @ jm_vec)
    if omega != 0:
        b = b - (1j * omega) * je_vec
    return b


def h_from_e(e, omega, Ce, jm_vec=None):
    """H = (i/ω)·Pμ⁻¹·(Cₑ e + jₘ) (model.jl:291-292)."""
    t = Ce @ e
    if jm_vec is not None:
        t = t + jm_vec
    return (1j / omega) * t


def e_from_h(h, omega, eps_diag_vec, Cm, je_vec=None):
    """E = (−i/ω)·Pε⁻¹·(Cₘ h − jₑ) (model.jl:281-284) with a diagonal Pε
    given by its values at the E samples (DOF order)."""
    t = Cm @ h
    if je_vec is not None:
        t = t - je_vec
    return (-1j / omega) * t / np.asarray(eps_diag_vec)


def create_Mcs(grid, sdl_e, sdl_m, kbloch=(0.0, 0.0, 0.0)):
    """Corner interpolation (create_Mcs, model.jl:287-306), restated from
    the roles given there — create_mean(isfwd, ∆l, ∆l′⁻¹): the mean of each
    component along its own axis, weighted by ∆l and scaled by ∆l′⁻¹/2:
      Mcₑ (isfwdₑ = boundft .!= EE = false, ∆l = s∆lₘ, ∆l′⁻¹ = 1/s∆lₑ):
          Ec_w[j] = (s∆lₘ[j−1]·E_w[j−1] + s∆lₘ[j]·E_w[j]) / (2·s∆lₑ[j])
      Mcₘ (isfwdₘ = boundft .!= HH = true, ∆l = s∆lₑ, ∆l′⁻¹ = 1/s∆lₘ):
          Hc_w[j] = (s∆lₑ[j]·H_w[j] + s∆lₑ[j+1]·H_w[j+1]) / (2·s∆lₘ[j])
    Ghosts as in the operator: E_w[−1] = E_w[0] with weight s∆lₘ[0] on a
    symmetry wall (the ε averaging's mirror), H_w[N] = 0 there; Bloch axes
    wrap with the phase e^{∓ikL}.  MaxwellBase's create_mean itself is not
    available here, so parity with it is unpinned."""
    N = grid.N
    n = 3 * grid.ncell
    ph = _bloch_phase(grid, kbloch)
    I, J, K = _ijk(N)
    idx = (I, J, K)
    ce, cm = _Coo(n), _Coo(n)
    for w in range(3):
        rows = _dof(w, I, J, K, N)
        t = idx[w]
        # E: backward
        inv = 1.0 / (2.0 * sdl_e[w][t])
        ce.add(rows, rows, sdl_m[w][t] * inv)
        nb = [I.copy(), J.copy(), K.copy()]
        g = t == 0
        if grid.isbloch[w]:
            nb[w] = np.where(g, N[w] - 1, t - 1)
            fac = np.where(g, 1.0 / ph[w], 1.0)
        else:
            nb[w] = np.where(g, 0, t - 1)
            fac = np.ones(I.shape, dtype=np.complex128)
        ce.add(rows, _dof(w, nb[0], nb[1], nb[2], N), sdl_m[w][nb[w]] * inv * fac)
        # H: forward
        inv = 1.0 / (2.0 * sdl_m[w][t])
        cm.add(rows, rows, sdl_e[w][t] * inv)
        nb = [I.copy(), J.copy(), K.copy()]
        g = t == N[w] - 1
        if grid.isbloch[w]:
            nb[w] = np.where(g, 0, t + 1)
            cm.add(rows, _dof(w, nb[0], nb[1], nb[2], N), sdl_e[w][nb[w]] * inv * np.where(g, ph[w], 1.0))
        else:
            keep = ~g
            nb[w] = np.where(g, 0, t + 1)
            val = sdl_e[w][nb[w]] * inv
            cm.add(rows[keep], _dof(w, nb[0], nb[1], nb[2], N)[keep], val[keep])
    return ce.csr(), cm.csr()


# --------------------------------------------------------------------------
# Material assignment and Kottke smoothing (src/model/full.jl:16-70)
# --------------------------------------------------------------------------
def volfrac_plane(lo, hi, n, r0):
    """Fraction of the box [lo, hi] on the side n·(x - r0) ≤ 0 (exact for a
    plane).  Closed form of Scardovelli & Zaleski (J. Comput. Phys. 164,
    2000), rearranged so that no term divides a vanishing quantity."""
    m = [0.0, 0.0, 0.0]
    d = 0.0
    for a in range(3):
        side = hi[a] - lo[a]
        ma = n[a] * side
        d += n[a] * (r0[a] - lo[a])
        if ma < 0.0:
            d -= ma
            ma = -ma
        m[a] = ma
    s = m[0] + m[1] + m[2]
    if s <= 0.0:
        return 0.5
    alpha = d / s
    if alpha <= 0.0:
        return 0.0
    if alpha >= 1.0:
        return 1.0
    m = sorted(x / s for x in m)
    tiny = 1e-12
    if m[0] < tiny * m[2]:
        m[0] = 0.0
    if m[1] < tiny * m[2]:
        m[1] = 0.0
    flip = alpha > 0.5
    if flip:
        alpha = 1.0 - alpha
    v = _sz_volume(m[0], m[1], m[2], alpha)
    return 1.0 - v if flip else v


def _sz_volume(m1, m2, m3, a):
    """Volume under m·y ≤ a in the unit cube, m1 ≤ m2 ≤ m3, Σm = 1, a ≤ 1/2."""
    m12 = m1 + m2
    if a < m1:
        t = a / m1
        return t * a * a / (6.0 * m2 * m3)
    if a < m2:
        return a * (a - m1) / (2.0 * m2 * m3) + m1 * m1 / (6.0 * m2 * m3)
    if a < min(m12, m3):
        q = a - m2
        base = (3.0 * a * a - 3.0 * a * m1 + m1 * m1) / (6.0 * m2 * m3)
        return base - (q / m1) * q * q / (6.0 * m2 * m3)
    if m3 < m12:
        q2 = a - m2
        q3 = a - m3
        base = (3.0 * a * a - 3.0 * a * m1 + m1 * m1) / (6.0 * m2 * m3)
        return base - ((q2 / m1) * q2 * q2 + (q3 / m1) * q3 * q3) / (6.0 * m2 * m3)
    return (2.0 * a - m12) / (2.0 * m3)


class Sphere:
    kind = "sphere"

    def __init__(self, c, r, eps):
        self.c = np.asarray(c, dtype=np.float64)
        self.r = float(r)
        self.eps = float(eps)

    def contains(self, X, Y, Z):
        dx = X - self.c[0]
        dy = Y - self.c[1]
        dz = Z - self.c[2]
        return (dx * dx + dy * dy) + dz * dz <= self.r * self.r

    def normal_point(self, xc):
        v = np.asarray(xc, dtype=np.float64) - self.c
        nr = math.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
        if nr == 0.0:
            n = np.array([1.0, 0.0, 0.0])
        else:
            n = v / nr
        return n, self.c + self.r * n


class CylinderZ:
    """A disk of the 2D models: the cylinder x²+y² ≤ r² unbounded in z (the
    z-invariant slice of a 2D shape).  Normal radial in the xy-plane."""
    kind = "cylz"

    def __init__(self, c, r, eps):
        self.c = np.asarray(c, dtype=np.float64)[:2]
        self.r = float(r)
        self.eps = float(eps)

    def contains(self, X, Y, Z):
        dx = X - self.c[0]
        dy = Y - self.c[1]
        return dx * dx + dy * dy <= self.r * self.r

    def normal_point(self, xc):
        v0 = xc[0] - self.c[0]
        v1 = xc[1] - self.c[1]
        nr = math.sqrt((v0 * v0 + v1 * v1) + 0.0 * 0.0)
        if nr == 0.0:
            n = np.array([1.0, 0.0, 0.0])
        else:
            n = np.array([v0 / nr, v1 / nr, 0.0])
        return n, np.array([self.c[0] + self.r * n[0], self.c[1] + self.r * n[1], xc[2]])


class Box:
    kind = "box"

    def __init__(self, lo, hi, eps):
        self.lo = np.asarray(lo, dtype=np.float64)
        self.hi = np.asarray(hi, dtype=np.float64)
        self.eps = float(eps)

    def contains(self, X, Y, Z):
        return ((X >= self.lo[0]) & (X <= self.hi[0]) & (Y >= self.lo[1]) & (Y <= self.hi[1])
                & (Z >= self.lo[2]) & (Z <= self.hi[2]))

    def normal_point(self, xc):
        best, bn, bp = -np.inf, None, None
        for a in range(3):
            for side in (0, 1):
                if side == 0:
                    dist = self.lo[a] - xc[a]
                    nv = -1.0
                    plane = self.lo[a]
                else:
                    dist = xc[a] - self.hi[a]
                    nv = 1.0
                    plane = self.hi[a]
                if dist > best:
                    best = dist
                    bn = np.zeros(3)
                    bn[a] = nv
                    bp = np.array(xc, dtype=np.float64)
                    bp[a] = plane
        return bn, bp


class DesignRegion:
    """Per-cell ε over cells [i0,i1)×[j0,j1)×[k0,k1) (convention A7)."""

    def __init__(self, lo_idx, hi_idx, eps_cells):
        self.lo = tuple(int(x) for x in lo_idx)
        self.hi = tuple(int(x) for x in hi_idx)
        self.eps = np.asarray(eps_cells, dtype=np.float64)
        assert self.eps.shape == tuple(h - l for l, h in zip(self.lo, self.hi))


def _ext_axes(grid, types):
    """Per-axis extended locations (N+1) for a sample set.  PRIM: l₀..l_N
    (ghost at the end); DUAL: ghost, d₀..d_{N-1}."""
    out = []
    for w in range(3):
        out.append(grid.lprim_full[w].copy() if types[w] == PRIM else grid.ldual_ext(w))
    return out


def object_index(grid, objects, types):
    """Object index (0 = background, q = q-th added object, last wins) at the
    (N+1)³ extended sample set of grid types ``types``; ghost entries follow
    the boundary: Bloch → periodic copy, PEC dual ghost → mirror copy of
    index 0, PEC primal ghost → evaluated on the boundary plane."""
    ax = _ext_axes(grid, types)
    X, Y, Z = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
    oind = np.zeros(X.shape, dtype=np.int32)
    for q, obj in enumerate(objects, start=1):
        oind[obj.contains(X, Y, Z)] = q
    for w in range(3):
        sl_dst = [slice(None)] * 3
        sl_src = [slice(None)] * 3
        if types[w] == PRIM:
            if grid.isbloch[w]:
                sl_dst[w] = grid.N[w]
                sl_src[w] = 0
                oind[tuple(sl_dst)] = oind[tuple(sl_src)]
        else:
            sl_dst[w] = 0
            sl_src[w] = grid.N[w] if grid.isbloch[w] else 1
            oind[tuple(sl_dst)] = oind[tuple(sl_src)]
    return oind


def _obj_eps(objects, eps_bg):
    return np.array([eps_bg] + [o.eps for o in objects], dtype=np.float64)


def _kottke(eps_fg, eps_bg, f, n):
    em = f * eps_fg + (1.0 - f) * eps_bg
    eh = 1.0 / (f / eps_fg + (1.0 - f) / eps_bg)
    return em * np.eye(3) + (eh - em) * np.outer(n, n)


def assign_smooth(grid, objects, eps_bg=1.0, design=None, return_debug=False):
    """Assign + smooth ε on the grid (calc_matparams!, full.jl:16-70).

    Returns eps_diag (Nx,Ny,Nz,3) real and eps_off (Nx,Ny,Nz,3) real
    (ε_xy, ε_yz, ε_zx at corners).  With return_debug, also the object-index
    arrays and smoothing masks (for bit-exact comparisons)."""
    N = grid.N
    epsq = _obj_eps(objects, eps_bg)
    eps_diag = np.zeros(tuple(N) + (3,))
    eps_off = np.zeros(tuple(N) + (3,))
    smask = np.zeros(tuple(N) + (4,), dtype=np.uint8)   # Exx, Eyy, Ezz, corner
    dbg = {}
    for w in range(3):
        # E_w samples: dual along w, primal elsewhere (assigned value)
        et = tuple(DUAL if a == w else PRIM for a in range(3))
        ht = tuple(PRIM if a == w else DUAL for a in range(3))
        oe = object_index(grid, objects, et)
        # E_w sample (i,j,k) sits at ext position i+1 along w (dual), i elsewhere
        sl = tuple(slice(1, N[a] + 1) if a == w else slice(0, N[a]) for a in range(3))
        assigned = epsq[oe[sl]]
        oh = object_index(grid, objects, ht)
        dbg[f"oind_E{w}"] = oe[sl].copy()
        dbg[f"oind_H{w}"] = oh
        eps_diag[..., w] = assigned
        lo_ax = [grid.lprim_full[a] if ht[a] == PRIM else grid.ldual_ext(a) for a in range(3)]
        cmin, cmax = _corner_minmax(oh, N)
        idx = np.argwhere(cmin != cmax)
        for (i, j, k) in idx:
            corners = oh[i:i + 2, j:j + 2, k:k + 2].ravel()
            lo = np.array([lo_ax[0][i], lo_ax[1][j], lo_ax[2][k]])
            hi = np.array([lo_ax[0][i + 1], lo_ax[1][j + 1], lo_ax[2][k + 1]])
            T = _smoothed_tensor(objects, epsq, corners, lo, hi)
            eps_diag[i, j, k, w] = T[w, w]
            smask[i, j, k, w] = 1
    # corners: primal³; voxel corners at cell centres (dual³)
    oc = object_index(grid, objects, (DUAL, DUAL, DUAL))
    dbg["oind_C"] = oc
    lo_ax = [grid.ldual_ext(a) for a in range(3)]
    cmin, cmax = _corner_minmax(oc, N)
    for (i, j, k) in np.argwhere(cmin != cmax):
        corners = oc[i:i + 2, j:j + 2, k:k + 2].ravel()
        lo = np.array([lo_ax[0][i], lo_ax[1][j], lo_ax[2][k]])
        hi = np.array([lo_ax[0][i + 1], lo_ax[1][j + 1], lo_ax[2][k + 1]])
        T = _smoothed_tensor(objects, epsq, corners, lo, hi)
        eps_off[i, j, k, 0] = T[0, 1]
        eps_off[i, j, k, 1] = T[1, 2]
        eps_off[i, j, k, 2] = T[2, 0]
        smask[i, j, k, 3] = 1
    if design is not None:
        _apply_design(grid, design, epsq, oc, eps_diag, eps_off, smask)
    if return_debug:
        dbg["smask"] = smask
        return eps_diag, eps_off, dbg
    return eps_diag, eps_off


def _corner_minmax(o, N):
    """min and max over the 2×2×2 ext block starting at each sample."""
    blocks = [o[a:a + N[0], b:b + N[1], c:c + N[2]] for a in (0, 1) for b in (0, 1) for c in (0, 1)]
    st = np.stack(blocks)
    return st.min(0), st.max(0)


def _smoothed_tensor(objects, epsq, corners, lo, hi):
    u = np.unique(corners)
    if len(u) == 2:
        fg = int(u.max())
        bgq = int(u.min())
        xc = 0.5 * (lo + hi)
        n, r0 = objects[fg - 1].normal_point(xc)
        f = volfrac_plane(lo, hi, n, r0)
        return _kottke(epsq[fg], epsq[bgq], f, n)
    return np.mean(epsq[corners]) * np.eye(3) * 1.0 if len(u) > 2 else epsq[u[0]] * np.eye(3)


def _apply_design(grid, design, epsq, oc, eps_diag, eps_off, smask):
    N = grid.N
    inreg = np.zeros(N, dtype=bool)
    sl = tuple(slice(design.lo[a], design.hi[a]) for a in range(3))
    inreg[sl] = True
    cellval = epsq[oc[1:, 1:, 1:]].copy()     # cell centres (dual index 0..N-1)
    cellval[sl] = design.eps
    for w in range(3):
        us = [a for a in range(3) if a != w]
        acc = np.zeros(N)
        touch = np.zeros(N, dtype=bool)
        for s0 in (-1, 0):
            for s1 in (-1, 0):
                idx = list(np.meshgrid(np.arange(N[0]), np.arange(N[1]), np.arange(N[2]), indexing="ij"))
                for a, s in zip(us, (s0, s1)):
                    t = idx[a] + s
                    if grid.isbloch[a]:
                        t = np.mod(t, N[a])
                    else:
                        t = np.where(t < 0, 0, t)
                    idx[a] = t
                acc += cellval[idx[0], idx[1], idx[2]]
                touch |= inreg[idx[0], idx[1], idx[2]]
        eps_diag[..., w] = np.where(touch, 0.25 * acc, eps_diag[..., w])
        smask[..., w] = np.where(touch, 2, smask[..., w])
    touchc = np.zeros(N, dtype=bool)
    for s in [(a, b, c) for a in (-1, 0) for b in (-1, 0) for c in (-1, 0)]:
        idx = list(np.meshgrid(np.arange(N[0]), np.arange(N[1]), np.arange(N[2]), indexing="ij"))
        for a in range(3):
            t = idx[a] + s[a]
            t = np.mod(t, N[a]) if grid.isbloch[a] else np.where(t < 0, 0, t)
            idx[a] = t
        touchc |= inreg[idx[0], idx[1], idx[2]]
    eps_off[touchc] = 0.0
    smask[..., 3] = np.where(touchc, 2, smask[..., 3])


def design_grad_chain(grid, design, g_diag):
    """Chain dL/dε_ww (Nx,Ny,Nz,3 real) back to the design cells (A7)."""
    N = grid.N
    lo, hi = design.lo, design.hi
    inreg = np.zeros(N, dtype=bool)
    inreg[tuple(slice(lo[a], hi[a]) for a in range(3))] = True
    out = np.zeros(N)
    for w in range(3):
        us = [a for a in range(3) if a != w]
        touch = np.zeros(N, dtype=bool)
        cells = []
        for s0 in (-1, 0):
            for s1 in (-1, 0):
                idx = list(np.meshgrid(np.arange(N[0]), np.arange(N[1]), np.arange(N[2]), indexing="ij"))
                for a, s in zip(us, (s0, s1)):
                    t = idx[a] + s
                    t = np.mod(t, N[a]) if grid.isbloch[a] else np.where(t < 0, 0, t)
                    idx[a] = t
                cells.append(idx)
                touch |= inreg[idx[0], idx[1], idx[2]]
        g = np.where(touch, 0.25 * g_diag[..., w], 0.0)
        for idx in cells:
            np.add.at(out, (idx[0], idx[1], idx[2]), np.where(inreg[idx[0], idx[1], idx[2]], g, 0.0))
    return out[tuple(slice(lo[a], hi[a]) for a in range(3))]


# --------------------------------------------------------------------------
# Whole-system helper
# --------------------------------------------------------------------------
class System:
    """Assembles A and b for a 3D model (ModelFull) under conventions A1-A9."""

    def __init__(self, grid, omega, Npml, objects=(), eps_bg=1.0, design=None,
                 pml_m=4.0, pml_R=1e-8, kbloch=(0.0, 0.0, 0.0)):
        self.grid = grid
        self.omega = omega
        self.kbloch = kbloch
        self.sdl_e, self.sdl_m = stretched_dl(grid, omega, Npml, pml_m, pml_R)
        self.eps_diag, self.eps_off, self.debug = assign_smooth(
            grid, list(objects), eps_bg, design, return_debug=True)
        self.Ce, self.Cm = create_curls(grid, self.sdl_e, self.sdl_m, kbloch)
        self.Peps = create_paramop(grid, self.eps_diag, self.eps_off, self.sdl_e, self.sdl_m, kbloch)
        self.A = create_A(omega, self.Peps, self.Ce, self.Cm)
        self.je = create_field_array(grid.N)

    def add_pointsrc(self, c, p, Idr=1.0):
        add_pointsrc(self.je, (PRIM, PRIM, PRIM), self.grid, c, p, Idr)

    def add_planesrc(self, n_axis, c, p, Jdn=1.0):
        add_planesrc(self.je, (PRIM, PRIM, PRIM), self.grid, n_axis, c, p, Jdn)

    def b(self):
        return create_b(self.omega, field_to_vec(self.je))


def adjoint_eps_grad(A, omega, e, g):
    """dL/dε_cc at every E_c sample, (3·Ncell,) real, for A e = b and the
    Wirtinger derivative g = ∂L/∂e (dL = 2·Re(gᵀ de)).  A = K − ω²·Pε
    (create_A, src/model/model.jl:225-246) gives ∂A/∂ε_cc = −ω² on the
    diagonal, hence de/dε_cc = ω²·A⁻¹(e_c u_c) and
    dL/dε_cc = 2·Re(ω²·λ_c·e_c) with Aᵀλ = g.  The reference has no adjoint;
    this restates the derivative of the operator it assembles.  Direct
    solve (small systems only)."""
    import scipy.sparse.linalg as spla
    lam = spla.spsolve(A.T.tocsc(), g)
    return 2.0 * np.real(omega ** 2 * lam * e), lam


# --------------------------------------------------------------------------
# Solver (FP64 BiCGSTAB; the reference itself leaves A\b to the user)
# --------------------------------------------------------------------------
def bicgstab(A, b, tol=1e-10, maxit=100000, x0=None):
    """Unpreconditioned BiCGSTAB (van der Vorst 1992) in complex128 with the
    unconjugated shadow product used by the GPU solver.  Returns
    (x, iterations, relres_history)."""
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - A @ x
    rh = r.copy()
    nb = np.linalg.norm(b)
    rho = alpha = om = 1.0 + 0j
    v = np.zeros_like(b)
    p = np.zeros_like(b)
    hist = [np.linalg.norm(r) / nb]
    for it in range(1, maxit + 1):
        rho_new = np.vdot(rh, r)
        beta = (rho_new / rho) * (alpha / om)
        p = r + beta * (p - om * v)
        v = A @ p
        alpha = rho_new / np.vdot(rh, v)
        s = r - alpha * v
        t = A @ s
        om = np.vdot(t, s) / np.vdot(t, t)
        x = x + alpha * p + om * s
        r = s - om * t
        rho = rho_new
        hist.append(np.linalg.norm(r) / nb)
        if hist[-1] < tol:
            return x, it, hist
    return x, maxit, hist
