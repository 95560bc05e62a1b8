"""Seeded synthetic models for the benchmark configurations.

There is no public dataset on this path; each configuration is generated
from ``numpy.random.default_rng(seed)`` with seed = 1000·(config index) +
instance, with the shapes, sizes and value distributions of the benchmark
definitions:

  1  vacuum 32³, 10-cell PML, λ = 20, z-dipole at the centre
  2  96³, 10-cell PML, 40 non-overlapping spheres r ~ U[3, 8] (ε = 12.25 in
     vacuum), x-polarised current sheet at z = 15, λ = 16
  3  24 instances with edges drawn from {48, …, 128}, 8-cell PML, 10–60
     spheres each, λ ~ U[12, 24], 1–4 dipoles with random orientation
  4  128×128×64 slab waveguide (ε = 12.25, 8 cells thick) with a 40×40×10
     design region of per-cell ε ~ U[1, 12.25]; y-polarised dipole at x = 20
  5  320³, 12-cell PML, 400 spheres r ~ U[4, 16], ε ∈ {1, 2.25, 12.25},
     λ = 24, 8 dipole right-hand sides

Spheres are rejection-sampled with a gap of at least 2 cells between
surfaces, so no voxel ever touches more than two materials.
"""
import numpy as np

from . import model as M
from .grid import uniform_grid


def _spheres(rng, N, npml, count, rlo, rhi, eps_choices, gap=2.0, max_tries=200000):
    out = []
    tries = 0
    lo = np.asarray([npml] * 3, dtype=float)
    hi = np.asarray(N, dtype=float) - npml
    while len(out) < count and tries < max_tries:
        tries += 1
        r = rng.uniform(rlo, rhi)
        if np.any(hi - lo <= 2 * r):
            continue
        c = rng.uniform(lo + r, hi - r)
        if all(np.linalg.norm(c - s[0]) > r + s[1] + gap for s in out):
            out.append((c, r, float(rng.choice(eps_choices))))
    return out


def config1(seed=0):
    N = (32, 32, 32)
    g = uniform_grid(N)
    om = 2 * np.pi / 20
    mdl = M.ModelFull(g)
    M.set_ωpml(mdl, om)
    M.set_Npml(mdl, ((10,) * 3, (10,) * 3))
    M.add_srce(mdl, M_point((16, 16, 16.5), (0, 0, 1)))
    return mdl, om


def M_point(c, p, Idr=1.0):
    from .sources import PointSrc
    return PointSrc(c, p, Idr)


def M_plane(n, c, p, Jdn=1.0):
    from .sources import PlaneSrc
    return PlaneSrc(n, c, p, Jdn)


def config2(seed=1000, nsph=40):
    N = (96, 96, 96)
    rng = np.random.default_rng(seed)
    g = uniform_grid(N)
    om = 2 * np.pi / 16
    mdl = M.ModelFull(g)
    M.set_ωpml(mdl, om)
    M.set_Npml(mdl, ((10,) * 3, (10,) * 3))
    for c, r, e in _spheres(rng, N, 10, nsph, 3.0, 8.0, [12.25]):
        M.add_obj(mdl, "dielectric", M.Sphere(c, r), ε=e)
    M.add_srce(mdl, M_plane((0, 0, 1), 15.0, (1, 0, 0)))
    return mdl, om


def config3_instance(q, seed_base=2000):
    rng = np.random.default_rng(seed_base + q)
    n = int(rng.choice([48, 64, 80, 96, 112, 128]))
    N = (n, n, n)
    g = uniform_grid(N)
    lam = rng.uniform(12.0, 24.0)
    om = 2 * np.pi / lam
    mdl = M.ModelFull(g)
    M.set_ωpml(mdl, om)
    M.set_Npml(mdl, ((8,) * 3, (8,) * 3))
    for c, r, e in _spheres(rng, N, 8, int(rng.integers(10, 61)), 3.0, 8.0, [12.25]):
        M.add_obj(mdl, "dielectric", M.Sphere(c, r), ε=e)
    rhs = []
    for _ in range(int(rng.integers(1, 5))):
        c = rng.uniform(10.0, n - 10.0, 3)
        p = rng.standard_normal(3)
        rhs.append((c, p / np.linalg.norm(p)))
    return mdl, om, rhs


def config4(seed=3000):
    N = (128, 128, 64)
    rng = np.random.default_rng(seed)
    g = uniform_grid(N)
    om = 2 * np.pi / 16
    mdl = M.ModelFull(g)
    M.set_ωpml(mdl, om)
    M.set_Npml(mdl, ((10,) * 3, (10,) * 3))
    zc = N[2] / 2
    M.add_obj(mdl, "slab", M.Box((-1.0, -1.0, zc - 4.0), (N[0] + 1.0, N[1] + 1.0, zc + 4.0)), ε=12.25)
    lo = (44, 44, 27)
    hi = (84, 84, 37)
    M.set_design(mdl, M.DesignRegion(lo, hi, rng.uniform(1.0, 12.25, (40, 40, 10))))
    M.add_srce(mdl, M_point((20.0, 64.0, zc), (0, 1, 0)))
    return mdl, om


def config4_mode(N=(128, 128, 64), x_plane=108, width=6.0, seed=3000):
    """Objective weights: a Gaussian E_y profile of width 6 cells centred on
    the slab, on the plane x = 108 (vector over all DOFs, zero elsewhere)."""
    rng = np.random.default_rng(seed + 1)
    y = np.arange(N[1]) + 0.5
    z = np.arange(N[2]) * 1.0
    yc = N[1] / 2 + rng.uniform(-1, 1)
    zc = N[2] / 2
    prof = np.exp(-((y[:, None] - yc) ** 2 + (z[None, :] - zc) ** 2) / (2 * width ** 2))
    F = np.zeros(tuple(N) + (3,), dtype=np.complex128)
    F[x_plane, :, :, 1] = prof
    return M.field_arr2vec(F)


def config5(seed=4000, nsph=400):
    N = (320, 320, 320)
    rng = np.random.default_rng(seed)
    g = uniform_grid(N)
    om = 2 * np.pi / 24
    mdl = M.ModelFull(g)
    M.set_ωpml(mdl, om)
    M.set_Npml(mdl, ((12,) * 3, (12,) * 3))
    for c, r, e in _spheres(rng, N, 12, nsph, 4.0, 16.0, [1.0, 2.25, 12.25]):
        M.add_obj(mdl, "dielectric", M.Sphere(c, r), ε=e)
    rhs = []
    for _ in range(8):
        c = rng.uniform(40.0, 280.0, 3)
        p = rng.standard_normal(3)
        rhs.append((c, p / np.linalg.norm(p)))
    return mdl, om, rhs


def dipole_rhs(mdl, om, c, p):
    """b for one dipole, leaving the model's own sources untouched."""
    je = mdl.je.copy()
    mdl.je[...] = 0
    M.add_srce(mdl, M_point(c, p))
    b = M.create_b(mdl, om)
    mdl.je[...] = je
    return b
