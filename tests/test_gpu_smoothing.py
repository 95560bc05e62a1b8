"""On-device assignment + Kottke smoothing against the oracle
(calc_matparams!, src/model/full.jl:16-70, conventions A4-A7).

Smoothing masks (which samples were Kottke-smoothed or design-controlled)
must be bit-identical; ε values within 1e-12 absolute (ε ≤ 12.25).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _objs(pkg, O, specs):
    """specs: ("s", c, r, eps) | ("b", lo, hi, eps) → (package objects, oracle objects)."""
    po, oo = [], []
    for sp in specs:
        if sp[0] == "s":
            po.append(pkg.model._Obj("m", pkg.Sphere(sp[1], sp[2]), sp[3]))
            oo.append(O.Sphere(sp[1], sp[2], sp[3]))
        else:
            po.append(pkg.model._Obj("m", pkg.Box(sp[1], sp[2]), sp[3]))
            oo.append(O.Box(sp[1], sp[2], sp[3]))
    return po, oo


def _run(pkg, O, grid, specs, eps_bg=1.0, design=None, omega=0.7, npml=((2, 2, 2), (2, 2, 2))):
    po, oo = _objs(pkg, O, specs)
    sdl_e, sdl_m = O.stretched_dl(grid, omega, npml)
    A = pkg.FDFDOperator(grid.N, omega, sdl_e, sdl_m, grid.isbloch)
    pd = None if design is None else pkg.DesignRegion(design.lo, design.hi, design.eps)
    A.smooth_objects(grid.lprim_full, po, eps_bg, pd)
    ed, eo, sm = A.get_eps()
    red, reo, dbg = O.assign_smooth(grid, oo, eps_bg, design, return_debug=True)
    return A, (ed, eo, sm), (red, reo, dbg["smask"]), sdl_e, sdl_m


def _check(got, ref):
    ed, eo, sm = got
    red, reo, rsm = ref
    assert np.array_equal(sm, rsm), np.argwhere(sm != rsm)[:10]
    assert np.max(np.abs(ed - red)) < 1e-12
    assert np.max(np.abs(eo - reo)) < 1e-12


def test_spheres_uniform(pkg, oracle):
    O = oracle
    g = O.uniform_grid((24, 22, 20))
    specs = [("s", (8.3, 9.1, 7.7), 4.2, 12.25), ("s", (15.6, 12.2, 11.9), 3.4, 2.25),
             ("s", (16.0, 11.0, 12.0), 2.0, 6.0)]          # overlaps the second: last wins
    A, got, ref, *_ = _run(pkg, O, g, specs)
    _check(got, ref)
    assert got[2][..., :3].sum() > 0 and got[2][..., 3].sum() > 0
    A.close()


def test_lattice_aligned_spheres(pkg, oracle):
    """Integer centres and radii: exact ties on the surface and normals with
    zero components (degenerate plane/voxel cuts)."""
    O = oracle
    g = O.uniform_grid((20, 20, 20))
    specs = [("s", (10.0, 10.0, 10.0), 5.0, 12.25), ("s", (4.5, 4.5, 15.0), 2.0, 4.0)]
    A, got, ref, *_ = _run(pkg, O, g, specs)
    _check(got, ref)
    A.close()


def test_nonuniform_spheres_and_box(pkg, oracle):
    O = oracle
    rng = np.random.default_rng(5)
    lp = tuple(np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, n))]) for n in (21, 18, 16))
    g = O.Grid(lp, (False, False, False))
    specs = [("b", (3.3, 2.1, 4.05), (14.2, 9.9, 8.8), 4.0), ("s", (9.0, 8.0, 7.0), 3.3, 12.25)]
    A, got, ref, *_ = _run(pkg, O, g, specs, eps_bg=1.5)
    _check(got, ref)
    A.close()


def test_bloch_axes(pkg, oracle):
    O = oracle
    g = O.uniform_grid((16, 14, 12), isbloch=(True, False, True))
    specs = [("s", (1.2, 7.0, 6.0), 3.1, 12.25), ("s", (10.0, 6.5, 11.4), 2.5, 2.25)]  # wrap in x and z
    A, got, ref, *_ = _run(pkg, O, g, specs, npml=((0, 2, 0), (0, 2, 0)))
    _check(got, ref)
    A.close()


def test_slab_with_design_region(pkg, oracle):
    O = oracle
    g = O.uniform_grid((32, 28, 20))
    rng = np.random.default_rng(4)
    design = O.DesignRegion((10, 8, 6), (20, 18, 13), rng.uniform(1.0, 12.25, (10, 10, 7)))
    specs = [("b", (-1.0, -1.0, 8.0), (33.0, 29.0, 12.0), 12.25)]
    A, got, ref, *_ = _run(pkg, O, g, specs, design=design)
    _check(got, ref)
    assert (got[2][..., :3] == 2).sum() > 0
    A.close()


def test_smoothed_operator_matches_oracle(pkg, oracle):
    """Full pipeline: GPU-smoothed ε → GPU matvec vs oracle assembly."""
    O = oracle
    g = O.uniform_grid((26, 24, 22))
    specs = [("s", (12.3, 11.1, 10.7), 5.2, 12.25), ("s", (6.0, 6.0, 15.0), 2.4, 2.25)]
    om = 2 * np.pi / 9
    npml = ((4, 4, 4), (4, 4, 4))
    A, got, ref, sdl_e, sdl_m = _run(pkg, O, g, specs, omega=om, npml=npml)
    _check(got, ref)
    S = O.System(g, om, npml, _objs(pkg, O, specs)[1])
    rng = np.random.default_rng(1)
    x = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    y = A @ x
    yr = S.A @ x
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < 1e-12
    A.close()
