"""GPU adjoint ε-gradient against the oracle and against finite differences.

eps_grad solves Aᵀλ = g with the transposed BiCGSTAB and forms
2·Re(ω²·λ·e) on the device; design_grad chains it to the design cells.
Tolerances: ≤ 1e-8 relative to the oracle (direct solves) for an FP64
adjoint solve at tol 1e-12; the chain ≤ 1e-13 relative; the end-to-end
design gradient within 1e-4 of central differences with h = 1e-4·ε (the
finite-difference check of the inverse-design workload).
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu

N = (16, 14, 12)
LO, HI = (5, 4, 4), (11, 10, 8)
OMEGA = 2 * np.pi / 6.0
NPML = ((3, 3, 3), (3, 3, 3))


def _objective(F, e):
    s = np.vdot(F, e)
    return abs(s) ** 2, np.conj(s) * np.conj(F)


@pytest.fixture(scope="module")
def case(pkg, oracle):
    O = oracle
    rng = np.random.default_rng(21)
    g = O.uniform_grid(N)
    eps_cells = rng.uniform(1.0, 12.25, tuple(h - l for l, h in zip(LO, HI)))
    sph = ((4.2, 9.8, 6.1), 2.4, 6.0)
    S = O.System(g, OMEGA, NPML, [O.Sphere(*sph)], 1.0, O.DesignRegion(LO, HI, eps_cells))
    S.add_pointsrc((3.5, 7.0, 6.0), (0.0, 1.0, 0.2))
    b = S.b()
    F = np.zeros(b.size, complex)
    F[1::3] = rng.standard_normal(b.size // 3) * (np.arange(b.size // 3) % N[0] == 12)
    e = spla.spsolve(S.A.tocsc(), b)
    L0, gv = _objective(F, e)
    grad, _ = O.adjoint_eps_grad(S.A, OMEGA, e, gv)
    return dict(S=S, b=b, F=F, e=e, g=gv, grad=grad, eps_cells=eps_cells, sph=sph, grid=g)


def _op(pkg, c, eps_cells=None):
    S = c["S"]
    A = pkg.FDFDOperator(N, OMEGA, S.sdl_e, S.sdl_m)
    objs = [pkg.model._Obj("m", pkg.Sphere(c["sph"][0], c["sph"][1]), c["sph"][2])]
    ec = c["eps_cells"] if eps_cells is None else eps_cells
    A.smooth_objects(c["grid"].lprim_full, objs, 1.0, pkg.DesignRegion(LO, HI, ec))
    return A


def test_eps_grad_matches_oracle(pkg, case):
    A = _op(pkg, case)
    grad, st = A.eps_grad(case["e"], case["g"], tol=1e-12, precision="fp64")
    ref = case["grad"].reshape(N[2], N[1], N[0], 3).transpose(2, 1, 0, 3)
    err = np.max(np.abs(grad - ref)) / np.max(np.abs(ref))
    assert err < 1e-8, (err, st)
    assert st["status"] == 0 and st["relres"] <= 1e-12
    A.close()


def test_eps_grad_mixed_precision(pkg, case):
    A = _op(pkg, case)
    grad, st = A.eps_grad(case["e"], case["g"], tol=1e-7, precision="mixed")
    ref = case["grad"].reshape(N[2], N[1], N[0], 3).transpose(2, 1, 0, 3)
    err = np.linalg.norm(grad - ref) / np.linalg.norm(ref)
    assert err < 1e-5, (err, st)
    A.close()


def test_design_chain_matches_oracle(pkg, oracle, case):
    A = _op(pkg, case)
    rng = np.random.default_rng(22)
    gd = rng.standard_normal(N + (3,))
    got = A.design_grad(gd)
    ref = oracle.design_grad_chain(case["grid"], oracle.DesignRegion(LO, HI, case["eps_cells"]), gd)
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    A.close()


def test_design_chain_wall_and_errors(pkg, oracle):
    """Region on the low walls (clamped indices); no region → error."""
    O = oracle
    g = O.uniform_grid((9, 8, 7))
    sdl_e, sdl_m = O.stretched_dl(g, 0.9, ((2, 2, 2), (2, 2, 2)))
    A = pkg.FDFDOperator(g.N, 0.9, sdl_e, sdl_m)
    with pytest.raises(ValueError):
        A.design_grad(np.zeros(g.N + (3,)))
    z = np.zeros(3 * g.ncell)
    assert A._lib.fdfd_design_grad(A._h, z.ctypes.data_as(pkg._lib._dp), z.ctypes.data_as(pkg._lib._dp)) == 1
    lo, hi = (0, 0, 0), (4, 3, 7)
    ec = np.random.default_rng(3).uniform(1, 4, (4, 3, 7))
    A.smooth_objects(g.lprim_full, [], 1.0, pkg.DesignRegion(lo, hi, ec))
    gd = np.random.default_rng(4).standard_normal(g.N + (3,))
    ref = O.design_grad_chain(g, O.DesignRegion(lo, hi, ec), gd)
    assert np.max(np.abs(A.design_grad(gd) - ref)) <= 1e-13 * np.max(np.abs(ref))
    A.close()


def test_design_gradient_finite_differences(pkg, case):
    """Whole GPU pipeline: smoothing → solve → adjoint → chain, against
    central differences of the GPU objective with h = 1e-4·ε."""
    b, F = case["b"], case["F"]

    def objective(ec):
        A = _op(pkg, case, ec)
        e, _ = A.solve(b, tol=1e-12, precision="fp64")
        A.close()
        return _objective(F, e)

    A = _op(pkg, case)
    e, _ = A.solve(b, tol=1e-12, precision="fp64")
    L0, gv = _objective(F, e)
    grad, _ = A.eps_grad(e, gv, tol=1e-12, precision="fp64")
    dg = A.design_grad(grad)
    A.close()
    rng = np.random.default_rng(23)
    cells = [tuple(rng.integers(0, HI[a] - LO[a]) for a in range(3)) for _ in range(6)]
    for cidx in cells:
        vals = []
        for sgn in (+1, -1):
            ec = case["eps_cells"].copy()
            h = 1e-4 * ec[cidx]
            ec[cidx] += sgn * h
            vals.append(objective(ec)[0])
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - dg[cidx]) <= 1e-4 * abs(dg[cidx]) + 1e-9 * L0, (cidx, fd, dg[cidx])
