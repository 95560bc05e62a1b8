"""The H-field formulation (ft = HH: A = Cₑ (Pε \\ Cₘ) − ω² Pμ, Pμ = I,
src/model/model.jl:238-240, 266-268) on the GPU against the oracle's
assembly, and against the E formulation: the H solve must reproduce
h_from_e of the E solve (both describe the same field)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu

CASES = [((15, 13, 11), (False, False, False), (0, 0, 0)), ((12, 14, 10), (True, False, True), (0.21, 0, -0.17))]


def _setup(pkg, O, N, bloch, kb, diag_only=True):
    g = O.Grid(tuple(np.arange(n + 1, dtype=float) for n in N), bloch)
    om = 2 * np.pi / 6.5
    npml = tuple(tuple(0 if bloch[w] else 2 for w in range(3)) for _ in range(2))
    sdl_e, sdl_m = O.stretched_dl(g, om, npml)
    rng = np.random.default_rng(17)
    eps = rng.uniform(1.0, 6.0, tuple(N) + (3,))
    Ce, Cm = O.create_curls(g, sdl_e, sdl_m, kb)
    ph = [np.exp(-1j * kb[w] * g.L[w]) for w in range(3)]
    A = pkg.FDFDOperator(N, om, sdl_e, sdl_m, bloch, ph)
    A.set_eps(eps)
    return g, om, eps, Ce, Cm, A


@pytest.mark.parametrize("N,bloch,kb", CASES)
def test_hh_operator(pkg, oracle, N, bloch, kb):
    O = oracle
    g, om, eps, Ce, Cm, A = _setup(pkg, O, N, bloch, kb)
    ev = O.field_to_vec(eps)
    Ahh = O.create_A_hh(om, ev, Ce, Cm)
    A.set_field_type("H")
    rng = np.random.default_rng(3)
    x = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    ref = Ahh @ x
    for prec, tol in (("c128", 1e-12), ("c64", 1e-5)):
        y = A.matvec(x, prec)
        assert np.max(np.abs(y - ref)) <= tol * np.max(np.abs(ref)), prec
    A.close()


def test_hh_solve_matches_e_solve(pkg, oracle):
    O = oracle
    N, bloch, kb = CASES[0]
    g, om, eps, Ce, Cm, A = _setup(pkg, O, N, bloch, kb)
    je = np.zeros(tuple(N) + (3,), complex)
    je[7, 6, 5, 2] = 1.0
    je[5, 8, 4, 0] = 0.5j
    jv = O.field_to_vec(je)
    b_e = -1j * om * jv
    e, st_e = A.solve(b_e, tol=1e-10, precision="fp64")
    h_ref = A.h_from_e(e)
    ev = O.field_to_vec(eps)
    b_h = O.create_b_hh(om, ev, Ce, jv)
    A.set_field_type("H")
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        h, st = A.solve(b_h, tol=tol, precision=prec)
        Ahh = O.create_A_hh(om, ev, Ce, Cm)
        assert np.linalg.norm(b_h - Ahh @ h) / np.linalg.norm(b_h) <= 1.01 * tol, (prec, st)
        assert np.linalg.norm(h - h_ref) / np.linalg.norm(h_ref) < 1e-5, prec
    with pytest.raises(pkg.FDFDError):
        A.solve(b_h, tol=1e-6, transpose=True)
    A.close()


def test_hh_rejects_offdiagonal(pkg, oracle):
    O = oracle
    g = O.uniform_grid((10, 9, 8))
    S = O.System(g, 1.0, ((2, 2, 2), (2, 2, 2)), [O.Sphere((5.1, 4.3, 3.9), 2.4, 6.0)])
    A = pkg.FDFDOperator(g.N, 1.0, S.sdl_e, S.sdl_m)
    A.set_eps(S.eps_diag, S.eps_off)
    with pytest.raises(pkg.FDFDError):
        A.set_field_type("H")
    A.close()
