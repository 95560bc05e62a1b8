"""GPU solver parity: x = A \\ b against the oracle (sparse direct solve in
complex128), in both precisions and both Krylov methods.

Tolerances: the true relative residual ‖b − A x‖/‖b‖, recomputed here with
the oracle's sparse A, must meet the requested tol; the field error against
the direct solve must be ≤ 1e-5 (relative 2-norm) at tol = 1e-7.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu


def _system(O, N=(16, 14, 12), spheres=True):
    g = O.uniform_grid(N)
    objs = [O.Sphere((8.2, 7.1, 6.3), 3.1, 6.0)] if spheres else []
    S = O.System(g, 2 * np.pi / 7.0, ((3, 3, 3), (3, 3, 3)), objs)
    S.add_pointsrc((7.6, 6.5, 6.0), (0.3, 0.2, 1.0))
    return S


def _op(pkg, S):
    A = pkg.FDFDOperator(S.grid.N, S.omega, S.sdl_e, S.sdl_m)
    A.set_eps(S.eps_diag, S.eps_off)
    return A


@pytest.fixture(scope="module")
def sysx(oracle):
    S = _system(oracle)
    b = S.b()
    xd = spla.spsolve(S.A.tocsc(), b)
    return S, b, xd


@pytest.mark.parametrize("precision,method", [("fp64", "bicgstab"), ("mixed", "bicgstab"), ("fp64", "cocg"),
                                              ("fp64", "bicgstabl"), ("mixed", "bicgstabl")])
def test_solve_matches_direct(pkg, sysx, precision, method):
    S, b, xd = sysx
    A = _op(pkg, S)
    tol = 1e-7
    x, st = A.solve(b, tol=tol, precision=precision, method=method)
    rel = np.linalg.norm(b - S.A @ x) / np.linalg.norm(b)
    assert rel <= tol * 1.01, (rel, st)
    assert abs(st[0]["relres"] - rel) < 1e-9 + 0.05 * rel
    ferr = np.linalg.norm(x - xd) / np.linalg.norm(xd)
    assert ferr < 1e-5, (ferr, st)
    if precision == "mixed":
        assert st[0]["refinements"] >= 1
    A.close()


def test_transpose_solve(pkg, sysx):
    S, b, _ = sysx
    A = _op(pkg, S)
    x, st = A.solve(b, tol=1e-8, precision="mixed", transpose=True)
    rel = np.linalg.norm(b - S.A.T @ x) / np.linalg.norm(b)
    assert rel <= 1e-8 * 1.01, (rel, st)
    A.close()


def test_multiple_rhs_and_x0(pkg, oracle, sysx):
    S, b, xd = sysx
    A = _op(pkg, S)
    b2 = np.stack([b, 2j * b, np.roll(b, 7)])
    x, st = A.solve(b2, tol=1e-7, precision="mixed")
    for q in range(3):
        rel = np.linalg.norm(b2[q] - S.A @ x[q]) / np.linalg.norm(b2[q])
        assert rel <= 1.01e-7, (q, rel)
    assert np.allclose(x[1], 2j * x[0], rtol=0, atol=1e-5 * np.abs(x[0]).max())
    # warm start from the converged answer: no iteration needed
    x3, st3 = A.solve(b, tol=1e-6, precision="mixed", x0=xd)
    assert st3[0]["iterations"] == 0
    A.close()


def test_zero_rhs_and_maxit(pkg, sysx):
    S, b, _ = sysx
    A = _op(pkg, S)
    x, st = A.solve(np.zeros_like(b), precision="mixed")
    assert np.all(x == 0) and st[0]["status"] == 0
    with pytest.raises(pkg.FDFDError) as ei:
        A.solve(b, tol=1e-12, precision="mixed", maxit=3, check_every=1)
    assert ei.value.code == 5
    assert ei.value.stats[0]["iterations"] >= 3
    A.close()


def test_graph_and_plain_agree(pkg, sysx):
    """The CUDA-graph replay and direct launches run the same recurrence."""
    S, b, _ = sysx
    A = _op(pkg, S)
    x1, s1 = A.solve(b, tol=1e-6, precision="fp64", use_graph=True, check_every=10)
    x2, s2 = A.solve(b, tol=1e-6, precision="fp64", use_graph=False, check_every=10)
    assert s1[0]["iterations"] == s2[0]["iterations"]
    assert np.array_equal(x1, x2)
    A.close()


def test_unsupported_cocg_forms_rejected(pkg, sysx):
    S, b, _ = sysx
    A = _op(pkg, S)
    for kw in ({"precision": "fp64", "transpose": True}, {"precision": "mixed"}):
        with pytest.raises(pkg.FDFDError) as ei:
            A.solve(b, method="cocg", **kw)
        assert ei.value.code == 2
    A.close()


@pytest.mark.parametrize("ell", [1, 2, 3, 4])
def test_bicgstabl_degrees(pkg, sysx, ell):
    """BiCGStab(ℓ) for every supported ℓ, mixed precision with reliable
    updates, transposed as well (the adjoint path)."""
    S, b, xd = sysx
    A = _op(pkg, S)
    for tr in (False, True):
        x, st = A.solve(b, tol=1e-8, precision="mixed", method="bicgstabl", ell=ell, transpose=tr)
        M = S.A.T if tr else S.A
        rel = np.linalg.norm(b - M @ x) / np.linalg.norm(b)
        assert rel <= 1e-8 * 1.01, (ell, tr, rel, st)
        assert st[0]["matvecs"] >= 2 * ell
    A.close()
