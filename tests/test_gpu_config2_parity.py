"""Parity at the benchmarked size: the 96³ dielectric-sphere scatterer
(40 spheres r ~ U[3, 8], ε = 12.25, 10-cell PML, λ = 16, x-polarised current
sheet at z = 15) — the workload bench.py times — against the oracle's
assembled system (create_A / create_b, src/model/model.jl:225-246, 251-274,
after calc_matparams!, src/model/full.jl:16-70).

* smoothing masks bit-identical, ε within 1e-12 absolute;
* b within 1e-14 relative;
* A x: complex128 ≤ 1e-12, complex64 ≤ 1e-5 relative (2-norm);
* the mixed-precision BiCGStab(4) solution meets a true relative residual of
  1e-6 on the oracle's own matrix (2 % slack for the different summation
  order of the CPU product)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2(pkg, oracle):
    O = oracle
    mdl, om = pkg.workloads.config2()
    A = pkg.create_A(mdl, om)
    g = O.uniform_grid(mdl.grid.N)
    objs = [O.Sphere(o.shape.c, o.shape.r, o.eps) for o in mdl.objects]
    S = O.System(g, om, mdl.Npml, objs)
    S.add_planesrc(2, 15.0, (1, 0, 0))
    yield pkg, mdl, om, A, S
    A.close()


def test_config2_smoothing_bit_exact(c2):
    pkg, mdl, om, A, S = c2
    ed, eo, sm = A.get_eps()
    assert np.array_equal(sm, S.debug["smask"]), np.argwhere(sm != S.debug["smask"])[:10]
    assert np.max(np.abs(ed - np.real(S.eps_diag))) < 1e-12
    assert np.max(np.abs(eo - np.real(S.eps_off))) < 1e-12
    assert np.count_nonzero(sm[..., :3] == 1) > 0 and np.count_nonzero(eo) > 0


def test_config2_rhs_and_matvec(c2):
    pkg, mdl, om, A, S = c2
    b = pkg.create_b(mdl, om)
    bo = S.b()
    assert np.linalg.norm(b - bo) <= 1e-14 * np.linalg.norm(bo)
    rng = np.random.default_rng(96)
    x = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    ref = S.A @ x
    for prec, tol in (("c128", 1e-12), ("c64", 1e-5)):
        y = A.matvec(x, prec)
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) <= tol, prec


def test_config2_mixed_solve_on_oracle_matrix(c2):
    pkg, mdl, om, A, S = c2
    b = S.b()
    x, st = A.solve(b, tol=1e-6, precision="mixed")
    assert st[0]["status"] == 0 and st[0]["relres"] <= 1e-6
    rel = np.linalg.norm(b - S.A @ x) / np.linalg.norm(b)
    assert rel <= 1.02e-6, rel
