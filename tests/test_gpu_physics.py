"""Physics sanity of the GPU path on the vacuum dipole workload (32³, 10-cell
PML, λ = 20, z-directed point current at the centre): the FP64 solve meets
1e-10 on the oracle's own matrix, the field decays by more than three
orders through the PML, and the PML reflects less than 1e-6 — the solution
in the 12³ interior agrees with the solution on a 64³ domain (same source,
same PML) to better than 1e-6 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(pkg, O, N, tol=1e-12):
    g = O.uniform_grid((N,) * 3)
    om = 2 * np.pi / 20.0
    S = O.System(g, om, ((10,) * 3, (10,) * 3))
    c = N / 2
    S.add_pointsrc((c, c, c + 0.5), (0, 0, 1))
    b = S.b()
    A = pkg.FDFDOperator(g.N, om, S.sdl_e, S.sdl_m)
    x, st = A.solve(b, tol=tol, precision="fp64")
    A.close()
    return S, b, x, st[0]


def test_vacuum_dipole_config1(pkg, oracle):
    O = oracle
    S32, b32, x32, st = _solve(pkg, O, 32, tol=1e-10)
    rel = np.linalg.norm(b32 - S32.A @ x32) / np.linalg.norm(b32)
    assert rel <= 1.01e-10, (rel, st)


def test_pml_decay_and_reflection(pkg, oracle):
    O = oracle
    S32, _, x32, _ = _solve(pkg, O, 32)
    S64, _, x64, _ = _solve(pkg, O, 64)
    E32 = O.vec_to_field(x32, S32.grid.N)
    E64 = O.vec_to_field(x64, S64.grid.N)
    a = E32[10:22, 10:22, 10:22]
    ref = E64[26:38, 26:38, 26:38]
    refl = np.linalg.norm(a - ref) / np.linalg.norm(ref)
    assert refl < 1e-6, refl
    outer = np.concatenate([E32[:2].ravel(), E32[-2:].ravel(), E32[:, :2].ravel(), E32[:, -2:].ravel(),
                            E32[:, :, :2].ravel(), E32[:, :, -2:].ravel()])
    assert np.abs(outer).max() < 1e-3 * np.abs(a).max()
