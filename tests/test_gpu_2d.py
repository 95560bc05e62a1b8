"""2D TE/TM models on the GPU (the z-invariant slice of the 3D operator)
against the oracle's slice blocks: disks and rectangles smoothed on the
device (masks bit-exact), operator ≤ 1e-12 in complex128 on the slice's
compact vectors, solves to the requested residual."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = (40, 36)
OMEGA = 2 * np.pi / 9.0


def _models(pkg, O, kind):
    M = pkg.ModelTE if kind == "TE" else pkg.ModelTM
    mdl = M(pkg.uniform_lprim2d(N))
    pkg.set_ωpml(mdl, OMEGA)
    pkg.set_Npml(mdl, ((6, 6), (6, 6)))
    specs = [("d", (14.3, 17.2), 5.1, 12.25), ("r", (22.0, 8.5), (31.5, 14.0), 4.0), ("d", (27.6, 24.9), 3.7, 2.25)]
    oo = []
    for sp in specs:
        if sp[0] == "d":
            pkg.add_obj(mdl, "m", pkg.Disk(sp[1], sp[2]), ε=sp[3])
            oo.append(O.CylinderZ(sp[1], sp[2], sp[3]))
        else:
            pkg.add_obj(mdl, "m", pkg.Rect(sp[1], sp[2]), ε=sp[3])
            oo.append(O.Box((sp[1][0], sp[1][1], -1e300), (sp[2][0], sp[2][1], 1e300), sp[3]))
    S = O.System(O.Grid(mdl.grid.lprim, mdl.grid.isbloch), OMEGA, mdl.Npml, oo)
    return mdl, S


def _block(S, comps):
    nc = S.grid.ncell
    idx = np.concatenate([[c + 3 * q for c in comps] for q in range(nc)]).astype(int)
    return S.A.tocsr()[idx][:, idx]


@pytest.mark.parametrize("kind", ["TE", "TM"])
def test_2d_operator_and_smoothing(pkg, oracle, kind):
    mdl, S = _models(pkg, oracle, kind)
    A = pkg.create_A(mdl, OMEGA)
    ed, eo, sm = A.get_eps()
    assert np.array_equal(sm, S.debug["smask"])
    assert np.max(np.abs(ed - S.eps_diag)) < 1e-12 and np.max(np.abs(eo - S.eps_off)) < 1e-12
    comps = mdl.comps
    B = _block(S, comps)
    rng = np.random.default_rng(9)
    x = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    y = A @ x
    ref = B @ x
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
    yt = A.rmatvec_transpose(x)
    assert np.max(np.abs(yt - B.T @ x)) <= 1e-12 * np.max(np.abs(ref))
    A.close()


@pytest.mark.parametrize("kind,prec", [("TE", "mixed"), ("TM", "mixed"), ("TE", "fp64")])
def test_2d_solve(pkg, oracle, kind, prec):
    mdl, S = _models(pkg, oracle, kind)
    comps = mdl.comps
    mdl.je[8, 18, 0, comps[-1]] = 1.0
    b = pkg.create_b(mdl, OMEGA)
    A = pkg.create_A(mdl, OMEGA)
    x, st = A.solve(b, tol=1e-8, precision=prec)
    B = _block(S, comps)
    rel = np.linalg.norm(b - B @ x) / np.linalg.norm(b)
    assert rel <= 1.01e-8, (rel, st)
    A.close()
