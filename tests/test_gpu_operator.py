"""GPU operator parity: y = A x from libfdfd_gb300 against the oracle's
assembled sparse A (the reference's create_A composition,
src/model/model.jl:235-237), on seeded inputs.

Tolerances: complex128 path ≤ 1e-12 relative (2-norm over the vector);
complex64 path ≤ 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def _nonuniform(N, seed):
    rng = np.random.default_rng(seed)
    return tuple(np.concatenate([[0.0], np.cumsum(rng.uniform(0.6, 1.4, n))]) for n in N)


def _case(O, kind):
    if kind == "vacuum8":
        g = O.uniform_grid((8, 8, 8))
        return O.System(g, 2 * np.pi / 5, ((2, 2, 2), (2, 2, 2))), {}
    if kind == "spheres_odd":
        g = O.Grid(_nonuniform((13, 10, 9), 1), (False, False, False))
        objs = [O.Sphere((6.1, 4.8, 4.4), 2.7, 12.25), O.Sphere((9.5, 6.0, 3.0), 1.6, 2.25)]
        return O.System(g, 2 * np.pi / 7, ((3, 2, 1), (1, 2, 3)), objs), {}
    if kind == "ragged":
        g = O.uniform_grid((37, 11, 5))
        objs = [O.Box((10.3, 2.2, 1.1), (25.7, 8.6, 3.9), 4.0)]
        return O.System(g, 2 * np.pi / 9, ((4, 0, 0), (3, 2, 1)), objs), {}
    if kind == "chunks":
        g = O.uniform_grid((40, 24, 70))
        objs = [O.Sphere((20.0, 12.0, 30.0), 6.3, 12.25), O.Sphere((12.0, 8.0, 50.0), 4.1, 2.25)]
        return O.System(g, 2 * np.pi / 10, ((5, 5, 5), (5, 5, 5)), objs), {}
    if kind == "bloch0":
        g = O.uniform_grid((9, 7, 6), isbloch=(True, True, True))
        objs = [O.Sphere((4.4, 3.1, 2.9), 2.2, 6.0)]
        return O.System(g, 2 * np.pi / 5, ((0, 0, 0), (0, 0, 0)), objs), {}
    if kind == "blochk":
        g = O.uniform_grid((10, 8, 6), isbloch=(True, False, True))
        objs = [O.Sphere((5.2, 4.1, 3.0), 2.0, 6.0)]
        k = (0.37, 0.0, -0.21)
        return O.System(g, 2 * np.pi / 5, ((0, 2, 0), (0, 2, 0)), objs, kbloch=k), {"kbloch": k}
    raise KeyError(kind)


def _make_op(pkg, S, kbloch=(0.0, 0.0, 0.0)):
    g = S.grid
    ph = tuple(np.exp(-1j * kbloch[w] * g.L[w]) for w in range(3))
    A = pkg.FDFDOperator(g.N, S.omega, S.sdl_e, S.sdl_m, g.isbloch, ph)
    A.set_eps(S.eps_diag, S.eps_off)
    return A


CASES = ["vacuum8", "spheres_odd", "ragged", "chunks", "bloch0", "blochk"]


@pytest.mark.parametrize("kind", CASES)
def test_matvec_parity(pkg, oracle, kind):
    S, kw = _case(oracle, kind)
    A = _make_op(pkg, S, **kw)
    x = _rand(A.n, 11)
    y_ref = S.A @ x
    y = A @ x
    err = np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)
    assert err < TOL64, err
    y32 = A.matvec(x, precision="c64")
    err32 = np.linalg.norm(y32 - y_ref) / np.linalg.norm(y_ref)
    assert err32 < TOL32, err32
    A.close()


@pytest.mark.parametrize("kind", ["vacuum8", "spheres_odd", "ragged", "bloch0"])
def test_transpose_parity(pkg, oracle, kind):
    S, kw = _case(oracle, kind)
    A = _make_op(pkg, S, **kw)
    x = _rand(A.n, 5)
    y_ref = S.A.T @ x
    y = A.T @ x
    err = np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)
    assert err < TOL64, err
    A.close()


@pytest.mark.parametrize("N", [(11, 9, 12), (12, 9, 12), (66, 17, 20)])
def test_random_tensor_everywhere(pkg, oracle, N):
    """Arbitrary ε diagonal and off-diagonal on every cell (walls included).
    Odd Nx runs the plain-load kernel, even Nx the TMA kernel."""
    O = oracle
    g = O.uniform_grid(N)
    sdl_e, sdl_m = O.stretched_dl(g, 2 * np.pi / 6, ((2, 3, 1), (2, 1, 3)))
    rng = np.random.default_rng(3)
    ed = rng.uniform(1.0, 12.0, N + (3,))
    eo = rng.uniform(-2.0, 2.0, N + (3,))
    Ce, Cm = O.create_curls(g, sdl_e, sdl_m)
    P = O.create_paramop(g, ed, eo, sdl_e, sdl_m)
    om = 2 * np.pi / 6
    Aref = O.create_A(om, P, Ce, Cm)
    A = pkg.FDFDOperator(g.N, om, sdl_e, sdl_m)
    A.set_eps(ed, eo)
    x = _rand(A.n, 9)
    y = A @ x
    err = np.linalg.norm(y - Aref @ x) / np.linalg.norm(Aref @ x)
    assert err < TOL64, err
    A.close()


def test_unit_vectors_index_map(pkg, oracle):
    """Bit-exact DOF index map: A e_q has non-zeros exactly where column q of
    the oracle's A does."""
    S, _ = _case(oracle, "spheres_odd")
    A = _make_op(pkg, S)
    rng = np.random.default_rng(0)
    Acsc = S.A.tocsc()
    for q in rng.choice(A.n, 12, replace=False):
        e = np.zeros(A.n, complex)
        e[q] = 1.0
        y = A @ e
        col = Acsc[:, q].toarray().ravel()
        assert np.array_equal(np.flatnonzero(np.abs(y) > 0), np.flatnonzero(np.abs(col) > 0)), q
        assert np.allclose(y, col, rtol=1e-13, atol=1e-14)
    A.close()


def test_eps_tensor_layout(pkg, oracle):
    """fdfd_set_eps_tensor reads the reference's (Nx,Ny,Nz,3,3) εarr."""
    S, _ = _case(oracle, "spheres_odd")
    g = S.grid
    epsarr = np.zeros(g.N + (3, 3), complex)
    for c in range(3):
        epsarr[..., c, c] = S.eps_diag[..., c]
    for p, (r, c) in enumerate(((0, 1), (1, 2), (2, 0))):
        epsarr[..., r, c] = S.eps_off[..., p]
        epsarr[..., c, r] = S.eps_off[..., p]
    A = pkg.FDFDOperator(g.N, S.omega, S.sdl_e, S.sdl_m)
    A.set_eps_tensor(epsarr)
    ed, eo, _ = A.get_eps()
    assert np.array_equal(ed, S.eps_diag) and np.array_equal(eo, S.eps_off)
    x = _rand(A.n, 2)
    assert np.linalg.norm(A @ x - S.A @ x) / np.linalg.norm(S.A @ x) < TOL64
    bad = epsarr.copy()
    bad[1, 1, 1, 0, 1] += 0.5
    with pytest.raises(pkg.FDFDError):
        A.set_eps_tensor(bad)
    A.close()


def test_residual_dev(pkg, oracle):
    """fdfd_residual_dev: r = b − A x and ‖r‖² in FP64 on device buffers."""
    torch = pytest.importorskip("torch")
    S, _ = _case(oracle, "spheres_odd")
    A = _make_op(pkg, S)
    x = _rand(A.n, 21)
    b = _rand(A.n, 22)
    dev = torch.device("cuda", 0)
    xd = torch.from_numpy(x.view(np.float64).reshape(-1, 2)).to(dev)
    bd = torch.from_numpy(b.view(np.float64).reshape(-1, 2)).to(dev)
    rd = torch.empty_like(xd)
    rr = A.residual_dev(xd.data_ptr(), bd.data_ptr(), rd.data_ptr())
    r_ref = b - S.A @ x
    r = rd.cpu().numpy().view(np.complex128).reshape(-1)
    assert np.linalg.norm(r - r_ref) / np.linalg.norm(r_ref) < TOL64
    assert abs(rr - np.vdot(r_ref, r_ref).real) / np.vdot(r_ref, r_ref).real < 1e-12
    A.close()


@pytest.mark.parametrize("kind", ["vacuum8", "chunks"])
@pytest.mark.parametrize("variant", ["0", "4"])
def test_tma_and_plain_kernels_agree(pkg, oracle, kind, variant, monkeypatch):
    """The first TMA kernel (variant 0) and the plain-load kernel run the same
    arithmetic: outputs are bitwise equal in both precisions.  The second TMA
    kernel (variant 4) sums the two corner terms of an off-diagonal output in
    another order: equal to 1e-15 (complex128) and 1e-6 (complex64) relative."""
    S, _ = _case(oracle, kind)
    monkeypatch.setenv("FDFD_OPERATOR_V2", variant)
    A1 = _make_op(pkg, S)
    monkeypatch.setenv("FDFD_DISABLE_TMA", "1")
    A2 = _make_op(pkg, S)
    x = _rand(A1.n, 31)
    if variant == "0":
        assert np.array_equal(A1 @ x, A2 @ x)
        assert np.array_equal(A1.matvec(x, "c64"), A2.matvec(x, "c64"))
    else:
        y1, y2 = A1 @ x, A2 @ x
        assert np.linalg.norm(y1 - y2) <= 1e-15 * np.linalg.norm(y2)
        y1, y2 = A1.matvec(x, "c64"), A2.matvec(x, "c64")
        assert np.linalg.norm(y1 - y2) <= 1e-6 * np.linalg.norm(y2)
    A1.close()
    A2.close()


@pytest.mark.parametrize("kc", [1, 2, 3, 5])
@pytest.mark.parametrize("kernel", ["tma2", "tma2_1row", "tma2_3slot", "tma1", "plain"])
def test_forced_z_chunks(pkg, oracle, monkeypatch, kc, kernel):
    """Every z-chunk length gives the oracle's A x in every operator kernel
    (the second TMA kernel in its layouts, the first TMA kernel, plain
    loads), on a grid of several x-y tiles so that interior CTAs start at
    planes 1, 2, … and must zero the z = 0 wall's pinned E themselves."""
    tma = kernel != "plain"
    monkeypatch.setenv("FDFD_OPERATOR_V2", {"tma2": "4", "tma2_1row": "1", "tma2_3slot": "2"}.get(kernel, "0"))
    g = oracle.uniform_grid((64, 48, 13))
    objs = [oracle.Sphere((30.2, 22.1, 6.3), 5.1, 12.25)]
    S = oracle.System(g, 2 * np.pi / 12, ((4, 4, 3), (4, 4, 3)), objs)
    monkeypatch.setenv("FDFD_KCHUNK", str(kc))
    monkeypatch.setenv("FDFD_DISABLE_TMA", "0" if tma else "1")
    A = _make_op(pkg, S)
    x = _rand(A.n, 29)
    ref = S.A @ x
    assert np.linalg.norm(A.matvec(x, "c128") - ref) / np.linalg.norm(ref) <= TOL64
    assert np.linalg.norm(A.matvec(x, "c64") - ref) / np.linalg.norm(ref) <= TOL32
    A.close()


@pytest.mark.parametrize("waves", [1, 2, 4])
@pytest.mark.parametrize("kernel", ["tma2", "tma2_1row"])
def test_balanced_schedules(pkg, oracle, monkeypatch, waves, kernel):
    """The second TMA kernel on a balanced z-chunk schedule (columns cut at
    even estimated cost, planes with off-diagonal terms weighing more,
    heaviest chunk first) gives the oracle's A x, and a mixed-precision solve
    through it (reducing epilogues on a one-dimensional grid of schedule
    entries) meets its tolerance on the oracle's matrix."""
    monkeypatch.setenv("FDFD_OPERATOR_V2", {"tma2": "4", "tma2_1row": "1"}[kernel])
    monkeypatch.setenv("FDFD_SCHEDULE", str(waves))
    g = oracle.uniform_grid((64, 48, 70))
    objs = [oracle.Sphere((20.0, 12.0, 30.0), 6.3, 12.25), oracle.Sphere((44.0, 30.0, 52.0), 4.1, 2.25)]
    S = oracle.System(g, 2 * np.pi / 10, ((5, 5, 5), (5, 5, 5)), objs)
    S.add_pointsrc((31.0, 23.0, 35.0), (0, 0, 1))
    A = _make_op(pkg, S)
    x = _rand(A.n, 31)
    ref = S.A @ x
    assert np.linalg.norm(A.matvec(x, "c128") - ref) / np.linalg.norm(ref) <= TOL64
    assert np.linalg.norm(A.matvec(x, "c64") - ref) / np.linalg.norm(ref) <= TOL32
    b = S.b()
    xs, st = A.solve(b, tol=1e-7, precision="mixed")
    assert st[0]["status"] == 0
    assert np.linalg.norm(b - S.A @ xs) / np.linalg.norm(b) <= 1.02e-7
    A.close()
