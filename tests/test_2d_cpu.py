"""2D TE/TM models as the z-invariant slice of the 3D operator, pinned on
the CPU: with one periodic cell along z the oracle's 3D operator splits
exactly into the TE block (Ex, Ey; Hz) and the TM block (Ez; Hx, Hy), and
each block equals the 2D Yee formulas of ModelTE/ModelTM (src/model/te.jl,
tm.jl) written out directly here."""
import numpy as np


def _slice_grid(O, N, bloch=(False, False)):
    lp = (np.arange(N[0] + 1, dtype=float), np.arange(N[1] + 1, dtype=float), np.array([0.0, 1.0]))
    return O.Grid(lp, (bloch[0], bloch[1], True))


def _system(O, N=(14, 12), eps=None, om=2 * np.pi / 7.0):
    g = _slice_grid(O, N)
    npml = ((3, 3, 0), (3, 3, 0))
    sdl_e, sdl_m = O.stretched_dl(g, om, npml)
    Ce, Cm = O.create_curls(g, sdl_e, sdl_m)
    P = O.create_paramop(g, eps, None, sdl_e, sdl_m)
    return g, O.create_A(om, P, Ce, Cm), sdl_e, sdl_m, om


def _idx(N, comps):
    cells = np.arange(N[0] * N[1])
    return np.concatenate([[c + 3 * q for c in comps] for q in cells]).astype(int)


def test_slice_decouples(oracle):
    rng = np.random.default_rng(1)
    N = (14, 12)
    eps = rng.uniform(1, 4, (N[0], N[1], 1, 3))
    g, A, *_ = _system(oracle, N, eps)
    A = A.tocsr()
    te, tm = _idx(N, (0, 1)), _idx(N, (2,))
    assert A[te][:, tm].count_nonzero() == 0
    assert A[tm][:, te].count_nonzero() == 0


def test_tm_block_is_2d_formula(oracle):
    rng = np.random.default_rng(2)
    N = (14, 12)
    eps = rng.uniform(1, 4, (N[0], N[1], 1, 3))
    g, A, se, sm, om = _system(oracle, N, eps)
    tm = _idx(N, (2,))
    Atm = A.tocsr()[tm][:, tm]
    e = rng.standard_normal(N) + 1j * rng.standard_normal(N)   # Ez[i, j]
    # curl E → H with pinned Ez (i = 0 or j = 0) and the PEC ghost Ez(N) = 0
    ez = e.copy()
    ez[0, :] = 0
    ez[:, 0] = 0
    ezp = np.zeros((N[0] + 1, N[1] + 1), complex)
    ezp[:N[0], :N[1]] = ez
    cmx, cmy, cex, cey = 1 / sm[0], 1 / sm[1], 1 / se[0], 1 / se[1]
    hx = cmy[None, :] * (ezp[:N[0], 1:] - ezp[:N[0], :N[1]])
    hy = -cmx[:, None] * (ezp[1:, :N[1]] - ezp[:N[0], :N[1]])
    # backward differences with the mirrored ghost H(−1) = H(0)
    hym = np.concatenate([hy[:1], hy[:-1]], axis=0)
    hxm = np.concatenate([hx[:, :1], hx[:, :-1]], axis=1)
    y = cex[:, None] * (hy - hym) - cey[None, :] * (hx - hxm)
    y[0, :] = 0
    y[:, 0] = 0
    y = y - om ** 2 * eps[:, :, 0, 2] * e
    got = (Atm @ np.ascontiguousarray(e.T).reshape(-1)).reshape(N[1], N[0]).T
    assert np.max(np.abs(got - y)) <= 1e-12 * np.max(np.abs(y))


def test_te_block_is_2d_formula(oracle):
    rng = np.random.default_rng(3)
    N = (14, 12)
    eps = rng.uniform(1, 4, (N[0], N[1], 1, 3))
    g, A, se, sm, om = _system(oracle, N, eps)
    te = _idx(N, (0, 1))
    Ate = A.tocsr()[te][:, te]
    ex = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    ey = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    exc, eyc = ex.copy(), ey.copy()
    exc[:, 0] = 0          # Ex tangential on the y = 0 wall: pinned
    eyc[0, :] = 0          # Ey tangential on the x = 0 wall: pinned
    exp_ = np.zeros((N[0], N[1] + 1), complex)
    exp_[:, :N[1]] = exc
    eyp = np.zeros((N[0] + 1, N[1]), complex)
    eyp[:N[0], :] = eyc
    cmx, cmy, cex, cey = 1 / sm[0], 1 / sm[1], 1 / se[0], 1 / se[1]
    hz = cmx[:, None] * (eyp[1:, :] - eyp[:N[0], :]) - cmy[None, :] * (exp_[:, 1:] - exp_[:, :N[1]])
    hzx = np.concatenate([hz[:1], hz[:-1]], axis=0)
    hzy = np.concatenate([hz[:, :1], hz[:, :-1]], axis=1)
    yx = cey[None, :] * (hz - hzy)
    yy = -cex[:, None] * (hz - hzx)
    yx[:, 0] = 0
    yy[0, :] = 0
    yx = yx - om ** 2 * eps[:, :, 0, 0] * ex
    yy = yy - om ** 2 * eps[:, :, 0, 1] * ey
    v = np.stack([ex, ey], axis=-1)
    got = (Ate @ np.ascontiguousarray(np.transpose(v, (1, 0, 2))).reshape(-1)).reshape(N[1], N[0], 2)
    got = np.transpose(got, (1, 0, 2))
    ref = np.stack([yx, yy], axis=-1)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
