"""Field post-processing on the GPU against the oracle: h_from_e
(src/model/model.jl:276-279) and the create_Mcs corner means (:287-306),
on PEC and Bloch grids with SC-PML, ≤ 1e-12 relative (FP64 both sides).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(O, bloch):
    rng = np.random.default_rng(31)
    lp = tuple(np.concatenate([[0.0], np.cumsum(rng.uniform(0.6, 1.4, n))]) for n in (13, 11, 9))
    return O.Grid(lp, bloch)


CASES = [((False, False, False), (0.0, 0.0, 0.0)), ((True, False, True), (0.13, 0.0, -0.21))]


@pytest.mark.parametrize("bloch,kb", CASES)
def test_h_from_e(pkg, oracle, bloch, kb):
    O = oracle
    g = _grid(O, bloch)
    om = 2 * np.pi / 6.5
    npml = ((0 if bloch[0] else 2, 2, 0 if bloch[2] else 2), (0 if bloch[0] else 2, 2, 0 if bloch[2] else 2))
    sdl_e, sdl_m = O.stretched_dl(g, om, npml)
    Ce, _ = O.create_curls(g, sdl_e, sdl_m, kb)
    ph = [np.exp(-1j * kb[w] * g.L[w]) for w in range(3)]
    A = pkg.FDFDOperator(g.N, om, sdl_e, sdl_m, bloch, ph)
    rng = np.random.default_rng(32)
    n = 3 * g.ncell
    e = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    jm = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for j in (None, jm):
        ref = O.h_from_e(e, om, Ce, j)
        got = A.h_from_e(e, j)
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    A.close()


@pytest.mark.parametrize("bloch,kb", CASES)
def test_corner_means(pkg, oracle, bloch, kb):
    O = oracle
    g = _grid(O, bloch)
    om = 2 * np.pi / 6.5
    npml = ((0 if bloch[0] else 2, 2, 0 if bloch[2] else 2), (0 if bloch[0] else 2, 2, 0 if bloch[2] else 2))
    sdl_e, sdl_m = O.stretched_dl(g, om, npml)
    Mce, Mcm = O.create_Mcs(g, sdl_e, sdl_m, kb)
    ph = [np.exp(-1j * kb[w] * g.L[w]) for w in range(3)]
    A = pkg.FDFDOperator(g.N, om, sdl_e, sdl_m, bloch, ph)
    rng = np.random.default_rng(33)
    n = 3 * g.ncell
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for field, M in (("E", Mce), ("H", Mcm)):
        ref = M @ v
        got = A.corner_mean(v, field)
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), field
    A.close()


@pytest.mark.parametrize("bloch,kb", CASES)
def test_e_from_h(pkg, oracle, bloch, kb):
    """e_from_h (model.jl:281-284) with a diagonal ε against the oracle, and
    its rejection of an off-diagonal ε (the reference's Pε \\ needs a
    diagonal one)."""
    O = oracle
    g = _grid(O, bloch)
    om = 2 * np.pi / 6.5
    npml = ((0 if bloch[0] else 2, 2, 0 if bloch[2] else 2), (0 if bloch[0] else 2, 2, 0 if bloch[2] else 2))
    sdl_e, sdl_m = O.stretched_dl(g, om, npml)
    _, Cm = O.create_curls(g, sdl_e, sdl_m, kb)
    ph = [np.exp(-1j * kb[w] * g.L[w]) for w in range(3)]
    A = pkg.FDFDOperator(g.N, om, sdl_e, sdl_m, bloch, ph)
    rng = np.random.default_rng(34)
    ed = rng.uniform(1.0, 12.25, g.N + (3,))
    A.set_eps(ed)
    n = 3 * g.ncell
    h = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    je = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for j in (None, je):
        ref = O.e_from_h(h, om, O.field_to_vec(ed), Cm, j)
        got = A.e_from_h(h, j)
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    eo = np.zeros(g.N + (3,))
    eo[2, 2, 2, 0] = 0.5
    A.set_eps(ed, eo)
    with pytest.raises(pkg.FDFDError):
        A.e_from_h(h)
    A.close()
