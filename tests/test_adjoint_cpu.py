"""The oracle's adjoint ε-gradient and design-cell chain, pinned on the CPU.

The reference has no adjoint, so the oracle's formula dL/dε_cc =
2·Re(ω²·λ_c·e_c) (Aᵀλ = g) is checked against central finite differences of
direct solves of the assembled A (create_A, src/model/model.jl:225-246), and
the design chain against the exact linear map of the design-region
assembly (per-cell ε averaged onto the E edges).
"""
import numpy as np
import scipy.sparse.linalg as spla


def _objective(F, e):
    s = np.vdot(F, e)            # Fᴴ e
    return abs(s) ** 2, np.conj(s) * np.conj(F)   # L, g = ∂L/∂e (Wirtinger)


def test_oracle_adjoint_matches_finite_differences(oracle):
    O = oracle
    g = O.uniform_grid((8, 7, 6))
    om = 2 * np.pi / 5.0
    S = O.System(g, om, ((2, 2, 2), (2, 2, 2)), [O.Sphere((4.1, 3.3, 2.9), 1.8, 6.0)])
    S.add_pointsrc((3.6, 3.5, 3.0), (0.2, 1.0, 0.4))
    b = S.b()
    rng = np.random.default_rng(11)
    F = rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size)
    e = spla.spsolve(S.A.tocsc(), b)
    L0, gv = _objective(F, e)
    grad, _ = O.adjoint_eps_grad(S.A, om, e, gv)
    assert L0 > 0
    for (i, j, k, c) in [(4, 3, 3, 0), (2, 5, 1, 2), (5, 2, 4, 1), (0, 3, 3, 1)]:
        vals = []
        for sgn in (+1, -1):
            ed = S.eps_diag.copy()
            hstep = 1e-6 * ed[i, j, k, c]
            ed[i, j, k, c] += sgn * hstep
            P = O.create_paramop(g, ed, S.eps_off, S.sdl_e, S.sdl_m)
            A2 = O.create_A(om, P, S.Ce, S.Cm)
            vals.append(_objective(F, spla.spsolve(A2.tocsc(), b))[0])
        fd = (vals[0] - vals[1]) / (2 * hstep)
        ad = grad[c + 3 * (i + g.N[0] * (j + g.N[1] * k))]
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-12 * L0, (i, j, k, c, fd, ad)


def test_design_chain_is_transpose_of_design_map(oracle):
    O = oracle
    g = O.uniform_grid((10, 9, 8))
    rng = np.random.default_rng(12)
    lo, hi = (3, 2, 0), (8, 6, 5)       # touches the z = 0 wall (index clamp)
    eps0 = rng.uniform(1.0, 12.25, tuple(h - l for l, h in zip(lo, hi)))
    objs = [O.Box((-1.0, -1.0, 3.0), (11.0, 10.0, 5.0), 4.0)]
    d0 = O.DesignRegion(lo, hi, eps0)
    ed0, _ = O.assign_smooth(g, objs, 1.0, d0)
    delta = rng.standard_normal(eps0.shape)
    ed1, _ = O.assign_smooth(g, objs, 1.0, O.DesignRegion(lo, hi, eps0 + delta))
    gd = rng.standard_normal(tuple(g.N) + (3,))
    lhs = np.sum(gd * (ed1 - ed0))
    rhs = np.sum(O.design_grad_chain(g, d0, gd) * delta)
    assert abs(lhs - rhs) <= 1e-12 * np.sum(np.abs(gd)), (lhs, rhs)


def test_corner_means_preserve_constants(oracle):
    """On a uniform grid without PML the two-point means reproduce a constant
    field: everywhere for E (mirror ghost), and for H except on the last
    plane, where the PEC ghost H_w[N] = 0 halves it."""
    O = oracle
    g = O.uniform_grid((6, 5, 4))
    sdl_e, sdl_m = O.stretched_dl(g, 1.0, ((0, 0, 0), (0, 0, 0)))
    Mce, Mcm = O.create_Mcs(g, sdl_e, sdl_m)
    one = np.ones(3 * g.ncell, complex)
    assert np.allclose(Mce @ one, 1.0, atol=1e-15)
    hc = O.vec_to_field(Mcm @ one, g.N)
    for w in range(3):
        last = [slice(None)] * 3
        last[w] = -1
        inner = [slice(None)] * 3
        inner[w] = slice(0, -1)
        assert np.allclose(hc[tuple(inner) + (w,)], 1.0, atol=1e-15)
        assert np.allclose(hc[tuple(last) + (w,)], 0.5, atol=1e-15)
