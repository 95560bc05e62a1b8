"""Source discretisation against the reference's own tests
(MaxwellFDFD.jl test/source.jl), for both the oracle and the package's host
mirror: the distweights known answers (fixture), the N = 1 Bloch property,
and the PlaneSrc / PointSrc conservation properties."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def kat():
    with open(os.path.join(HERE, "golden", "distweights_kat.json")) as f:
        return json.load(f)


@pytest.fixture(params=["oracle", "package"])
def impl(request, pkg, oracle):
    if request.param == "oracle":
        return oracle.distweights, oracle.PRIM, oracle.DUAL
    return pkg.distweights, pkg.PRIM, pkg.DUAL


def test_distweights_known_answers(kat, impl):
    dw, PRIM, DUAL = impl
    assert len(kat["cases"]) == 38
    for c in kat["cases"]:
        gt = PRIM if c["gt"] == "PRIM" else DUAL
        l = np.array(kat[c["gt"]]["l"])
        dl = np.array(kat[c["gt"]]["dl"])
        if c["throws"]:
            with pytest.raises(ValueError):
                dw(c["c"], gt, kat["domain"], l, dl, c["isbloch"])
            continue
        ind, wt = dw(c["c"], gt, kat["domain"], l, dl, c["isbloch"])
        assert [i + 1 for i in ind] == c["ind"], (c, ind)
        assert np.allclose(wt, c["wt"], rtol=1e-14, atol=0), (c, wt)


def test_distweights_single_point_bloch(impl):
    """test/source.jl:106-120: N = 1 with Bloch gives ind = [1,1] and a total
    weight 1/∆l wherever c lies."""
    dw, PRIM, DUAL = impl
    rng = np.random.default_rng(0)
    for c in 2 * rng.random(8):
        ind, wt = dw(c, PRIM, (0, 2), np.array([0.0]), np.array([9.0]), True)
        assert list(ind) == [0, 0] and np.isclose(sum(wt), 1 / 9)
        ind, wt = dw(c, DUAL, (0, 2), np.array([1.0]), np.array([10.0]), True)
        assert list(ind) == [0, 0] and np.isclose(sum(wt), 1 / 10)
    with pytest.raises(ValueError):
        dw(0.5, PRIM, (0, 2), np.array([0.0]), np.array([9.0]), False)


def _grids(which, lib):
    b = (True, True, True)
    if which == "coarse":
        return lib.Grid((np.arange(-10, 11.0),) * 3, b)
    if which == "fine":
        return lib.Grid((np.arange(-10, 10.25, 0.5),) * 3, b)
    raise KeyError(which)


def _add_plane(side, lib, g, src):
    if side == "oracle":
        j = lib.create_field_array(g.N)
        lib.add_planesrc(j, (lib.PRIM,) * 3, g, *src)
    else:
        j = np.zeros(g.N + (3,), complex)
        lib.PlaneSrc(*src).add_to(j, (lib.PRIM,) * 3, g)
    return j


def _add_point(side, lib, g, c, p):
    if side == "oracle":
        j = lib.create_field_array(g.N)
        lib.add_pointsrc(j, (lib.PRIM,) * 3, g, c, p, 1.0)
    else:
        j = np.zeros(g.N + (3,), complex)
        lib.PointSrc(c, p).add_to(j, (lib.PRIM,) * 3, g)
    return j


@pytest.mark.parametrize("side", ["oracle", "package"])
def test_planesrc_conservation(side, pkg, oracle):
    """test/source.jl:123-170."""
    lib = oracle if side == "oracle" else pkg
    n = np.array([0, 0, 1])
    if side == "oracle":
        src = (2, 0.0, [1, 0, 0])
    else:
        src = (n, 0.0, [1, 0, 0])
    g = _grids("coarse", lib)
    j = _add_plane(side, lib, g, src)
    assert np.max(np.abs(j)) == 1.0
    assert np.all(j[..., 1] == 0) and np.all(j[..., 2] == 0)
    gf = _grids("fine", lib)
    jf = _add_plane(side, lib, gf, src)
    assert np.isclose(j[0, :, :, 0].sum() * 1.0, jf[0, :, :, 0].sum() * 0.25)
    assert np.max(np.abs(jf)) == 2.0
    rng = np.random.default_rng(1)
    z = np.sort(rng.random(21)) * 20
    z -= z.mean()
    gn = lib.Grid((np.arange(-10, 11.0), np.arange(-10, 11.0), z), (True, True, True))
    jn = _add_plane(side, lib, gn, src)
    dy = gn.dl[lib.PRIM][1]
    dz = gn.dl[lib.PRIM][2]
    assert np.isclose(j[0, :, :, 0].sum(), (jn[0, :, :, 0] * np.outer(dy, dz)).sum())


@pytest.mark.parametrize("side", ["oracle", "package"])
def test_pointsrc_conservation(side, pkg, oracle):
    """test/source.jl:172-230."""
    lib = oracle if side == "oracle" else pkg
    c, p = [0.7, 0.7, 0.7], np.array([1.0, 1.0, 1.0])
    pn = p / np.linalg.norm(p)
    for which, dv in (("coarse", 1.0), ("fine", 0.125)):
        g = _grids(which, lib)
        j = _add_point(side, lib, g, c, p)
        for w in range(3):
            assert np.count_nonzero(j[..., w]) == 8
            assert np.isclose(j[..., w].sum() * dv, pn[w], rtol=1e-15, atol=0)
    rng = np.random.default_rng(2)
    ax = []
    for _ in range(3):
        a = np.sort(rng.random(21)) * 20
        ax.append(a - (a.mean() - 0.7))
    gn = lib.Grid(tuple(ax), (True, True, True))
    jn = _add_point(side, lib, gn, c, p)
    g = _grids("coarse", lib)
    j = _add_point(side, lib, g, c, p)
    dx = gn.dl[lib.PRIM][0]
    dy = gn.dl[lib.PRIM][1]
    dz = gn.dl[lib.DUAL][2]
    vol = dx[:, None, None] * dy[None, :, None] * dz[None, None, :]
    assert np.isclose(j[..., 2].sum(), (jn[..., 2] * vol).sum())


def test_package_sources_match_oracle(pkg, oracle):
    """The product's host source assembly equals the oracle's on random
    non-uniform grids, both boundary kinds, and arbitrary placements."""
    rng = np.random.default_rng(7)
    for trial in range(20):
        N = tuple(int(v) for v in rng.integers(4, 9, 3))
        bloch = tuple(bool(v) for v in rng.integers(0, 2, 3))
        lp = tuple(np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, n))]) for n in N)
        go, gp = oracle.Grid(lp, bloch), pkg.Grid(lp, bloch)
        c = [rng.uniform(lp[a][0], lp[a][-1]) for a in range(3)]
        p = rng.standard_normal(3)
        jo = oracle.create_field_array(N)
        oracle.add_pointsrc(jo, (oracle.PRIM,) * 3, go, c, p, 1.3 - 0.2j)
        jp = np.zeros(N + (3,), complex)
        pkg.PointSrc(c, p, 1.3 - 0.2j).add_to(jp, (pkg.PRIM,) * 3, gp)
        assert np.allclose(jo, jp, rtol=1e-14, atol=1e-15), trial
        ax = int(rng.integers(0, 3))
        nvec = np.eye(3)[ax]
        jo = oracle.create_field_array(N)
        oracle.add_planesrc(jo, (oracle.PRIM,) * 3, go, ax, c[ax], p, 0.5j)
        jp = np.zeros(N + (3,), complex)
        pkg.PlaneSrc(nvec, c[ax], p, 0.5j).add_to(jp, (pkg.PRIM,) * 3, gp)
        assert np.allclose(jo, jp, rtol=1e-14, atol=1e-15), trial
