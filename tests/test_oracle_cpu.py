"""CPU checks of the oracle's restated MaxwellBase arithmetic and of the
package's host-side set-up (no GPU needed)."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest
import scipy.sparse as sp


def _sym_weights(O, S):
    g = S.grid
    I, J, K = np.meshgrid(*[np.arange(n) for n in g.N], indexing="ij")
    idx = (I, J, K)
    VE = np.zeros(g.N + (3,), complex)
    for w in range(3):
        u, v = [a for a in range(3) if a != w]
        VE[..., w] = S.sdl_m[w][idx[w]] * S.sdl_e[u][idx[u]] * S.sdl_e[v][idx[v]]
    return O.field_to_vec(VE)


def test_curl_of_gradient_vanishes(oracle):
    """Cₑ·∇φ = 0 for φ supported away from the walls, PML included."""
    O = oracle
    g = O.uniform_grid((14, 12, 10))
    S = O.System(g, 2 * np.pi / 6, ((3, 3, 3), (3, 3, 3)))
    rng = np.random.default_rng(0)
    phi = np.zeros((15, 13, 11))
    phi[2:-2, 2:-2, 2:-2] = rng.standard_normal((11, 9, 7))
    E = np.zeros(g.N + (3,), complex)
    E[..., 0] = (phi[1:, :-1, :-1] - phi[:-1, :-1, :-1]) / S.sdl_m[0][:, None, None]
    E[..., 1] = (phi[:-1, 1:, :-1] - phi[:-1, :-1, :-1]) / S.sdl_m[1][None, :, None]
    E[..., 2] = (phi[:-1, :-1, 1:] - phi[:-1, :-1, :-1]) / S.sdl_m[2][None, None, :]
    e = O.field_to_vec(E)
    assert np.linalg.norm(S.Ce @ e) < 1e-12 * np.linalg.norm(e)


def test_symmetrised_operator(oracle):
    """V_E·A is complex symmetric (the reason the transpose kernel is S A S⁻¹)."""
    O = oracle
    g = O.Grid(tuple(np.concatenate([[0.0], np.cumsum(np.random.default_rng(3).uniform(0.7, 1.3, n))])
                     for n in (11, 10, 9)), (False, False, False))
    S = O.System(g, 2 * np.pi / 5, ((2, 3, 1), (1, 2, 3)), [O.Sphere((5.0, 5.0, 4.0), 2.5, 12.25)])
    SA = sp.diags(_sym_weights(O, S)) @ S.A
    assert abs(SA - SA.T).max() <= 1e-14 * abs(SA).max()
    assert np.count_nonzero(S.eps_off) > 0


def test_e_from_h_inverts_h_from_e_on_a_solution(oracle):
    """For A e = b = −iω jₑ with a diagonal Pε (model.jl:264-284):
    e_from_h(h_from_e(e)) = e exactly, the identity the two restated
    formulas must satisfy."""
    import scipy.sparse.linalg as spla
    O = oracle
    g = O.uniform_grid((7, 6, 5))
    om = 2 * np.pi / 4.5
    S = O.System(g, om, ((1, 2, 1), (2, 1, 1)))
    rng = np.random.default_rng(41)
    ed = rng.uniform(1.0, 12.25, g.N + (3,))
    sdl_e, sdl_m = S.sdl_e, S.sdl_m
    Ce, Cm = O.create_curls(g, sdl_e, sdl_m)
    P = O.create_paramop(g, ed, None, sdl_e, sdl_m)
    A = O.create_A(om, P, Ce, Cm)
    n = 3 * g.ncell
    je = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    je[O.field_to_vec(O.pinned_mask(g))] = 0.0
    e = spla.spsolve(A.tocsc(), O.create_b(om, je))
    back = O.e_from_h(O.h_from_e(e, om, Ce), om, O.field_to_vec(ed), Cm, je)
    assert np.max(np.abs(back - e)) <= 1e-9 * np.max(np.abs(e))


def test_h_formulation_describes_the_e_solution(oracle):
    """The oracle's H formulation (create_A_hh, create_b_hh; model.jl:238-240,
    266-268) solved directly gives h_from_e of the E solution, and e_from_h
    of it gives the E solution back (diagonal ε, jₘ = 0)."""
    import scipy.sparse.linalg as spla
    O = oracle
    g = O.uniform_grid((6, 7, 5))
    om = 2 * np.pi / 4.0
    S = O.System(g, om, ((1, 1, 2), (2, 1, 1)))
    rng = np.random.default_rng(43)
    ed = rng.uniform(1.0, 12.25, g.N + (3,))
    ev = O.field_to_vec(ed)
    Ce, Cm = O.create_curls(g, S.sdl_e, S.sdl_m)
    A = O.create_A(om, O.create_paramop(g, ed, None, S.sdl_e, S.sdl_m), Ce, Cm)
    n = 3 * g.ncell
    je = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    je[O.field_to_vec(O.pinned_mask(g))] = 0.0
    e = spla.spsolve(A.tocsc(), O.create_b(om, je))
    h = spla.spsolve(O.create_A_hh(om, ev, Ce, Cm).tocsc(), O.create_b_hh(om, ev, Ce, je))
    href = O.h_from_e(e, om, Ce)
    assert np.max(np.abs(h - href)) <= 1e-9 * np.max(np.abs(href))
    assert np.max(np.abs(O.e_from_h(h, om, ev, Cm, je) - e)) <= 1e-9 * np.max(np.abs(e))


def test_pinned_rows(oracle):
    """Tangential E on the negative PEC planes: row = −ω² ε, column decoupled."""
    O = oracle
    g = O.uniform_grid((6, 5, 4))
    S = O.System(g, 1.1, ((1, 1, 1), (1, 1, 1)))
    M = O.field_to_vec(O.pinned_mask(g))
    A = S.A.tocsr()
    for q in np.flatnonzero(M)[:40]:
        row = A.getrow(q)
        assert row.nnz == 1 and row.indices[0] == q
        assert np.isclose(row.data[0], -(1.1 ** 2) * O.field_to_vec(S.eps_diag)[q])


def test_volume_fraction_against_sampling(oracle):
    O = oracle
    rng = np.random.default_rng(4)
    for _ in range(25):
        lo = rng.uniform(-1, 0, 3)
        hi = lo + rng.uniform(0.5, 2.0, 3)
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        r0 = lo + rng.uniform(0, 1, 3) * (hi - lo)
        f = O.volfrac_plane(lo, hi, n, r0)
        P = lo + rng.random((200000, 3)) * (hi - lo)
        fmc = np.mean((P - r0) @ n <= 0)
        assert abs(f - fmc) < 6e-3
        assert abs(O.volfrac_plane(lo, hi, -n, r0) - (1 - f)) < 1e-12
    # axis-aligned and two-zero-component normals are exact
    assert O.volfrac_plane([0, 0, 0], [1, 1, 1], [0, 0, 1.0], [0, 0, 0.3]) == pytest.approx(0.3, abs=1e-15)
    assert O.volfrac_plane([0, 0, 0], [2, 1, 1], [1.0, 0, 0], [0.5, 0, 0]) == pytest.approx(0.25, abs=1e-15)
    s = np.sqrt(0.5)
    assert O.volfrac_plane([0, 0, 0], [1, 1, 1], [s, s, 0.0], [0.5, 0.5, 0]) == pytest.approx(0.5, abs=1e-15)


def test_kottke_limits(oracle):
    O = oracle
    n = np.array([0.6, 0.0, 0.8])
    assert np.allclose(O._kottke(12.25, 1.0, 1.0, n), 12.25 * np.eye(3))
    assert np.allclose(O._kottke(12.25, 1.0, 0.0, n), np.eye(3))
    T = O._kottke(4.0, 1.0, 0.5, n)
    assert np.allclose(T, T.T)
    assert np.isclose(n @ T @ n, 1 / (0.5 / 4 + 0.5 / 1))      # harmonic mean along n
    t = np.array([0.0, 1.0, 0.0])
    assert np.isclose(t @ T @ t, 2.5)                           # arithmetic mean across


def test_smoothing_masks_and_priority(oracle):
    O = oracle
    g = O.uniform_grid((16, 16, 16))
    big = O.Sphere((8.0, 8.0, 8.0), 5.0, 4.0)
    small = O.Sphere((8.0, 8.0, 8.0), 2.0, 9.0)     # added last: wins inside
    ed, eo, dbg = O.assign_smooth(g, [big, small], 1.0, return_debug=True)
    assert dbg["oind_C"][9, 9, 9] == 2                      # cell centre (8.5, 8.5, 8.5)
    assert ed[8, 8, 8, 0] == 9.0                            # deep inside the small sphere
    assert ed[0, 0, 0, 0] == 1.0
    sm = dbg["smask"]
    assert sm[..., :3].sum() > 0 and sm[..., 3].sum() > 0
    assert np.all(ed >= 1.0 - 1e-12) and np.all(ed <= 9.0 + 1e-12)


def test_design_chain_rule(oracle):
    """dL/dε_cell from design_grad_chain equals finite differences of the
    assembled ε (A7 is linear in the cell values)."""
    O = oracle
    g = O.uniform_grid((12, 10, 8))
    rng = np.random.default_rng(9)
    vals = rng.uniform(1, 12, (4, 3, 2))
    des = O.DesignRegion((4, 3, 3), (8, 6, 5), vals)
    objs = [O.Box((-1, -1, 2.5), (13, 11, 5.5), 6.0)]
    ed0, _ = O.assign_smooth(g, objs, 1.0, des)
    gdiag = rng.standard_normal(ed0.shape)
    chain = O.design_grad_chain(g, des, gdiag)
    for (a, b, c) in [(0, 0, 0), (3, 2, 1), (1, 1, 0), (2, 0, 1)]:
        v2 = vals.copy()
        v2[a, b, c] += 0.1
        ed1, _ = O.assign_smooth(g, objs, 1.0, O.DesignRegion(des.lo, des.hi, v2))
        fd = np.sum(gdiag * (ed1 - ed0)) / 0.1
        assert np.isclose(chain[a, b, c], fd, rtol=1e-10, atol=1e-12)


def test_pml_profile(pkg, oracle):
    g = pkg.uniform_grid((30, 20, 10))
    om = 0.8
    Npml = ((5, 4, 0), (6, 0, 3))
    s = pkg.grid.sfactor(g, 0, pkg.PRIM, om, Npml)
    assert np.all(s[5:25] == 1.0)            # primal planes 5 and 24 lie on the inner faces
    assert np.all(np.imag(s[:5]) < 0) and np.all(np.imag(s[25:]) < 0)
    smax = -(4 + 1) * np.log(1e-8) / (2 * 5)
    assert np.isclose(s[0], 1 + smax / (1j * om))
    # host mirror == oracle
    go = oracle.uniform_grid((30, 20, 10))
    se1, sm1 = pkg.create_stretched_dl(g, om, Npml)
    se2, sm2 = oracle.stretched_dl(go, om, Npml)
    for a, b in zip(se1 + sm1, se2 + sm2):
        assert np.array_equal(a, b)


def test_host_grid_matches_oracle(pkg, oracle):
    rng = np.random.default_rng(11)
    for bloch in [(False, False, False), (True, False, True)]:
        lp = tuple(np.concatenate([[-1.0], -1.0 + np.cumsum(rng.uniform(0.4, 1.6, n))]) for n in (7, 5, 9))
        a, b = pkg.Grid(lp, bloch), oracle.Grid(lp, bloch)
        for gt in (0, 1):
            for w in range(3):
                assert np.array_equal(a.l[gt][w], b.l[gt][w])
                assert np.array_equal(a.dl[gt][w], b.dl[gt][w])
        assert np.array_equal(a.bounds[0], b.bounds[0]) and np.array_equal(a.L, b.L)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    m = bench.max_over_ranks(1.5 + rank, ws)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, m))


def test_bench_replicas_max_over_ranks():
    """The N > 1 path of bench.py: each replica reports its time, the job
    time is the maximum over ranks (world_size 2 over gloo)."""
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert out == {0: 2.5, 1: 2.5}


def test_native_csr_baseline_matches_oracle(oracle):
    """The OpenMP CSR SpMV/BiCGSTAB (the benchmark's CPU baseline) against
    scipy and the oracle's own BiCGSTAB on the same assembled A."""
    from oracle.csr_native import NativeCSR
    O = oracle
    g = O.uniform_grid((10, 9, 8))
    S = O.System(g, 2 * np.pi / 6.0, ((2, 2, 2), (2, 2, 2)), [O.Sphere((5.1, 4.2, 3.9), 2.2, 6.0)])
    S.add_pointsrc((4.6, 4.5, 4.0), (0.2, 0.1, 1.0))
    b = S.b()
    M = NativeCSR(S.A, threads=2)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size)
    assert np.max(np.abs(M.matvec(x) - S.A @ x)) <= 1e-13 * np.max(np.abs(S.A @ x))
    xo, ito, _ = O.bicgstab(S.A, b, tol=1e-8, maxit=5000)
    xn, itn, rel = M.bicgstab(b, tol=1e-8, maxit=5000)
    assert rel < 1e-8 and abs(itn - ito) <= max(3, ito // 20), (itn, ito)
    assert np.linalg.norm(b - S.A @ xn) / np.linalg.norm(b) < 1e-7


def test_native_bicgstabl_converges(oracle):
    """The CPU baseline's BiCGStab(ℓ) reaches the tolerance on the same
    system and, like the GPU solver, needs fewer operator applications than
    BiCGSTAB there."""
    from oracle.csr_native import NativeCSR
    O = oracle
    g = O.uniform_grid((12, 11, 10))
    S = O.System(g, 2 * np.pi / 5.0, ((2, 2, 2), (2, 2, 2)), [O.Sphere((6.1, 5.2, 4.9), 2.6, 12.25)])
    S.add_pointsrc((5.6, 5.5, 5.0), (0.2, 0.1, 1.0))
    b = S.b()
    M = NativeCSR(S.A, threads=2)
    _, it, _ = M.bicgstab(b, tol=1e-8, maxit=20000)
    for ell in (1, 2, 4):
        x, mv, rel = M.bicgstabl(b, ell=ell, tol=1e-8, maxmv=40000)
        assert rel < 1e-8, (ell, mv)
        assert np.linalg.norm(b - S.A @ x) / np.linalg.norm(b) < 1e-7
        if ell == 4:
            assert mv <= 2 * it, (mv, it)
