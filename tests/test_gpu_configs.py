"""Full-size benchmark configurations as parity cases, through properties
that do not depend on size.

* Uneven batch (24 instances, edges 48–128, 8-cell PML, 10–60 spheres,
  1–4 dipoles): the whole batch in one fdfd_solve_multi call; and three 48³
  instances solved concurrently from separate host threads, one handle
  each.  Every right-hand side meets 1e-6 on the FP64 residual recomputed by
  the GPU, and one instance per grid size on the oracle's assembled
  matrix.
* 320³ with 400 spheres (ε ∈ {1, 2.25, 12.25}): on-device smoothing, then
  complex64 against complex128 application, the transpose identity
  uᵀ(A v) = (Aᵀu)ᵀ v in complex128, and a capped solve whose reported
  residual matches the FP64 residual recomputed independently.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C3_48 = (1, 6, 20)   # instances of the uneven batch with 48³ grids


def _solve_instance(pkg, q, out):
    wl = pkg.workloads
    mdl, om, rhs = wl.config3_instance(q)
    A = pkg.create_A(mdl, om)
    res = []
    for c, p in rhs:
        b = wl.dipole_rhs(mdl, om, c, p)
        x, st = A.solve(b, tol=1e-6, precision="mixed")
        res.append((b, x, st[0]))
    # FP64 residual on the GPU, independent of the solver's own bookkeeping
    chk = []
    for b, x, st in res:
        r = b - A.matvec(x)
        chk.append(np.linalg.norm(r) / np.linalg.norm(b))
    A.close()
    out[q] = (mdl, om, res, chk)


def test_uneven_batch_concurrent(pkg, oracle):
    out = {}
    threads = [threading.Thread(target=_solve_instance, args=(pkg, q, out)) for q in C3_48]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert sorted(out) == sorted(C3_48)
    for q in C3_48:
        mdl, om, res, chk = out[q]
        assert len(res) >= 1
        for (b, x, st), rel in zip(res, chk):
            assert st["status"] == 0 and st["relres"] <= 1e-6, (q, st)
            assert rel <= 1.01e-6, (q, rel)
    # one instance against the oracle's assembled matrix
    O = oracle
    mdl, om, res, _ = out[C3_48[-1]]
    g = O.uniform_grid(mdl.grid.N)
    objs = [O.Sphere(o.shape.c, o.shape.r, o.eps) for o in mdl.objects]
    S = O.System(g, om, mdl.Npml, objs)
    for b, x, st in res:
        rel = np.linalg.norm(b - S.A @ x) / np.linalg.norm(b)
        assert rel <= 1.02e-6, rel


@pytest.fixture(scope="module")
def big(pkg):
    mdl, om, rhs = pkg.workloads.config5()
    A = pkg.create_A(mdl, om)
    yield pkg, mdl, om, rhs, A
    A.close()


def test_320_smoothing_and_precisions(big):
    import torch
    pkg, mdl, om, rhs, A = big
    ed, eo, sm = A.get_eps()
    assert ed.min() >= 1.0 - 1e-12 and ed.max() <= 12.25 + 1e-12
    assert np.count_nonzero(sm[..., :3] == 1) > 0 and np.count_nonzero(eo) > 0
    del ed, eo, sm
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(5)
    x64 = torch.randn(A.n, 2, device=dev, dtype=torch.float64, generator=g)
    y64 = torch.empty_like(x64)
    x32 = x64.float()
    y32 = torch.empty_like(x32)
    A.matvec_dev(x64.data_ptr(), y64.data_ptr(), "c128")
    A.matvec_dev(x32.data_ptr(), y32.data_ptr(), "c64")
    A.sync()
    rel = (torch.linalg.vector_norm(y32.double() - y64) / torch.linalg.vector_norm(y64)).item()
    assert rel < 1e-5, rel


def test_320_transpose_identity(big):
    pkg, mdl, om, rhs, A = big
    rng = np.random.default_rng(6)
    u = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    v = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
    lhs = np.dot(u, A.matvec(v))
    rhs_ = np.dot(A.rmatvec_transpose(u), v)
    assert abs(lhs - rhs_) <= 1e-10 * abs(lhs), (lhs, rhs_)


def test_320_capped_solve_residual(big):
    import torch
    pkg, mdl, om, rhs, A = big
    c, p = rhs[0]
    b = pkg.workloads.dipole_rhs(mdl, om, c, p)
    dev = torch.device("cuda", 0)
    bd = torch.from_numpy(b.view(np.float64).reshape(-1, 2)).to(dev)
    xd = torch.zeros_like(bd)
    with pytest.raises(pkg.FDFDError) as ei:
        A.solve_dev(bd.data_ptr(), xd.data_ptr(), tol=1e-6, precision="mixed", maxit=400)
    assert ei.value.code == 5  # not converged within the cap
    r = torch.empty_like(bd)
    rr = A.residual_dev(xd.data_ptr(), bd.data_ptr(), r.data_ptr())
    rel = rr ** 0.5 / np.linalg.norm(b)
    assert 0 < rel < 1.0


def test_batch_of_rhs_on_concurrent_streams(pkg, oracle):
    """All right-hand sides of one 48³ instance at once, one worker stream
    each: the same answers as the one-by-one solve."""
    wl = pkg.workloads
    mdl, om, rhs = wl.config3_instance(C3_48[0])
    A = pkg.create_A(mdl, om)
    B = np.stack([wl.dipole_rhs(mdl, om, c, p) for c, p in rhs])
    xs, sts = A.solve(B, tol=1e-7, precision="mixed")
    xb, stb = A.solve(B, tol=1e-7, precision="mixed", workers=len(rhs))
    for q in range(len(rhs)):
        assert stb[q]["status"] == 0 and stb[q]["relres"] <= 1e-7, stb[q]
        rel = np.linalg.norm(B[q] - A.matvec(xb[q])) / np.linalg.norm(B[q])
        assert rel <= 1.01e-7, (q, rel)
        assert np.linalg.norm(xb[q] - xs[q]) / np.linalg.norm(xs[q]) < 1e-5
    A.close()


def test_config3_all_instances_in_one_multi_solve(pkg, oracle):
    """The whole uneven batch — all 24 instances (edges 48–128, 10–60
    spheres, λ ~ U[12, 24]) with each of their 1–4 dipole right-hand sides —
    in one fdfd_solve_multi call (one parent CUDA graph per round).  Every
    entry meets 1e-6 on its FP64 residual recomputed by the GPU, and one
    instance of every grid size meets it on the oracle's assembled matrix."""
    import torch
    wl = pkg.workloads
    dev = torch.device("cuda", 0)
    ops, entries, bufs = [], [], []
    for q in range(24):
        mdl, om, rhs = wl.config3_instance(q)
        A = pkg.create_A(mdl, om)
        ops.append((A, mdl, om))
        for c, p in rhs:
            b = wl.dipole_rhs(mdl, om, c, p)
            bd = torch.from_numpy(b.view(np.float64).reshape(-1, 2)).to(dev)
            xd = torch.zeros_like(bd)
            entries.append((A, bd.data_ptr(), xd.data_ptr()))
            bufs.append((q, b, bd, xd))
    assert len(entries) >= 24
    stats = pkg.solve_multi(entries, tol=1e-6, precision="mixed")
    seen = {}
    for (q, b, bd, xd), st in zip(bufs, stats):
        assert st["status"] == 0 and st["relres"] <= 1e-6, (q, st)
        A = ops[q][0]
        r = torch.empty_like(bd)
        rr = A.residual_dev(xd.data_ptr(), bd.data_ptr(), r.data_ptr())
        assert rr ** 0.5 / np.linalg.norm(b) <= 1.01e-6, q
        seen.setdefault(A.N[0], (q, b, xd))
    O = oracle
    for n, (q, b, xd) in sorted(seen.items()):
        A, mdl, om = ops[q]
        g = O.uniform_grid(mdl.grid.N)
        objs = [O.Sphere(o.shape.c, o.shape.r, o.eps) for o in mdl.objects]
        S = O.System(g, om, mdl.Npml, objs)
        x = xd.cpu().numpy().view(np.complex128).reshape(-1)
        rel = np.linalg.norm(b - S.A @ x) / np.linalg.norm(b)
        assert rel <= 1.02e-6, (n, q, rel)
    for A, _, _ in ops:
        A.close()
