"""Failure handling of the C ABI, made to happen without faulting, trapping
or hanging the GPU:

* a NaN in the right-hand side or in the initial guess → FDFD_ERR_NONFINITE
  (the host reads ‖b‖² and the first true residual before iterating);
* a device allocation that fails → FDFD_ERR_NOMEM, simulated on the host by
  the FDFD_FAIL_ALLOC_BYTES hook (requests of at least that many bytes fail
  without reaching the CUDA runtime), and the handle works again once the
  hook is lifted;
* a bounded device-side wait that runs out → FDFD_ERR_TIMEOUT: with
  FDFD_WAIT_LIMIT_CLOCKS=0 each pipeline wait of the TMA operator kernel
  tests its mbarrier once instead of waiting, so a block that finds its
  first plane not yet landed stops, waits (with the full ~1 s limit) for the
  copies it already issued and raises the error flag; a fresh handle then
  applies the operator correctly (the context stays usable)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FDFD_ERR_NOMEM, FDFD_ERR_NONFINITE, FDFD_ERR_TIMEOUT = 4, 8, 9


def _system(O, N, seed=3):
    g = O.uniform_grid(N)
    om = 2 * np.pi / 8.0
    S = O.System(g, om, ((3, 3, 3), (3, 3, 3)), [O.Sphere(tuple(n / 2 + 0.3 for n in N), min(N) / 4, 6.0)])
    S.add_pointsrc(tuple(n / 2 for n in N), (0, 0, 1))
    return S


def _operator(pkg, S):
    A = pkg.FDFDOperator(S.grid.N, S.omega, S.sdl_e, S.sdl_m)
    A.set_eps(S.eps_diag, S.eps_off)
    return A


@pytest.mark.parametrize("where", ["b", "x0"])
def test_nonfinite_input_is_reported(pkg, oracle, where):
    S = _system(oracle, (16, 14, 12))
    A = _operator(pkg, S)
    b = S.b()
    x0 = None
    if where == "b":
        b = b.copy()
        b[17] = np.nan
    else:
        x0 = np.zeros_like(b)
        x0[5] = complex(np.inf, 0.0)
    with pytest.raises(pkg.FDFDError) as ei:
        A.solve(b, tol=1e-8, precision="mixed", x0=x0)
    assert ei.value.code == FDFD_ERR_NONFINITE
    # the handle is still usable
    x, st = A.solve(S.b(), tol=1e-8, precision="fp64")
    assert np.linalg.norm(S.b() - S.A @ x) / np.linalg.norm(S.b()) < 1e-7
    A.close()


def test_allocation_failure_is_reported(pkg, oracle, monkeypatch):
    S = _system(oracle, (24, 24, 24))
    A = _operator(pkg, S)                     # created with no hook set
    n = 3 * S.grid.ncell
    # any buffer the size of one complex64 vector or more fails
    monkeypatch.setenv("FDFD_FAIL_ALLOC_BYTES", str(8 * n))
    with pytest.raises(pkg.FDFDError) as ei:
        A.solve(S.b(), tol=1e-8, precision="mixed")
    assert ei.value.code == FDFD_ERR_NOMEM
    assert "cudaMalloc" in str(ei.value)
    monkeypatch.delenv("FDFD_FAIL_ALLOC_BYTES")
    x, st = A.solve(S.b(), tol=1e-8, precision="mixed")
    assert np.linalg.norm(S.b() - S.A @ x) / np.linalg.norm(S.b()) < 1e-7
    A.close()


def test_bounded_wait_reports_timeout(pkg, oracle, monkeypatch):
    N = (64, 64, 64)      # 256 thread blocks of the TMA kernel (even N[0]: TMA path)
    S = _system(oracle, N)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(3 * S.grid.ncell) + 1j * rng.standard_normal(3 * S.grid.ncell)
    monkeypatch.setenv("FDFD_KCHUNK", "4")          # no autotuning launches at create
    monkeypatch.setenv("FDFD_WAIT_LIMIT_CLOCKS", "0")
    A = _operator(pkg, S)
    with pytest.raises(pkg.FDFDError) as ei:
        A.matvec(x, precision="c64")
    assert ei.value.code == FDFD_ERR_TIMEOUT
    A.close()
    monkeypatch.delenv("FDFD_WAIT_LIMIT_CLOCKS")
    monkeypatch.delenv("FDFD_KCHUNK")
    B = _operator(pkg, S)
    y = B.matvec(x, precision="c64")
    ref = S.A @ x
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-5
    B.close()


def test_multi_solve_reports_a_nonfinite_entry(pkg, oracle):
    """fdfd_solve_multi with one NaN right-hand side among good ones: the call
    reports FDFD_ERR_NONFINITE, the other entries are still solved."""
    import torch
    S = _system(oracle, (16, 14, 12))
    A = _operator(pkg, S)
    dev = torch.device("cuda", 0)
    b = S.b()
    bad = b.copy()
    bad[3] = np.nan
    bufs = []
    for v in (b, bad, 2.0 * b):
        bd = torch.from_numpy(v.view(np.float64).reshape(-1, 2)).to(dev)
        bufs.append((bd, torch.zeros_like(bd)))
    with pytest.raises(pkg.FDFDError) as ei:
        pkg.solve_multi([(A, bd.data_ptr(), xd.data_ptr()) for bd, xd in bufs], tol=1e-8, precision="mixed")
    assert ei.value.code == FDFD_ERR_NONFINITE
    st = ei.value.stats
    assert st[1]["status"] == FDFD_ERR_NONFINITE
    for q in (0, 2):
        assert st[q]["status"] == 0 and st[q]["relres"] <= 1e-8
        x = bufs[q][1].cpu().numpy().view(np.complex128).reshape(-1)
        bq = b if q == 0 else 2.0 * b
        assert np.linalg.norm(bq - S.A @ x) / np.linalg.norm(bq) < 1.02e-8
    A.close()
