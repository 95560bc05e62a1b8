"""fdfd_residual_dev_noalloc — the residual entry point for callers that
cannot allocate device memory (their GPU memory belongs to a framework's
caching pool, or a cudaMalloc's implicit synchronisation would stall their
pipeline).  Called through the C ABI (ctypes) and compared with
fdfd_residual_dev, which computes the same r = b − A x and ‖r‖² with the
handle's own reduction buffer, on two calls in a row.  Tolerance: 1e-12
relative (the complex128 operator tolerance of the other tests).

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_noalloc_residual_matches_allocating_entry_point(pkg, oracle):
    torch = pytest.importorskip("torch")
    O = oracle
    lib = pkg._lib.load()
    g = O.uniform_grid((40, 24, 30))
    S = O.System(g, 2 * np.pi / 9, ((4, 4, 4), (4, 4, 4)),
                 [O.Sphere((20.2, 12.1, 15.3), 6.1, 12.25), O.Sphere((8.0, 8.0, 8.0), 3.0, 2.25)])
    A = pkg.FDFDOperator(g.N, S.omega, S.sdl_e, S.sdl_m)
    A.set_eps(S.eps_diag, S.eps_off)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(12)
    r_ref = None
    for call in range(2):
        x = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
        b = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
        xd = torch.from_numpy(x.view(np.float64).reshape(-1, 2)).to(dev)
        bd = torch.from_numpy(b.view(np.float64).reshape(-1, 2)).to(dev)
        r1 = torch.zeros_like(xd)
        r2 = torch.full_like(xd, float("nan"))
        n1, n2 = C.c_double(), C.c_double()
        torch.cuda.synchronize()
        assert lib.fdfd_residual_dev(A._h, C.c_void_p(xd.data_ptr()), C.c_void_p(bd.data_ptr()),
                                     C.c_void_p(r1.data_ptr()), C.byref(n1)) == 0
        free_before = torch.cuda.mem_get_info(dev)[0]
        assert lib.fdfd_residual_dev_noalloc(A._h, C.c_void_p(xd.data_ptr()), C.c_void_p(bd.data_ptr()),
                                             C.c_void_p(r2.data_ptr()), C.byref(n2)) == 0
        if call == 1:
            # after the first call's one-time set-up, nothing is allocated
            assert torch.cuda.mem_get_info(dev)[0] == free_before
        a = r1.cpu().numpy().view(np.complex128).reshape(-1)
        c = r2.cpu().numpy().view(np.complex128).reshape(-1)
        assert np.linalg.norm(c - a) / np.linalg.norm(a) <= TOL
        assert abs(n2.value - n1.value) / n1.value <= TOL
        r_ref = b - S.A @ x
        assert np.linalg.norm(c - r_ref) / np.linalg.norm(r_ref) <= TOL
    A.close()


def test_noalloc_residual_lengthens_short_z_chunks(pkg, monkeypatch):
    """With the z-chunk forced to one plane, a 128×128×260 grid needs 16640
    thread blocks, more than the fixed scratch's 16384 partial slots; the
    call lengthens the chunk until the grid fits and still matches
    fdfd_residual_dev (which sizes its own buffer), on two calls in a row."""
    torch = pytest.importorskip("torch")
    lib = pkg._lib.load()
    N = (128, 128, 260)
    monkeypatch.setenv("FDFD_KCHUNK", "1")
    g = pkg.uniform_grid(N)
    om = 2 * np.pi / 20
    mdl = pkg.ModelFull(g)
    pkg.set_ωpml(mdl, om)
    pkg.set_Npml(mdl, ((8,) * 3, (8,) * 3))
    A = pkg.create_A(mdl, om)
    monkeypatch.delenv("FDFD_KCHUNK")
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev).manual_seed(3)
    for call in range(2):
        xd = torch.randn(A.n, 2, device=dev, dtype=torch.float64, generator=gen)
        bd = torch.randn(A.n, 2, device=dev, dtype=torch.float64, generator=gen)
        r1 = torch.zeros_like(xd)
        r2 = torch.full_like(xd, float("nan"))
        n1, n2 = C.c_double(), C.c_double()
        torch.cuda.synchronize()
        assert lib.fdfd_residual_dev(A._h, C.c_void_p(xd.data_ptr()), C.c_void_p(bd.data_ptr()),
                                     C.c_void_p(r1.data_ptr()), C.byref(n1)) == 0
        assert lib.fdfd_residual_dev_noalloc(A._h, C.c_void_p(xd.data_ptr()), C.c_void_p(bd.data_ptr()),
                                             C.c_void_p(r2.data_ptr()), C.byref(n2)) == 0
        assert (torch.linalg.vector_norm(r2 - r1) / torch.linalg.vector_norm(r1)).item() <= TOL
        assert abs(n2.value - n1.value) / n1.value <= TOL
    A.close()
