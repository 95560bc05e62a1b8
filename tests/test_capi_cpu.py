"""The C ABI without a GPU: the library loads, exports every symbol that
include/fdfd_gb300.h declares, and rejects bad input with status codes
(no compute calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdfd_gb300.h")


@pytest.fixture(scope="module")
def lib(pkg):
    if not os.path.exists(pkg._lib.LIBPATH):
        import __graft_entry__ as ge
        ge._load_module("fdfd_gb300_build", os.path.join(ge.PKG_DIR, "build.py")).build()
    return pkg._lib.load()


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fdfd_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(lib, pkg):
    names = _declared()
    assert len(names) >= 15
    for nm in names:
        assert hasattr(lib, nm), f"{nm} declared in the header but not exported"
    # the ctypes binding covers every declared entry point
    assert set(names) <= set(pkg._lib.SIGNATURES)


def test_no_undeclared_exports(lib, pkg):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", pkg._lib.LIBPATH], capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r"\bT (fdfd_[a-z0-9_]+)\b", out)))
    assert exported == _declared()


def test_bad_arguments_rejected(lib, pkg):
    L = pkg._lib
    assert lib.fdfd_create(None, None) == L.FDFD_ERR_ARG
    d = L.fdfd_desc()
    h = C.c_void_p()
    assert lib.fdfd_create(C.byref(d), C.byref(h)) == L.FDFD_ERR_ARG     # N = 0
    assert b"N must be" in lib.fdfd_last_error(None)
    arrs = [np.ones(4, complex) for _ in range(6)]
    for w in range(3):
        d.N[w] = 4
        d.sdl_e[w] = L.dptr(arrs[w])
        d.sdl_m[w] = L.dptr(arrs[3 + w])
    d.order_cmpfirst = 1
    d.boundft[1] = L.FDFD_HH
    assert lib.fdfd_create(C.byref(d), C.byref(h)) == L.FDFD_ERR_UNSUPPORTED
    d.boundft[1] = L.FDFD_EE
    d.order_cmpfirst = 0
    assert lib.fdfd_create(C.byref(d), C.byref(h)) == L.FDFD_ERR_UNSUPPORTED
    assert lib.fdfd_matvec(None, None, None, 0) == L.FDFD_ERR_ARG
    assert lib.fdfd_solve(None, None, None, 1, None, None) == L.FDFD_ERR_ARG
    assert lib.fdfd_sync(None) == L.FDFD_ERR_ARG
    lib.fdfd_destroy(None)  # no-op


def test_no_device_reports_status(lib, pkg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.FDFDError) as ei:
        pkg.FDFDOperator((4, 4, 4), 1.0, [np.ones(4)] * 3, [np.ones(4)] * 3)
    assert ei.value.code == pkg._lib.FDFD_ERR_NO_DEVICE


def test_default_opts(lib, pkg):
    o = pkg._lib.default_opts()
    assert o.method == pkg._lib.FDFD_BICGSTABL and o.ell == 4 and o.precision == pkg._lib.FDFD_PREC_MIXED
    assert o.tol == 1e-6 and o.delta == 0.1 and o.use_graph == 1
    assert lib.fdfd_version().startswith(b"fdfd_gb300")
