"""ctypes binding of libfdfd_gb300.so (declared in include/fdfd_gb300.h).

The library is built in-tree by build.py.  Loading fails loudly when it is
missing: there is no CPU fallback for the operator or the solver.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libfdfd_gb300.so")

FDFD_OK = 0
FDFD_ERR_ARG = 1
FDFD_ERR_UNSUPPORTED = 2
FDFD_ERR_CUDA = 3
FDFD_ERR_NOMEM = 4
FDFD_ERR_NOT_CONVERGED = 5
FDFD_ERR_BREAKDOWN = 6
FDFD_ERR_NO_DEVICE = 7
FDFD_ERR_NONFINITE = 8
FDFD_ERR_TIMEOUT = 9
FDFD_C128, FDFD_C64 = 0, 1
FDFD_EE, FDFD_HH = 0, 1
FDFD_PREC_FP64, FDFD_PREC_MIXED = 0, 1
FDFD_BICGSTAB, FDFD_COCG, FDFD_BICGSTABL = 0, 1, 2
FDFD_SHAPE_SPHERE, FDFD_SHAPE_BOX, FDFD_SHAPE_CYLZ = 0, 1, 2
FDFD_SLICE_NONE, FDFD_SLICE_TE, FDFD_SLICE_TM = 0, 1, 2

_dp = C.POINTER(C.c_double)


class fdfd_desc(C.Structure):
    _fields_ = [("N", C.c_int32 * 3), ("isbloch", C.c_int32 * 3), ("boundft", C.c_int32 * 3),
                ("order_cmpfirst", C.c_int32), ("device", C.c_int32), ("slice2d", C.c_int32),
                ("omega", C.c_double * 2), ("e_ikl", (C.c_double * 2) * 3),
                ("sdl_e", _dp * 3), ("sdl_m", _dp * 3)]


class fdfd_object(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32), ("eps", C.c_double), ("p", C.c_double * 6)]


class fdfd_design(C.Structure):
    _fields_ = [("lo", C.c_int32 * 3), ("hi", C.c_int32 * 3), ("eps_cells", _dp)]


class fdfd_solve_opts(C.Structure):
    _fields_ = [("method", C.c_int32), ("precision", C.c_int32), ("tol", C.c_double), ("maxit", C.c_int64),
                ("delta", C.c_double), ("x0_given", C.c_int32), ("check_every", C.c_int32),
                ("transpose", C.c_int32), ("use_graph", C.c_int32), ("ell", C.c_int32)]


class fdfd_stats(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("matvecs", C.c_int64), ("refinements", C.c_int32),
                ("status", C.c_int32), ("relres", C.c_double), ("time_ms", C.c_double),
                ("launches", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# exported symbol → (restype, argtypes)
SIGNATURES = {
    "fdfd_create": (C.c_int, [C.POINTER(fdfd_desc), C.POINTER(C.c_void_p)]),
    "fdfd_destroy": (None, [C.c_void_p]),
    "fdfd_last_error": (C.c_char_p, [C.c_void_p]),
    "fdfd_version": (C.c_char_p, []),
    "fdfd_stream": (C.c_void_p, [C.c_void_p]),
    "fdfd_sync": (C.c_int, [C.c_void_p]),
    "fdfd_set_eps_tensor": (C.c_int, [C.c_void_p, _dp]),
    "fdfd_set_eps": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fdfd_smooth_objects": (C.c_int, [C.c_void_p, _dp * 3, C.POINTER(fdfd_object), C.c_int32, C.c_double,
                                      C.POINTER(fdfd_design)]),
    "fdfd_get_eps": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_uint8)]),
    "fdfd_matvec": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int32]),
    "fdfd_matvec_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "fdfd_matvec_transpose": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int32]),
    "fdfd_solve": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int32, C.POINTER(fdfd_solve_opts),
                             C.POINTER(fdfd_stats)]),
    "fdfd_solve_batch": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int32, C.c_int32, C.POINTER(fdfd_solve_opts),
                                   C.POINTER(fdfd_stats)]),
    "fdfd_solve_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(fdfd_solve_opts),
                                 C.POINTER(fdfd_stats)]),
    "fdfd_default_opts": (None, [C.POINTER(fdfd_solve_opts)]),
    "fdfd_residual_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "fdfd_residual_dev_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.POINTER(C.c_double)]),
    "fdfd_eps_grad": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.POINTER(fdfd_solve_opts), C.POINTER(fdfd_stats)]),
    "fdfd_eps_grad_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(fdfd_solve_opts), C.POINTER(fdfd_stats)]),
    "fdfd_design_grad": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fdfd_h_from_e": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "fdfd_set_field_type": (C.c_int, [C.c_void_p, C.c_int32]),
    "fdfd_h_from_e_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fdfd_e_from_h": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "fdfd_e_from_h_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fdfd_corner_mean": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp]),
    "fdfd_corner_mean_dev": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "fdfd_solve_multi": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                  C.POINTER(fdfd_solve_opts), C.c_void_p]),
    "fdfd_design_grad_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
}


class FDFDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[fdfd status {code}] {msg}")
        self.code = code


_lib = None


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise FDFDError(-1, f"{LIBPATH} is missing: build it with build.py (no CPU fallback exists)")
    lib = C.CDLL(LIBPATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc, handle=None):
    if rc != FDFD_OK:
        msg = load().fdfd_last_error(handle)
        raise FDFDError(rc, msg.decode() if msg else "")


def dptr(a):
    """double* to a C-contiguous float64/complex128 numpy array."""
    assert a.flags["C_CONTIGUOUS"] and a.dtype in (np.float64, np.complex128), (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def default_opts(**kw):
    o = fdfd_solve_opts()
    load().fdfd_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown solver option {k}")
        setattr(o, k, v)
    return o
