"""GB300-native FDFD operator and solver behind MaxwellFDFD.jl's API.

The hot path — applying and solving A = Cₘ·Cₑ − ω²·Pε on the 3D Yee grid
with SC-PML and subpixel-smoothed ε (src/model/model.jl:238-287 of the
reference) — runs in libfdfd_gb300.so (CUDA, sm_103a) through the C ABI in
include/fdfd_gb300.h.  This package is the host-side mirror of the
reference's model/source API plus a ctypes binding of that ABI.
"""
from . import _lib
from ._lib import FDFDError, load
from .grid import DUAL, PRIM, Grid, PMLParam, create_stretched_dl, uniform_grid
from .model import (EE, HH, Box, DesignRegion, Disk, ModelFull, ModelTE, ModelTM, Rect, Sphere, add_obj, add_srce,
                    clear_objs, clear_srcs, create_A, create_b, create_linsys, create_stretched_dls, field_arr2vec,
                    field_arr2vec_2d, set_boundft, set_design, set_kbloch, set_Npml, set_ωpml, uniform_lprim2d,
                    vec2field_arr, vec2field_arr_2d)
from .operator import FDFDOperator, solve_multi
from . import workloads
from .sources import PlaneSrc, PointSrc, distweights

__all__ = [
    "FDFDError", "load", "Grid", "PMLParam", "uniform_grid", "create_stretched_dl", "PRIM", "DUAL", "EE", "HH",
    "ModelFull", "Sphere", "Box", "DesignRegion", "add_obj", "add_srce", "clear_objs", "clear_srcs", "create_A",
    "create_b", "create_linsys", "create_stretched_dls", "set_boundft", "set_design", "set_kbloch", "set_Npml",
    "set_ωpml", "field_arr2vec", "vec2field_arr", "FDFDOperator", "solve_multi", "PlaneSrc", "PointSrc", "distweights",
    "ModelTE", "ModelTM", "Disk", "Rect", "uniform_lprim2d", "field_arr2vec_2d", "vec2field_arr_2d",
]
