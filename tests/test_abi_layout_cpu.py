"""The ctypes structures of the Python binding against the C header's own
layout: a small C program, compiled here with gcc against
include/fdfd_gb300.h, prints each struct's size and field offsets, and the
ctypes classes must agree byte for byte."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "fdfd_desc": ["N", "isbloch", "boundft", "order_cmpfirst", "device", "slice2d", "omega", "e_ikl", "sdl_e",
                  "sdl_m"],
    "fdfd_object": ["kind", "pad", "eps", "p"],
    "fdfd_design": ["lo", "hi", "eps_cells"],
    "fdfd_solve_opts": ["method", "precision", "tol", "maxit", "delta", "x0_given", "check_every", "transpose",
                        "use_graph", "ell"],
    "fdfd_stats": ["iterations", "matvecs", "refinements", "status", "relres", "time_ms", "launches"],
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "fdfd_gb300.h"', "int main(void) {"]
    for s, fields in STRUCTS.items():
        lines.append(f'  printf("{s} size %zu\\n", sizeof({s}));')
        for f in fields:
            lines.append(f'  printf("{s} {f} %zu\\n", offsetof({s}, {f}));')
    lines += ["  return 0;", "}"]
    src = d / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "abi"
    subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        s, f, v = line.split()
        layout[(s, f)] = int(v)
    return layout


@pytest.mark.parametrize("name", sorted(STRUCTS))
def test_ctypes_layout_matches_header(pkg, c_layout, name):
    cls = getattr(pkg._lib, name)
    assert ctypes.sizeof(cls) == c_layout[(name, "size")]
    assert [f for f, _ in cls._fields_] == STRUCTS[name]
    for f in STRUCTS[name]:
        assert getattr(cls, f).offset == c_layout[(name, f)], f
