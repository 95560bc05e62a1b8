"""The Julia binding (maxwellfdm.jl_gb300/julia/MaxwellFDFDGPU.jl) against
the C header it mirrors: every struct passed by ccall has the header
struct's fields in the same order with the same widths (so Julia's C layout
matches), and every symbol it calls is declared in the header.  Julia is not
installed, so the file is read as text."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdfd_gb300.h")
JULIA = os.path.join(ROOT, "maxwellfdm.jl_gb300", "julia", "MaxwellFDFDGPU.jl")

_C2J = {"int32_t": "Int32", "int64_t": "Int64", "double": "Float64", "uint8_t": "UInt8"}


def _c_struct(text, name):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # comments may hold braces
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r";", text)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = re.sub(r"/\*.*?\*/", "", line).strip()
        if not line:
            continue
        d = re.match(r"(const\s+)?(\w+)\s*(\*?)\s*(\w+)((?:\[\d+\])*)\s*;", line)
        assert d, line
        base = "Ptr{%s}" % _C2J[d.group(2)] if d.group(3) else _C2J[d.group(2)]
        count = 1
        for dim in re.findall(r"\[(\d+)\]", d.group(5)):
            count *= int(dim)
        fields.append((d.group(4), base if count == 1 else "NTuple{%d,%s}" % (count, base)))
    return fields


def _julia_struct(text, name):
    m = re.search(r"(?:Base\.@kwdef\s+)?struct " + name + r"\n(.*?)\nend", text, re.S)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("#")[0].strip()
        if not line:
            continue
        f = re.match(r"(\w+)::([^=\s]+)", line)
        assert f, line
        fields.append((f.group(1), f.group(2)))
    return fields


@pytest.fixture(scope="module")
def texts():
    with open(HEADER) as f:
        h = f.read()
    with open(JULIA) as f:
        j = f.read()
    return h, j


@pytest.mark.parametrize("cname,jname", [("fdfd_desc", "FDFDDesc"), ("fdfd_solve_opts", "SolveOpts"),
                                         ("fdfd_stats", "SolveStats")])
def test_struct_layouts_match(texts, cname, jname):
    h, j = texts
    c = _c_struct(h, cname)
    jl = _julia_struct(j, jname)
    assert [t for _, t in jl] == [t for _, t in c]
    assert [n for n, _ in jl] == [n for n, _ in c]


def test_called_symbols_are_declared(texts):
    h, j = texts
    called = set(re.findall(r"ccall\(\(:(\w+)", j))
    assert called
    declared = set(re.findall(r"\b(fdfd_\w+)\s*\(", h))
    assert called <= declared, called - declared


def test_rrule_for_the_solve(texts):
    """The binding defines ChainRulesCore reverse rules for the solve with
    respect to ε (solve_with_eps) and b (A \\ b); their pullbacks run the
    transposed GPU solve (transpose = 1 in the options they pass)."""
    _, j = texts
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(solve_with_eps\), A::FDFDOperator", j)
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(\\\), A::FDFDOperator", j)
    pb = re.search(r"function solve_pullback\(.*?\nend", j, re.S).group(0)
    assert "opts.use_graph" in pb and ", 1,\n" in pb    # the transpose flag
    assert "2 .* real.((A.ω^2) .* λ .* e)" in j          # ε̄ = 2Re(ω²λe)
    assert "2 .* conj.(λ)" in j                            # b̄ = 2 conj(λ)


def test_device_residual_wrappers(texts):
    _, j = texts
    assert "ccall((:fdfd_residual_dev," in j
    assert "ccall((:fdfd_residual_dev_noalloc," in j
