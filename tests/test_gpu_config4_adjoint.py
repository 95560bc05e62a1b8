"""The inverse-design gradient workload: 128×128×64 grid, 10-cell PML, a slab
waveguide (ε = 12.25, 8 cells thick), a 40×40×10 design region of per-cell
ε ~ U[1, 12.25] (seeded), a y-polarised dipole at x = 20, and the objective
L = |Σ over the plane x = 108 of conj(E_mode)·E|² with a Gaussian E_mode of
width 6 cells.  The gradient dL/dε over the design region comes from one
transposed GPU solve (fdfd_eps_grad) chained to the cells (fdfd_design_grad)
— the derivative of create_A (src/model/model.jl:225-246) through the
design-region ε convention (calc_matparams!, src/model/full.jl:16-70).

* central differences with h = 1e-4·ε on 32 seeded design cells: ≤ 1e-4
  relative (2-norm over the 32 cells), every cell within 1e-3 of its own
  value plus 1e-4 of the largest;
* the CPU sparse-operator adjoint — the oracle's assembled Aᵀ solved by the
  OpenMP CSR BiCGStab(4) to 1e-11, the same 2·Re(ω²·λ·e) and the same
  design chain in numpy — ≤ 1e-6 relative to the largest component."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H_REL = 1e-4


@pytest.fixture(scope="module")
def c4(pkg):
    wl = pkg.workloads
    mdl, om = wl.config4()
    A = pkg.create_A(mdl, om)
    b = pkg.create_b(mdl, om)
    F = wl.config4_mode()
    e, st = A.solve(b, tol=1e-11, precision="fp64")
    assert st[0]["status"] == 0
    s = np.vdot(F, e)
    g = np.conj(s) * np.conj(F)
    grad, st = A.eps_grad(e, g, tol=1e-11, precision="fp64")
    assert st["status"] == 0 and st["relres"] <= 1e-11
    dg = A.design_grad(grad)
    yield dict(pkg=pkg, mdl=mdl, om=om, A=A, b=b, F=F, e=e, g=g, grad=grad, dg=dg, L=abs(s) ** 2)
    A.close()


def _objective(c, eps_cells):
    """L at perturbed design ε: the design is re-smoothed on the same handle
    and the solve starts from the unperturbed field."""
    pkg, mdl, A = c["pkg"], c["mdl"], c["A"]
    d = pkg.DesignRegion(mdl.design.lo, mdl.design.hi, eps_cells)
    A.smooth_objects(mdl.grid.lprim, mdl.objects, mdl.eps_bg, d)
    x, st = A.solve(c["b"], tol=1e-11, precision="mixed", x0=c["e"])
    assert st[0]["status"] == 0, st
    return abs(np.vdot(c["F"], x)) ** 2


def test_config4_gradient_matches_central_differences(c4):
    rng = np.random.default_rng(3004)
    eps0 = np.array(c4["mdl"].design.eps, dtype=np.float64)
    shape = eps0.shape
    cells = [tuple(int(rng.integers(0, n)) for n in shape) for _ in range(32)]
    fd, ad = [], []
    for q in cells:
        h = H_REL * eps0[q]
        ep = eps0.copy()
        ep[q] += h
        em = eps0.copy()
        em[q] -= h
        fd.append((_objective(c4, ep) - _objective(c4, em)) / (2 * h))
        ad.append(c4["dg"][q])
    # restore the handle's design
    pkg, mdl = c4["pkg"], c4["mdl"]
    c4["A"].smooth_objects(mdl.grid.lprim, mdl.objects, mdl.eps_bg, pkg.DesignRegion(mdl.design.lo, mdl.design.hi, eps0))
    fd, ad = np.array(fd), np.array(ad)
    assert np.linalg.norm(fd - ad) <= 1e-4 * np.linalg.norm(ad), (fd, ad)
    # per cell: the difference quotient's noise (solves to 1e-11 relative,
    # divided by 2h) is about 1e-5 of the largest component
    assert np.all(np.abs(fd - ad) <= 1e-3 * np.abs(ad) + 1e-4 * np.abs(ad).max()), (fd, ad)


def test_config4_gradient_matches_cpu_sparse_adjoint(c4, oracle):
    from oracle.build_oracle import build
    from oracle.csr_native import NativeCSR
    build()
    O = oracle
    mdl, om = c4["mdl"], c4["om"]
    N = mdl.grid.N
    zc = N[2] / 2
    g = O.uniform_grid(N)
    objs = [O.Box((-1.0, -1.0, zc - 4.0), (N[0] + 1.0, N[1] + 1.0, zc + 4.0), 12.25)]
    design = O.DesignRegion(mdl.design.lo, mdl.design.hi, np.array(mdl.design.eps, dtype=np.float64))
    S = O.System(g, om, mdl.Npml, objs, 1.0, design)
    S.add_pointsrc((20.0, 64.0, zc), (0, 1, 0))
    assert np.linalg.norm(S.b() - c4["b"]) <= 1e-14 * np.linalg.norm(S.b())
    M = NativeCSR(S.A.T.tocsr())
    lam, mv, rel = M.bicgstabl(c4["g"], ell=4, tol=1e-11, maxmv=400000)
    assert rel <= 1e-11
    gd = 2.0 * np.real(om ** 2 * lam * c4["e"])
    gcell = O.vec_to_field(gd.astype(np.complex128), N).real
    dg_cpu = O.design_grad_chain(g, design, gcell)
    dg = c4["dg"]
    assert dg_cpu.shape == dg.shape
    assert np.max(np.abs(dg_cpu - dg)) <= 1e-6 * np.max(np.abs(dg_cpu))
