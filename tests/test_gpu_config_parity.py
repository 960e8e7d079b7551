"""Per-application parity with the oracle at the benchmark configurations'
own shapes: the kernels the benchmarks time (block sizes, packed
right-hand sides, s-matrix tiles, grid sizes) are the ones checked here.

* Wilson-clover 32^4 with the 32^4 benchmark's recipe (gauge exp(i 0.3 H),
  mass 0.05, csw 1.0, boundary phases [1, 1, 1, -1]): M, Mdag, Meooe and
  MooeeInv (and daggers) from both parities.
* Mobius 16^3 x 32, Ls 12, b 1.5, c 0.5, M5 1.8, mass 0.01, gauge exp(i 0.4 H)
  from the device generator, 12 right-hand sides packed in one field
  (Ls * n_rhs = 144 threads per 4D site, the shape of the 12-source
  propagator benchmark): M, Mdag, Meooe, Mooee, MooeeInv (and daggers) from
  both parities, every right-hand side; the physical import and export.
* The 32^3 x 64, Ls 16 benchmark operator's shape (Ls 16, mass 0.005, two
  packed right-hand sides) on a 16^3 x 32 lattice the oracle handles quickly.

Tolerances as in test_gpu_parity.py: relative 1e-13 per application in FP64
and double-float (the reference's fingerprint tolerance,
tests/qcd/fermion_operators.py:527), 1e-6 in FP32, 3e-3 for FP16 storage.
The oracle's result of each application is computed once and compared with
every precision.  The procedure follows the reference's operator tests
(tests/qcd/fermion_operators.py:847-908, tests/qcd/domain_wall.py:309-347).
"""
import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # collected on CPU hosts, skipped there
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

TOL = {"double": 1e-13, "double_float": 1e-13, "single": 1e-6, "half": 3e-3}
PREC = {"double": g.double, "double_float": g.double_float, "single": g.single, "half": g.half}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _compare(ref, ops, src_nat, n_rhs, names_full, names_eo, extra=()):
    """Apply every opcode on the GPU for each precision, then the oracle once
    per right-hand side, and compare.  src_nat: list of natural arrays (one
    per rhs).  Returns the worst relative error per precision."""
    par = o.parity_of_sites(ref.dims)
    worst = {k: 0.0 for k in ops}
    srcs = {}
    for k, op in ops.items():
        s = op.F_lattice()
        for r in range(n_rhs):
            s.set_natural(src_nat[r], r)
        srcs[k] = s
    cases = [(name, None) for name in names_full]
    cases += [(name, sp) for name in names_eo for sp in (g.even, g.odd)]
    for name, sp in cases:
        outs = {}
        for k, op in ops.items():
            dst = op.F_lattice()
            if sp is None:
                op._apply(name, dst, srcs[k])
            else:
                dp = sp.inv() if name.startswith("Meooe") else sp
                op._apply(name, dst.half(dp), srcs[k].half(sp))
            outs[k] = dst
        torch.cuda.synchronize()
        for r in range(n_rhs):
            if sp is None:
                want = ref.apply(name, src_nat[r])
            else:
                dp = sp.inv() if name.startswith("Meooe") else sp
                mask = (par == sp.code).reshape((-1,) + (1,) * (src_nat[r].ndim - 1))
                want = ref.apply(name, src_nat[r] * mask, dp.code)
            for k, dst in outs.items():
                e = rel(dst.get_natural(r), want)
                worst[k] = max(worst[k], e)
                assert e < TOL[k], (name, None if sp is None else sp.name, r, k, e)
        del outs
    return worst


@pytest.fixture(scope="module")
def wilson_clover_32():
    dims = [32, 32, 32, 32]
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3(grid, 0.3, 4321)
    p = dict(mass=0.05, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])
    ref = o.wilson_clover(U.U, dims, **p)
    return U, p, ref


def test_wilson_clover_32x32x32x32_every_precision(wilson_clover_32):
    U, p, ref = wilson_clover_32
    op64 = g.qcd.fermion.wilson_clover(U, p)
    ops = {"double": op64, "double_float": op64.converted(g.double_float), "single": op64.converted(g.single)}
    rng = np.random.default_rng(7)
    V = ref.V
    src = [rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))]
    _compare(ref, ops, src, 1, ["M", "Mdag"], ["Meooe", "MeooeDag", "MooeeInv", "MooeeInvDag"])


def _mobius_case(dims, Ls, mass, n_rhs, seed, precs):
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3_device(grid, 0.4, seed)
    p = dict(Ls=Ls, b=1.5, c=0.5, M5=1.8, mass_plus=mass, mass_minus=mass,
             boundary_phases=[1.0, 1.0, 1.0, -1.0], n_rhs=n_rhs)
    ref = o.mobius(U.host(), dims, Ls=Ls, b=1.5, c=0.5, M5=1.8, mass=mass, boundary_phases=[1, 1, 1, -1])
    op64 = g.qcd.fermion.mobius(U, p)
    ops = {k: (op64 if k == "double" else op64.converted(PREC[k])) for k in precs}
    rng = np.random.default_rng(seed)
    shape = ref.shape()
    src = [rng.standard_normal(shape) + 1j * rng.standard_normal(shape) for _ in range(n_rhs)]
    return ref, ops, src


def test_mobius_16x16x16x32_Ls12_12_packed_sources():
    dims, Ls, n_rhs = [16, 16, 16, 32], 12, 12
    ref, ops, src = _mobius_case(dims, Ls, 0.01, n_rhs, 4242, ["double", "double_float", "single", "half"])
    _compare(ref, ops, src, n_rhs, ["M", "Mdag"],
             ["Meooe", "MeooeDag", "Mooee", "MooeeDag", "MooeeInv", "MooeeInvDag"])
    # physical import (4D -> 5D: walls, then Dminus) and export, every rhs
    rng = np.random.default_rng(99)
    V = ref.V
    s4 = [rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3)) for _ in range(n_rhs)]
    for k, op in ops.items():
        a = op.U_lattice()
        for r in range(n_rhs):
            a.set_natural(s4[r], r)
        b5 = op.ImportPhysicalFermionSource(a)
        x5 = op.F_lattice()
        for r in range(n_rhs):
            x5.set_natural(src[r], r)
        q = op.ExportPhysicalFermionSolution(x5)
        for r in range(n_rhs):
            assert rel(b5.get_natural(r), ref.import_physical_source(s4[r])) < TOL[k], ("import", k, r)
            assert rel(q.get_natural(r), ref.export_physical_solution(src[r])) < TOL[k], ("export", k, r)


def test_mobius_Ls16_two_packed_sources_shape():
    dims, Ls, n_rhs = [16, 16, 16, 32], 16, 2
    ref, ops, src = _mobius_case(dims, Ls, 0.005, n_rhs, 777, ["double", "double_float", "single"])
    _compare(ref, ops, src, n_rhs, ["M", "Mdag"], ["Meooe", "MeooeDag", "MooeeInv", "MooeeInvDag"])
