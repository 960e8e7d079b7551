"""Multi-shift CG on the eo2_ne normal matrix (lib/gpt/algorithms/inverter/multi_shift_cg.py)
against the oracle: every shifted system (Mpc^+ Mpc + s) x = b is checked
with the oracle's own opcodes, Mpc = 1 - Meooe MooeeInv Meooe MooeeInv on the
odd sites (the Schur complement of lib/gpt/algorithms/preconditioner/
schur_complement_two.py), Mpc^+ the same with the adjoint opcodes."""
import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

EVEN, ODD = 0, 1


def _mpc_ne(ref, x):
    t = ref.apply("MooeeInv", x, ODD)
    z = ref.apply("MooeeInv", ref.apply("Meooe", t, EVEN), EVEN)
    w = x - ref.apply("Meooe", z, ODD)
    u = ref.apply("MooeeInvDag", ref.apply("MeooeDag", w, EVEN), EVEN)
    return w - ref.apply("MooeeInvDag", ref.apply("MeooeDag", u, ODD), ODD)


@pytest.mark.parametrize("kind,params", [
    ("wilson_clover", dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])),
    ("mobius", dict(Ls=4, b=1.5, c=0.5, M5=1.8, mass_plus=0.1, mass_minus=0.1, boundary_phases=[1.0, 1.0, 1.0, -1.0])),
])
def test_multishift_solves_every_shift(kind, params):
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 23).U
    grid = g.grid(dims, g.double)
    Uf = g.qcd.gauge.gauge_field(grid, U)
    op = g.qcd.fermion.wilson_clover(Uf, params) if kind == "wilson_clover" else g.qcd.fermion.mobius(Uf, params)
    ref = o.wilson_clover(U, dims, **params) if kind == "wilson_clover" else o.mobius(U, dims, **params)
    par = o.parity_of_sites(dims).reshape((-1,) + (1,) * (len(ref.shape()) - 1))
    r = np.random.default_rng(4)
    b_np = (r.standard_normal(ref.shape()) + 1j * r.standard_normal(ref.shape())) * (par == ODD)
    B = op.F_lattice()
    B[:] = b_np
    shifts = [0.0, 0.003, 0.05, 0.4, 2.0]
    ms = g.algorithms.inverter.multi_shift_cg({"eps": 1e-10, "maxiter": 4000, "shifts": shifts})
    X = ms(g.qcd.fermion.preconditioner.eo2_ne()(op).Mpc)(B.half(g.odd))
    assert ms.last.converged and not ms.last.breakdown
    for j, s in enumerate(shifts):
        F = op.F_lattice()
        F.half(g.odd).tensor.copy_(X[j].tensor)
        x = F[:]
        assert np.abs(x * (par == EVEN)).max() == 0.0
        res = _mpc_ne(ref, x) + s * x - b_np
        assert np.linalg.norm(res) / np.linalg.norm(b_np) < 1e-9, (j, s)
        assert ms.last.residual_sq[j] <= 1e-20


def test_normal_matrix_matches_the_oracle():
    dims = [4, 4, 4, 8]
    params = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 29).U
    Uf = g.qcd.gauge.gauge_field(g.grid(dims, g.double), U)
    op = g.qcd.fermion.wilson_clover(Uf, params)
    ref = o.wilson_clover(U, dims, **params)
    par = o.parity_of_sites(dims).reshape(-1, 1, 1)
    r = np.random.default_rng(2)
    x_np = (r.standard_normal(ref.shape()) + 1j * r.standard_normal(ref.shape())) * (par == ODD)
    Xl = op.F_lattice()
    Xl[:] = x_np
    Y = g.qcd.fermion.preconditioner.eo2_ne()(op).Mpc(Xl.half(g.odd))
    F = op.F_lattice()
    F.half(g.odd).tensor.copy_(Y.tensor)
    want = _mpc_ne(ref, x_np)
    assert np.linalg.norm(F[:] - want) / np.linalg.norm(want) < 1e-13


def test_generic_cg_on_a_shifted_operator():
    """inverter.cg on a matrix operator that is not a native normal matrix
    (here Mpc^+ Mpc + s, composed in Python): the reference's recursion
    (cg.py:47-105) driven from the host over the device vector algebra; its
    solution of every shifted system is checked with the oracle's opcodes,
    and on Mpc itself it agrees with the device-resident CG."""
    dims = [4, 4, 4, 8]
    params = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 31).U
    op = g.qcd.fermion.wilson_clover(g.qcd.gauge.gauge_field(g.grid(dims, g.double), U), params)
    ref = o.wilson_clover(U, dims, **params)
    par = o.parity_of_sites(dims).reshape(-1, 1, 1)
    r = np.random.default_rng(6)
    b_np = (r.standard_normal(ref.shape()) + 1j * r.standard_normal(ref.shape())) * (par == ODD)
    B = op.F_lattice()
    B[:] = b_np
    b = B.half(g.odd)
    Mpc = g.qcd.fermion.preconditioner.eo2_ne()(op).Mpc
    inv = g.algorithms.inverter
    for s in (0.0, 0.05):
        def shifted(dst, src, s=s):
            Mpc(dst, src)
            g.axpby(dst, s, src, 1.0, dst)

        cg = inv.cg({"eps": 1e-10, "maxiter": 2000})
        x = cg(shifted)(b)
        assert cg.last.converged and cg.last.iterations > 0
        F = op.F_lattice()
        F.half(g.odd).tensor.copy_(x.tensor)
        res = _mpc_ne(ref, F[:]) + s * F[:] - b_np
        assert np.linalg.norm(res) / np.linalg.norm(b_np) < 1e-9, s
        if s == 0.0:
            cgn = inv.cg({"eps": 1e-10, "maxiter": 2000})
            xn = cgn(Mpc)(b)
            assert abs(cgn.last.iterations - cg.last.iterations) <= 1
            d = (xn.tensor.view(torch.float64) - x.tensor.view(torch.float64)).norm()
            assert d <= 1e-8 * xn.tensor.view(torch.float64).norm()
