"""MADWF (lib/gpt/qcd/fermion/preconditioner/mixed_dwf.py) and its
fifth-dimension moves, following the reference's test
tests/qcd/domain_wall.py:134-163: an approximate outer Mobius solve from an
inner zmobius solve agrees with the exact propagator to eps^2 < 5e-4, a
second right-hand side gives the same result, and defect correction around
MADWF reaches the exact propagator (eps^2 < 1e-10).  With inner = outer the
algorithm is exact.  The chiral shift P and the slice copy are checked
against numpy on natural fields, the solves against the oracle's Mobius M."""
import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402
from gpt_gb300 import _lib, core  # noqa: E402

DIMS = [4, 4, 4, 8]
MOBIUS = dict(mass=0.08, M5=1.8, b=1.5, c=0.5, Ls=12, boundary_phases=[1.0, 1.0, 1.0, 1.0])
# zmobius approximation of the Ls = 12, b + c = 2 Mobius operator over the
# kernel spectrum of the reference's test (tests/qcd/domain_wall.py:91-112)
OMEGA = [0.17661651536320583 + 0.14907774771612217j, 0.23027432016909377 - 0.03530801572584271j,
         0.3368765581549033, 0.7305711010541054, 1.1686138337986505 + 0.3506492418109086j,
         1.1686138337986505 - 0.3506492418109086j, 0.994175013717952, 0.5029903152251229,
         0.23027432016909377 + 0.03530801572584271j, 0.17661651536320583 - 0.14907774771612217j]
ZMOBIUS = dict(mass=0.08, M5=1.8, b=1.0, c=0.0, omega=OMEGA, boundary_phases=[1.0, 1.0, 1.0, 1.0])


def _rand(shape, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(shape) + 1j * r.standard_normal(shape)


def _field(op, arr):
    F = op.F_lattice()
    F[:] = arr
    return F


def _gauge(eps=0.9, seed=17):
    return g.qcd.gauge.random_su3(g.grid(DIMS, g.double), eps, seed)


def _p_numpy(x, offset):
    """dst_s = P- x_s + P+ x_{s+offset} on natural [V][Ls][4][3] arrays."""
    y = x.copy()
    y[:, :, 0:2] = np.roll(x, -offset, axis=1)[:, :, 0:2]
    return y


@pytest.mark.parametrize("prec,tol", [("double", 0.0), ("double_float", 1e-14), ("single", 1e-6)])
def test_chiral_shift_and_slice_copy_match_numpy(prec, tol):
    U = _gauge()
    op = g.qcd.fermion.mobius(U, dict(MOBIUS, Ls=6))
    op = op if prec == "double" else op.converted(getattr(g, prec))
    small = g.qcd.fermion.mobius(U, dict(MOBIUS, Ls=4))
    small = small if prec == "double" else small.converted(getattr(g, prec))
    x = _rand(op.F_lattice()[:].shape, 3)
    X = _field(op, x)
    L = _lib.load()
    for off in (1, -1, 2):
        Y = op.F_lattice()
        _lib.check(L.gbf_chiral_shift(X.layout.op, X.ptr, Y.ptr, off, 2, core.stream_ptr()))
        want = _p_numpy(x, off)
        assert np.abs(Y[:] - want).max() <= tol * np.abs(want).max()
    # P^+ P = 1
    Y, Z = op.F_lattice(), op.F_lattice()
    _lib.check(L.gbf_chiral_shift(X.layout.op, X.ptr, Y.ptr, 1, 2, core.stream_ptr()))
    _lib.check(L.gbf_chiral_shift(Y.layout.op, Y.ptr, Z.ptr, -1, 2, core.stream_ptr()))
    assert np.abs(Z[:] - x).max() <= tol * np.abs(x).max()
    # slices 1, 2 of the Ls = 6 field -> slices 2, 3 of an Ls = 4 field, times -0.5
    s0 = _rand(small.F_lattice()[:].shape, 4)
    S = _field(small, s0)
    _lib.check(L.gbf_copy_slices(S.layout.op, S.ptr, 2, X.layout.op, X.ptr, 1, 2, -0.5, 2, core.stream_ptr()))
    want = s0.copy()
    want[:, 2:4] = -0.5 * x[:, 1:3]
    assert np.abs(S[:] - want).max() <= max(tol, 1e-15) * np.abs(want).max()
    # out-of-range slices are rejected before any launch
    assert L.gbf_copy_slices(S.layout.op, S.ptr, 3, X.layout.op, X.ptr, 0, 2, 1.0, 2, core.stream_ptr()) == 1


def _solvers(eps):
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    return inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": eps, "maxiter": 4000}))


def test_madwf_with_the_outer_operator_inside_is_exact():
    """inner = outer: MADWF reproduces D^-1 src (checked against the
    oracle's Mobius M on the full 5D solution)."""
    U = _gauge()
    qm = g.qcd.fermion.mobius(U, dict(MOBIUS, Ls=6))
    slv = _solvers(1e-11)
    src_np = _rand(qm.F_lattice()[:].shape, 5)
    src = _field(qm, src_np)
    x = g.qcd.fermion.preconditioner.mixed_dwf(slv, slv, qm)(qm)(src)[:]
    ref = o.mobius(U.U, DIMS, **dict(MOBIUS, Ls=6))
    res = src_np - ref.apply("M", x)
    assert np.sqrt(o.norm2(res) / o.norm2(src_np)) < 1e-8
    x_exact = slv(qm)(src)[:]
    assert np.linalg.norm(x - x_exact) / np.linalg.norm(x_exact) < 1e-8


def test_madwf_zmobius_inner_approximates_the_mobius_propagator():
    """tests/qcd/domain_wall.py:134-163 on a 4^3 x 8 lattice: zmobius Ls = 10
    inside a Mobius Ls = 12 solve."""
    U = _gauge()
    qm = g.qcd.fermion.mobius(U, MOBIUS)
    qz = g.qcd.fermion.zmobius(U, ZMOBIUS)
    assert qz.Ls == 10
    slv_5d = _solvers(1e-5)
    slv_e = _solvers(1e-8)
    inv = g.algorithms.inverter
    mdwf = g.qcd.fermion.preconditioner.mixed_dwf(slv_5d, slv_5d, qz)
    src4 = _rand((int(np.prod(DIMS)), 4, 3), 6)
    S = qm.U_lattice()
    S[:] = src4
    exact = qm.propagator(slv_e)(S)[:]
    madwf = qm.propagator(mdwf)(S)[:]
    eps2 = np.linalg.norm(madwf - exact) ** 2 / np.linalg.norm(exact) ** 2
    assert eps2 < 5e-4, eps2
    again = qm.propagator(mdwf)(S)[:]
    assert np.linalg.norm(again - madwf) ** 2 / np.linalg.norm(madwf) ** 2 < 1e-13
    dc = qm.propagator(inv.defect_correcting(mdwf, eps=1e-6, maxiter=10))(S)[:]
    eps2 = np.linalg.norm(dc - exact) ** 2 / np.linalg.norm(exact) ** 2
    assert eps2 < 1e-10, eps2


def test_bulk_propagator_projects_to_the_propagator():
    """qm.bulk_propagator_to_propagator * qm.bulk_propagator(slv) ==
    qm.propagator(slv) (tests/qcd/domain_wall.py:171-176)."""
    U = _gauge()
    qm = g.qcd.fermion.mobius(U, dict(MOBIUS, Ls=6))
    slv = _solvers(1e-10)
    src4 = _rand((int(np.prod(DIMS)), 4, 3), 8)
    S = qm.U_lattice()
    S[:] = src4
    bulk = qm.bulk_propagator(slv)(S)
    assert bulk.layout is qm.F_layout
    via_bulk = qm.bulk_propagator_to_propagator(bulk)[:]
    direct = qm.propagator(slv)(S)[:]
    assert np.linalg.norm(via_bulk - direct) / np.linalg.norm(direct) < 1e-12


def test_J5q_matches_numpy_midpoint():
    """qm.J5q(psi) = P+ psi_{Ls/2-1} + P- psi_{Ls/2} (mobius.py:55-61) on a
    random 5D field, against numpy on the natural layout."""
    U = _gauge()
    qm = g.qcd.fermion.mobius(U, dict(MOBIUS, Ls=6))
    x = _rand(qm.F_lattice()[:].shape, 9)  # [V, Ls, 4, 3]
    got = qm.J5q(_field(qm, x))[:]
    want = np.concatenate([x[:, 2, 0:2], x[:, 3, 2:4]], axis=1)
    assert np.array_equal(got, want)
