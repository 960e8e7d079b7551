"""Deflation (lib/gpt/algorithms/inverter/deflate.py over modes/matrix.py),
sequence (sequence.py) and CG with a guess on the eo2_ne normal operator
(cg.py:48-68), following the reference's own test
tests/algorithms/implicitly_restarted_lanczos.py:82-112: the low-mode
approximation inverts the operator on its eigenvectors, and CG started from
the deflated guess converges in fewer iterations to the same tolerance.

The eigenvectors are inputs here: the lowest eigenpairs of the dense normal
matrix Mpc^+ Mpc built column by column with the oracle's opcodes on a 4^4
lattice (1536 unknowns) and diagonalised by numpy.  Residuals are checked
with the oracle as well."""
import ctypes

import numpy as np
import pytest

import oracle as o
from gpt_gb300 import _lib


def test_mode_and_guess_entry_points_reject_null_arguments():
    L = _lib.load()
    f = (ctypes.c_double * 2)(1.0, 0.0)
    assert L.gbf_modes_apply(None, None, None, f, 1, None, None, 1, None) == 1
    assert b"null" in L.gbf_last_error()
    p = _lib.gbf_cg_params(1e-8, 10, 0, 0)
    assert L.gbf_solve_normal_cg(None, None, None, ctypes.byref(p), None, None) == 1
    assert L.gbf_eo2ne_prepare(None, None, None, None) == 1
    assert L.gbf_eo2ne_reconstruct(None, None, None, None, None) == 1


torch = pytest.importorskip("torch")
gpu = pytest.mark.gpu

EVEN, ODD = 0, 1
DIMS = [4, 4, 4, 4]
PARAMS = dict(mass=-0.2, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _mpc_ne(ref, x):
    t = ref.apply("MooeeInv", x, ODD)
    z = ref.apply("MooeeInv", ref.apply("Meooe", t, EVEN), EVEN)
    w = x - ref.apply("Meooe", z, ODD)
    u = ref.apply("MooeeInvDag", ref.apply("MeooeDag", w, EVEN), EVEN)
    return w - ref.apply("MooeeInvDag", ref.apply("MeooeDag", u, ODD), ODD)


_cache = {}


def _system():
    """Gauge field, oracle, odd-site index map and the lowest eigenpairs of the
    dense normal matrix (built once per session)."""
    if "sys" in _cache:
        return _cache["sys"]
    import gpt_gb300 as g

    U = g.qcd.gauge.random_su3(g.grid(DIMS), 0.4, 41).U
    ref = o.wilson_clover(U, DIMS, **PARAMS)
    par = o.parity_of_sites(DIMS)
    odd = np.nonzero(par == ODD)[0]
    shape = ref.shape()
    n = odd.size * 12
    A = np.empty((n, n), dtype=np.complex128)
    for c in range(n):
        e = np.zeros(shape, dtype=np.complex128)
        e[odd[c // 12], (c % 12) // 3, c % 3] = 1.0
        A[:, c] = _mpc_ne(ref, e)[odd].reshape(-1)
    lam, vec = np.linalg.eigh(0.5 * (A + A.conj().T))
    _cache["sys"] = (U, ref, par, odd, A, lam, vec)
    return _cache["sys"]


def _half(op, g, arr_odd, odd):
    """An odd-site half lattice of op holding arr_odd ([n_odd, 4, 3])."""
    full = np.zeros(op.F_lattice()[:].shape, dtype=np.complex128)
    full[odd] = arr_odd
    F = op.F_lattice()
    F[:] = full
    return F.half(g.odd)


def _numpy_of_half(op, g, h, odd):
    F = op.F_lattice()
    F.half(g.odd).tensor.copy_(h.tensor)
    full = F[:]
    assert np.abs(np.delete(full, odd, axis=0)).max() == 0.0
    return full[odd]


@gpu
@pytest.mark.parametrize("prec,tol", [("double", 1e-13), ("double_float", 1e-12), ("single", 2e-6)])
def test_modes_matrix_matches_numpy(prec, tol):
    """dst = sum_n left_n <right_n, src> f_n for 11 modes (one full block of
    eight and a remainder), distinct left and right modes, complex f."""
    _need_gpu()
    import gpt_gb300 as g

    U, ref, par, odd, A, lam, vec = _system()
    op = g.qcd.fermion.wilson_clover(g.qcd.gauge.gauge_field(g.grid(DIMS, g.double), U), PARAMS)
    op = op if prec == "double" else op.converted(getattr(g, prec))
    r = np.random.default_rng(5)
    shp = (odd.size, 4, 3)
    rnd = lambda: r.standard_normal(shp) + 1j * r.standard_normal(shp)  # noqa: E731
    L = [rnd() for _ in range(11)]
    R = [rnd() for _ in range(11)]
    ev = list(r.uniform(0.5, 2.0, 11))
    f = lambda x: 1.0 / x + 0.25j * x  # noqa: E731
    src = rnd()
    want = sum(L[i] * np.vdot(R[i], src) * f(ev[i]) for i in range(11))
    lg = [_half(op, g, a, odd) for a in L]
    rg = [_half(op, g, a, odd) for a in R]
    m = g.algorithms.modes.matrix(lg, rg, ev, f)
    got = _numpy_of_half(op, g, m(_half(op, g, src, odd)), odd)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < tol


@gpu
def test_low_mode_approximation_inverts_on_eigenvectors():
    """lma = deflate(evec, evals)(Mpc): evals[i] * lma * evec[i] = evec[i]
    (implicitly_restarted_lanczos.py:82-88)."""
    _need_gpu()
    import gpt_gb300 as g

    U, ref, par, odd, A, lam, vec = _system()
    op = g.qcd.fermion.wilson_clover(g.qcd.gauge.gauge_field(g.grid(DIMS, g.double), U), PARAMS)
    w = g.qcd.fermion.preconditioner.eo2_ne()(op)
    nev = 12
    evec = [_half(op, g, vec[:, i].reshape(-1, 4, 3), odd) for i in range(nev)]
    lma = g.algorithms.inverter.deflate(evec, lam[:nev])(w.Mpc)
    for i in range(nev):
        y = _numpy_of_half(op, g, lma(evec[i]), odd)
        v = vec[:, i].reshape(-1, 4, 3)
        assert np.linalg.norm(lam[i] * y - v) ** 2 / np.linalg.norm(v) ** 2 * lam[i] < 5e-10


@gpu
def test_deflated_cg_needs_fewer_iterations():
    """sequence(deflate(evec, evals), cg) against cg on the normal operator
    (implicitly_restarted_lanczos.py:90-112), both to eps 1e-8; the residual
    is checked with the oracle's normal matrix."""
    _need_gpu()
    import gpt_gb300 as g

    U, ref, par, odd, A, lam, vec = _system()
    op = g.qcd.fermion.wilson_clover(g.qcd.gauge.gauge_field(g.grid(DIMS, g.double), U), PARAMS)
    w = g.qcd.fermion.preconditioner.eo2_ne()(op)
    inv = g.algorithms.inverter
    r = np.random.default_rng(8)
    b = r.standard_normal((odd.size, 4, 3)) + 1j * r.standard_normal((odd.size, 4, 3))
    start = _half(op, g, b, odd)
    cg = inv.cg({"eps": 1e-8, "maxiter": 1000})
    x_cg = _numpy_of_half(op, g, cg(w.Mpc)(start), odd)
    n_cg = len(cg.history)
    res = A @ x_cg.reshape(-1) - b.reshape(-1)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 1.5e-8 and cg.last.converged

    nev = 24
    evec = [_half(op, g, vec[:, i].reshape(-1, 4, 3), odd) for i in range(nev)]
    defl = inv.sequence(inv.deflate(evec, lam[:nev]), cg)
    x_d = _numpy_of_half(op, g, defl(w.Mpc)(start), odd)
    n_defl = len(cg.history)
    res = A @ x_d.reshape(-1) - b.reshape(-1)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 1.5e-8 and cg.last.converged
    assert n_defl < n_cg

    # the deflated guess alone: its residual has no component along the modes
    lma = inv.deflate(evec, lam[:nev])(w.Mpc)
    x0 = _numpy_of_half(op, g, lma(start), odd).reshape(-1)
    r0 = b.reshape(-1) - A @ x0
    assert np.abs(vec[:, :nev].conj().T @ r0).max() < 1e-10 * np.linalg.norm(b)


@gpu
def test_cg_guess_edge_cases():
    """A guess that already solves the system returns after zero iterations;
    a zero source gives the zero solution (cg.py:66-68)."""
    _need_gpu()
    import gpt_gb300 as g

    U, ref, par, odd, A, lam, vec = _system()
    op = g.qcd.fermion.wilson_clover(g.qcd.gauge.gauge_field(g.grid(DIMS, g.double), U), PARAMS)
    w = g.qcd.fermion.preconditioner.eo2_ne()(op)
    inv = g.algorithms.inverter
    r = np.random.default_rng(9)
    b = r.standard_normal((odd.size, 4, 3)) + 1j * r.standard_normal((odd.size, 4, 3))
    start = _half(op, g, b, odd)
    cg = inv.cg({"eps": 1e-8, "maxiter": 1000})
    x = cg(w.Mpc)(start)
    n1 = cg.last.iterations
    cg(w.Mpc)(x, start)  # x is the guess: already converged
    assert cg.last.iterations == 0 and cg.last.converged and n1 > 0
    x2 = _half(op, g, b, odd)  # a non-zero guess for a zero source
    cg(w.Mpc)(x2, _half(op, g, 0 * b, odd))
    assert cg.last.iterations == 0 and np.abs(_numpy_of_half(op, g, x2, odd)).max() == 0.0


@gpu
def test_preconditioned_deflated_solve_matches_the_oracle():
    """preconditioned(eo2_ne(), sequence(deflate(evec, evals), cg)) on the
    full operator: R and L S on the device around the deflated CG; the true
    residual of M x = src with the oracle's M."""
    _need_gpu()
    import gpt_gb300 as g

    U, ref, par, odd, A, lam, vec = _system()
    op = g.qcd.fermion.wilson_clover(g.qcd.gauge.gauge_field(g.grid(DIMS, g.double), U), PARAMS)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    r = np.random.default_rng(12)
    src_np = r.standard_normal(ref.shape()) + 1j * r.standard_normal(ref.shape())
    src = op.F_lattice()
    src[:] = src_np
    nev = 24
    evec = [_half(op, g, vec[:, i].reshape(-1, 4, 3), odd) for i in range(nev)]
    cg_plain = inv.cg({"eps": 1e-10, "maxiter": 1000})
    x_plain = inv.preconditioned(pc.eo2_ne(), cg_plain)(op)(src)[:]
    cg = inv.cg({"eps": 1e-10, "maxiter": 1000})
    x = inv.preconditioned(pc.eo2_ne(), inv.sequence(inv.deflate(evec, lam[:nev]), cg))(op)(src)[:]
    assert cg.last.converged and cg.last.iterations < cg_plain.last.iterations
    for sol in (x, x_plain):
        res = src_np - ref.apply("M", sol)
        assert np.sqrt(o.norm2(res) / o.norm2(src_np)) < 1e-8
    assert np.linalg.norm(x - x_plain) / np.linalg.norm(x_plain) < 1e-8
