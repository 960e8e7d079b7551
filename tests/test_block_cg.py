"""Block CG over packed right-hand sides (lib/gpt/algorithms/inverter/block_cg.py:36-149)
against the oracle's per-rhs solves, and against the packed independent CG.

Tolerances: the solutions agree with the oracle's FP64 eo2_ne CG solution to
1e-8 relative at eps = 1e-10 (the reference's own CG/true-residual check,
tests/qcd/fermion_operators.py:158-167), and the true residual of M x = b in
FP64 is below 1e-8.
"""
import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

WC = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])
MOB = dict(Ls=6, b=1.5, c=0.5, M5=1.8, mass_plus=0.1, mass_minus=0.1, boundary_phases=[1.0, 1.0, 1.0, -1.0])


def _rand(shape, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(shape) + 1j * r.standard_normal(shape)


def _ops(kind, params, dims, nrhs, prec):
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3(grid, 0.4, 17)
    mk = g.qcd.fermion.wilson_clover if kind == "wilson_clover" else g.qcd.fermion.mobius
    packed = mk(U, dict(params, n_rhs=nrhs))
    if prec is not g.double:
        packed = packed.converted(prec)
    ref = o.wilson_clover(U.U, dims, **params) if kind == "wilson_clover" else o.mobius(U.U, dims, **params)
    return packed, ref


@pytest.mark.parametrize("kind,params,nrhs,prec", [
    ("wilson_clover", WC, 4, "double"),
    ("wilson_clover", WC, 12, "double"),
    ("mobius", MOB, 3, "double"),
    ("wilson_clover", WC, 4, "double_float"),
])
def test_block_cg_matches_oracle_solves(kind, params, nrhs, prec):
    dims = [4, 4, 4, 8]
    P = {"double": g.double, "double_float": g.double_float}[prec]
    op, ref = _ops(kind, params, dims, nrhs, P)
    shape = op.F_lattice()[:].shape[1:] if nrhs > 1 else op.F_lattice()[:].shape
    srcs = [_rand(shape, 60 + k) for k in range(nrhs)]
    B = op.F_lattice()
    for k in range(nrhs):
        B.set_natural(srcs[k], k)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    bcg = inv.block_cg({"eps": 1e-10, "maxiter": 1000})
    X = inv.preconditioned(pc.eo2_ne(), bcg)(op)(B)
    assert bcg.last.converged and not bcg.last.breakdown
    for k in range(nrhs):
        x = X.get_natural(k)
        r = srcs[k] - ref.apply("M", x)
        assert np.sqrt(o.norm2(r) / o.norm2(srcs[k])) < 1e-8, k
        x_ref, _, _ = ref.eo2ne_cg(srcs[k], 1e-12, 4000)
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8, k


def test_block_cg_needs_no_more_iterations_than_packed_cg():
    """The shared Krylov space converges all right-hand sides in at most as
    many iterations as the slowest independent CG."""
    dims = [4, 4, 4, 8]
    nrhs = 6
    op, _ = _ops("wilson_clover", dict(WC, mass=0.02), dims, nrhs, g.double)
    shape = op.F_lattice()[:].shape[1:]
    B = op.F_lattice()
    for k in range(nrhs):
        B.set_natural(_rand(shape, 80 + k), k)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": 1e-10, "maxiter": 4000})
    inv.preconditioned(pc.eo2_ne(), cg)(op)(B)
    bcg = inv.block_cg({"eps": 1e-10, "maxiter": 4000})
    inv.preconditioned(pc.eo2_ne(), bcg)(op)(B)
    assert cg.last.converged and bcg.last.converged
    assert bcg.last.iterations <= cg.last.iterations


@pytest.mark.parametrize("kind,params,nrhs,dims", [
    ("wilson_clover", WC, 4, [4, 4, 4, 8]),
    # k = 12 packed sources in 5D (the 12-source propagator's shape): the
    # register-tiled FP32 Gram with 3 x 3 entry blocks per thread
    ("mobius", dict(MOB, Ls=4), 12, [4, 4, 4, 8]),
    ("wilson_clover", WC, 7, [4, 4, 4, 8]),
])
def test_block_cg_single_precision_inner_in_defect_correction(kind, params, nrhs, dims):
    op, ref = _ops(kind, params, dims, nrhs, g.double)
    shape = op.F_lattice()[:].shape[1:]
    srcs = [_rand(shape, 90 + k) for k in range(nrhs)]
    B = op.F_lattice()
    for k in range(nrhs):
        B.set_natural(srcs[k], k)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    inner = inv.preconditioned(pc.eo2_ne(), inv.block_cg({"eps": 1e-5, "maxiter": 1000}))
    dc = inv.defect_correcting(inv.mixed_precision(inner, g.single, g.double), eps=1e-10, maxiter=20)
    X = dc(op)(B)
    for k in range(nrhs):
        r = srcs[k] - ref.apply("M", X.get_natural(k))
        assert np.sqrt(o.norm2(r) / o.norm2(srcs[k])) < 1e-10, k


def test_block_cg_reports_breakdown_for_dependent_sources():
    dims = [4, 4, 4, 4]
    op, _ = _ops("wilson_clover", WC, dims, 3, g.double)
    shape = op.F_lattice()[:].shape[1:]
    s = _rand(shape, 5)
    B = op.F_lattice()
    B.set_natural(s, 0)
    B.set_natural(s, 1)  # identical: the residual block has rank 2
    B.set_natural(_rand(shape, 6), 2)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    bcg = inv.block_cg({"eps": 1e-10, "maxiter": 100})
    inv.preconditioned(pc.eo2_ne(), bcg)(op)(B)
    assert bcg.last.breakdown and not bcg.last.converged
