"""Parity of the CUDA path (through the C ABI of libgbferm.so) with the CPU
oracle and with the reference's Grid fingerprints.

Tolerances: FP64 relative 1e-13 per application (the reference's own
fingerprint tolerance, tests/qcd/fermion_operators.py:527); FP32 relative
1e-6 (fp32 eps 1e-7 x 10; the reference uses 1e-7 x 100 in
fermion_operators.py:530-604).
"""
import json
import os

import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # collected on CPU hosts, skipped there
    pytest.skip("needs a GPU", allow_module_level=True)

import gpt_gb300 as g  # noqa: E402

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
# double_float (h + l of two FP32 words, 48-bit significand) is held to the
# FP64 tolerance
TOL = {"double": 1e-13, "double_float": 1e-13, "single": 1e-6}
PREC = {"double": g.double, "double_float": g.double_float, "single": g.single}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def gpu_op(kind, U, dims, prec, **p):
    grid = g.grid(dims, g.double)
    Uf = g.qcd.gauge.gauge_field(grid, U)
    if kind == "wilson_clover":
        op = g.qcd.fermion.wilson_clover(Uf, p)
    elif kind == "wilson_twisted_mass":
        op = g.qcd.fermion.wilson_twisted_mass(Uf, p)
    elif kind == "zmobius":
        op = g.qcd.fermion.zmobius(Uf, p)
    else:
        op = g.qcd.fermion.mobius(Uf, p)
    return op if prec is g.double else op.converted(prec)


def to_gpu(op, arr, five=True):
    lat = op.F_lattice() if five else op.U_lattice()
    lat[:] = arr
    return lat


def rand_field(shape, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(shape) + 1j * r.standard_normal(shape)


# ---------------------------------------------------------------------------
# Grid fingerprints reproduced on the GPU
# ---------------------------------------------------------------------------
def _fp_fields(dims, Ls=None):
    fp = GOLD["fingerprints"]
    rng = o.random(fp["seed"])
    g4 = o.grid(dims)
    U = rng.gauge(g4)
    f = {"U": U}
    if Ls:
        g5 = o.grid([Ls] + dims)
        f["src5"], f["dst5"] = rng.spincolor(g5), rng.spincolor(g5)
    f["src4"], f["dst4"] = rng.spincolor(g4), rng.spincolor(g4)
    return f


@pytest.mark.parametrize("prec", ["double", "double_float"])
@pytest.mark.parametrize("name", ["wilson", "wilson_clover"])
def test_gpu_wilson_clover_fingerprints(name, prec):
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp[name]
    f = _fp_fields(dims)
    op = gpu_op("wilson_clover", f["U"], dims, PREC[prec], **case["params"])
    src = to_gpu(op, f["src4"])
    for tag, ref in case["matrices"].items():
        dst = op.M(src) if tag == "" else op.Mdiag(src)
        X = np.vdot(f["dst4"].ravel(), dst[:].ravel())
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (name, tag, X)


@pytest.mark.parametrize("prec", ["double", "double_float"])
def test_gpu_zmobius_fingerprint(prec):
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp["zmobius"]
    p = case["params"]
    f = _fp_fields(dims, len(p["omega"]))
    op = gpu_op("zmobius", f["U"], dims, PREC[prec], **p)
    src5 = to_gpu(op, f["src5"])
    src4 = to_gpu(op, f["src4"], five=False)
    for tag, ref in case["matrices"].items():
        if tag == ".ImportPhysicalFermionSource":
            out = op.ImportPhysicalFermionSource(src4)
        elif tag == "":
            out = op.M(src5)
        else:
            out = op.Mdiag(src5)
        X = np.vdot(f["dst5"].ravel(), out[:].ravel())
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (tag, X)


@pytest.mark.parametrize("prec", ["double", "double_float"])
def test_gpu_twisted_mass_fingerprint(prec):
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp["wilson_twisted_mass"]
    f = _fp_fields(dims)
    op = gpu_op("wilson_twisted_mass", f["U"], dims, PREC[prec], **case["params"])
    src = to_gpu(op, f["src4"])
    for tag, ref in case["matrices"].items():
        dst = op.M(src) if tag == "" else op.Mdiag(src)
        X = np.vdot(f["dst4"].ravel(), dst[:].ravel())
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (tag, X)


@pytest.mark.parametrize("prec", ["double", "double_float"])
@pytest.mark.parametrize("name", ["mobius", "mobius_axial_mass"])
def test_gpu_mobius_fingerprints(name, prec):
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp[name]
    f = _fp_fields(dims, case["params"]["Ls"])
    op = gpu_op("mobius", f["U"], dims, PREC[prec], **case["params"])
    src5 = to_gpu(op, f["src5"])
    src4 = to_gpu(op, f["src4"], five=False)
    for tag, ref in case["matrices"].items():
        if tag == ".ImportPhysicalFermionSource":
            out = op.ImportPhysicalFermionSource(src4)
        elif tag == "":
            out = op.M(src5)
        else:
            out = op.Mdiag(src5)
        X = np.vdot(f["dst5"].ravel(), out[:].ravel())
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (name, tag, X)


# ---------------------------------------------------------------------------
# every opcode against the oracle
# ---------------------------------------------------------------------------
WC = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])
WC_ANISO = dict(mass=-0.2, csw_r=1.2, csw_t=0.7, xi_0=1.3, nu=2.1, boundary_phases=[1.0, -1.0, 1j, np.exp(0.3j)])
MOB = dict(Ls=6, b=1.5, c=0.5, M5=1.8, mass_plus=0.05, mass_minus=0.09, boundary_phases=[1.0, 1.0, 1.0, -1.0])
TM = dict(mass=0.1, mu=0.3, boundary_phases=[1.0, 1.0, 1.0, -1.0])
ZMOB = dict(omega=[0.8 + 0.3j, 1.1 - 0.2j, 0.6, 1.4 + 0.1j], b=1.2, c=0.3, M5=1.8, mass=0.07,
            boundary_phases=[1.0, 1.0, 1.0, -1.0])
# inner extents Ls * n_rhs >= 8 run the shared-memory link hop in FP32/FP16
MOB8 = dict(MOB, Ls=8)
ZMOB8 = dict(ZMOB, omega=ZMOB["omega"] + [0.9 - 0.1j, 1.2, 0.7 + 0.2j, 1.05])


def _oracle(kind, U, dims, p):
    if kind == "wilson_clover":
        return o.wilson_clover(U, dims, **p)
    if kind == "wilson_twisted_mass":
        return o.wilson_twisted_mass(U, dims, **p)
    if kind == "zmobius":
        return o.zmobius(U, dims, **{k: v for k, v in p.items() if k != "n_rhs"})
    return o.mobius(U, dims, **{k: v for k, v in p.items() if k != "n_rhs"})


@pytest.mark.parametrize("prec", ["double", "double_float", "single"])
@pytest.mark.parametrize("kind,params,dims", [
    ("wilson_clover", WC, [4, 4, 4, 8]),
    ("wilson_clover", WC_ANISO, [4, 2, 6, 4]),
    ("wilson_clover", dict(mass=0.3, boundary_phases=[1, 1, 1, -1]), [2, 2, 2, 2]),
    ("mobius", MOB, [4, 4, 2, 4]),
    ("mobius", MOB8, [4, 2, 6, 4]),
    ("wilson_twisted_mass", TM, [4, 4, 4, 8]),
    ("zmobius", ZMOB, [4, 4, 2, 4]),
    ("zmobius", ZMOB8, [4, 4, 2, 4]),
])
def test_opcodes_vs_oracle(kind, params, dims, prec):
    P = PREC[prec]
    tol = TOL[prec]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 11).U
    ref = _oracle(kind, U, dims, params)
    op = gpu_op(kind, U, dims, P, **params)
    src_np = rand_field(ref.shape(), 5)
    par = o.parity_of_sites(dims)
    src = to_gpu(op, src_np)
    for name in ["M", "Mdag", "Mdiag", "Dhop", "DhopDag"] + (["Dminus", "DminusDag"] if "mobius" in kind else []):
        dst = op.F_lattice()
        op._apply(name, dst, src)
        want = ref.apply(name, src_np)
        assert rel(dst[:], want) < tol, name
    for name in ["Meooe", "MeooeDag", "Mooee", "MooeeDag", "MooeeInv", "MooeeInvDag"]:
        for sp in [g.even, g.odd]:
            dp = sp.inv() if name.startswith("Meooe") else sp
            s_np = src_np * (par == sp.code).reshape((-1,) + (1,) * (src_np.ndim - 1))
            s = to_gpu(op, s_np)
            dst = op.F_lattice()
            op._apply(name, dst.half(dp), s.half(sp))
            want = ref.apply(name, s_np, dp.code)
            assert rel(dst[:], want) < tol, (name, sp)


@pytest.mark.parametrize("prec", ["double", "double_float", "single"])
@pytest.mark.parametrize("kind,params", [("mobius", MOB), ("zmobius", ZMOB)])
def test_mobius_import_export(prec, kind, params):
    P = PREC[prec]
    dims = [4, 4, 4, 4]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 3).U
    ref = _oracle(kind, U, dims, params)
    op = gpu_op(kind, U, dims, P, **params)
    s4 = rand_field((ref.V, 4, 3), 1)
    out = op.ImportPhysicalFermionSource(to_gpu(op, s4, five=False))
    assert rel(out[:], ref.import_physical_source(s4)) < TOL[prec]
    s5 = rand_field(ref.shape(), 2)
    q = op.ExportPhysicalFermionSolution(to_gpu(op, s5))
    assert rel(q[:], ref.export_physical_solution(s5)) < TOL[prec]
    # opcodes 2013 / 2015: the walls alone, and their adjoint
    u = op.ImportUnphysicalFermion(to_gpu(op, s4, five=False))
    assert rel(u[:], ref.import_unphysical(s4)) < TOL[prec]
    e = op.ExportPhysicalFermionSource(to_gpu(op, s5))
    assert rel(e[:], ref.export_physical_source(s5)) < TOL[prec]
    e2 = op.ImportUnphysicalFermion.adj()(to_gpu(op, s5))
    assert np.array_equal(e2[:], e[:])


def test_reconstruct12_matches_full_links():
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 4).U
    a = gpu_op("wilson_clover", U, dims, g.single, reconstruct=1, **WC)
    b = gpu_op("wilson_clover", U, dims, g.single, reconstruct=0, **WC)
    s = rand_field((int(np.prod(dims)), 4, 3), 3)
    x = a.M(to_gpu(a, s))[:]
    y = b.M(to_gpu(b, s))[:]
    assert rel(x, y) < 2e-6


def test_multi_rhs_packed_equals_single():
    dims = [4, 4, 4, 4]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 8).U
    single = gpu_op("wilson_clover", U, dims, g.double, **WC)
    packed = gpu_op("wilson_clover", U, dims, g.double, n_rhs=3, **WC)
    srcs = [rand_field((int(np.prod(dims)), 4, 3), 20 + k) for k in range(3)]
    P = packed.F_lattice()
    for k in range(3):
        P.set_natural(srcs[k], k)
    out = packed.M(P)
    for k in range(3):
        want = single.M(to_gpu(single, srcs[k]))[:]
        assert rel(out.get_natural(k), want) < 1e-15


# ---------------------------------------------------------------------------
# solvers
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["double", "double_float"])
@pytest.mark.parametrize("kind,params", [("wilson_clover", WC), ("mobius", dict(MOB, mass_plus=0.1, mass_minus=0.1)),
                                         ("wilson_twisted_mass", TM), ("zmobius", ZMOB)])
def test_eo2ne_cg_vs_oracle(kind, params, prec):
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 21).U
    ref = _oracle(kind, U, dims, params)
    op = gpu_op(kind, U, dims, PREC[prec], **params)
    b = rand_field(ref.shape(), 9)
    x_ref, it_ref, _ = ref.eo2ne_cg(b, 1e-10, 2000)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": 1e-10, "maxiter": 2000})
    slv = inv.preconditioned(pc.eo2_ne(), cg)(op)
    x = slv(to_gpu(op, b))[:]
    assert cg.last.converged
    assert abs(cg.last.iterations - it_ref) <= 2
    r = b - ref.apply("M", x)
    assert np.sqrt(o.norm2(r) / o.norm2(b)) < 1e-8
    assert rel(x, x_ref) < 1e-8


@pytest.mark.parametrize("outer", ["double", "double_float"])
def test_mixed_precision_defect_correction(outer):
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 2).U
    ref = o.wilson_clover(U, dims, **dict(WC, mass=0.05))
    op = gpu_op("wilson_clover", U, dims, PREC[outer], **dict(WC, mass=0.05))
    b = rand_field(ref.shape(), 4)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    inner = inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": 1e-5, "maxiter": 1000}))
    dc = inv.defect_correcting(inv.mixed_precision(inner, g.single, PREC[outer]), eps=1e-10, maxiter=20)
    slv = dc(op)
    x = slv(to_gpu(op, b))[:]
    r = b - ref.apply("M", x)
    assert np.sqrt(o.norm2(r) / o.norm2(b)) < 1e-10
    x_ref, _, _ = ref.eo2ne_cg(b, 1e-12, 4000)
    assert rel(x, x_ref) < 1e-8


def test_propagator_wilson_and_mobius():
    dims = [4, 4, 4, 4]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 5).U
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    for kind, params in [("wilson_clover", WC), ("mobius", dict(MOB, mass_plus=0.1, mass_minus=0.1))]:
        ref = _oracle(kind, U, dims, params)
        op = gpu_op(kind, U, dims, g.double, **params)
        prop = op.propagator(inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": 1e-11, "maxiter": 4000})))
        s4 = rand_field((ref.V, 4, 3), 7)
        q = prop(to_gpu(op, s4, five=False))[:]
        if kind == "wilson_clover":
            want, _, _ = ref.eo2ne_cg(s4, 1e-12, 4000)
        else:
            x5, _, _ = ref.eo2ne_cg(ref.import_physical_source(s4), 1e-12, 4000)
            want = ref.export_physical_solution(x5)
        assert rel(q, want) < 1e-8, kind


@pytest.mark.parametrize("kind,params,nrhs", [
    ("wilson_clover", WC, 3),
    ("mobius", dict(MOB, mass_plus=0.1, mass_minus=0.1), 2),
])
def test_packed_multi_rhs_cg_equals_separate_solves(kind, params, nrhs):
    """All right-hand sides iterate together (shared links, per-rhs scalars);
    each converges exactly as its own single-rhs solve."""
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 12).U
    single = gpu_op(kind, U, dims, g.double, **params)
    packed = gpu_op(kind, U, dims, g.double, n_rhs=nrhs, **params)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    shape = single.F_lattice()[:].shape
    srcs = [rand_field(shape, 40 + k) * (k + 1) for k in range(nrhs)]
    P = packed.F_lattice()
    for k in range(nrhs):
        P.set_natural(srcs[k], k)
    cgp = inv.cg({"eps": 1e-10, "maxiter": 2000})
    X = inv.preconditioned(pc.eo2_ne(), cgp)(packed)(P)
    assert cgp.last.converged
    its = []
    for k in range(nrhs):
        cgs = inv.cg({"eps": 1e-10, "maxiter": 2000})
        x = inv.preconditioned(pc.eo2_ne(), cgs)(single)(to_gpu(single, srcs[k]))[:]
        its.append(cgs.last.iterations)
        assert rel(X.get_natural(k), x) < 1e-12
    assert cgp.last.iterations == max(its)


@pytest.mark.parametrize("kind,params,nrhs,dims", [
    ("wilson_clover", WC, 8, [4, 4, 4, 8]),
    ("wilson_clover", WC, 12, [8, 4, 4, 4]),
    ("mobius", dict(MOB, mass_plus=0.1, mass_minus=0.1), 2, [4, 4, 4, 8]),
    # 2048 tiles of one 4D site: more than a wave of resident blocks, so the
    # reducing launches loop over tiles
    ("mobius", dict(MOB, Ls=12, mass_plus=0.1, mass_minus=0.1), 12, [8, 8, 8, 8]),
])
def test_packed_single_precision_inner_solve_vs_oracle(kind, params, nrhs, dims):
    """Packed right-hand sides with an FP32 inner operator (the shared-memory
    link hop, reducing launches included): M per rhs within the FP32
    tolerance, and the defect-corrected mixed solve of every rhs to the FP64
    oracle's true residual 1e-10."""
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 31).U
    ref = _oracle(kind, U, dims, params)
    packed = gpu_op(kind, U, dims, g.double, n_rhs=nrhs, **params)
    p32 = packed.converted(g.single)
    srcs = [rand_field(ref.shape(), 60 + k) for k in range(nrhs)]
    P, P32 = packed.F_lattice(), p32.F_lattice()
    for k in range(nrhs):
        P.set_natural(srcs[k], k)
        P32.set_natural(srcs[k], k)
    out = p32.M(P32)
    for k in range(nrhs):
        assert rel(out.get_natural(k), ref.apply("M", srcs[k])) < TOL["single"], k
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    dc = inv.defect_correcting(inv.mixed_precision(inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": 1e-5, "maxiter": 4000})),
                                                   g.single, g.double), eps=1e-10, maxiter=40)
    X = dc(packed)(P)
    for k in range(nrhs):
        r = srcs[k] - ref.apply("M", X.get_natural(k))
        assert np.sqrt(o.norm2(r) / o.norm2(srcs[k])) < 1e-10, k


def test_half_precision_storage_operator():
    """FP16 spinor storage with a per-site FP32 scale: M agrees with FP32 to
    the storage precision (2^-11 relative per component)."""
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 13).U
    s = rand_field((int(np.prod(dims)), 4, 3), 5)
    ref = o.wilson_clover(U, dims, **WC).apply("M", s)
    for kind, P, tol in [("wilson_clover", g.single, 1e-6), ("wilson_clover", g.half, 3e-3)]:
        op = gpu_op(kind, U, dims, P, **WC)
        out = op.M(to_gpu(op, s))[:]
        assert rel(out, ref) < tol, P


def test_reductions_bitwise_deterministic():
    dims = [8, 8, 8, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 6).U
    op = gpu_op("wilson_clover", U, dims, g.double, **WC)
    b = to_gpu(op, rand_field((int(np.prod(dims)), 4, 3), 1))
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    slv = inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": 1e-8, "maxiter": 500}))(op)
    x1 = slv(b).tensor.clone()
    x2 = slv(b).tensor.clone()
    assert torch.equal(x1, x2)
    n1, n2 = g.norm2(b), g.norm2(b)
    assert n1 == n2


@pytest.mark.parametrize("prec,tol", [(g.double, 1e-14), (g.double_float, 1e-13), (g.single, 1e-6)])
def test_vector_algebra_matches_numpy(prec, tol):
    """norm2, inner_product, axpy and the fused axpy_norm2 and
    inner_product_norm2 (lib/gpt/core/transform.py:101-153) against numpy on
    full fields, one and three packed right-hand sides."""
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 8).U
    V = int(np.prod(dims))
    for nrhs in (1, 3):
        op = gpu_op("wilson_clover", U, dims, g.double, **dict(WC, n_rhs=nrhs))
        op = op if prec is g.double else op.converted(prec)
        xs = [rand_field((V, 4, 3), 10 + k) for k in range(nrhs)]
        ys = [rand_field((V, 4, 3), 20 + k) for k in range(nrhs)]
        x, y = op.F_lattice(), op.F_lattice()
        x[:] = xs[0] if nrhs == 1 else np.stack(xs)
        y[:] = ys[0] if nrhs == 1 else np.stack(ys)
        a = [0.3 - 0.7j, 1.5 + 0.2j, -0.4j][:nrhs]
        d = op.F_lattice()
        n2 = g.axpy_norm2(d, a if nrhs > 1 else a[0], x, y)
        n2 = [n2] if nrhs == 1 else n2
        got = d[:] if nrhs > 1 else [d[:]]
        for k in range(nrhs):
            want = a[k] * xs[k] + ys[k]
            assert np.linalg.norm(got[k] - want) / np.linalg.norm(want) < tol
            assert abs(n2[k] / np.vdot(want, want).real - 1) < tol
        ip, nx = g.inner_product_norm2(x, y)
        ip, nx = ([ip], [nx]) if nrhs == 1 else (ip, nx)
        for k in range(nrhs):
            assert abs(ip[k] - np.vdot(xs[k], ys[k])) / abs(np.vdot(xs[k], ys[k])) < tol
            assert abs(nx[k] / np.vdot(xs[k], xs[k]).real - 1) < tol


@pytest.mark.parametrize("kind,params", [("wilson_clover", WC), ("mobius", dict(MOB, mass_plus=0.1, mass_minus=0.1))])
def test_device_loop_equals_host_checked_graphs(kind, params):
    """The CG loop as host-checked graphs (the default 16 and 8 iterations),
    as one conditional-while graph on the device and as plain host launches
    (profile) runs the same kernels: bitwise equal solutions and the same
    iteration count."""
    dims = [4, 4, 4, 8]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.4, 33).U
    op = gpu_op(kind, U, dims, g.double, **params)
    b = to_gpu(op, rand_field(op.F_lattice()[:].shape, 3))
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    out = []
    for K, prof in ((0, False), (8, False), (-1, False), (-1, False), (0, True)):
        cg = inv.cg({"eps": 1e-10, "maxiter": 2000, "iterations_per_graph": K, "profile": prof})
        x = inv.preconditioned(pc.eo2_ne(), cg)(op)(b)
        assert cg.last.converged
        out.append((cg.last.iterations, x[:]))
    assert len({o[0] for o in out}) == 1
    assert all(np.array_equal(out[0][1], o[1]) for o in out[1:])


def test_cg_maxiter_reports_not_converged():
    dims = [4, 4, 4, 4]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 6).U
    op = gpu_op("wilson_clover", U, dims, g.double, **WC)
    b = to_gpu(op, rand_field((int(np.prod(dims)), 4, 3), 1))
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": 1e-14, "maxiter": 3})
    inv.preconditioned(pc.eo2_ne(), cg)(op)(b)
    assert cg.last.iterations == 3 and not cg.last.converged
    cg2 = inv.cg({"eps": 1e-14, "maxiter": 3, "fail_if_not_converged": True})
    with pytest.raises(ValueError):
        inv.preconditioned(pc.eo2_ne(), cg2)(op)(b)


def test_zero_source_gives_zero_solution():
    dims = [4, 4, 4, 4]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 6).U
    op = gpu_op("wilson_clover", U, dims, g.double, **WC)
    b = op.F_lattice()
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": 1e-10, "maxiter": 100})
    x = inv.preconditioned(pc.eo2_ne(), cg)(op)(b)
    assert cg.last.iterations == 0
    assert float(np.abs(x[:]).max()) == 0.0


def test_api_errors_are_raised():
    dims = [4, 4, 4, 4]
    U = g.qcd.gauge.random_su3(g.grid(dims), 0.3, 6).U
    op = gpu_op("wilson_clover", U, dims, g.double, **WC)
    a = op.F_lattice()
    with pytest.raises(g._lib.GBFError):
        op._apply("M", a, a)  # src == dst is rejected as in the reference
    with pytest.raises(ValueError):
        g.grid([3, 4, 4, 4])
