"""Pin the CPU oracle to the reference's own golden values.

The golden numbers live in tests/golden/reference_goldens.json (extracted from
the lehner/gpt test files by tests/golden/make_reference_goldens.py).  Passing
these tests means the oracle reproduces gpt's RNG bit-exactly and Grid's
Wilson, Wilson-clover and Mobius operators to the reference's fingerprint
tolerance (relative 1e-13, tests/qcd/fermion_operators.py:527).
"""
import hashlib
import json
import os
import struct

import numpy as np
import pytest

import oracle as o

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def test_sha256_matches_hashlib():
    data = GOLD["sha256"]["input"].encode()
    assert o.sha256_words(data) == list(struct.unpack(">8I", hashlib.sha256(data).digest()))
    for n in [0, 1, 55, 56, 63, 64, 65, 119, 120, 200]:
        d = bytes((i * 7 + 3) % 256 for i in range(n))
        assert o.sha256_words(d) == list(struct.unpack(">8I", hashlib.sha256(d).digest()))


def test_plaquette_goldens():
    # tests/random/simple.py:17-31: one engine, three grids in sequence
    rng = o.random(GOLD["plaquette"]["seed"])
    for case in GOLD["plaquette"]["cases"]:
        g = o.grid(case["grid"])
        U = rng.gauge(g, case["scale"])
        if case.get("single"):
            U = U.astype(np.complex64).astype(np.complex128)
        p = o.plaquette(U, g.dims)
        assert abs(p - case["plaquette"]) ** 2 < case["tol_sq"]
        for mu in range(4):
            dev = np.einsum("vji,vjk->vik", U[mu].conj(), U[mu]) - np.eye(3)
            assert np.linalg.norm(dev) ** 2 / np.linalg.norm(U[mu]) ** 2 < case["tol_sq"]


def _pick(v, dims, coords):
    v = v[:, 0].reshape(dims[::-1])
    return np.array([v[tuple(c[::-1])].real for c in coords])


def test_normal_samples_and_choice():
    # tests/random/simple.py:38-141: a fresh engine draws zn/normal scalars,
    # then samples a complex field twice (second time after 1000 refills)
    ns = GOLD["normal_samples"]
    rng = o.random(ns["seed"])
    for _ in range(10000):
        rng.zn()
    for _ in range(10000):
        rng.zn(n=3)
    for _ in range(10000):
        rng.normal()
    g = o.grid(ns["grid"])
    v = rng.normal(g)
    assert np.linalg.norm(_pick(v, ns["grid"], ns["coords"]) - ns["after_0"]) < ns["tol"]
    for _ in range(1000):
        v = rng.normal(g)
    assert np.linalg.norm(_pick(v, ns["grid"], ns["coords"]) - ns["after_1000"]) < ns["tol"]
    assert rng.choice(["A", "B", "C"], 10) == GOLD["choice"]["abc_10"]
    assert list(rng.choice(np.array([1, 2, 3]), 5)) == GOLD["choice"]["123_5"]


def _fingerprint_fields(dims, Ls=None):
    fp = GOLD["fingerprints"]
    rng = o.random(fp["seed"])
    g4 = o.grid(dims)
    U = rng.gauge(g4)
    f = {"U": U}
    if Ls is not None:
        g5 = o.grid([Ls] + dims)
        f["src5"], f["dst5"] = rng.spincolor(g5), rng.spincolor(g5)
    f["src4"], f["dst4"] = rng.spincolor(g4), rng.spincolor(g4)
    return f


@pytest.mark.parametrize("name", ["wilson", "wilson_clover"])
def test_wilson_clover_fingerprints(name):
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp[name]
    f = _fingerprint_fields(dims)
    op = o.wilson_clover(f["U"], dims, **case["params"])
    for tag, ref in case["matrices"].items():
        opname = {"": "M", ".Mdiag": "Mdiag"}[tag]
        X = o.inner(f["dst4"], op.apply(opname, f["src4"]))
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (name, tag, X)


def test_wilson_twisted_mass_fingerprint():
    """tests/qcd/fermion_operators.py:366-386, 519-523: Grid's WilsonTMFermion."""
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp["wilson_twisted_mass"]
    f = _fingerprint_fields(dims)
    op = o.wilson_twisted_mass(f["U"], dims, **case["params"])
    for tag, ref in case["matrices"].items():
        opname = {"": "M", ".Mdiag": "Mdiag"}[tag]
        X = o.inner(f["dst4"], op.apply(opname, f["src4"]))
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (tag, X)


def test_zmobius_fingerprint():
    """tests/qcd/fermion_operators.py:400-426: Grid's ZMobiusFermion, complex
    per-slice b_s, c_s from omega (lib/gpt/qcd/fermion/zmobius.py:31-34), the
    c_s K term scaled by the output slice."""
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp["zmobius"]
    p = case["params"]
    f = _fingerprint_fields(dims, Ls=len(p["omega"]))
    op = o.zmobius(f["U"], dims, **p)
    for tag, ref in case["matrices"].items():
        if tag == ".ImportPhysicalFermionSource":
            X = o.inner(f["dst5"], op.import_physical_source(f["src4"]))
        else:
            X = o.inner(f["dst5"], op.apply("M" if tag == "" else "Mdiag", f["src5"]))
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (tag, X)


@pytest.mark.parametrize("name", ["mobius", "mobius_axial_mass"])
def test_mobius_fingerprints(name):
    fp = GOLD["fingerprints"]
    dims = fp["grid"]
    case = fp[name]
    p = case["params"]
    f = _fingerprint_fields(dims, Ls=p["Ls"])
    op = o.mobius(f["U"], dims, **p)
    for tag, ref in case["matrices"].items():
        if tag == ".ImportPhysicalFermionSource":
            X = o.inner(f["dst5"], op.import_physical_source(f["src4"]))
        else:
            X = o.inner(f["dst5"], op.apply({"": "M", ".Mdiag": "Mdiag"}[tag], f["src5"]))
        assert abs(X - complex(*ref)) / abs(X) < fp["rel_tol"], (name, tag, X)


def test_eo_decomposition_identities():
    # M restricted to a parity equals Mooee + Meooe (fermion_operators.py:677-695)
    dims = [4, 4, 4, 8]
    U = o.synthetic_gauge(dims, 0.5, 7)
    rng = np.random.default_rng(1)
    src = rng.standard_normal((np.prod(dims), 4, 3)) + 1j * rng.standard_normal((np.prod(dims), 4, 3))
    for op in [o.wilson_clover(U, dims, mass=0.1, csw_r=1.0, csw_t=1.0),
               o.mobius(U, dims, Ls=4, b=1.5, c=0.5, M5=1.8, mass=0.05)]:
        s = src if op.n5 == 1 else np.repeat(src[:, None], op.n5, axis=1) * (1 + np.arange(op.n5))[None, :, None, None]
        full = op.apply("M", s)
        for p in [o.EVEN, o.ODD]:
            part = op.apply("Meooe", s, p) + op.apply("Mooee", s, p)
            mask = o.parity_of_sites(dims) == p
            assert np.linalg.norm((full - part)[mask]) / np.linalg.norm(full[mask]) < 1e-14
        # adjoint consistency <a, M b> = conj(<b, M^+ a>)
        a = np.roll(s, 3)
        for m, md in [("M", "Mdag"), ("Dhop", "DhopDag")]:
            x1 = o.inner(a, op.apply(m, s))
            x2 = np.conj(o.inner(s, op.apply(md, a)))
            assert abs(x1 - x2) / abs(x1) < 1e-13
        # inverse consistency of Mooee
        for p in [o.EVEN, o.ODD]:
            y = op.apply("MooeeInv", op.apply("Mooee", s, p), p)
            mask = o.parity_of_sites(dims) == p
            assert np.linalg.norm((y - s)[mask]) / np.linalg.norm(s[mask]) < 1e-13


def test_unphysical_import_and_physical_source_export():
    """Opcodes 2013 and 2015 (lib/gpt/qcd/fermion/operator/base.py:147-164):
    ImportPhysicalFermionSource = Dminus ImportUnphysicalFermion (its wall
    placement is pinned by the reference's .ImportPhysicalFermionSource
    fingerprint above), and ExportPhysicalFermionSource is the adjoint of
    ImportUnphysicalFermion, as lib/gpt/qcd/fermion/preconditioner/physical.py:36-39
    uses it (the adjoint of the physical import = ExportPhysicalFermionSource
    Dminus^+).  Wilson: both are copies."""
    dims = [4, 4, 2, 4]
    U = o.synthetic_gauge(dims, 0.4, 5)
    rng = np.random.default_rng(8)
    V = int(np.prod(dims))
    e = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    for m in [o.mobius(U, dims, Ls=6, b=1.5, c=0.5, M5=1.8, mass=0.1),
              o.zmobius(U, dims, omega=[0.8 + 0.3j, 1.1, 0.6 - 0.1j, 1.4], b=1.2, c=0.3, M5=1.8, mass=0.07)]:
        p = rng.standard_normal(m.shape()) + 1j * rng.standard_normal(m.shape())
        a = o.inner(m.import_unphysical(e), p)
        b = o.inner(e, m.export_physical_source(p))
        assert abs(a - b) / abs(a) < 1e-14
        y = m.import_physical_source(e)
        assert np.linalg.norm(m.apply("Dminus", m.import_unphysical(e)) - y) / np.linalg.norm(y) < 1e-15
        # physical.py:36-39: <Import_phys e, p> = <e, ExportSource(Dminus^+ p)>
        c = o.inner(y, p)
        d = o.inner(e, m.export_physical_source(m.apply("DminusDag", p)))
        assert abs(c - d) / abs(c) < 1e-13
    w = o.wilson_clover(U, dims, mass=0.1, csw_r=1.0, csw_t=1.0)
    for name in ["ImportUnphysicalFermion", "ExportPhysicalFermionSource"]:
        assert np.array_equal(w.apply(name, e), e)


def test_oracle_solvers_true_residual():
    dims = [4, 4, 4, 8]
    U = o.synthetic_gauge(dims, 0.5, 3)
    rng = np.random.default_rng(2)
    op = o.wilson_clover(U, dims, mass=0.1, csw_r=1.0, csw_t=1.0, with_single=True)
    src = rng.standard_normal((op.V, 4, 3)) + 1j * rng.standard_normal((op.V, 4, 3))
    x, it, res = op.eo2ne_cg(src, 1e-10, 1000)
    assert it > 0
    r = src - op.apply("M", x)
    assert np.sqrt(o.norm2(r) / o.norm2(src)) < 1e-8
    x2, it2, nout, tres = op.defect_correcting(src, 1e-10, 20, 1e-5, 1000)
    assert tres < 1e-10
    assert np.sqrt(o.norm2(x - x2) / o.norm2(x)) < 1e-8


# ---------------------------------------------------------------------------
# solve-level goldens: point-source propagators of the RNG's gauge fields
# (single precision links, as in the reference), contracted to correlators
# ---------------------------------------------------------------------------
def _point_propagator_correlator(solve_column, V, point_index, n_t, per_slice):
    corr = np.zeros(n_t)
    extra = []
    for col in range(12):
        src = np.zeros((V, 4, 3), dtype=np.complex128)
        src[point_index, col // 3, col % 3] = 1.0
        x4, aux = solve_column(src)
        corr += (np.abs(x4.reshape(n_t, per_slice, 12)) ** 2).sum(axis=(1, 2))
        extra.append(aux)
    return corr, extra


def test_wilson_point_correlator_golden():
    """tests/qcd/fermion_operators.py:190-218: the eo2_ne propagator of a
    point source on g.qcd.gauge.random(rng "test") links in single precision,
    kappa 0.137, boundary phases exp(i k), contracted to
    sum_x tr(D(x) D(x)^+) per time slice, within the reference's 1e-5."""
    G = GOLD["wilson_correlator"]
    dims = G["grid"]
    g = o.grid(dims)
    U = o.random(G["seed"]).gauge(g, G["gauge_scale"]).astype(np.complex64).astype(np.complex128)
    ph = [complex(np.cos(k), np.sin(k)) for k in G["boundary_phases_exp_i"]]
    w = o.wilson_clover(U, dims, kappa=G["kappa"], boundary_phases=ph)
    p = G["point"]
    idx = p[0] + dims[0] * (p[1] + dims[1] * (p[2] + dims[2] * p[3]))

    def solve(src):
        x, it, res = w.eo2ne_cg(src, 1e-8, 5000)
        return x, it

    corr, its = _point_propagator_correlator(solve, g.V, idx, dims[3], g.V // dims[3])
    assert np.linalg.norm(corr - np.array(G["correlator"])) < G["tol"]


def test_mobius_point_correlator_and_J5q_goldens():
    """tests/qcd/domain_wall.py:171-274: Mobius (Ls 12, b 1.5, c 0.5, M5 1.8,
    mass 0.08) propagator of a point source, Import -> eo2_ne CG -> Export,
    on g.qcd.gauge.random(rng "test", scale 2) links in single precision:
    the correlator sum_x tr(D D^+) per time slice (eps_qm < 1e-5) and the
    midpoint density J5q = P+ psi_{Ls/2-1} + P- psi_{Ls/2} of the 5D
    solution (mobius.py:55-61) contracted the same way (within 1e-5); and
    the correlator of the zmobius operator of domain_wall.py:91-112 against
    the same golden (eps_qz < 5e-4)."""
    G = GOLD["mobius_correlators"]
    dims = G["grid"]
    g = o.grid(dims)
    U = o.random(G["seed"]).gauge(g, G["gauge_scale"]).astype(np.complex64).astype(np.complex128)
    prm = G["params"]
    Ls = int(prm["Ls"])
    qm = o.mobius(U, dims, Ls=Ls, b=prm["b"], c=prm["c"], M5=prm["M5"], mass=prm["mass"],
                  boundary_phases=prm["boundary_phases"])
    p = G["point"]
    idx = p[0] + dims[0] * (p[1] + dims[1] * (p[2] + dims[2] * p[3]))
    n_t, per = dims[3], g.V // dims[3]
    j5 = np.zeros(n_t)

    def solve(src):
        x5, it, res = qm.eo2ne_cg(qm.import_physical_source(src), 1e-7, 20000)
        mid = np.concatenate([x5[:, Ls // 2 - 1, 0:2], x5[:, Ls // 2, 2:4]], axis=1)  # [V, 4, 3]
        return qm.export_physical_solution(x5), mid

    corr, mids = _point_propagator_correlator(solve, g.V, idx, n_t, per)
    for mid in mids:
        j5 += (np.abs(mid.reshape(n_t, per, 12)) ** 2).sum(axis=(1, 2))
    assert np.linalg.norm(corr - np.array(G["correlator"])) / len(corr) < G["correlator_tol"]
    assert np.linalg.norm(j5 - np.array(G["J5q"])) < G["J5q_tol"]
    # the J5q values are O(1e-5): check them relatively as well
    assert np.abs(j5 / np.array(G["J5q"]) - 1).max() < 1e-3
    # zmobius (Ls 10, complex omega) approximating this Mobius operator: its
    # correlator against the same golden, the reference's eps_qz < 5e-4
    zp = G["zmobius_params"]
    qz = o.zmobius(U, dims, omega=zp["omega"], b=zp["b"], c=zp["c"], M5=zp["M5"], mass=zp["mass"],
                   boundary_phases=zp["boundary_phases"])

    def solve_z(src):
        x5, it, res = qz.eo2ne_cg(qz.import_physical_source(src), 1e-6, 20000)
        return qz.export_physical_solution(x5), it

    corr_z, _ = _point_propagator_correlator(solve_z, g.V, idx, n_t, per)
    assert np.linalg.norm(corr_z - np.array(G["correlator"])) / len(corr_z) < G["zmobius_correlator_tol"]
