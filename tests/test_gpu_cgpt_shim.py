"""The cgpt-signature functions of gpt_gb300.cgpt (create / update / set_mass
/ delete / apply_fermion_operator, lib/cgpt/lib/operators.cc:34-107) on
numpy natural-layout lattices, every opcode of
lib/cgpt/lib/operators/types.h that the hot path uses (2001-2015, 3001, 3002,
4001, 4002) against the oracle; relative 1e-13 in FP64 (the reference's
fingerprint tolerance, tests/qcd/fermion_operators.py:527)."""
import numpy as np
import pytest

import oracle as o

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # collected on CPU hosts, skipped there
    pytest.skip("needs a GPU", allow_module_level=True)

from gpt_gb300 import cgpt  # noqa: E402
from gpt_gb300.qcd import gauge as G  # noqa: E402
from gpt_gb300 import core  # noqa: E402

TOL = 1e-13
DIMS = [4, 4, 2, 4]
PHASES = [1.0, 1.0, 1.0, -1.0]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _fields(shape, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(shape) + 1j * r.standard_normal(shape)


def _gauge(seed):
    return G.random_su3(core.grid(DIMS), 0.4, seed).U


def _check_all_opcodes(ptr, ref, five):
    V = ref.V
    shape = ref.shape()
    par = o.parity_of_sites(DIMS).reshape((-1,) + (1,) * (len(shape) - 1))
    src = _fields(shape, 1)
    # full-lattice opcodes
    for code, name in [(2001, "M"), (2002, "Mdag"), (2009, "Mdiag"), (2010, "Dminus"), (2011, "DminusDag"),
                       (3001, "Dhop"), (4001, "DhopDag")]:
        dst = np.zeros(shape, np.complex128)
        assert cgpt.apply_fermion_operator(ptr, code, [src], [dst]) == 0.0
        if not five and name.startswith("Dminus"):
            want = src  # Wilson: Dminus is the identity (reference/wilson_clover.py:174-176)
        else:
            want = ref.apply(name, src)
        assert rel(dst, want) < TOL, name
    # even-odd opcodes on checkerboarded lattices
    for code, name, flip in [(2003, "Meooe", True), (2004, "MeooeDag", True), (2005, "Mooee", False),
                             (2006, "MooeeDag", False), (2007, "MooeeInv", False), (2008, "MooeeInvDag", False),
                             (3002, "DhopEO", True), (4002, "DhopEODag", True)]:
        for sp in (0, 1):
            s = cgpt.checkerboarded(src * (par == sp), sp)
            dst = cgpt.checkerboarded(np.zeros(shape, np.complex128), sp)
            cgpt.apply_fermion_operator(ptr, code, [s], [dst])
            dp = 1 - sp if flip else sp
            assert dst.parity == dp
            if name.startswith("DhopEO"):
                # the hopping term alone, from parity sp to dp
                want = ref.apply("Dhop" if name == "DhopEO" else "DhopDag", np.asarray(s)) * (par == dp)
            else:
                want = ref.apply(name, np.asarray(s), dp)
            assert rel(np.asarray(dst), want) < TOL, (name, sp)
    # imports and exports (4D <-> 5D; copies for Wilson)
    s4 = _fields((V, 4, 3), 2)
    for code, fn in [(2012, "import_physical_source"), (2013, "import_unphysical")]:
        dst = np.zeros(shape, np.complex128)
        cgpt.apply_fermion_operator(ptr, code, [s4], [dst])
        want = getattr(ref, fn)(s4) if five else s4
        assert rel(dst, want) < TOL, code
    for code, fn in [(2014, "export_physical_solution"), (2015, "export_physical_source")]:
        dst = np.zeros((V, 4, 3), np.complex128)
        cgpt.apply_fermion_operator(ptr, code, [src], [dst])
        want = getattr(ref, fn)(src) if five else src
        assert rel(dst, want) < TOL, code


def test_wilson_clover_through_cgpt_signatures():
    U = _gauge(3)
    p = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=PHASES, cF=1, isAnisotropic=False, xi_0=1.0, nu=1.0)
    ptr = cgpt.create_fermion_operator("wilson_clover", "double", dict(p, U_grid=DIMS, U=[U[mu] for mu in range(4)]))
    try:
        _check_all_opcodes(ptr, o.wilson_clover(U, DIMS, **p), False)
        # set_mass (implementation.h:21-29) then update with a new field, as
        # interface.py:40-44 re-uses a pooled operator
        cgpt.set_mass_fermion_operator(ptr, {"mass": -0.05})
        src = _fields((int(np.prod(DIMS)), 4, 3), 4)
        dst = np.zeros_like(src)
        cgpt.apply_fermion_operator(ptr, 2001, [src], [dst])
        assert rel(dst, o.wilson_clover(U, DIMS, **dict(p, mass=-0.05)).apply("M", src)) < TOL
        s = cgpt.checkerboarded(src * (o.parity_of_sites(DIMS) == 1)[:, None, None], 1)
        cgpt.apply_fermion_operator(ptr, 2007, [s], [dst])
        assert rel(dst, o.wilson_clover(U, DIMS, **dict(p, mass=-0.05)).apply("MooeeInv", np.asarray(s), 1)) < TOL
        U2 = _gauge(5)
        cgpt.update_fermion_operator(ptr, {"U": U2})
        cgpt.apply_fermion_operator(ptr, 2001, [src], [dst])
        assert rel(dst, o.wilson_clover(U2, DIMS, **dict(p, mass=-0.05)).apply("M", src)) < TOL
    finally:
        assert cgpt.delete_fermion_operator(ptr) == 0
    with pytest.raises(RuntimeError):
        cgpt.apply_fermion_operator(ptr, 2001, [src], [dst])


def test_mobius_through_cgpt_signatures():
    U = _gauge(6)
    Ls = 6
    p = dict(mass_plus=0.05, mass_minus=0.09, b=1.5, c=0.5, M5=1.8, boundary_phases=PHASES)
    ptr = cgpt.create_fermion_operator("mobius", "double", dict(p, U_grid=DIMS, F_grid=[Ls] + DIMS, U=U))
    try:
        _check_all_opcodes(ptr, o.mobius(U, DIMS, Ls=Ls, **p), True)
        cgpt.set_mass_fermion_operator(ptr, {"mass_plus": 0.02, "mass_minus": 0.03})
        ref = o.mobius(U, DIMS, Ls=Ls, **dict(p, mass_plus=0.02, mass_minus=0.03))
        src = _fields(ref.shape(), 7)
        dst = np.zeros_like(src)
        cgpt.apply_fermion_operator(ptr, 2001, [src], [dst])
        assert rel(dst, ref.apply("M", src)) < TOL
    finally:
        cgpt.delete_fermion_operator(ptr)


def test_multi_rhs_wilson_and_errors():
    U = _gauge(8)
    p = dict(mass=0.2, csw_r=1.0, csw_t=1.0, boundary_phases=PHASES)
    n = 3
    ptr = cgpt.create_fermion_operator("wilson_clover", "double",
                                       dict(p, U_grid=DIMS, F_grid=[n] + DIMS, multi_rhs=True, Ls=n, U=U))
    try:
        ref = o.wilson_clover(U, DIMS, **p)
        V = ref.V
        src = _fields((V, n, 4, 3), 9)
        dst = np.zeros_like(src)
        cgpt.apply_fermion_operator(ptr, 2001, [src], [dst])
        for k in range(n):
            assert rel(dst[:, k], ref.apply("M", np.ascontiguousarray(src[:, k]))) < TOL
        with pytest.raises(RuntimeError, match="checkerboarded"):
            cgpt.apply_fermion_operator(ptr, 2003, [src], [dst])
    finally:
        cgpt.delete_fermion_operator(ptr)
    with pytest.raises(RuntimeError, match="Unknown precision"):
        cgpt.create_fermion_operator("wilson_clover", "quad", dict(p, U_grid=DIMS, U=U))
