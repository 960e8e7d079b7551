"""CPU oracle for the gpt fermion-matrix hot path -- TEST INFRASTRUCTURE ONLY.

This package is the oracle for the CUDA path in ``gpt_gb300``.  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference leg of
``bench.py`` may import it; the product never does.

It wraps ``oracle.cpp`` (a C++17/OpenMP restatement of the reference's
algorithms, each function citing the reference file it follows) with numpy:

* gpt's random number generator (``lib/cgpt/lib/random/*.h``), bit-exact, so
  the reference's own golden values can be reproduced: RNG samples
  (``tests/random/simple.py:66-127``), plaquettes (``tests/random/simple.py:17-31``)
  and the Grid-produced operator fingerprints of
  ``tests/qcd/fermion_operators.py:338-524``.  Parity is therefore pinned to
  the reference's Grid operator through those golden values.
* Wilson-clover and Mobius operators, eo2_ne CG and defect correction.

Layouts ("natural", shared with the product's host interface):
  spinor   complex128 array [V, 4, 3] (site = x0 + L0*(x1 + L1*(x2 + L2*x3)))
  5D field complex128 array [V, Ls, 4, 3]
  gauge    complex128 array [4, V, 3, 3]
"""
import ctypes
import itertools
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

OPCODES = {
    "M": 2001, "Mdag": 2002, "Meooe": 2003, "MeooeDag": 2004, "Mooee": 2005, "MooeeDag": 2006,
    "MooeeInv": 2007, "MooeeInvDag": 2008, "Mdiag": 2009, "Dminus": 2010, "DminusDag": 2011,
    "ImportPhysicalFermionSource": 2012, "ImportUnphysicalFermion": 2013, "ExportPhysicalFermionSolution": 2014,
    "ExportPhysicalFermionSource": 2015,
    "Dhop": 3001, "DhopDag": 4001,
}
EVEN, ODD, FULL = 0, 1, 2
DIST = {"normal": 0, "cnormal": 1, "uniform_real": 2, "uniform_int": 3, "zn": 4}


def build(force=False):
    """Compile oracle.cpp into liboracle.so (g++, OpenMP)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src):
        return _LIB_PATH
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", _LIB_PATH + ".tmp", src]
    subprocess.check_call(cmd)
    os.replace(_LIB_PATH + ".tmp", _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P, D, I, L_ = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_long
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_rng_new.restype = P
        L.orc_rng_new.argtypes = [ctypes.c_char_p]
        L.orc_rng_free.argtypes = [P]
        L.orc_rng_scalar.argtypes = [P, I, D, D, P]
        L.orc_rng_sample.argtypes = [P, ctypes.c_char_p, I, P, I, D, D, I, P]
        L.orc_sha256.argtypes = [P, ctypes.c_size_t, P]
        L.orc_gauge_random.argtypes = [P, ctypes.c_char_p, P, D, P]
        L.orc_field_exp_i.argtypes = [P, L_]
        L.orc_plaquette.restype = D
        L.orc_plaquette.argtypes = [P, P]
        L.orc_wilson_clover_new.restype = P
        L.orc_wilson_clover_new.argtypes = [P, P, D, D, D, D, D, P, I]
        L.orc_wilson_twisted_mass_new.restype = P
        L.orc_wilson_twisted_mass_new.argtypes = [P, P, D, D, P, I]
        L.orc_zmobius_new.restype = P
        L.orc_zmobius_new.argtypes = [P, P, I, P, P, D, D, D, P, I, I]
        L.orc_mobius_new.restype = P
        L.orc_mobius_new.argtypes = [P, P, I, D, D, D, D, D, P, I]
        L.orc_op_free.argtypes = [P]
        L.orc_op_apply.argtypes = [P, I, P, P, I]
        L.orc_mobius_import.argtypes = [P, P, P, I]
        L.orc_eo2ne_cg.argtypes = [P, P, P, D, I, P]
        L.orc_eo2ne_cg_single.argtypes = [P, P, P, D, I, P]
        L.orc_defect_correcting.argtypes = [P, P, P, D, I, D, I, P, P]
        L.orc_num_threads.restype = I
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def num_threads():
    return lib().orc_num_threads()


def sha256_words(data: bytes):
    """SHA-256 state words H0..H7 of ``data`` (restated, checked against hashlib)."""
    buf = np.frombuffer(data, dtype=np.uint8).copy() if len(data) else np.zeros(1, np.uint8)
    out = np.zeros(8, np.uint32)
    lib().orc_sha256(_ptr(buf), len(data), _ptr(out))
    return [int(x) for x in out]


# ---------------------------------------------------------------------------
# grids and the random number generator
# ---------------------------------------------------------------------------
class grid:
    """A lattice geometry; each instance owns its own random stream key
    (the reference keys its per-grid streams by grid object)."""

    _counter = itertools.count()

    def __init__(self, dims):
        self.dims = [int(d) for d in dims]
        self.key = f"grid{next(grid._counter)}".encode()
        self.V = int(np.prod(self.dims))

    @property
    def L4(self):
        return self.dims[-4:]


class random:
    """gpt.random(seed) restated (engine "vectorized_ranlux24_389_64")."""

    def __init__(self, seed):
        self.obj = lib().orc_rng_new(seed.encode())

    def __del__(self):
        if getattr(self, "obj", None):
            lib().orc_rng_free(self.obj)
            self.obj = None

    def _lattice(self, g, dist, p0, p1, n_per_site):
        dims = np.array(g.dims, dtype=np.int64)
        out = np.zeros((g.V, n_per_site), dtype=np.complex128)
        _check(lib().orc_rng_sample(self.obj, g.key, len(g.dims), _ptr(dims), DIST[dist], p0, p1, n_per_site, _ptr(out)))
        return out

    def _scalar(self, dist, p0, p1):
        out = np.zeros(2, dtype=np.float64)
        _check(lib().orc_rng_scalar(self.obj, DIST[dist], p0, p1, _ptr(out)))
        return complex(out[0], out[1])

    # lattice samplers: n_per_site complex numbers per site
    def cnormal(self, g, n_per_site=12, mu=0.0, sigma=1.0):
        return self._lattice(g, "cnormal", mu, sigma, n_per_site)

    def normal(self, g=None, n_per_site=1, mu=0.0, sigma=1.0):
        if g is None:
            return self._scalar("normal", mu, sigma).real
        return self._lattice(g, "normal", mu, sigma, n_per_site)

    def uniform_real(self, g=None, n_per_site=1, min=0.0, max=1.0):
        if g is None:
            return self._scalar("uniform_real", min, max).real
        return self._lattice(g, "uniform_real", min, max, n_per_site)

    def uniform_int(self, min=0, max=1):
        return int(self._scalar("uniform_int", min, max).real)

    def zn(self, n=2):
        return self._scalar("zn", n, 0)

    def choice(self, array, n):
        if isinstance(array, np.ndarray):
            return np.take(array, [self.uniform_int(min=0, max=len(array) - 1) for i in range(n)], axis=0)
        return [array[self.uniform_int(min=0, max=len(array) - 1)] for i in range(n)]

    def gauge(self, g, scale=1.0):
        """g.qcd.gauge.random(grid, rng, scale): [4, V, 3, 3] SU(3) links."""
        dims = np.array(g.dims, dtype=np.int64)
        U = np.zeros((4, g.V, 3, 3), dtype=np.complex128)
        _check(lib().orc_gauge_random(self.obj, g.key, _ptr(dims), float(scale), _ptr(U)))
        return U

    def spincolor(self, g):
        """rng.cnormal(g.vspincolor(grid)) in natural layout."""
        a = self.cnormal(g, 12)
        if len(g.dims) == 5:  # [Ls, x, y, z, t] grid: s fastest
            return a.reshape(g.V // g.dims[0], g.dims[0], 4, 3)
        return a.reshape(g.V, 4, 3)


def plaquette(U, dims):
    U = np.ascontiguousarray(U, dtype=np.complex128)
    d = np.array(dims, dtype=np.int64)
    return lib().orc_plaquette(_ptr(U), _ptr(d))


def field_exp_i(X):
    """exp(i X) of a [V, 3, 3] field with the reference's global scaling rule."""
    X = np.ascontiguousarray(X, dtype=np.complex128).copy()
    _check(lib().orc_field_exp_i(_ptr(X), X.shape[0]))
    return X


# ---------------------------------------------------------------------------
# geometry helpers
# ---------------------------------------------------------------------------
def coords(dims):
    V = int(np.prod(dims))
    s = np.arange(V)
    out = []
    for L in dims:
        out.append(s % L)
        s = s // L
    return np.stack(out, axis=1)


def parity_of_sites(dims):
    return coords(dims).sum(axis=1) % 2


def _phases(boundary_phases):
    ph = np.zeros(8, dtype=np.float64)
    for mu, p in enumerate(boundary_phases):
        ph[2 * mu] = complex(p).real
        ph[2 * mu + 1] = complex(p).imag
    return ph


# ---------------------------------------------------------------------------
# operators
# ---------------------------------------------------------------------------
class _op:
    n5 = 1

    def __del__(self):
        if getattr(self, "obj", None):
            lib().orc_op_free(self.obj)
            self.obj = None

    def shape(self):
        return (self.V, 4, 3) if self.n5 == 1 else (self.V, self.n5, 4, 3)

    def apply(self, name, src, parity=FULL):
        """Apply an opcode to a natural-layout full-lattice field.  For the
        even-odd opcodes ``parity`` is the output parity; other sites are 0."""
        src = np.ascontiguousarray(src, dtype=np.complex128)
        dst = np.zeros(self.shape(), dtype=np.complex128)
        _check(lib().orc_op_apply(self.obj, OPCODES[name], _ptr(src), _ptr(dst), parity))
        return dst

    def eo2ne_cg(self, src, eps, maxiter):
        """preconditioned(eo2_ne(), cg(eps, maxiter)) applied to src."""
        src = np.ascontiguousarray(src, dtype=np.complex128)
        x = np.zeros(self.shape(), dtype=np.complex128)
        res = np.zeros(1)
        it = lib().orc_eo2ne_cg(self.obj, _ptr(src), _ptr(x), eps, maxiter, _ptr(res))
        if it <= -1000000000:
            raise RuntimeError(lib().orc_last_error().decode())
        return x, it, float(res[0])

    def eo2ne_cg_single(self, src, eps, maxiter):
        """The same solve with the single-precision operator (needs with_single=True)."""
        src = np.ascontiguousarray(src, dtype=np.complex128)
        x = np.zeros(self.shape(), dtype=np.complex128)
        res = np.zeros(1)
        it = lib().orc_eo2ne_cg_single(self.obj, _ptr(src), _ptr(x), eps, maxiter, _ptr(res))
        if it <= -1000000000:
            raise RuntimeError(lib().orc_last_error().decode())
        return x, it, float(res[0])

    def defect_correcting(self, src, eps, maxouter, eps_inner, maxinner):
        """defect_correcting(mixed_precision(preconditioned(eo2_ne, cg(eps_inner)), single, double), eps)."""
        src = np.ascontiguousarray(src, dtype=np.complex128)
        x = np.zeros(self.shape(), dtype=np.complex128)
        res = np.zeros(1)
        nout = np.zeros(1, dtype=np.int32)
        it = lib().orc_defect_correcting(self.obj, _ptr(src), _ptr(x), eps, maxouter, eps_inner, maxinner, _ptr(res), _ptr(nout))
        if it < 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return x, it, int(nout[0]), float(res[0])


class wilson_clover(_op):
    """g.qcd.fermion.wilson_clover / reference.wilson_clover parameters."""

    def __init__(self, U, dims, kappa=None, mass=None, csw_r=0.0, csw_t=0.0, xi_0=1.0, nu=1.0,
                 boundary_phases=(1, 1, 1, -1), with_single=False, **_ignored):
        if kappa is not None:
            assert mass is None
            mass = 1.0 / kappa / 2.0 - 4.0
        self.dims = list(dims)
        self.V = int(np.prod(dims))
        self.U = np.ascontiguousarray(U, dtype=np.complex128)
        d = np.array(dims, dtype=np.int64)
        ph = _phases(boundary_phases)
        self.obj = lib().orc_wilson_clover_new(_ptr(self.U), _ptr(d), float(mass), float(csw_r), float(csw_t),
                                               float(xi_0), float(nu), _ptr(ph), int(with_single))
        if not self.obj:
            raise RuntimeError(lib().orc_last_error().decode())


class wilson_twisted_mass(_op):
    """g.qcd.fermion.wilson_twisted_mass parameters (lib/gpt/qcd/fermion/wilson.py:99-107):
    Wilson hop, Mooee = (4 + mass) + i mu g5."""

    def __init__(self, U, dims, mass, mu, boundary_phases=(1, 1, 1, -1), with_single=False, **_ignored):
        self.dims = list(dims)
        self.V = int(np.prod(dims))
        self.U = np.ascontiguousarray(U, dtype=np.complex128)
        d = np.array(dims, dtype=np.int64)
        ph = _phases(boundary_phases)
        self.obj = lib().orc_wilson_twisted_mass_new(_ptr(self.U), _ptr(d), float(mass), float(mu), _ptr(ph),
                                                     int(with_single))
        if not self.obj:
            raise RuntimeError(lib().orc_last_error().decode())


class mobius(_op):
    """g.qcd.fermion.mobius parameters (b_s = b, c_s = c for all s)."""

    def __init__(self, U, dims, Ls, b, c, M5, mass=None, mass_plus=None, mass_minus=None,
                 boundary_phases=(1, 1, 1, -1), with_single=False, **_ignored):
        if mass is not None:
            mass_plus = mass_minus = mass
        self.dims = list(dims)
        self.V = int(np.prod(dims))
        self.n5 = int(Ls)
        self.U = np.ascontiguousarray(U, dtype=np.complex128)
        d = np.array(dims, dtype=np.int64)
        ph = _phases(boundary_phases)
        self.obj = lib().orc_mobius_new(_ptr(self.U), _ptr(d), int(Ls), float(b), float(c), float(M5),
                                        float(mass_plus), float(mass_minus), _ptr(ph), int(with_single))
        if not self.obj:
            raise RuntimeError(lib().orc_last_error().decode())

    # P+ on s=0 and P- on s=Ls-1, then Dminus: the convention that reproduces
    # the reference's ImportPhysicalFermionSource fingerprint
    IMPORT_VARIANT = 3

    def import_physical_source(self, src4, variant=None):
        v = self.IMPORT_VARIANT if variant is None else variant
        src4 = np.ascontiguousarray(src4, dtype=np.complex128)
        out = np.zeros(self.shape(), dtype=np.complex128)
        _check(lib().orc_mobius_import(self.obj, _ptr(src4), _ptr(out), int(v)))
        return out

    def export_physical_solution(self, x5):
        x5 = np.ascontiguousarray(x5, dtype=np.complex128)
        out = np.zeros((self.V, 4, 3), dtype=np.complex128)
        _check(lib().orc_op_apply(self.obj, OPCODES["ExportPhysicalFermionSolution"], _ptr(x5), _ptr(out), FULL))
        return out

    def import_unphysical(self, src4):
        """Opcode 2013: the walls of the physical import (P+ eta on s = 0,
        P- eta on s = Ls-1) without Dminus."""
        return self.import_physical_source(src4, variant=self.IMPORT_VARIANT & 1)

    def export_physical_source(self, x5):
        """Opcode 2015: P+ psi_0 + P- psi_{Ls-1}, the adjoint of import_unphysical."""
        x5 = np.ascontiguousarray(x5, dtype=np.complex128)
        out = np.zeros((self.V, 4, 3), dtype=np.complex128)
        _check(lib().orc_op_apply(self.obj, OPCODES["ExportPhysicalFermionSource"], _ptr(x5), _ptr(out), FULL))
        return out



class zmobius(mobius):
    """g.qcd.fermion.zmobius parameters (lib/gpt/qcd/fermion/zmobius.py:59-78):
    Ls = len(omega), per-slice complex b_s = ((b + c) / omega_s + (b - c)) / 2,
    c_s = ((b + c) / omega_s - (b - c)) / 2.  col_scale selects which slice
    index scales the c_s K term (output slice by default)."""

    def __init__(self, U, dims, omega, b, c, M5, mass=None, mass_plus=None, mass_minus=None,
                 boundary_phases=(1, 1, 1, -1), with_single=False, col_scale=False, **_ignored):
        if mass is not None:
            mass_plus = mass_minus = mass
        om = [complex(*w) if isinstance(w, (list, tuple)) else complex(w) for w in omega]
        Ls = len(om)
        bs = np.array([0.5 * ((b + c) / w + (b - c)) for w in om], dtype=np.complex128)
        cs = np.array([0.5 * ((b + c) / w - (b - c)) for w in om], dtype=np.complex128)
        self.bs, self.cs = bs, cs
        self.dims = list(dims)
        self.V = int(np.prod(dims))
        self.n5 = Ls
        self.U = np.ascontiguousarray(U, dtype=np.complex128)
        d = np.array(dims, dtype=np.int64)
        ph = _phases(boundary_phases)
        self.obj = lib().orc_zmobius_new(_ptr(self.U), _ptr(d), int(Ls), _ptr(bs), _ptr(cs), float(M5),
                                         float(mass_plus), float(mass_minus), _ptr(ph), int(with_single),
                                         int(bool(col_scale)))
        if not self.obj:
            raise RuntimeError(lib().orc_last_error().decode())

def inner(a, b):
    return complex(np.vdot(a.ravel(), b.ravel()))


def norm2(a):
    return float(np.vdot(a.ravel(), a.ravel()).real)


def synthetic_gauge(dims, eps, seed):
    """The benchmark gauge recipe: U = exp(i eps H), H Hermitian traceless with
    complex-Gaussian entries (numpy PCG64 seeded).  Same arrays feed the GPU
    and the oracle, so parity does not depend on this choice."""
    V = int(np.prod(dims))
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.standard_normal((4 * V, 3, 3)) + 1j * rng.standard_normal((4 * V, 3, 3))
    H = 0.5 * (A + np.conj(np.swapaxes(A, 1, 2)))
    tr = np.trace(H, axis1=1, axis2=2).real / 3.0
    H -= tr[:, None, None] * np.eye(3)[None]
    w, v = np.linalg.eigh(H)
    U = np.einsum("nij,nj,nkj->nik", v, np.exp(1j * eps * w), np.conj(v))
    return U.reshape(4, V, 3, 3)
