"""Fermion operators: g.qcd.fermion.wilson_clover, wilson_twisted_mass and mobius.

Mirrors lib/gpt/qcd/fermion/wilson.py:63-96 (parameter handling, kappa ->
mass), lib/gpt/qcd/fermion/mobius.py:25-117 and the operator object of
lib/gpt/qcd/fermion/operator/base.py:28-306 (method names, .converted(),
.updated(), .propagator(), .even_odd_sites_decomposed()).  Every method maps
to an opcode of the native library (lib/gpt/qcd/fermion/operator/interface.py:88-91
-> cgpt apply_fermion_operator), here gbf_apply of libgbferm.so.
"""
import copy as _copy
import ctypes

import numpy as np

from .. import _lib
from .. import core
from .gauge import gauge_field


class matrix_operator:
    """A linear map dst = A(src) on lattices, with optional adjoint/inverse."""

    def __init__(self, mat, adj_mat=None, inv_mat=None, adj_inv_mat=None, otype=None):
        self.mat = mat
        self.adj_mat = adj_mat
        self.inv_mat = inv_mat
        self.adj_inv_mat = adj_inv_mat

    def __call__(self, first, second=None):
        if second is None:
            src = first
            dst = self._new_dst(src)
            self.mat(dst, src)
            return dst
        self.mat(first, second)
        return first

    def _new_dst(self, src):
        return src.new()

    def __mul__(self, src):
        return self(src)

    def _with_dst(self, new_dst, new_dst_adj):
        if new_dst is not None:
            self._new_dst = new_dst
        self._new_dst_adj = new_dst_adj
        return self

    def adj(self):
        # operators between different vector spaces (the 4D <-> 5D imports and
        # exports) create the adjoint's destination in the other space
        nd = getattr(self, "_new_dst_adj", None)
        od = self.__dict__.get("_new_dst")
        return matrix_operator(self.adj_mat, self.mat, self.adj_inv_mat, self.inv_mat)._with_dst(nd, od)

    def inv(self):
        return matrix_operator(self.inv_mat, self.adj_inv_mat, self.mat, self.adj_mat)


def _params_struct(name, p, dims, Ls, n_rhs):
    s = _lib.gbf_params()
    for i in range(4):
        s.dims[i] = dims[i]
    s.Ls = Ls
    s.n_rhs = n_rhs
    ph = p.get("boundary_phases", [1, 1, 1, 1])
    for mu in range(4):
        s.boundary_phases[2 * mu] = complex(ph[mu]).real
        s.boundary_phases[2 * mu + 1] = complex(ph[mu]).imag
    s.reconstruct = int(p.get("reconstruct", -1))
    if name == "wilson_twisted_mass":
        s.mass = float(p["mass"])
        s.mu = float(p["mu"])
        s.xi_0 = s.nu = 1.0
    elif name == "wilson_clover":
        s.mass = float(p["mass"])
        s.csw_r = float(p.get("csw_r", 0.0))
        s.csw_t = float(p.get("csw_t", 0.0))
        s.xi_0 = float(p.get("xi_0", 1.0) or 1.0)
        s.nu = float(p.get("nu", 1.0) or 1.0)
        s.isAnisotropic = int(bool(p.get("isAnisotropic", False)))
    else:
        s.mass_plus = float(p["mass_plus"])
        s.mass_minus = float(p["mass_minus"])
        s.b = float(p["b"])
        s.c = float(p["c"])
        s.M5 = float(p["M5"])
        s.xi_0 = s.nu = 1.0
        if name == "zmobius":
            om = np.array([complex(w) for w in p["omega"]], dtype=np.complex128)
            s.keep_omega = om  # alive until gbf_create has read it
            s.omega = om.ctypes.data
    return s


class fermion_operator(matrix_operator):
    """Native fermion operator (cgpt_fermion_operator analogue)."""

    def __init__(self, name, U, params, precision=None, daggered=False, clover_from=None):
        self.name = name
        self.U = U
        self.params = dict(params)
        self.daggered = daggered
        prec = precision if precision is not None else U.grid.precision
        self.U_grid = U.grid.converted(prec)
        self.precision = prec
        self.Ls = int(params.get("Ls", 1)) if name in ("mobius", "zmobius") else 1
        self.n_rhs = int(params.get("n_rhs", 1))
        dims = self.U_grid.fdimensions
        self.F_layout = core.layout.get(self.U_grid, self.Ls, self.n_rhs, five_d=name in ("mobius", "zmobius"))
        self.U_layout = core.layout.get(self.U_grid, 1, self.n_rhs, five_d=False)
        L = _lib.load()
        s = _params_struct(name, self.params, dims, self.Ls, self.n_rhs)
        h = ctypes.c_void_p()
        _lib.check(L.gbf_create(name.encode(), prec.code, ctypes.byref(s), ctypes.byref(h)))
        self.obj = h
        uptr, on_dev = U.ptr()
        if clover_from is not None:
            _lib.check(L.gbf_update_gauge_from(self.obj, ctypes.c_void_p(uptr), on_dev, clover_from.obj, core.stream_ptr()))
        else:
            _lib.check(L.gbf_update_gauge(self.obj, ctypes.c_void_p(uptr), on_dev, core.stream_ptr()))
        self._register()

    def __del__(self):
        try:
            if getattr(self, "obj", None) is not None:
                _lib.load().gbf_delete(self.obj)
                self.obj = None
        except Exception:
            pass

    # ---- fields ----
    def F_lattice(self, cb=core.full):
        return core.lattice(self.F_layout, cb)

    def U_lattice(self, cb=core.full):
        return core.lattice(self.U_layout, cb)

    # ---- opcode application (interface.py:88-91) ----
    def _apply(self, opname, dst, src):
        code = _lib.OPCODES[opname]
        sp = src.cb.code
        _lib.check(_lib.load().gbf_apply(self.obj, code, _lib.ptrs([src.ptr]), _lib.ptrs([dst.ptr]), 1, sp, core.stream_ptr()))
        if opname in ("Meooe", "MeooeDag", "DhopEO", "DhopEODag"):
            dst.cb = src.cb.inv()
        elif src.cb is not core.full:
            dst.cb = src.cb

    def _op(self, name, name_dag, new_dst=None, inv=None, inv_dag=None, new_dst_adj=None):
        def m(n):
            return (lambda dst, src: self._apply(n, dst, src)) if n else None

        a, ad, i, idg = m(name), m(name_dag), m(inv), m(inv_dag)
        if self.daggered:
            a, ad, i, idg = ad, a, idg, i
            if new_dst_adj is not None:
                new_dst, new_dst_adj = new_dst_adj, new_dst
        return matrix_operator(a, ad, i, idg)._with_dst(new_dst, new_dst_adj)

    def _register(self):
        # base.py:84-169 (method registry)
        self.M = self._op("M", "Mdag")
        self.mat = self.M.mat
        self.adj_mat = self.M.adj_mat
        self.inv_mat = None
        self.adj_inv_mat = None
        self.Meooe = self._op("Meooe", "MeooeDag")
        self.Mooee = self._op("Mooee", "MooeeDag", inv="MooeeInv", inv_dag="MooeeInvDag")
        self.DhopEO = self._op("DhopEO", "DhopEODag")
        self.Dhop = self._op("Dhop", "DhopDag")
        self.Mdiag = self._op("Mdiag", None)
        self.Dminus = self._op("Dminus", "DminusDag")
        to_F = lambda src: self.F_lattice()
        to_U = lambda src: self.U_lattice()
        self.ImportPhysicalFermionSource = self._op("ImportPhysicalFermionSource", None, new_dst=to_F)
        self.ExportPhysicalFermionSolution = self._op("ExportPhysicalFermionSolution", None, new_dst=to_U)
        # opcodes 2013 / 2015 (base.py:147-164): the walls of the physical
        # import without Dminus, and its adjoint
        self.ImportUnphysicalFermion = self._op("ImportUnphysicalFermion", "ExportPhysicalFermionSource",
                                                new_dst=to_F, new_dst_adj=to_U)
        self.ExportPhysicalFermionSource = self._op("ExportPhysicalFermionSource", "ImportUnphysicalFermion",
                                                    new_dst=to_U, new_dst_adj=to_F)

    # ---- base.py:219-260 ----
    def converted(self, precision):
        # same links and clover at another precision: the clover term is
        # converted from this operator instead of rebuilt
        return type(self)(self.U, self.params, precision=precision, daggered=self.daggered, clover_from=self)

    def updated(self, U):
        return type(self)(U, self.params, precision=self.precision, daggered=self.daggered)

    def modified(self, **params):
        """The same operator with some parameters replaced (base.py:221-228),
        for example modified(mass=1.0) for the Pauli-Villars operator of
        MADWF; mass sets both Mobius masses, as the factories do."""
        p = {**self.params, **params}
        if "mass" in params and self.name in ("mobius", "zmobius"):
            p["mass_plus"] = p["mass_minus"] = float(params["mass"])
        if "kappa" in params and self.name in ("wilson_clover", "wilson_twisted_mass"):
            p["mass"] = 1.0 / float(params["kappa"]) / 2.0 - 4.0
            p.pop("kappa")
        return type(self)(self.U, p, precision=self.precision, daggered=self.daggered)

    def adj(self):
        return type(self)(self.U, self.params, precision=self.precision, daggered=not self.daggered)

    def propagator(self, solver):
        """base.py:270-286: Export * solver(op) * Import."""
        exp, imp = self.ExportPhysicalFermionSolution, self.ImportPhysicalFermionSource
        inv_matrix = solver(self)

        def prop(dst, src):
            t = imp(src)
            x = inv_matrix(t)
            exp(dst, x)

        return matrix_operator(prop)

    def bulk_propagator(self, solver):
        """Domain-wall operators (mobius.py:118-135): solver(op) * Import, the
        5D solution; bulk_propagator_to_propagator (= Export) projects it to
        the 4D propagator."""
        if self.name not in ("mobius", "zmobius"):
            raise NotImplementedError("bulk_propagator is defined for the domain-wall operators")
        imp = self.ImportPhysicalFermionSource
        inv_matrix = solver(self)

        def prop(dst, src):
            inv_matrix(dst, imp(src))

        m = matrix_operator(prop)
        m._new_dst = lambda src: self.F_lattice()
        return m

    def J5q(self, src5):
        """The midpoint density of a domain-wall field (mobius.py:55-61):
        dst4 = P+ psi_{Ls/2-1} + P- psi_{Ls/2}, as the chiral shift P^+
        (slice s gets P- psi_s + P+ psi_{s-1}) followed by a copy of slice
        Ls/2 into a 4D field."""
        if self.name not in ("mobius", "zmobius"):
            raise NotImplementedError("J5q is defined for the domain-wall operators")
        L = _lib.load()
        y = self.F_lattice()
        _lib.check(L.gbf_chiral_shift(src5.layout.op, src5.ptr, y.ptr, -1, 2, core.stream_ptr()))
        dst = self.U_lattice()
        _lib.check(L.gbf_copy_slices(dst.layout.op, dst.ptr, 0, y.layout.op, y.ptr, self.Ls // 2, 1, 1.0, 2,
                                     core.stream_ptr()))
        return dst

    @property
    def bulk_propagator_to_propagator(self):
        """mobius.py:69: the 4D solution P- psi_0 + P+ psi_{Ls-1} of a 5D field."""
        return self.ExportPhysicalFermionSolution

    def even_odd_sites_decomposed(self, parity):
        return _even_odd_sites(self, parity)

    def link_bytes(self):
        """Bytes per stored link (144 FP64, 72 FP32, 48 FP32 reconstruct-12)."""
        return _lib.load().gbf_link_bytes(self.obj)

    def tune(self, force=False):
        """Choose the kernels' block sizes for this operator by timing them
        (or re-apply the cached choice); returns {"tag", "params", "results"}."""
        from .. import tune as _tune

        return _tune.tune(self, force=force)

    # native eo2_ne + block CG on the device (gbf_solve_eo2ne_block_cg)
    def _solve_eo2ne_block_cg(self, dst, src, eps, maxiter, graph_iterations=0, profile=0):
        p = _lib.gbf_cg_params(float(eps), int(maxiter), 0, 0)
        r = _lib.gbf_cg_result()
        _lib.check(_lib.load().gbf_solve_eo2ne_block_cg(self.obj, src.ptr, dst.ptr, ctypes.byref(p), ctypes.byref(r),
                                                        core.stream_ptr()))
        return r

    # native eo2_ne + CG on the device (gbf_solve_eo2ne_cg)
    def _solve_eo2ne_cg(self, dst, src, eps, maxiter, graph_iterations=0, profile=0):
        p = _lib.gbf_cg_params(float(eps), int(maxiter), int(graph_iterations), int(profile))
        r = _lib.gbf_cg_result()
        _lib.check(_lib.load().gbf_solve_eo2ne_cg(self.obj, src.ptr, dst.ptr, ctypes.byref(p), ctypes.byref(r), core.stream_ptr()))
        return r


class _even_odd_sites:
    """base.py:288-306: DD = Mooee|D, CC = Mooee|C, CD/DC = Meooe."""

    def __init__(self, op, parity):
        self.op = op
        self.D = parity
        self.C = parity.inv()
        self.DD = op.Mooee
        self.CC = op.Mooee
        self.CD = op.Meooe
        self.DC = op.Meooe


def _std_params(params, kw):
    p = dict(params or {})
    p.update(kw)
    return p


def wilson_clover(U, params=None, **kw):
    """g.qcd.fermion.wilson_clover (lib/gpt/qcd/fermion/wilson.py:63-96)."""
    p = _std_params(params, kw)
    p = _copy.deepcopy(p)
    if p.get("kappa") is not None:
        assert p.get("mass") is None
        p["mass"] = 1.0 / p["kappa"] / 2.0 - 4.0
        del p["kappa"]
    p.setdefault("csw_r", 0.0)
    p.setdefault("csw_t", 0.0)
    p.setdefault("cF", 1)
    p.setdefault("n_rhs", 1)
    bp = p.get("boundary_phases")
    if bp is None:
        raise ValueError("boundary_phases required")
    if bp[-1] == 0.0:
        raise NotImplementedError("open boundary conditions are not implemented on this path")
    if p.get("cF", 1) != 1.0:
        raise ValueError("cF only with open boundaries (wilson.py:89-90)")
    return wilson_clover_operator(U, p)


class wilson_clover_operator(fermion_operator):
    def __init__(self, U, params, precision=None, daggered=False, clover_from=None):
        super().__init__("wilson_clover", U, params, precision, daggered, clover_from)


def wilson_twisted_mass(U, params=None, **kw):
    """g.qcd.fermion.wilson_twisted_mass (lib/gpt/qcd/fermion/wilson.py:99-107):
    the Wilson hop with Mooee = (4 + mass) + i mu gamma5 (Grid's WilsonTMFermion
    through lib/cgpt/lib/operators/wilson_twisted_mass.h:19-45)."""
    p = _std_params(params, kw)
    for k in ("mass", "mu", "boundary_phases"):
        if p.get(k) is None:
            raise ValueError(f"{k} required")
    p.setdefault("n_rhs", 1)
    return wilson_twisted_mass_operator(U, p)


class wilson_twisted_mass_operator(fermion_operator):
    def __init__(self, U, params, precision=None, daggered=False, clover_from=None):
        super().__init__("wilson_twisted_mass", U, params, precision, daggered)


def mobius(U, params=None, **kw):
    """g.qcd.fermion.mobius (lib/gpt/qcd/fermion/mobius.py:25-46, 325-327)."""
    p = _std_params(params, kw)
    if p.get("mass") is not None:
        p["mass_plus"] = p["mass"]
        p["mass_minus"] = p["mass"]
    if p.get("omega") is not None:
        # per-slice Cayley coefficients from omega (the c_s of
        # mobius.py:34-46 with omega): the zmobius operator
        return zmobius(U, p)
    p.setdefault("n_rhs", 1)
    return mobius_operator(U, p)


def zmobius(U, params=None, **kw):
    """g.qcd.fermion.zmobius (lib/gpt/qcd/fermion/zmobius.py:59-78): Ls =
    len(omega), complex per-slice b_s, c_s from omega, b and c."""
    p = _std_params(params, kw)
    if p.get("omega") is None:
        raise ValueError("omega required")
    p["omega"] = [complex(*w) if isinstance(w, (list, tuple)) else complex(w) for w in p["omega"]]
    p["Ls"] = len(p["omega"])
    if p.get("mass") is not None:
        p["mass_plus"] = p["mass"]
        p["mass_minus"] = p["mass"]
    p.setdefault("n_rhs", 1)
    return zmobius_operator(U, p)


class zmobius_operator(fermion_operator):
    def __init__(self, U, params, precision=None, daggered=False, clover_from=None):
        super().__init__("zmobius", U, params, precision, daggered)


class mobius_operator(fermion_operator):
    def __init__(self, U, params, precision=None, daggered=False, clover_from=None):
        super().__init__("mobius", U, params, precision, daggered)


# ---------------------------------------------------------------------------
# preconditioners (lib/gpt/qcd/fermion/preconditioner/even_odd_sites.py:61-72)
# ---------------------------------------------------------------------------
class preconditioner:
    class eo2_ne:
        """normal_equation(schur_complement_two(op, even_odd_sites_decomposed(parity)))."""

        def __init__(self, params=None, parity=None):
            par = (params or {}).get("parity", parity) if params else parity
            self.parity = par if par is not None else core.odd
            if self.parity is not core.odd:
                raise NotImplementedError("eo2_ne is implemented for parity = odd (the reference default)")

        def __call__(self, op):
            return _eo2_ne_matrix(op, self.parity)

    class mixed_dwf:
        """MADWF (lib/gpt/qcd/fermion/preconditioner/mixed_dwf.py:29-108, the
        algorithm of arXiv:1111.5059): an approximate inverse of the outer
        domain-wall operator from a solve with a cheaper inner one (another
        Ls or zmobius), through the Pauli-Villars operators (mass 1) and the
        chiral shift P.  solver and solver_pv are inverters of full 5D
        operators (for example preconditioned(eo2_ne(), cg(...))); all
        fifth-dimension moves run on the device (gbf_chiral_shift,
        gbf_copy_slices).  Inner and outer operators share the precision."""

        def __init__(self, solver, solver_pv, dwf_inner):
            self.solver = solver
            self.solver_pv = solver_pv
            self.dwf_inner = dwf_inner
            self.dwf_inner_pv = dwf_inner.modified(mass=1.0)

        def __call__(self, dwf_outer):
            inner, inner_pv = self.dwf_inner, self.dwf_inner_pv
            if inner.precision is not dwf_outer.precision:
                raise ValueError("inner and outer domain-wall operators must share the precision")
            if inner.n_rhs != dwf_outer.n_rhs or inner.U_grid.fdimensions != dwf_outer.U_grid.fdimensions:
                raise ValueError("inner and outer domain-wall operators must share the 4D grid and n_rhs")
            outer_pv = dwf_outer.modified(mass=1.0)
            inv_outer_pv = self.solver_pv(outer_pv)
            inv_inner = self.solver(inner)
            L = _lib.load()

            def P(dst, src, offset):
                # offset 1: P (mixed_dwf.py:56-57); offset -1: P^+ = P^-1 (:59-60)
                _lib.check(L.gbf_chiral_shift(src.layout.op, src.ptr, dst.ptr, offset, src.nhalves(), core.stream_ptr()))

            def slice0(dst, src, scale):
                _lib.check(L.gbf_copy_slices(dst.layout.op, dst.ptr, 0, src.layout.op, src.ptr, 0, 1, float(scale),
                                             src.nhalves(), core.stream_ptr()))

            def one(dst, src):
                # c_s = P^+ D_PV,outer^-1 src
                c = dwf_outer.F_lattice()
                P(c, inv_outer_pv(src), -1)
                # y0' = [P^+ D_inner^-1 D_PV,inner P (c_0, 0, ..., 0)]_0 on the inner Ls
                wi = inner.F_lattice()
                slice0(wi, c, 1.0)
                a = inner.F_lattice()
                P(a, wi, 1)
                y = inv_inner(inner_pv.M(a))
                y0 = inner.F_lattice()
                P(y0, y, -1)
                # y1 = P^+ D_PV,outer^-1 D_outer P (-y0', c_1, ..., c_{Ls-1})
                wo = c.copy()
                slice0(wo, y0, -1.0)
                e = dwf_outer.F_lattice()
                P(e, wo, 1)
                y1 = dwf_outer.F_lattice()
                P(y1, inv_outer_pv(dwf_outer.M(e)), -1)
                # dst = P (y0', y1_1, ..., y1_{Ls-1})
                slice0(y1, y0, 1.0)
                P(dst, y1, 1)
                dst.cb = core.full

            def inv(dst, src):
                if isinstance(src, (list, tuple)):
                    for d, s_ in zip(dst, src):
                        one(d, s_)
                else:
                    one(dst, src)

            m = matrix_operator(inv, inv_mat=dwf_outer.mat)
            m._new_dst = lambda src: ([dwf_outer.F_lattice() for _ in src] if isinstance(src, (list, tuple))
                                      else dwf_outer.F_lattice())
            return m


class _eo2_ne_matrix:
    """The eo2_ne-preconditioned system of `op`; `Mpc` is the normal matrix
    Mpc^+ Mpc on half lattices of the odd sites
    (lib/gpt/algorithms/preconditioner/normal_equation.py:35-65), applied by
    gbf_apply_eo2ne_normal."""

    def __init__(self, op, parity):
        self.op = op
        self.parity = parity

        def _ne(dst, src):
            if src.cb is not core.odd:
                raise ValueError("Mpc acts on odd-site half lattices")
            _lib.check(_lib.load().gbf_apply_eo2ne_normal(op.obj, src.ptr, dst.ptr, core.stream_ptr()))
            dst.cb = core.odd

        self.Mpc = matrix_operator(_ne, _ne)
        self.Mpc._new_dst = lambda src: op.F_lattice(core.odd)
        self.Mpc.native_op = op
