"""Krylov inverters of the hot path: cg, preconditioned, defect_correcting,
mixed_precision (lib/gpt/algorithms/inverter/cg.py:24-117,
preconditioned.py:24-54, defect_correcting.py:23-142, mixed_precision.py:23-32),
and the adjacent solver layers block_cg, multi_shift_cg, deflate and
sequence (block_cg.py, multi_shift_cg.py, deflate.py, sequence.py).

preconditioned(eo2_ne(), cg(...)) on a native fermion operator runs as one
device-resident solve (prepare, CG in CUDA graphs, reconstruction) through
gbf_solve_eo2ne_cg.  defect_correcting and mixed_precision compose on the
host exactly as in the reference, with all vector algebra on the device.
"""
import math

from .. import core
from ..qcd import fermion as _fermion


class cg:
    """gpt.algorithms.inverter.cg(eps, maxiter): CG on the eo2_ne normal
    equations; convergence when |r|^2 <= eps^2 |b|^2 (cg.py:70, 103)."""

    def __init__(self, params=None, eps=1e-15, maxiter=1000000, fail_if_not_converged=False, iterations_per_graph=0,
                 profile=False, eps_abs=None, miniter=0, prec=None):
        p = dict(params or {})
        self.eps = p.get("eps", eps)
        self.maxiter = p.get("maxiter", maxiter)
        self.fail_if_not_converged = p.get("fail_if_not_converged", fail_if_not_converged)
        # for the generic CG on any matrix operator (cg.py:25-34)
        self.eps_abs = p.get("eps_abs", eps_abs)
        self.miniter = p.get("miniter", miniter)
        self.prec = p.get("prec", prec)
        # iterations_per_graph K > 0: CUDA graphs of K iterations with a host
        # convergence check between them; 0: the library's default K (16);
        # -1: the whole CG loop on the device (one CUDA graph with a
        # conditional while node).  profile: no graphs, every kernel
        # launched from the host between CUDA events
        self.iterations_per_graph = p.get("iterations_per_graph", iterations_per_graph)
        self.profile = bool(p.get("profile", profile))
        self.history = []
        self.last = None
        self.total_iterations = 0

    def modified(self, **params):
        d = dict(eps=self.eps, maxiter=self.maxiter, fail_if_not_converged=self.fail_if_not_converged,
                 iterations_per_graph=self.iterations_per_graph, profile=self.profile, eps_abs=self.eps_abs,
                 miniter=self.miniter, prec=self.prec)
        d.update(params)
        return cg(d)

    def __call__(self, mat):
        """cg(mat).  For the eo2_ne normal operator of a native operator
        (preconditioner.eo2_ne()(op).Mpc): the whole CG on the device starting
        from the destination as the guess (gbf_solve_normal_cg; the
        reference's guess handling, cg.py:48-68: r = src - mat psi, zero
        source -> zero solution); a guess that already meets the tolerance
        returns after zero iterations.  For any other Hermitian positive
        definite matrix operator (a composed or shifted operator, a user
        operator): the recursion of cg.py:47-105 driven from the host, every
        vector operation and reduction on the device (norm2, inner_product,
        axpy_norm2, axpby), the matrix applied through its own callable."""
        op = getattr(mat, "native_op", None)
        if op is None:
            return self._generic(mat)
        import ctypes

        from .. import _lib
        me = self

        def inv(dst, src):
            if src.cb is not core.odd or dst.cb is not core.odd:
                raise ValueError("the eo2_ne normal operator acts on odd-site half lattices")
            p = _lib.gbf_cg_params(float(me.eps), int(me.maxiter), int(me.iterations_per_graph), int(me.profile))
            r = _lib.gbf_cg_result()
            _lib.check(_lib.load().gbf_solve_normal_cg(op.obj, src.ptr, dst.ptr, ctypes.byref(p), ctypes.byref(r),
                                                       core.stream_ptr()))
            me.last = r
            me.history = [None] * r.iterations
            me.total_iterations += r.iterations
            if me.fail_if_not_converged and not r.converged:
                raise ValueError("FATAL error: CG not converged")

        m = _fermion.matrix_operator(inv, inv_mat=mat.mat)
        m._new_dst = lambda src: op.F_lattice(core.odd)
        m.accept_guess = True
        return m


    def _generic(self, mat):
        import types

        me = self
        apply = mat.mat if hasattr(mat, "mat") and mat.mat is not None else mat
        prec = self.prec(mat) if self.prec is not None else None

        def per_rhs(v, n):
            return list(v) if isinstance(v, (list, tuple)) else [v] * n

        def inv(psi, src):
            if src is psi:
                raise ValueError("src and psi must differ (cg.py:49)")
            n = src.layout.n_rhs
            p, mmp, r = src.new(), src.new(), src.new()
            z = src.new() if prec is not None else None
            apply(mmp, psi)
            core.axpby(r, -1.0, mmp, 1.0, src)
            if prec is not None:
                z[:] = 0
                prec(z, r)
                core.copy(p, z)
                cp = [x.real for x in per_rhs(core.inner_product(r, z), n)]
            else:
                core.copy(p, r)
                cp = per_rhs(core.norm2(p), n)
            ssq = per_rhs(core.norm2(src), n)
            res_info = types.SimpleNamespace(iterations=0, converged=0, breakdown=0,
                                             residual_sq=[0.0] * n)
            me.last = res_info
            me.history = []
            if all(v == 0.0 for v in ssq):
                psi[:] = 0
                res_info.converged = 1
                return
            rsq = [me.eps ** 2 * v for v in ssq]
            done = [False] * n
            for k in range(me.maxiter):
                c = cp
                apply(mmp, p)
                d = [x.real for x in per_rhs(core.inner_product(p, mmp), n)]
                a = [0.0 if done[j] or d[j] == 0.0 else c[j] / d[j] for j in range(n)]
                if any(not done[j] and not (d[j] > 0.0) for j in range(n)):
                    res_info.breakdown = 1
                if prec is not None:
                    core.axpby(r, [-x for x in a], mmp, 1.0, r)
                    z[:] = 0
                    prec(z, r)
                    cp = [x.real for x in per_rhs(core.inner_product(r, z), n)]
                else:
                    cp = per_rhs(core.axpy_norm2(r, [-x for x in a], mmp, r), n)
                b = [0.0 if done[j] or c[j] == 0.0 else cp[j] / c[j] for j in range(n)]
                core.axpby(psi, a, p, 1.0, psi)
                core.axpby(p, b, p, 1.0, z if prec is not None else r)
                res = [abs(x) for x in cp]
                me.history.append(max(res[j] / ssq[j] for j in range(n) if ssq[j] > 0))
                res_info.iterations = k + 1
                res_info.residual_sq = [res[j] / ssq[j] if ssq[j] > 0 else 0.0 for j in range(n)]
                if k + 1 >= me.miniter:
                    for j in range(n):
                        if me.eps_abs is not None and res[j] <= me.eps_abs ** 2:
                            done[j] = True
                        if res[j] <= rsq[j]:
                            done[j] = True
                    if all(done):
                        res_info.converged = 1
                        break
                if res_info.breakdown:
                    break
            me.total_iterations += res_info.iterations
            if me.fail_if_not_converged and not res_info.converged:
                raise ValueError("FATAL error: CG not converged")

        m = _fermion.matrix_operator(inv, inv_mat=apply)
        new_dst = getattr(mat, "_new_dst", None)
        if new_dst is not None:
            m._new_dst = new_dst
        m.accept_guess = True
        return m


class block_cg(cg):
    """gpt.algorithms.inverter.block_cg(eps, maxiter) (block_cg.py:36-149):
    the packed right-hand sides of an n_rhs operator share one Krylov space;
    converged when max_b |r_b|^2 / |b_b|^2 <= eps^2 as recorded by the block
    recursion.  Runs on the device through preconditioned(eo2_ne(), ...)."""

    def modified(self, **params):
        d = dict(eps=self.eps, maxiter=self.maxiter, fail_if_not_converged=self.fail_if_not_converged)
        d.update(params)
        return block_cg(d)

    def __call__(self, mat):
        raise NotImplementedError("block_cg runs on the device through preconditioned(eo2_ne(), block_cg(...))")


class multi_shift_cg:
    """gpt.algorithms.inverter.multi_shift_cg(eps, maxiter, shifts)
    (multi_shift_cg.py:51-144): solves (mat + s_j) x_j = src for all shifts
    with one Krylov space.  Runs on the device for the eo2_ne normal matrix of
    a native operator (preconditioner.eo2_ne()(op).Mpc); mat(dst_list, src)
    fills one odd-site half lattice per shift."""

    def __init__(self, params=None, eps=1e-15, maxiter=1000000, shifts=()):
        p = dict(params or {})
        self.eps = p.get("eps", eps)
        self.maxiter = p.get("maxiter", maxiter)
        self.shifts = [float(s) for s in p.get("shifts", shifts)]
        self.last = None

    def __call__(self, mat):
        op = getattr(mat, "native_op", None)
        if op is None:
            raise NotImplementedError("multi_shift_cg runs on the device for preconditioner.eo2_ne()(op).Mpc")
        import ctypes

        from .. import _lib
        me = self

        def inv(dst, src):
            n = len(me.shifts)
            if len(dst) != n:
                raise ValueError(f"expected {n} destination lattices")
            sh = (ctypes.c_double * n)(*me.shifts)
            p = _lib.gbf_cg_params(float(me.eps), int(me.maxiter), 0, 0)
            r = _lib.gbf_cg_result()
            _lib.check(_lib.load().gbf_solve_eo2ne_multishift(op.obj, src.ptr, _lib.ptrs([d.ptr for d in dst]), sh, n,
                                                              ctypes.byref(p), ctypes.byref(r), core.stream_ptr()))
            for d in dst:
                d.cb = core.odd
            me.last = r

        m = _fermion.matrix_operator(inv)
        m._new_dst = lambda src: [op.F_lattice(core.odd) for _ in me.shifts]
        return m


class deflate:
    """gpt.algorithms.inverter.deflate(evec, ev) (deflate.py:23-32): the
    low-mode part sum_n evec_n evec_n^+ / ev_n of the inverse, as a mode
    matrix applied on the device (algorithms.modes.matrix).  Used alone it is
    the low-mode approximation; in sequence(deflate(...), cg(...)) it is the
    guess from which the CG starts."""

    def __init__(self, evec, ev, params=None, block=16):
        self.evec = list(evec)
        self.ev = [float(x) if complex(x).imag == 0 else complex(x) for x in ev]
        self.block = (params or {}).get("block", block)

    def __call__(self, matrix):
        from . import modes
        m = modes.matrix(self.evec, self.evec, self.ev, lambda x: 1.0 / x, block=self.block)
        m.accept_guess = False
        return m


class sequence:
    """gpt.algorithms.inverter.sequence(*inverters) (sequence.py:23-42): the
    inverters of one matrix applied in turn to the same (dst, src), each
    later one starting from the result of the one before."""

    def __init__(self, *inverters):
        self.inverters = inverters

    def __call__(self, outer_mat):
        mats = [i(outer_mat) for i in self.inverters]

        def inv(dst, src):
            for m in mats:
                m(dst, src)

        m = _fermion.matrix_operator(inv, inv_mat=getattr(outer_mat, "mat", None))
        m._new_dst = mats[0]._new_dst
        m.accept_guess = True
        return m


class preconditioned:
    """M^-1 = L Mpc^-1 R + S (preconditioned.py:28-54)."""

    def __init__(self, preconditioner, inverter, params=None):
        self.preconditioner = preconditioner
        self.inverter = inverter

    def __call__(self, op):
        if not isinstance(self.preconditioner, _fermion.preconditioner.eo2_ne):
            raise NotImplementedError("the device path implements the eo2_ne preconditioner")
        if not isinstance(op, _fermion.fermion_operator):
            raise TypeError("expected a native fermion operator")
        if op.daggered:
            raise NotImplementedError("solves with the daggered operator are not on this path")
        inv = self.inverter
        if not isinstance(inv, cg):
            return self._composed(op)

        solve = op._solve_eo2ne_block_cg if isinstance(inv, block_cg) else op._solve_eo2ne_cg

        def mat(dst, src):
            r = solve(dst, src, inv.eps, inv.maxiter, inv.iterations_per_graph, int(inv.profile))
            inv.last = r
            inv.history = [None] * r.iterations
            inv.total_iterations += r.iterations
            if inv.fail_if_not_converged and not r.converged:
                raise ValueError("FATAL error: CG not converged")

        def new_dst(src):
            return op.F_lattice()

        m = _fermion.matrix_operator(mat, inv_mat=op.mat)
        m._new_dst = new_dst
        return m

    def _composed(self, op):
        """L Mpc^-1 R + S around any inverter of the normal operator (for
        example sequence(deflate(...), cg(...))): R and L S on the device
        (gbf_eo2ne_prepare / gbf_eo2ne_reconstruct), the inverter on
        preconditioner.eo2_ne()(op).Mpc with a zero guess."""
        from .. import _lib
        inner = self.inverter(self.preconditioner(op).Mpc)

        def mat(dst, src):
            b = op.F_lattice(core.odd)
            _lib.check(_lib.load().gbf_eo2ne_prepare(op.obj, src.ptr, b.ptr, core.stream_ptr()))
            y = op.F_lattice(core.odd)
            inner(y, b)
            _lib.check(_lib.load().gbf_eo2ne_reconstruct(op.obj, src.ptr, y.ptr, dst.ptr, core.stream_ptr()))
            dst.cb = core.full

        m = _fermion.matrix_operator(mat, inv_mat=op.mat)
        m._new_dst = lambda src: op.F_lattice()
        return m


class mixed_precision:
    """Run the inner inverter on op.converted(inner_precision) and convert
    source and solution (mixed_precision.py:23-32, matrix_operator.py:139-178)."""

    def __init__(self, inverter, inner_precision, outer_precision):
        self.inverter = inverter
        self.inner_precision = inner_precision
        self.outer_precision = outer_precision

    def __call__(self, op):
        inner_op = op.converted(self.inner_precision)
        inner = self.inverter(inner_op)
        self.inner_op = inner_op

        def mat(dst, src):
            cs = inner_op.F_lattice()
            core.convert(cs, src)
            cd = inner(cs)
            core.convert(dst, cd)

        m = _fermion.matrix_operator(mat, inv_mat=op.mat)
        m._new_dst = lambda src: op.F_lattice()
        return m


class defect_correcting:
    """Outer defect correction (defect_correcting.py:85-130): residual
    s = src - M psi in the outer precision, s normalised by |src|, inner
    solve, psi += d |src|; stops when max_j |s_j| / |src_j| < eps."""

    def __init__(self, inner_inverter, params=None, eps=1e-15, maxiter=1000000):
        p = dict(params or {})
        self.eps = p.get("eps", eps)
        self.maxiter = p.get("maxiter", maxiter)
        self.inner_inverter = inner_inverter
        self.history = []

    def __call__(self, outer_mat):
        inner_inv_mat = self.inner_inverter(outer_mat)
        me = self

        def mat(psi, src):
            n = src.layout.n_rhs
            ns = core.norm2(src)
            ns = [ns] if n == 1 else ns
            ns = [x if x != 0.0 else 1.0 for x in ns]
            s = src.new()
            t = src.new()
            me.history = []
            psi_zero = core.norm2(psi)
            psi_zero = all(v == 0.0 for v in ([psi_zero] if n == 1 else psi_zero))
            for i in range(me.maxiter):
                if i == 0 and psi_zero:
                    core.copy(s, src)  # src - M * 0, without applying M
                else:
                    outer_mat(t, psi)
                    core.axpby(s, -1.0, t, 1.0, src)
                nd = core.norm2(s)
                nd = [nd] if n == 1 else nd
                eps = max(math.sqrt(nd[j] / ns[j]) for j in range(n))
                me.history.append(eps)
                if eps < me.eps:
                    break
                core.axpby(s, [1.0 / math.sqrt(x) for x in ns], s)
                d = inner_inv_mat(s)
                core.axpby(psi, [math.sqrt(x) for x in ns], d, 1.0, psi)

        m = _fermion.matrix_operator(mat, inv_mat=outer_mat.mat)
        m._new_dst = lambda src: outer_mat.F_lattice()
        return m
