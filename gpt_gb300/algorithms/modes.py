"""Mode representations of matrices (lib/gpt/algorithms/modes/matrix.py:25-67):

    A = sum_n left[n] right[n]^+ f(evals[n])

applied on the device by gbf_modes_apply: the inner products <right[n], src>
(blocks of eight modes per pass over the sites, deterministic FP64
reductions), then the linear combination of the left modes.  The modes are
fields of one layout and checkerboard (for example the odd-site eigenvectors
of the eo2_ne normal operator).
"""
import ctypes

from .. import _lib, core
from ..qcd import fermion as _fermion


def _as_list(x):
    return (list(x), True) if isinstance(x, (list, tuple)) else ([x], False)


def matrix(left, right, evals, f, params=None, block=16, linear_combination_block=8):
    """The reference's block sizes are accepted for compatibility; the device
    kernels use their own block of eight modes."""
    left, right = list(left), list(right)
    if not (len(left) == len(right) and 0 < len(left) <= len(evals)):
        raise ValueError("need as many left as right modes and an eigenvalue for each")
    lay, cb = left[0].layout, left[0].cb
    for v in left + right:
        if v.layout is not lay or v.cb is not cb:
            raise ValueError("all modes must share one layout and checkerboard")
    n = len(left)
    fv = [complex(f(evals[i])) for i in range(n)]
    fa = (ctypes.c_double * (2 * n))(*[c for z in fv for c in (z.real, z.imag)])
    lp = _lib.ptrs([v.ptr for v in left])
    rp = _lib.ptrs([v.ptr for v in right])

    def approx(dst, src):
        dl, _ = _as_list(dst)
        sl, _ = _as_list(src)
        if len(dl) != len(sl):
            raise ValueError("as many destinations as sources")
        for d, s in zip(dl, sl):
            if s is d or s.ptr == d.ptr:
                raise ValueError("src and dst must differ")
            if s.layout is not lay or s.cb is not cb or d.layout is not lay:
                raise ValueError("src and dst must have the modes' layout and checkerboard")
            _lib.check(_lib.load().gbf_modes_apply(lay.op, lp, rp, fa, n, s.ptr, d.ptr, s.nhalves(),
                                                   core.stream_ptr()))
            d.cb = cb

    m = _fermion.matrix_operator(approx)
    m._new_dst = lambda src: [s.new() for s in src] if isinstance(src, (list, tuple)) else src.new()
    m.modes = (left, right, fv)
    return m
