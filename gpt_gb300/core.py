"""Core objects of the gpt-compatible host layer: precisions, grids, field
layouts, lattices and vector algebra (lib/gpt/core/grid.py,
lib/gpt/core/precision.py, lib/gpt/core/transform.py:101-153).

A ``lattice`` is a fermion field in the library's internal device layout
(see include/gbferm.h); ``lattice[:]`` reads or writes it in gpt's natural
host layout, complex128 [V, (Ls,) 4, 3].  All arithmetic runs on the GPU
through libgbferm.so; PyTorch only provides device memory and streams.
"""
import ctypes
import threading

import numpy as np
import torch

from . import _lib


class precision:
    def __init__(self, name, code, eps, nbytes):
        self.name = name
        self.code = code
        self.eps = eps
        self.nbytes = nbytes

    def __repr__(self):
        return self.name


double = precision("double", _lib.GBF_DOUBLE, 1e-15, 192)
single = precision("single", _lib.GBF_SINGLE, 1e-7, 96)
half = precision("half", _lib.GBF_HALF, 1e-3, 52)
# FP64-class accuracy on the FP32 pipe: each real is h + l of two FP32 words
# (no counterpart in the reference, whose precisions are single and double)
double_float = precision("double_float", _lib.GBF_DOUBLE_FLOAT, 4e-15, 192)


class checkerboard:
    def __init__(self, name, code):
        self.name = name
        self.code = code

    def inv(self):
        return odd if self is even else even

    def __repr__(self):
        return self.name


even = checkerboard("even", _lib.GBF_EVEN)
odd = checkerboard("odd", _lib.GBF_ODD)
full = checkerboard("full", _lib.GBF_FULL)


class grid:
    """4D lattice geometry with a precision (g.grid(fdimensions, precision))."""

    def __init__(self, fdimensions, prec=double):
        self.fdimensions = [int(d) for d in fdimensions]
        assert len(self.fdimensions) == 4
        for d in self.fdimensions:
            if d < 2 or d % 2:
                raise ValueError("lattice dimensions must be even and >= 2")
        self.precision = prec
        self.gsites = int(np.prod(self.fdimensions))

    def converted(self, prec):
        return grid(self.fdimensions, prec)

    def __eq__(self, other):
        return isinstance(other, grid) and self.fdimensions == other.fdimensions and self.precision is other.precision

    def __hash__(self):
        return hash((tuple(self.fdimensions), self.precision.name))

    def __repr__(self):
        return f"grid({self.fdimensions}, {self.precision})"


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


_layout_cache = {}


class _native_handle:
    """A native operator handle (the vector-algebra workspace of a layout),
    deleted with the object."""

    def __init__(self, h):
        self.h = h

    def __del__(self):
        try:
            _lib.load().gbf_delete(self.h)
        except Exception:
            pass


class layout:
    """Field layout = (4D grid, Ls, n_rhs).  Owns light-weight native
    operator handles used for vector algebra on fields of this layout, one
    per thread: a handle carries reduction workspace, and the C ABI allows one
    thread per handle at a time (worker threads of the serving loop reduce
    fields of the same layout concurrently on their own streams)."""

    _create_lock = threading.Lock()

    def __init__(self, g, Ls=1, n_rhs=1):
        self.grid = g
        self.Ls = int(Ls)
        self.n_rhs = int(n_rhs)
        self.five_d = self.Ls > 1 or False
        self._local = threading.local()

    @staticmethod
    def get(g, Ls=1, n_rhs=1, five_d=None):
        key = (tuple(g.fdimensions), g.precision.name, int(Ls), int(n_rhs), bool(five_d))
        with layout._create_lock:
            lay = _layout_cache.get(key)
            if lay is None:
                lay = layout(g, Ls, n_rhs)
                lay.five_d = bool(five_d) if five_d is not None else Ls > 1
                _layout_cache[key] = lay
        return lay

    @property
    def op(self):
        hd = getattr(self._local, "handle", None)
        if hd is None:
            L = _lib.load()
            p = _lib.gbf_params()
            for i in range(4):
                p.dims[i] = self.grid.fdimensions[i]
            p.Ls = self.Ls
            p.n_rhs = self.n_rhs
            p.xi_0 = p.nu = 1.0
            p.b, p.c, p.M5 = 1.0, 0.0, 0.0
            p.reconstruct = -1
            h = ctypes.c_void_p()
            name = b"mobius" if self.five_d else b"wilson_clover"
            _lib.check(L.gbf_create(name, self.grid.precision.code, ctypes.byref(p), ctypes.byref(h)))
            hd = _native_handle(h)
            self._local.handle = hd
        return hd.h

    def half_bytes(self):
        N = self.grid.gsites // 2 * self.Ls * self.n_rhs
        return self.grid.precision.nbytes * N

    def natural_shape(self):
        V = self.grid.gsites
        return (V, self.Ls, 4, 3) if self.five_d else (V, 4, 3)



class lattice:
    """A fermion field (vspincolor; 5D for Mobius) in the internal layout.

    cb = full: [even half][odd half]; cb = even/odd: one half."""

    def __init__(self, lay, cb=full, tensor=None):
        self.layout = lay
        self.cb = cb
        nb = lay.half_bytes() * (2 if cb is full else 1)
        if tensor is None:
            tensor = torch.zeros(nb, dtype=torch.uint8, device="cuda")
        assert tensor.numel() == nb and tensor.dtype == torch.uint8
        self.tensor = tensor

    @property
    def grid(self):
        return self.layout.grid

    @property
    def ptr(self):
        return self.tensor.data_ptr()

    def half(self, p):
        assert self.cb is full
        hb = self.layout.half_bytes()
        return lattice(self.layout, p, self.tensor[p.code * hb:(p.code + 1) * hb])

    def checkerboard(self, cb=None):
        if cb is None:
            return self.cb
        assert (cb is full) == (self.cb is full)
        self.cb = cb
        return self

    def nhalves(self):
        return 2 if self.cb is full else 1

    def new(self):
        return lattice(self.layout, self.cb)

    def copy(self):
        return lattice(self.layout, self.cb, self.tensor.clone())

    # natural host layout access, rhs by rhs
    def set_natural(self, arr, rhs=0):
        assert self.cb is full
        arr = np.ascontiguousarray(arr, dtype=np.complex128).reshape(self.layout.natural_shape())
        dev = torch.from_numpy(arr.view(np.float64)).to("cuda", non_blocking=False)
        L = _lib.load()
        _lib.check(L.gbf_field_import(self.layout.op, dev.data_ptr(), self.ptr, rhs, int(self.layout.five_d), stream_ptr()))
        torch.cuda.current_stream().synchronize()

    def get_natural(self, rhs=0):
        assert self.cb is full
        shape = self.layout.natural_shape()
        dev = torch.zeros(int(np.prod(shape)) * 2, dtype=torch.float64, device="cuda")
        L = _lib.load()
        _lib.check(L.gbf_field_export(self.layout.op, self.ptr, dev.data_ptr(), rhs, int(self.layout.five_d), stream_ptr()))
        return dev.cpu().numpy().view(np.complex128).reshape(shape)

    def __setitem__(self, key, value):
        if key != slice(None):
            raise NotImplementedError("only lattice[:] = value is supported")
        if np.isscalar(value) and value == 0:
            self.tensor.zero_()
            return
        value = np.asarray(value)
        if value.shape == self.layout.natural_shape():
            self.set_natural(value, 0)
        else:
            for r in range(self.layout.n_rhs):
                self.set_natural(value[r], r)

    def __getitem__(self, key):
        if key != slice(None):
            raise NotImplementedError("only lattice[:] is supported")
        if self.layout.n_rhs == 1:
            return self.get_natural(0)
        return np.stack([self.get_natural(r) for r in range(self.layout.n_rhs)])


def vspincolor(g, Ls=1, n_rhs=1, cb=full):
    return lattice(layout.get(g, Ls, n_rhs, five_d=Ls > 1), cb)


# ---------------------------------------------------------------------------
# vector algebra (per right-hand side; double accumulation, fixed order)
# ---------------------------------------------------------------------------
def _n(x):
    return x.layout.n_rhs


def norm2(x):
    """|x|^2 per packed right-hand side (lib/gpt/core/foundation/lattice/__init__.py:28-39)."""
    out = (ctypes.c_double * 16)()
    _lib.check(_lib.load().gbf_norm2(x.layout.op, x.ptr, x.nhalves(), out, stream_ptr()))
    r = [out[i] for i in range(_n(x))]
    return r[0] if len(r) == 1 else r


def inner_product(x, y):
    """<x, y> = sum conj(x) y per right-hand side."""
    re = (ctypes.c_double * 16)()
    im = (ctypes.c_double * 16)()
    _lib.check(_lib.load().gbf_inner(x.layout.op, x.ptr, y.ptr, x.nhalves(), re, im, stream_ptr()))
    r = [complex(re[i], im[i]) for i in range(_n(x))]
    return r[0] if len(r) == 1 else r


def _vec(a, n):
    if np.isscalar(a):
        return [a] * n
    return list(a)


def axpby(out, a, x, b=None, y=None):
    """out = a x + b y  (a complex, b real; per rhs or scalars)."""
    n = _n(x)
    a = _vec(a, n)
    are = _lib.darr([complex(v).real for v in a])
    aim = _lib.darr([complex(v).imag for v in a])
    bb = _lib.darr([float(v) for v in _vec(b if b is not None else 0.0, n)])
    _lib.check(_lib.load().gbf_axpby(out.layout.op, out.ptr, are, aim, x.ptr, bb, y.ptr if y is not None else None,
                                     x.nhalves(), stream_ptr()))
    return out


def axpy(out, a, x, y):
    """gpt.axpy: out = a x + y."""
    return axpby(out, a, x, 1.0, y)


def axpy_norm2(out, a, x, y):
    """gpt.axpy_norm2 (lib/gpt/core/transform.py:139-153): out = a x + y and
    |out|^2 per rhs, in one fused pass (gbf_axpy_norm2)."""
    n = _n(x)
    a = _vec(a, n)
    are = _lib.darr([complex(v).real for v in a])
    aim = _lib.darr([complex(v).imag for v in a])
    res = (ctypes.c_double * 16)()
    _lib.check(_lib.load().gbf_axpy_norm2(out.layout.op, out.ptr, are, aim, x.ptr, y.ptr, x.nhalves(), res,
                                          stream_ptr()))
    r = [res[i] for i in range(n)]
    return r[0] if n == 1 else r


def inner_product_norm2(x, y):
    """gpt.inner_product_norm2 (transform.py:121-131): (<x, y>, |x|^2)."""
    return inner_product(x, y), norm2(x)


def copy(dst, src):
    dst.tensor.copy_(src.tensor)
    return dst


def convert(dst, src, scale=1.0):
    """Precision conversion between layouts of equal geometry (optionally scaled)."""
    _lib.check(_lib.load().gbf_convert(dst.layout.op, dst.ptr, src.layout.op, src.ptr, float(scale), src.nhalves(),
                                       stream_ptr()))
    return dst
