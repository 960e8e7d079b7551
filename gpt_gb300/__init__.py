"""gpt_gb300 -- GB300-native fermion-matrix hot path of gpt (lehner/gpt).

Drop-in for gpt's Wilson-clover / Mobius Dslash and the eo2_ne-preconditioned
CG: ``g.qcd.fermion.wilson_clover`` / ``g.qcd.fermion.mobius``,
``g.qcd.fermion.preconditioner.eo2_ne``, ``g.algorithms.inverter.cg``,
``preconditioned``, ``defect_correcting`` and ``mixed_precision`` keep gpt's
names and parameters; the arithmetic runs in hand-written sm_103a CUDA
kernels of libgbferm.so (C ABI: include/gbferm.h).  PyTorch provides device
memory and streams only.
"""
from .core import (
    precision, double, single, half, double_float, even, odd, full, grid, layout, lattice, vspincolor,
    norm2, inner_product, axpy, axpby, axpy_norm2, inner_product_norm2, copy, convert,
)
from . import _lib
from . import qcd
from . import algorithms
from . import io
from .io import save, format


def load(path=None):
    """g.load(path): read a gauge-field file (NERSC format, gpt_gb300.io);
    g.load() without a path loads (building if needed) the native library and
    raises if it is unavailable."""
    if path is None:
        return _lib.load()
    return io.load(path)
