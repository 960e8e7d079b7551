"""ctypes binding of libgbferm.so (the C ABI declared in include/gbferm.h).

The library is the only compute path: if it cannot be loaded the import
fails loudly -- there is no CPU or PyTorch fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbferm.so")

GBF_DOUBLE, GBF_SINGLE, GBF_HALF, GBF_DOUBLE_FLOAT = 0, 1, 2, 3
GBF_EVEN, GBF_ODD, GBF_FULL = 0, 1, 2

OPCODES = {
    "M": 2001, "Mdag": 2002, "Meooe": 2003, "MeooeDag": 2004, "Mooee": 2005, "MooeeDag": 2006,
    "MooeeInv": 2007, "MooeeInvDag": 2008, "Mdiag": 2009, "Dminus": 2010, "DminusDag": 2011,
    "ImportPhysicalFermionSource": 2012, "ImportUnphysicalFermion": 2013, "ExportPhysicalFermionSolution": 2014,
    "ExportPhysicalFermionSource": 2015,
    "Dhop": 3001, "DhopEO": 3002, "DhopDag": 4001, "DhopEODag": 4002,
}


class gbf_params(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int * 4),
        ("Ls", ctypes.c_int),
        ("n_rhs", ctypes.c_int),
        ("mass", ctypes.c_double),
        ("csw_r", ctypes.c_double),
        ("csw_t", ctypes.c_double),
        ("xi_0", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("isAnisotropic", ctypes.c_int),
        ("boundary_phases", ctypes.c_double * 8),
        ("mass_plus", ctypes.c_double),
        ("mass_minus", ctypes.c_double),
        ("b", ctypes.c_double),
        ("c", ctypes.c_double),
        ("M5", ctypes.c_double),
        ("reconstruct", ctypes.c_int),
        ("mu", ctypes.c_double),
        ("omega", ctypes.c_void_p),
    ]


class gbf_cg_params(ctypes.Structure):
    _fields_ = [("eps", ctypes.c_double), ("maxiter", ctypes.c_int), ("iterations_per_graph", ctypes.c_int),
                ("profile", ctypes.c_int)]


class gbf_cg_result(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("breakdown", ctypes.c_int),
        ("residual_sq", ctypes.c_double * 16),
        ("kernel_ms", ctypes.c_double * 3),
        ("kernel_launches", ctypes.c_int * 3),
    ]


_lib = None


def load():
    """Load libgbferm.so, building it first when sources are newer (nvcc)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import _build

    try:
        _build.build()
    except Exception as e:  # no nvcc here: use a prebuilt library if present
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libgbferm.so is missing and could not be built: {e}") from e
    try:
        L = ctypes.CDLL(LIB_PATH)
    except OSError as e:
        raise ImportError(f"cannot load {LIB_PATH}: {e}") from e
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    PP = ctypes.POINTER(ctypes.c_void_p)
    DP = ctypes.POINTER(ctypes.c_double)
    sig = {
        "gbf_create": (I, [ctypes.c_char_p, I, ctypes.POINTER(gbf_params), ctypes.POINTER(P)]),
        "gbf_update_gauge": (I, [P, P, I, P]),
        "gbf_update_gauge_from": (I, [P, P, I, P, P]),
        "gbf_set_mass": (I, [P, D, D]),
        "gbf_delete": (I, [P]),
        "gbf_apply": (I, [P, I, PP, PP, I, I, P]),
        "gbf_field_bytes": (I, [P, I, ctypes.POINTER(ctypes.c_size_t)]),
        "gbf_field_import": (I, [P, P, P, I, I, P]),
        "gbf_field_export": (I, [P, P, P, I, I, P]),
        "gbf_norm2": (I, [P, P, I, DP, P]),
        "gbf_inner": (I, [P, P, P, I, DP, DP, P]),
        "gbf_axpby": (I, [P, P, DP, DP, P, DP, P, I, P]),
        "gbf_convert": (I, [P, P, P, P, D, I, P]),
        "gbf_solve_eo2ne_cg": (I, [P, P, P, ctypes.POINTER(gbf_cg_params), ctypes.POINTER(gbf_cg_result), P]),
        "gbf_solve_eo2ne_block_cg": (I, [P, P, P, ctypes.POINTER(gbf_cg_params), ctypes.POINTER(gbf_cg_result), P]),
        "gbf_apply_eo2ne_normal": (I, [P, P, P, P]),
        "gbf_solve_eo2ne_multishift": (I, [P, P, PP, DP, I, ctypes.POINTER(gbf_cg_params), ctypes.POINTER(gbf_cg_result), P]),
        "gbf_solve_normal_cg": (I, [P, P, P, ctypes.POINTER(gbf_cg_params), ctypes.POINTER(gbf_cg_result), P]),
        "gbf_eo2ne_prepare": (I, [P, P, P, P]),
        "gbf_eo2ne_reconstruct": (I, [P, P, P, P, P]),
        "gbf_modes_apply": (I, [P, PP, PP, DP, I, P, P, I, P]),
        "gbf_chiral_shift": (I, [P, P, P, I, I, P]),
        "gbf_axpy_norm2": (I, [P, P, DP, DP, P, P, I, DP, P]),
        "gbf_copy_slices": (I, [P, P, I, P, P, I, I, ctypes.c_double, I, P]),
        "gbf_last_error": (ctypes.c_char_p, []),
        "gbf_stream_sync": (I, [P]),
        "gbf_launch_count": (ctypes.c_ulonglong, []),
        "gbf_link_bytes": (I, [P]),
        "gbf_tune": (I, [P, P, ctypes.POINTER(ctypes.c_int), DP]),
        "gbf_set_tuning": (I, [P, ctypes.POINTER(ctypes.c_int)]),
        "gbf_random_gauge": (I, [ctypes.POINTER(ctypes.c_int), D, ctypes.c_ulonglong, P, P]),
        "gbf_random_spinor": (I, [ctypes.c_longlong, ctypes.c_ulonglong, P, P]),
        "gbf_norm2_noalloc": (I, [I, P, ctypes.c_longlong, I, DP, P]),
        "gbf_norm2_noalloc_error": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class GBFError(RuntimeError):
    """Raised for a non-zero return code of the C ABI (mirrors cgpt's
    RuntimeError from lib/cgpt/lib/exception.h:21-39)."""


def check(rc):
    if rc != 0:
        msg = load().gbf_last_error().decode()
        raise GBFError(f"gbferm error {rc}: {msg}")


def darr(values, n=16):
    a = (ctypes.c_double * n)()
    for i, v in enumerate(values):
        a[i] = v
    return a


def ptrs(ps):
    a = (ctypes.c_void_p * max(1, len(ps)))()
    for i, p in enumerate(ps):
        a[i] = p
    return a
