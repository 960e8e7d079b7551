"""cgpt's fermion-operator functions, with cgpt's own signatures, on top of
libgbferm.so.

The reference reaches its fermion operators through five functions of its
native module (lib/cgpt/lib/operators.cc:34-107), called from
lib/gpt/qcd/fermion/operator/interface.py:29-103:

    create_fermion_operator(name, precision, params) -> ptr
    update_fermion_operator(ptr, params) -> 0
    set_mass_fermion_operator(ptr, params) -> 0
    delete_fermion_operator(ptr) -> 0
    apply_fermion_operator(ptr, opcode, src, dst) -> float

This module exports the same five functions with the same argument order
and meaning, so a caller written against cgpt's interface (see
INTEGRATION.md) can switch to the GB300 library by importing this module in
its place.  What differs is only the representation of grids and lattices,
which in the reference are pointers to Grid objects:

* a grid is its dimensions: params["U_grid"] = [L0, L1, L2, L3] and, for
  five-dimensional operators, params["F_grid"] = [Ls, L0, L1, L2, L3] (gpt
  inserts the fifth dimension first, lib/gpt/qcd/fermion/operator/base.py:47-52);
* a lattice is a numpy complex128 array in gpt's natural layout: a 4D
  fermion [V, 4, 3], a 5D (or multi-rhs Wilson) fermion [V, Ls, 4, 3], a
  gauge link [V, 3, 3] (params["U"] is the list of the four links, or one
  [4, V, 3, 3] array); site index x0 + L0 (x1 + L1 (x2 + L2 x3));
* an even-odd (checkerboarded) lattice is a ``checkerboarded`` array: the
  full natural shape with its checkerboard (0 even, 1 odd) attached; only its
  sites of that parity are read, and an even-odd result is written to the
  sites of its parity with the others set to zero.

precision is "single" or "double" as in the reference, or this library's
"half" (FP16 storage with a per-site scale) and "double_float" (FP64-class
arithmetic on the FP32 pipe).  Errors raise RuntimeError with the library's
message (cgpt's EXPORT turns C++ exceptions into RuntimeError,
lib/cgpt/lib/exception.h:21-39).  Every call runs on the current CUDA stream
and returns after the results are in host memory.
"""
import ctypes

import numpy as np

from . import _lib

_PREC = {"double": _lib.GBF_DOUBLE, "single": _lib.GBF_SINGLE, "half": _lib.GBF_HALF,
         "double_float": _lib.GBF_DOUBLE_FLOAT}
_EO_OPCODES = {2003, 2004, 2005, 2006, 2007, 2008, 3002, 4002}
_PARITY_FLIP = {2003, 2004, 3002, 4002}  # Meooe / DhopEO write the other parity
_FROM_4D = {2012, 2013}  # ImportPhysicalFermionSource, ImportUnphysicalFermion
_TO_4D = {2014, 2015}    # ExportPhysicalFermionSolution, ExportPhysicalFermionSource


class checkerboarded(np.ndarray):
    """A natural-layout array that holds one checkerboard (0 even, 1 odd):
    the counterpart of a gpt lattice on a red-black grid."""

    def __new__(cls, array, parity):
        obj = np.asarray(array, dtype=np.complex128).view(cls)
        obj.parity = int(parity)
        return obj

    def __array_finalize__(self, obj):
        self.parity = getattr(obj, "parity", None)


class _state:
    def __init__(self, name, precision, handle, dims, Ls, n_rhs, five_d):
        self.name = name
        self.precision = precision
        self.h = handle
        self.dims = list(dims)
        self.V = int(np.prod(dims))
        self.Ls = Ls
        self.n_rhs = n_rhs
        self.five_d = five_d


_ops = {}


def _err(msg):
    raise RuntimeError(msg)


def _check(rc):
    if rc != 0:
        _err(_lib.load().gbf_last_error().decode())


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def _gauge(params, V):
    U = params.get("U")
    if U is None:
        _err("params has no gauge field 'U'")
    if isinstance(U, (list, tuple)):
        if len(U) != 4:
            _err("params['U'] must hold the four links U_mu")
        U = np.stack([np.asarray(u, dtype=np.complex128).reshape(V, 3, 3) for u in U])
    U = np.ascontiguousarray(U, dtype=np.complex128)
    if U.size != 4 * V * 9:
        _err(f"gauge field of {U.size} complex numbers does not match 4 x {V} x 3 x 3")
    return U.reshape(4, V, 3, 3)


def _struct(name, params, dims, Ls, n_rhs):
    s = _lib.gbf_params()
    for i in range(4):
        s.dims[i] = dims[i]
    s.Ls = Ls if name in ("mobius", "zmobius") else 1
    s.n_rhs = n_rhs
    ph = params.get("boundary_phases", [1, 1, 1, 1])
    for mu in range(4):
        s.boundary_phases[2 * mu] = complex(ph[mu]).real
        s.boundary_phases[2 * mu + 1] = complex(ph[mu]).imag
    s.reconstruct = int(params.get("reconstruct", -1))
    s.xi_0 = s.nu = 1.0
    if name in ("wilson_clover", "wilson_twisted_mass"):
        if params.get("mass") is None:
            _err("params has no 'mass' (the caller converts kappa, lib/gpt/qcd/fermion/wilson.py:78-81)")
        s.mass = float(params["mass"])
        if float(params.get("cF", 1.0) or 1.0) != 1.0:
            _err("cF != 1 (open boundary conditions) is not supported")
    if name == "wilson_clover":
        s.csw_r = float(params.get("csw_r") or 0.0)
        s.csw_t = float(params.get("csw_t") or 0.0)
        s.isAnisotropic = int(bool(params.get("isAnisotropic", False)))
        s.xi_0 = float(params.get("xi_0") or 1.0)
        s.nu = float(params.get("nu") or 1.0)
    elif name == "wilson_twisted_mass":
        s.mu = float(params["mu"])
    elif name in ("mobius", "zmobius"):
        s.mass_plus = float(params["mass_plus"])
        s.mass_minus = float(params["mass_minus"])
        s.b = float(params["b"])
        s.c = float(params["c"])
        s.M5 = float(params["M5"])
        if name == "zmobius":
            om = np.array([complex(w) for w in params["omega"]], dtype=np.complex128)
            s.keep_omega = om  # alive until gbf_create has read it
            s.omega = om.ctypes.data
    return s


def create_fermion_operator(name, precision, params):
    """cgpt create_fermion_operator (operators.cc:34-57): returns the operator
    as an integer handle.  name: "wilson_clover", "wilson_twisted_mass",
    "mobius" or "zmobius"; the gauge field params["U"] is copied to the
    device, as Grid's ImportGauge copies it."""
    if precision not in _PREC:
        _err("Unknown precision")
    dims = [int(d) for d in params.get("U_grid", [])]
    if len(dims) != 4:
        _err("params['U_grid'] must give the four lattice dimensions")
    five = name in ("mobius", "zmobius")
    F = [int(d) for d in params.get("F_grid", dims)]
    Ls, n_rhs = 1, 1
    if five:
        Ls = int(params.get("Ls", F[0] if len(F) == 5 else 0))
        if name == "zmobius" and "omega" in params:
            Ls = len(params["omega"])
        if Ls < 1:
            _err("five-dimensional operator without Ls (params['F_grid'] = [Ls, L0, L1, L2, L3])")
    elif params.get("multi_rhs"):
        # multi-rhs Wilson-clover: the right-hand sides form the first
        # dimension of F_grid (lib/gpt/qcd/fermion/wilson.py:82-86)
        n_rhs = int(params.get("Ls", F[0] if len(F) == 5 else 1))
    L = _lib.load()
    s = _struct(name, params, dims, Ls, n_rhs)
    h = ctypes.c_void_p()
    _check(L.gbf_create(name.encode(), _PREC[precision], ctypes.byref(s), ctypes.byref(h)))
    st = _state(name, precision, h, dims, Ls, n_rhs, five)
    try:
        U = _gauge(params, st.V)
        _check(L.gbf_update_gauge(h, ctypes.c_void_p(U.ctypes.data), 0, ctypes.c_void_p(_stream())))
    except Exception:
        L.gbf_delete(h)
        raise
    _ops[h.value] = st
    return h.value


def _get(ptr):
    st = _ops.get(int(ptr))
    if st is None:
        _err("unknown fermion operator")
    return st


def update_fermion_operator(ptr, params):
    """cgpt update_fermion_operator (operators.cc:59-70): import a new gauge
    field (links, clover term and inverse rebuilt on the device)."""
    st = _get(ptr)
    U = _gauge(params, st.V)
    _check(_lib.load().gbf_update_gauge(st.h, ctypes.c_void_p(U.ctypes.data), 0, ctypes.c_void_p(_stream())))
    return 0


def set_mass_fermion_operator(ptr, params):
    """cgpt set_mass_fermion_operator (operators.cc:72-83 and
    lib/cgpt/lib/operators/implementation.h:21-45): Wilson-type operators
    take params["mass"], domain-wall operators params["mass_plus"] and
    params["mass_minus"]."""
    st = _get(ptr)
    L = _lib.load()
    if st.five_d:
        _check(L.gbf_set_mass(st.h, float(params["mass_plus"]), float(params["mass_minus"])))
    else:
        _check(L.gbf_set_mass(st.h, float(params["mass"]), float(params["mass"])))
    return 0


def delete_fermion_operator(ptr):
    """cgpt delete_fermion_operator (operators.cc:85-94)."""
    st = _ops.pop(int(ptr), None)
    if st is None:
        _err("unknown fermion operator")
    _check(_lib.load().gbf_delete(st.h))
    return 0


def _device(nbytes):
    import torch

    return torch.zeros(int(nbytes), dtype=torch.uint8, device="cuda")


def _natural_rhs(st, arr, four_d):
    """Split a natural array into per-rhs arrays of the library's natural
    import layout ([V, 12] for 4D fields, [V, Ls, 12] for 5D)."""
    a = np.ascontiguousarray(arr, dtype=np.complex128)
    if four_d or not st.five_d:
        if st.n_rhs == 1:
            return [a.reshape(st.V, 12)]
        a = a.reshape(st.V, st.n_rhs, 12)
        return [np.ascontiguousarray(a[:, k]) for k in range(st.n_rhs)]
    return [a.reshape(st.V, st.Ls, 12)]


def _upload(st, arr, full, four_d):
    import torch

    L = _lib.load()
    for k, part in enumerate(_natural_rhs(st, arr, four_d)):
        dev = torch.from_numpy(part.view(np.float64).reshape(-1)).to("cuda")
        _check(L.gbf_field_import(st.h, ctypes.c_void_p(dev.data_ptr()), ctypes.c_void_p(full.data_ptr()), k,
                                  int(st.five_d and not four_d), ctypes.c_void_p(_stream())))
        torch.cuda.current_stream().synchronize()


def _download(st, full, out, four_d):
    import torch

    L = _lib.load()
    per = st.V * 12 * (st.Ls if (st.five_d and not four_d) else 1)
    parts = []
    for k in range(st.n_rhs if not st.five_d or four_d else 1):
        dev = torch.zeros(2 * per, dtype=torch.float64, device="cuda")
        _check(L.gbf_field_export(st.h, ctypes.c_void_p(full.data_ptr()), ctypes.c_void_p(dev.data_ptr()), k,
                                  int(st.five_d and not four_d), ctypes.c_void_p(_stream())))
        parts.append(dev.cpu().numpy().view(np.complex128))
    if len(parts) == 1:
        res = parts[0]
    else:
        res = np.stack([p.reshape(st.V, 12) for p in parts], axis=1)
    out[...] = res.reshape(out.shape)


def _field_bytes(st, which):
    n = ctypes.c_size_t()
    _check(_lib.load().gbf_field_bytes(st.h, which, ctypes.byref(n)))
    return n.value


def apply_fermion_operator(ptr, opcode, src, dst):
    """cgpt apply_fermion_operator (operators.cc:96-107, unary.h:20-48): apply
    `opcode` to each src[i], writing dst[i] in place (lists of equal length;
    argument order src, dst as at the C level, interface.py:88-91).  Returns
    0.0, the value of every opcode implemented here (Grid's void unary
    operations)."""
    st = _get(ptr)
    opcode = int(opcode)
    if len(src) != len(dst):
        _err("src and dst lists differ in length")
    L = _lib.load()
    full5 = _field_bytes(st, 1)
    half5 = _field_bytes(st, 0)
    full4 = _field_bytes(st, 2)
    for s_arr, d_arr in zip(src, dst):
        if not isinstance(d_arr, np.ndarray) or d_arr.dtype != np.complex128 or not d_arr.flags.writeable:
            _err("dst lattices must be writable complex128 numpy arrays")
        in4, out4 = opcode in _FROM_4D, opcode in _TO_4D
        S = _device(full4 if in4 else full5)
        D = _device(full4 if out4 else full5)
        _upload(st, s_arr, S, in4)
        sp = _lib.GBF_FULL
        sptr, dptr = S.data_ptr(), D.data_ptr()
        if opcode in _EO_OPCODES:
            sp = getattr(s_arr, "parity", None)
            if sp not in (0, 1):
                _err(f"opcode {opcode} acts on a checkerboarded lattice (cgpt.checkerboarded(array, parity))")
            dp = 1 - sp if opcode in _PARITY_FLIP else sp
            sptr += sp * half5
            dptr += dp * half5
        _check(L.gbf_apply(st.h, opcode, _lib.ptrs([sptr]), _lib.ptrs([dptr]), 1, sp, ctypes.c_void_p(_stream())))
        _download(st, D, d_arr, out4)
        if opcode in _EO_OPCODES and isinstance(d_arr, checkerboarded):
            d_arr.parity = 1 - sp if opcode in _PARITY_FLIP else sp
    return 0.0
