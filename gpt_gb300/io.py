"""Gauge-field files in the NERSC format: g.load(path) / g.save(path, U,
g.format.nersc()) for the links the fermion operators import.

Follows the reference's reader and writer (lib/gpt/core/io/nersc_io.py:24-380):

* a text header between BEGIN_HEADER and END_HEADER of `KEY = value` lines
  with DIMENSION_1..4, DATATYPE (4D_SU3_GAUGE_3x3: full matrices,
  4D_SU3_GAUGE: the first two rows, the third rebuilt as the complex
  conjugate of their cross product, lib/cgpt/lib/munge.h:21-39),
  FLOATING_POINT (IEEE64BIG/LITTLE, IEEE32BIG/LITTLE), CHECKSUM, PLAQUETTE
  and LINK_TRACE;
* then the links site by site (x fastest), mu = 0..3 per site, each matrix
  row-major, complex numbers as (re, im);
* CHECKSUM is the sum modulo 2^32 of the data's 32-bit words in host byte
  order before the third row is rebuilt (lib/cgpt/lib/checksums/nersc.h:19-31);
* PLAQUETTE and LINK_TRACE are checked to the digits the header gives
  (nersc_io.py:226-246); files are written as IEEE64BIG 3x3.

The byte swapping, reordering and row reconstruction are vectorised numpy on
the host (the file system bounds this path; the links then go to the device
through gbf_update_gauge)."""
import datetime
import getpass
import os
import socket

import numpy as np

from . import core
from .qcd import gauge as _gauge


class format:
    class nersc:
        def __init__(self, params=None, **kw):
            p = {"id": "gpt_gb300", "label": "", "sequence_number": 1}
            p.update(params or {})
            p.update(kw)
            self.params = p


_FP = {
    "IEEE64BIG": (">f8", core.double),
    "IEEE64LITTLE": ("<f8", core.double),
    "IEEE64": ("<f8", core.double),
    "IEEE32BIG": (">f4", core.single),
    "IEEE32LITTLE": ("<f4", core.single),
    "IEEE32": ("<f4", core.single),
}


def _read_header(path):
    with open(path, "rb") as f:
        first = f.readline()
        try:
            if first.decode("utf-8").strip() != "BEGIN_HEADER":
                return None
        except UnicodeDecodeError:
            return None
        meta = {}
        while True:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: no END_HEADER")
            line = line.decode("utf-8").strip()
            if line == "END_HEADER":
                break
            key, val = line.split("=", 1)
            meta[key.strip()] = val.strip()
        return meta, f.tell()


def checksum(words):
    """NERSC checksum: sum of the uint32 words modulo 2^32."""
    w = np.ascontiguousarray(words).view(np.uint32)
    return int(w.sum(dtype=np.uint64) & 0xFFFFFFFF)


def reconstruct_third_row(m):
    """[..., 2, 3] complex -> [..., 3, 3] with row 2 = conj(row0 x row1)."""
    out = np.empty(m.shape[:-2] + (3, 3), dtype=m.dtype)
    out[..., :2, :] = m
    a, b = m[..., 0, :], m[..., 1, :]
    out[..., 2, 0] = np.conj(a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1])
    out[..., 2, 1] = np.conj(a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2])
    out[..., 2, 2] = np.conj(a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0])
    return out


def link_trace(U):
    """Re tr U / 3 averaged over sites and directions (nersc_io.py:239-241)."""
    H = U.host()
    return float(np.real(np.trace(H, axis1=2, axis2=3)).sum() / H.shape[1] / 3 / 4)


def _digits_tolerance(text, eps):
    frac = text.split(".")[1].lower().split("e")[0] if "." in text else ""
    return max(1e2 * eps, 10.0 ** (-len(frac) + 2))


def load(path):
    """Read a NERSC gauge file into a gauge_field (grid precision from the file)."""
    h = _read_header(path)
    if h is None:
        raise NotImplementedError(f"{path}: not a NERSC file")
    meta, offset = h
    dims = [int(meta[f"DIMENSION_{i + 1}"]) for i in range(4)]
    dtype, prec = _FP[meta["FLOATING_POINT"]]
    kind = meta["DATATYPE"]
    rows = {"4D_SU3_GAUGE_3x3": 3, "4D_SU3_GAUGE": 2}.get(kind)
    if rows is None:
        raise NotImplementedError(f"{path}: data type {kind}")
    V = int(np.prod(dims))
    raw = np.fromfile(path, dtype=dtype, offset=offset)
    if raw.size != V * 4 * rows * 3 * 2:
        raise ValueError(f"{path}: {raw.size} numbers, expected {V * 4 * rows * 3 * 2}")
    host = raw.astype(raw.dtype.newbyteorder("="))  # host byte order
    cs = checksum(host)
    cs_exp = int(meta["CHECKSUM"], 16)
    if cs != cs_exp:
        raise ValueError(f"{path}: checksum {cs:x} != {cs_exp:x}")
    m = host.astype(np.float64).view(np.complex128).reshape(V, 4, rows, 3)
    if rows == 2:
        m = reconstruct_third_row(m)
    U = _gauge.gauge_field(core.grid(dims, prec), np.ascontiguousarray(np.transpose(m, (1, 0, 2, 3))))
    U.metadata = meta
    eps = prec.eps
    P, L = _gauge.plaquette(U), link_trace(U)
    if abs(P - float(meta["PLAQUETTE"])) >= _digits_tolerance(meta["PLAQUETTE"], eps):
        raise ValueError(f"{path}: plaquette {P} != header {meta['PLAQUETTE']}")
    if abs(L - float(meta["LINK_TRACE"])) >= _digits_tolerance(meta["LINK_TRACE"], eps):
        raise ValueError(f"{path}: link trace {L} != header {meta['LINK_TRACE']}")
    return U


def save(path, U, fmt=None):
    """Write a gauge_field as NERSC 4D_SU3_GAUGE_3x3 IEEE64BIG (nersc_io.py:263-380)."""
    fmt = fmt if fmt is not None else format.nersc()
    p = fmt.params
    H = U.host()
    dims = U.grid.fdimensions
    data = np.ascontiguousarray(np.transpose(H, (1, 0, 2, 3)))  # [site][mu][3][3]
    cs = checksum(data.view(np.float64))
    L, P = link_trace(U), _gauge.plaquette(U)
    now = datetime.datetime.now(datetime.timezone.utc).strftime("%c %Z")
    header = "\n".join([
        "BEGIN_HEADER", "HDR_VERSION = 1.0", "DATATYPE = 4D_SU3_GAUGE_3x3", "STORAGE_FORMAT =",
        *[f"DIMENSION_{i + 1} = {dims[i]}" for i in range(4)],
        f"LINK_TRACE = {L:.15g}", f"PLAQUETTE  = {P:.15g}",
        *[f"BOUNDARY_{i + 1} = PERIODIC" for i in range(4)],
        f"CHECKSUM =   {cs:x}", "SCIDAC_CHECKSUMA =          0", "SCIDAC_CHECKSUMB =          0",
        f"ENSEMBLE_ID = {p['id']}", f"ENSEMBLE_LABEL = {p['label']}", f"SEQUENCE_NUMBER = {p['sequence_number']}",
        f"CREATOR = {getpass.getuser()}", f"CREATOR_HARDWARE = {socket.gethostname()}",
        f"CREATION_DATE = {now}", f"ARCHIVE_DATE = {now}", "FLOATING_POINT = IEEE64BIG", "END_HEADER", ""])
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "wb") as f:
        f.write(header.encode("utf-8"))
        data.view(np.float64).astype(">f8").tofile(f)
    os.replace(tmp, path)
