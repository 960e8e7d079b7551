"""Gauge-field files: g.load(path) / g.save(path, U, fmt) for the links the
fermion operators import, in the NERSC format and in LIME containers (ILDG
files, and gpt's own lime format for gauge fields).

NERSC:

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

LIME (lib/gpt/core/io/lime_io/load.py:28-234, save.py:105-223; the ILDG
branch of lib/cgpt/lib/io/ildg.h):

* a sequence of records, each a 144-byte header (magic 0x456789ab, version 1,
  MB/ME flags, data length, 128-byte type name; big-endian) followed by the
  data padded to a multiple of 8 bytes;
* ILDG files: an `ildg-format` XML record (field su3gauge, precision 64 or
  32, lx ly lz lt) and `ildg-binary-data`; gpt's lime files: `gpt-format`
  (grid, n = 4, otype) and `gpt-binary-data`;
* the binary data: sites in lexicographic order (x fastest), per site the
  four links mu = x, y, z, t, each 3x3 row-major, complex (re, im),
  big-endian IEEE;
* `scidac-checksum` (suma, sumb): per-site CRC32 of the site's bytes as
  stored, rotated left by (site mod 29) resp. (site mod 31), XOR over the
  sites (lime_io/scidac.py:23-46).

The byte swapping, reordering and row reconstruction are vectorised numpy on
the host (the file system bounds this path; the links then go to the device
through gbf_update_gauge)."""
import datetime
import getpass
import os
import socket
import struct
import xml.etree.ElementTree as ET
import zlib

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

    class lime:
        """gpt's lime format (lib/gpt/core/io/save.py:31-35): extra text
        records `tags` written in `tag_order`, the links under
        binary_data_tag, then scidac-checksum and gpt-format."""

        def __init__(self, params=None, **kw):
            p = {"binary_data_tag": "gpt-binary-data", "tags": {}, "tag_order": []}
            p.update(params or {})
            p.update(kw)
            self.params = p

    class ildg:
        """An ILDG file: ildg-format, ildg-binary-data (precision 64 or 32),
        scidac-checksum."""

        def __init__(self, params=None, **kw):
            p = {"precision": 64, "lfn": ""}
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


# ---------------------------------------------------------------------------
# LIME containers
# ---------------------------------------------------------------------------
LIME_MAGIC = 0x456789AB


def _lime_records(path):
    """{type: (offset, size)} of the records of a LIME file, or None."""
    rec = {}
    size_all = os.path.getsize(path)
    with open(path, "rb") as f:
        head = f.read(4)
        if len(head) < 4 or struct.unpack(">L", head)[0] != LIME_MAGIC:
            return None
        pos = 0
        while pos < size_all:
            f.seek(pos)
            h = f.read(144)
            if len(h) < 144:
                raise ValueError(f"{path}: truncated LIME record header")
            magic, version, _flags, size = struct.unpack(">LHHQ", h[:16])
            if magic != LIME_MAGIC or version != 1:
                raise ValueError(f"{path}: bad LIME record header at byte {pos}")
            tag = h[16:144].split(b"\0", 1)[0].decode("utf-8")
            if pos + 144 + size > size_all:
                raise ValueError(f"{path}: truncated LIME record {tag}")
            rec[tag] = (pos + 144, size)
            pos += 144 + size + ((8 - size % 8) % 8)
    return rec


def _lime_text(path, rec, tag):
    off, size = rec[tag]
    with open(path, "rb") as f:
        f.seek(off)
        return f.read(size).decode("utf-8").strip("\0")


def _xml_dict(text):
    d = {}
    for child in ET.fromstring(text):
        t = child.tag
        if t.startswith("{"):
            t = t[t.index("}") + 1:]
        d[t] = (child.text or "").strip()
    return d


def scidac_checksums(site_bytes):
    """(suma, sumb) of the binary data, one row of bytes per site in
    lexicographic order (lime_io/scidac.py:23-46)."""
    nsite = site_bytes.shape[0]
    crc = np.fromiter((zlib.crc32(site_bytes[i].tobytes()) for i in range(nsite)), dtype=np.uint64, count=nsite)
    idx = np.arange(nsite, dtype=np.uint64)
    out = []
    for m in (29, 31):
        k = idx % np.uint64(m)
        rot = ((crc << k) | (crc >> (np.uint64(32) - k))) & np.uint64(0xFFFFFFFF)
        out.append(int(np.bitwise_xor.reduce(rot)) if nsite else 0)
    return out[0], out[1]


_GAUGE_OTYPES = ("ot_matrix_su_n_fundamental_group(3)", "ot_matrix_color(3)")


def _load_lime(path, rec):
    if "ildg-format" in rec:
        d = _xml_dict(_lime_text(path, rec, "ildg-format"))
        if d.get("field") != "su3gauge":
            raise NotImplementedError(f"{path}: ILDG field {d.get('field')}")
        dims = [int(d["lx"]), int(d["ly"]), int(d["lz"]), int(d["lt"])]
        bits = int(d["precision"])
    elif "gpt-format" in rec:
        d = _xml_dict(_lime_text(path, rec, "gpt-format"))
        parts = d["grid"].split(";")
        if len(parts) != 3 or int(d["n"]) != 4 or d["otype"].split(";")[0] not in _GAUGE_OTYPES:
            raise NotImplementedError(f"{path}: only gauge fields (4 colour matrices on a full 4D grid) are read")
        dims = [int(x) for x in parts[0].strip("[]").split(",")]
        bits = {"double": 64, "single": 32}[parts[1]]
    else:
        raise NotImplementedError(f"{path}: LIME file without ildg-format or gpt-format record")
    if len(dims) != 4:
        raise NotImplementedError(f"{path}: {len(dims)}-dimensional grid")
    tags = [t for t in rec if t.endswith("-binary-data")]
    if len(tags) != 1:
        raise ValueError(f"{path}: expected one *-binary-data record, found {tags}")
    off, size = rec[tags[0]]
    V = int(np.prod(dims))
    word = 8 if bits == 64 else 4
    site = 4 * 9 * 2 * word
    if size != V * site:
        raise ValueError(f"{path}: binary data of {size} bytes, expected {V * site}")
    raw = np.fromfile(path, dtype=np.uint8, count=size, offset=off).reshape(V, site)
    if "scidac-checksum" in rec:
        c = _xml_dict(_lime_text(path, rec, "scidac-checksum"))
        a, b = scidac_checksums(raw)
        if a != int(c["suma"], 16) or b != int(c["sumb"], 16):
            raise ValueError(f"{path}: scidac checksum {a:x} {b:x} != {c['suma'].strip()} {c['sumb'].strip()}")
    vals = raw.reshape(-1).view(">f8" if bits == 64 else ">f4").astype(np.float64)
    m = vals.view(np.complex128).reshape(V, 4, 3, 3)
    prec = core.double if bits == 64 else core.single
    U = _gauge.gauge_field(core.grid(dims, prec), np.ascontiguousarray(np.transpose(m, (1, 0, 2, 3))))
    U.metadata = dict(d)
    return U


def _lime_record(f, tag, data, first, last):
    flags = (0x8000 if first else 0) | (0x4000 if last else 0)
    f.write(struct.pack(">LHHQ", LIME_MAGIC, 1, flags, len(data)))
    t = tag.encode("utf-8") + b"\0"
    if len(t) > 128:
        raise ValueError(f"LIME record type too long: {tag}")
    f.write(t + b"\0" * (128 - len(t)))
    f.write(data)
    f.write(b"\0" * ((8 - len(data) % 8) % 8))


def _xml_text(root, d):
    r = ET.Element(root)
    for k, v in d.items():
        ET.SubElement(r, k).text = str(v)
    return ET.tostring(r, encoding="utf-8", xml_declaration=True)


def _save_lime(path, U, fmt):
    """gpt lime (format.lime) or ILDG (format.ildg) file of a gauge field."""
    H = U.host()
    dims = U.grid.fdimensions
    ildg = isinstance(fmt, format.ildg)
    bits = int(fmt.params["precision"]) if ildg else (64 if U.grid.precision is core.double else 32)
    if bits not in (32, 64):
        raise ValueError("ILDG precision is 32 or 64")
    data = np.ascontiguousarray(np.transpose(H, (1, 0, 2, 3)))  # [site][mu][3][3]
    raw = data.view(np.float64).astype(">f8" if bits == 64 else ">f4")
    V = int(np.prod(dims))
    site_bytes = raw.view(np.uint8).reshape(V, -1)
    a, b = scidac_checksums(site_bytes)
    records = []
    if ildg:
        records.append(("ildg-format", _xml_text("ildgFormat", {
            "version": "1.0", "field": "su3gauge", "precision": bits,
            "lx": dims[0], "ly": dims[1], "lz": dims[2], "lt": dims[3]})))
        if fmt.params.get("lfn"):
            records.append(("ildg-data-lfn", str(fmt.params["lfn"]).encode("utf-8")))
        records.append(("ildg-binary-data", raw.tobytes()))
    else:
        p = fmt.params
        for t in p["tag_order"]:
            records.append((t, str(p["tags"][t]).encode("utf-8")))
        records.append((p["binary_data_tag"], raw.tobytes()))
    records.append(("scidac-checksum", _xml_text("scidacChecksum", {"version": "1.0", "suma": f"{a:8x}",
                                                                    "sumb": f"{b:8x}"})))
    if not ildg:
        grid_desc = f"[{','.join(str(x) for x in dims)}];{'double' if bits == 64 else 'single'};full"
        records.append(("gpt-format", _xml_text("gptFormat", {
            "grid": grid_desc, "n": 4, "otype": "ot_matrix_su_n_fundamental_group(3);full"})))
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "wb") as f:
        for i, (t, d) in enumerate(records):
            _lime_record(f, t, d, i == 0, i == len(records) - 1)
    os.replace(tmp, path)


def load(path):
    """Read a NERSC or LIME (ILDG, gpt lime) gauge file into a gauge_field
    (grid precision from the file)."""
    rec = _lime_records(path)
    if rec is not None:
        return _load_lime(path, rec)
    h = _read_header(path)
    if h is None:
        raise NotImplementedError(f"{path}: neither a NERSC nor a LIME file")
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
    """Write a gauge_field: NERSC 4D_SU3_GAUGE_3x3 IEEE64BIG
    (nersc_io.py:263-380, the default), gpt lime (format.lime) or ILDG
    (format.ildg)."""
    fmt = fmt if fmt is not None else format.nersc()
    if isinstance(fmt, (format.lime, format.ildg)):
        return _save_lime(path, U, fmt)
    if not isinstance(fmt, format.nersc):
        raise NotImplementedError(f"format {type(fmt).__name__}")
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
