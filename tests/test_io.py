"""Gauge files: NERSC (lib/gpt/core/io/nersc_io.py) and LIME containers
(lib/gpt/core/io/lime_io: gpt's lime format and ILDG files with SciDAC
checksums).  The reference's round-trip tests are tests/io/io.py:198-216
(save, load, relative difference < 1e-14); here the round trips are exact."""
import os

import numpy as np
import pytest

import gpt_gb300 as g
from gpt_gb300 import io as gio


def _field(dims=(4, 4, 4, 8), seed=7):
    return g.qcd.gauge.random_su3(g.grid(list(dims)), 0.4, seed)


def _write(path, meta, data, dtype):
    lines = ["BEGIN_HEADER"] + [f"{k} = {v}" for k, v in meta.items()] + ["END_HEADER", ""]
    with open(path, "wb") as f:
        f.write("\n".join(lines).encode())
        np.asarray(data, dtype=np.float64).astype(dtype).tofile(f)


def _meta(U, kind, fp, cs):
    d = U.grid.fdimensions
    return {"HDR_VERSION": "1.0", "DATATYPE": kind, **{f"DIMENSION_{i + 1}": d[i] for i in range(4)},
            "LINK_TRACE": f"{gio.link_trace(U):.15g}", "PLAQUETTE": f"{g.qcd.gauge.plaquette(U):.15g}",
            "CHECKSUM": f"{cs:x}", "FLOATING_POINT": fp}


def test_round_trip_is_exact(tmp_path):
    U = _field()
    fn = str(tmp_path / "ckpoint_lat.10")
    g.save(fn, U, g.format.nersc(id="test", sequence_number=10))
    V = g.load(fn)
    assert V.grid.fdimensions == U.grid.fdimensions and V.grid.precision is g.double
    assert np.array_equal(V.host(), U.host())
    assert V.metadata["DATATYPE"] == "4D_SU3_GAUGE_3x3" and V.metadata["FLOATING_POINT"] == "IEEE64BIG"
    assert V.metadata["SEQUENCE_NUMBER"] == "10"


def test_two_row_storage_rebuilds_the_third_row(tmp_path):
    U = _field(seed=3)
    H = U.host()
    two = np.ascontiguousarray(np.transpose(H, (1, 0, 2, 3))[:, :, :2, :])  # [site][mu][2][3]
    cs = gio.checksum(two.view(np.float64))
    fn = str(tmp_path / "two_rows")
    _write(fn, _meta(U, "4D_SU3_GAUGE", "IEEE64LITTLE", cs), two.view(np.float64).ravel(), "<f8")
    V = g.load(fn)
    assert np.abs(V.host() - H).max() < 1e-14


def test_single_precision_big_endian(tmp_path):
    U = _field(seed=5)
    data = np.transpose(U.host(), (1, 0, 2, 3)).astype(np.complex64)
    cs = gio.checksum(np.ascontiguousarray(data).view(np.float32))
    fn = str(tmp_path / "single")
    meta = _meta(U, "4D_SU3_GAUGE_3x3", "IEEE32BIG", cs)
    meta["PLAQUETTE"] = f"{g.qcd.gauge.plaquette(U):.6f}"
    meta["LINK_TRACE"] = f"{gio.link_trace(U):.6f}"
    _write(fn, meta, data.view(np.float32).ravel(), ">f4")
    V = g.load(fn)
    assert V.grid.precision is g.single
    assert np.abs(V.host() - U.host()).max() < 1e-6


def test_corrupt_files_are_rejected(tmp_path):
    U = _field(seed=9)
    fn = str(tmp_path / "ck")
    g.save(fn, U)
    raw = bytearray(open(fn, "rb").read())
    raw[-5] ^= 0x40  # flip a bit of the last number
    bad = str(tmp_path / "ck_bad")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        g.load(bad)
    text = open(fn, "rb").read()
    plaq = text.replace(b"PLAQUETTE  = 0.", b"PLAQUETTE  = 0.9", 1)
    wrong = str(tmp_path / "ck_plaq")
    open(wrong, "wb").write(plaq)
    with pytest.raises(ValueError, match="plaquette"):
        g.load(wrong)
    other = str(tmp_path / "not_nersc")
    open(other, "wb").write(b"\x00\x01binary")
    with pytest.raises(NotImplementedError):
        g.load(other)


@pytest.mark.gpu
def test_loaded_field_gives_the_same_operator(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    U = _field(dims=(8, 8, 8, 8), seed=11)
    fn = str(tmp_path / "ck8")
    g.save(fn, U)
    V = g.load(fn)
    p = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1])
    a, b = g.qcd.fermion.wilson_clover(U, p), g.qcd.fermion.wilson_clover(V, p)
    r = np.random.default_rng(1)
    s = r.standard_normal((8 ** 4, 4, 3)) + 1j * r.standard_normal((8 ** 4, 4, 3))
    x, y = a.F_lattice(), b.F_lattice()
    x[:] = s
    y[:] = s
    assert np.array_equal(a.M(x)[:], b.M(y)[:])


# ---------------------------------------------------------------------------
# LIME containers: gpt's lime format (the reference's round trip,
# tests/io/io.py:208-216) and ILDG files (lime_io/load.py ildg-format branch)
# ---------------------------------------------------------------------------
def _lime_rec(tag, data):
    import struct

    h = struct.pack(">LHHQ", 0x456789AB, 1, 0xC000, len(data)) + tag.encode() + b"\0" * (128 - len(tag))
    return h + data + b"\0" * ((8 - len(data) % 8) % 8)


def _scidac_ref(site_bytes):
    """Independent statement of the SciDAC checksum (lime_io/scidac.py:23-33)
    with binascii and Python integers."""
    import binascii

    a = b = 0
    for i, row in enumerate(site_bytes):
        c = binascii.crc32(bytes(row)) & 0xFFFFFFFF
        for m, acc in ((29, "a"), (31, "b")):
            k = i % m
            r = ((c << k) | (c >> (32 - k))) & 0xFFFFFFFF
            if acc == "a":
                a ^= r
            else:
                b ^= r
    return a, b


def test_lime_round_trip_is_exact(tmp_path):
    U = _field(seed=21)
    fn = str(tmp_path / "lime.0000")
    g.save(fn, U, g.format.lime())
    V = g.load(fn)
    assert V.grid.fdimensions == U.grid.fdimensions and V.grid.precision is g.double
    assert np.array_equal(V.host(), U.host())
    assert V.metadata["otype"].startswith("ot_matrix_su_n_fundamental_group(3)")


@pytest.mark.parametrize("bits", [64, 32])
def test_ildg_round_trip(tmp_path, bits):
    U = _field(seed=22)
    fn = str(tmp_path / f"ildg{bits}")
    g.save(fn, U, g.format.ildg(precision=bits))
    V = g.load(fn)
    assert V.grid.precision is (g.double if bits == 64 else g.single)
    if bits == 64:
        assert np.array_equal(V.host(), U.host())
    else:
        assert np.abs(V.host() - U.host()).max() < 1e-6


def test_hand_built_ildg_file_with_namespaces_and_extra_records(tmp_path):
    """An ILDG file as other writers produce it (namespaced XML, xlf-info and
    lfn records, checksum written before the data), checked with an
    independent statement of the SciDAC checksum."""
    U = _field(dims=(4, 2, 2, 6), seed=23)
    d = U.grid.fdimensions
    data = np.ascontiguousarray(np.transpose(U.host(), (1, 0, 2, 3))).view(np.float64).astype(">f8")
    site_bytes = data.view(np.uint8).reshape(int(np.prod(d)), -1)
    a, b = _scidac_ref(site_bytes)
    assert (a, b) == gio.scidac_checksums(site_bytes)
    fmt = (f'<?xml version="1.0" encoding="UTF-8"?><ildgFormat xmlns="http://www.lqcd.org/ildg" '
           f'xmlns:xsi="http://www.w3.org/2001/XMLSchema-instance"><version>1.0</version><field>su3gauge</field>'
           f'<precision>64</precision><lx>{d[0]}</lx><ly>{d[1]}</ly><lz>{d[2]}</lz><lt>{d[3]}</lt></ildgFormat>')
    cs = f"<?xml version='1.0'?><scidacChecksum><version>1.0</version><suma>{a:x}</suma><sumb>{b:x}</sumb></scidacChecksum>"
    blob = (_lime_rec("xlf-info", b"plaquette = 0.5\n") + _lime_rec("ildg-format", fmt.encode())
            + _lime_rec("scidac-checksum", cs.encode()) + _lime_rec("ildg-data-lfn", b"lfn://test/1")
            + _lime_rec("ildg-binary-data", data.tobytes()))
    fn = str(tmp_path / "ext.ildg")
    open(fn, "wb").write(blob)
    V = g.load(fn)
    assert V.grid.fdimensions == list(d) and np.array_equal(V.host(), U.host())


def test_corrupt_lime_files_are_rejected(tmp_path):
    U = _field(seed=24)
    fn = str(tmp_path / "ck.ildg")
    g.save(fn, U, g.format.ildg())
    raw = bytearray(open(fn, "rb").read())
    i = raw.index(b"ildg-binary-data") + 128 + 100  # inside the binary data
    raw[i] ^= 0x01
    bad = str(tmp_path / "bad.ildg")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        g.load(bad)
    short = str(tmp_path / "short.ildg")
    open(short, "wb").write(open(fn, "rb").read()[:-4096])
    with pytest.raises(ValueError, match="truncated"):
        g.load(short)
    other = str(tmp_path / "prop.lime")
    fmt = b"<ildgFormat><version>1.0</version><field>diracFermion</field><precision>64</precision></ildgFormat>"
    open(other, "wb").write(_lime_rec("ildg-format", fmt) + _lime_rec("ildg-binary-data", b"\0" * 64))
    with pytest.raises(NotImplementedError):
        g.load(other)
