"""NERSC gauge files (lib/gpt/core/io/nersc_io.py; the reference's round-trip
test is tests/io/io.py:198-206: save, load, relative difference < 1e-14)."""
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
