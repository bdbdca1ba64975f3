"""Gauge-file formats on the CPU. ILDG / SciDAC: the oracle's restatement pinned (CRC-32 check value,
checksum rotation, LIME framing, write/read round trip) and the library's host-side LIME
and XML parsing (gb_ildg_read_header, no device work) on files the oracle writes.
openQCD: the header parser (gb_openqcd_read_header)."""
import zlib

import numpy as np
import pytest

import grid_gb300 as g
from oracle import ildg

DIMS = (2, 2, 4, 4)


def test_crc32_check_value_and_rotation():
    # the CRC-32 check value of the IEEE 802.3 / zlib polynomial
    assert zlib.crc32(b"123456789") == 0xCBF43926
    # two sites: site 0 is not rotated, site 1 by one bit in both sums (1 % 29 = 1 % 31 = 1)
    sb = np.frombuffer(b"abcdefgh" * 2, dtype=np.uint8).reshape(2, 8).copy()
    sb[1, 0] = ord("z")
    c0, c1 = zlib.crc32(sb[0].tobytes()), zlib.crc32(sb[1].tobytes())
    r1 = ((c1 << 1) | (c1 >> 31)) & 0xFFFFFFFF
    assert ildg.scidac_checksum(sb) == (c0 ^ r1, c0 ^ r1)


@pytest.mark.parametrize("precision", [64, 32])
def test_oracle_round_trip_and_framing(tmp_path, precision):
    U = g.random_gauge(DIMS, 0.5, 5)
    path = tmp_path / "cfg.lime"
    suma, sumb = ildg.write(path, U, DIMS, precision, lfn="lfn://test/1")
    raw = path.read_bytes()
    assert raw[:4] == bytes([0x45, 0x67, 0x89, 0xAB]) and len(raw) % 8 == 0
    recs = ildg.lime_records(path)
    types = [r[0] for r in recs]
    assert types == ["scidac-private-file-xml", "scidac-file-xml", "scidac-private-record-xml", "scidac-record-xml",
                     "ildg-format", "ildg-data-lfn", "ildg-binary-data", "scidac-checksum"]
    assert [(r[1], r[2]) for r in recs] == [(True, False), (False, True), (True, False), (False, False),
                                            (False, False), (False, False), (False, False), (False, True)]
    V, meta = ildg.read(path)
    want = U if precision == 64 else U.astype(np.complex64).astype(np.complex128)
    assert np.array_equal(V, want)
    assert (meta["suma"], meta["sumb"]) == (suma, sumb) == (meta["suma_computed"], meta["sumb_computed"])
    assert meta["lfn"] == "lfn://test/1" and meta["dims"] == list(DIMS) and meta["field"] == "su3gauge"


def test_library_parses_oracle_records(tmp_path):
    U = g.random_gauge(DIMS, 0.5, 6)
    path = tmp_path / "cfg.lime"
    suma, sumb = ildg.write(path, U, DIMS, 32, lfn="conf.100")
    h = g.ildg_read_header(path)
    assert list(h.dims) == list(DIMS) and h.precision == 32 and h.field == b"su3gauge" and h.lfn == b"conf.100"
    assert h.has_checksum == 1 and (h.scidac_suma, h.scidac_sumb) == (suma, sumb)
    assert h.has_plaquette == 1 and h.data_bytes == int(np.prod(DIMS)) * 72 * 4
    rec = [r for r in ildg.lime_records(path) if r[0] == "ildg-binary-data"][0]
    assert h.data_offset == rec[3]
    # no checksum record: parsed, flagged
    ildg.write(tmp_path / "nock.lime", U, DIMS, 64, with_checksum=False)
    assert g.ildg_read_header(tmp_path / "nock.lime").has_checksum == 0
    # a truncated file and a file that is not LIME are refused
    (tmp_path / "short.lime").write_bytes(path.read_bytes()[:-100])
    (tmp_path / "junk.lime").write_bytes(b"BEGIN_HEADER\n" + b"x" * 200)
    for bad in ("short.lime", "junk.lime"):
        with pytest.raises(g.GridError):
            g.ildg_read_header(tmp_path / bad)


def test_library_parses_openqcd_header(tmp_path):
    """openQCD header (OpenQcdIO.h:43-75) on the host: int32 Nt Nx Ny Nz (Grid order back
    to x y z t) and the plaquette divided by Nc; implausible extents are refused."""
    import ctypes

    from oracle import openqcd
    dims = (4, 6, 4, 8)
    U = g.random_gauge(dims, 0.5, 7)
    path = tmp_path / "cfg.oq"
    plaq = openqcd.write(path, U, dims)
    d = (ctypes.c_int * 4)()
    p = ctypes.c_double()
    assert g.lib.gb_openqcd_read_header(str(path).encode(), d, ctypes.byref(p)) == 0
    assert tuple(d) == dims and abs(p.value - plaq) < 1e-15
    (tmp_path / "swapped.oq").write_bytes(path.read_bytes()[:4][::-1] + path.read_bytes()[4:])
    assert g.lib.gb_openqcd_read_header(str(tmp_path / "swapped.oq").encode(), d, ctypes.byref(p)) != 0
