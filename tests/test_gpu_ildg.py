"""ILDG / SciDAC gauge files (Grid/parallelIO/IldgIO.h) through the library's device
reader and writer against the oracle's numpy restatement (zlib CRC-32): files the oracle
writes read back bit-exact (64-bit) or as rounded (32-bit) with the same SciDAC
checksums and statistics; files the library writes carry the checksums and usqcdInfo the
oracle computes; corrupted or checksum-less files are refused."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import ildg, nersc

pytestmark = pytest.mark.gpu

DIMS = (4, 6, 4, 8)


@pytest.mark.parametrize("precision", [64, 32])
def test_read_oracle_file(gpu_available, tmp_path, precision):
    U = g.random_gauge(DIMS, 0.6, 21)
    path = tmp_path / "cfg.lime"
    suma, sumb = ildg.write(path, U, DIMS, precision, lfn="lfn://ens/cfg.1000")
    V, h = g.ildg_read(path)
    want, meta = ildg.read(path)
    assert np.array_equal(V, want)
    if precision == 64:
        assert np.array_equal(V, U)
    assert (h.scidac_suma_computed, h.scidac_sumb_computed) == (suma, sumb) == (h.scidac_suma, h.scidac_sumb)
    plaq, tr = nersc.plaquette_and_trace(want, DIMS)
    assert abs(h.plaquette_computed - plaq) < 1e-12 and abs(h.link_trace_computed - tr) < 1e-12
    assert h.lfn == b"lfn://ens/cfg.1000"


@pytest.mark.parametrize("precision", [64, 32])
def test_write_read_by_oracle(gpu_available, tmp_path, precision):
    U = g.random_gauge(DIMS, 0.4, 22)
    path = tmp_path / "out.lime"
    g.ildg_write(path, U, DIMS, precision, lfn="run7")
    types = [r[0] for r in ildg.lime_records(path)]
    assert types == ["scidac-private-file-xml", "scidac-file-xml", "scidac-private-record-xml", "scidac-record-xml",
                     "ildg-format", "ildg-data-lfn", "ildg-binary-data", "scidac-checksum"]
    V, meta = ildg.read(path)
    want = U if precision == 64 else U.astype(np.complex64).astype(np.complex128)
    assert np.array_equal(V, want)
    assert (meta["suma"], meta["sumb"]) == (meta["suma_computed"], meta["sumb_computed"])
    plaq, tr = nersc.plaquette_and_trace(U, DIMS)
    assert abs(meta["plaquette"] - plaq) < 1e-12 and abs(meta["link_trace"] - tr) < 1e-12
    assert meta["lfn"] == "run7" and meta["precision"] == precision
    # and back through the library
    W, h = g.ildg_read(path)
    assert np.array_equal(W, want)


def test_corrupt_and_unchecked_files(gpu_available, tmp_path):
    U = g.random_gauge(DIMS, 0.5, 23)
    path = tmp_path / "cfg.lime"
    ildg.write(path, U, DIMS, 64)
    rec = [r for r in ildg.lime_records(path) if r[0] == "ildg-binary-data"][0]
    raw = bytearray(path.read_bytes())
    raw[rec[3] + 1000] ^= 0x10
    bad = tmp_path / "bad.lime"
    bad.write_bytes(bytes(raw))
    with pytest.raises(g.GridError):
        g.ildg_read(bad)
    V, h = g.ildg_read(bad, check=False)
    assert (h.scidac_suma_computed, h.scidac_sumb_computed) != (h.scidac_suma, h.scidac_sumb)
    ildg.write(tmp_path / "nock.lime", U, DIMS, 64, with_checksum=False)
    with pytest.raises(g.GridError):
        g.ildg_read(tmp_path / "nock.lime")
    # a wrong plaquette in usqcdInfo is refused, as Grid asserts
    ildg.write(tmp_path / "plaq.lime", U, DIMS, 64, plaquette=(0.123, 0.456))
    with pytest.raises(g.GridError):
        g.ildg_read(tmp_path / "plaq.lime")
