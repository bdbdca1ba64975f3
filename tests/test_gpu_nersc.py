"""NERSC gauge files (Grid/parallelIO/NerscIO.h) through the library's device reader and
writer against the oracle's numpy restatement: files the oracle writes read back to the
same field (bit-exact for 64-bit 3x3 payloads, within rounding otherwise) with the same
checksum, plaquette and link trace; files the library writes carry the payload checksum
and statistics the oracle computes; a corrupted payload is refused."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import nersc

pytestmark = pytest.mark.gpu

DIMS = (4, 6, 4, 8)


@pytest.mark.parametrize("fmt", ["IEEE64BIG", "IEEE64", "IEEE32BIG", "IEEE32"])
@pytest.mark.parametrize("two_row", [False, True])
def test_read_oracle_file(gpu_available, tmp_path, fmt, two_row):
    U = g.random_gauge(DIMS, 0.6, 11)
    path = tmp_path / "cfg"
    csum, plaq, tr = nersc.write(path, U, DIMS, two_row, fmt)
    V, h = g.nersc_read(path)
    want, _, _ = nersc.read(path)
    assert h.checksum_computed == csum == h.checksum
    # the statistics of the field as stored (rounded to 32 bits for IEEE32 files)
    plaq, tr = nersc.plaquette_and_trace(want, DIMS)
    assert abs(h.plaquette_computed - plaq) < 1e-12 and abs(h.link_trace_computed - tr) < 1e-12
    if fmt.startswith("IEEE64") and not two_row:
        assert np.array_equal(V, U)
    assert np.max(np.abs(V - want)) < 1e-14


@pytest.mark.parametrize("two_row,bits,big", [(False, 64, True), (True, 64, True), (False, 32, False), (True, 32, True)])
def test_write_read_by_oracle(gpu_available, tmp_path, two_row, bits, big):
    U = g.random_gauge(DIMS, 0.4, 12)
    path = tmp_path / "out"
    g.nersc_write(path, U, DIMS, two_row=two_row, bits=bits, big_endian=big)
    V, hdr, csum = nersc.read(path)
    assert int(hdr["CHECKSUM"], 16) == csum
    plaq, tr = nersc.plaquette_and_trace(U, DIMS)
    assert abs(float(hdr["PLAQUETTE"]) - plaq) < 1e-9 and abs(float(hdr["LINK_TRACE"]) - tr) < 1e-9
    assert np.max(np.abs(V - U)) < (1e-13 if bits == 64 else 1e-6)
    W, h = g.nersc_read(path)  # and our own reader accepts it
    assert np.max(np.abs(W - V)) < 1e-14


def test_corrupted_payload_is_refused(gpu_available, tmp_path):
    U = g.random_gauge(DIMS, 0.6, 13)
    path = tmp_path / "bad"
    nersc.write(path, U, DIMS, False, "IEEE64BIG")
    raw = bytearray(path.read_bytes())
    raw[-5] ^= 0x40
    path.write_bytes(bytes(raw))
    with pytest.raises(g.GridError) as e:
        g.nersc_read(path)
    assert e.value.status == 9
    V, h = g.nersc_read(path, check=False)
    assert h.checksum_computed != h.checksum


def test_gauge_stats(gpu_available):
    assert np.allclose(g.gauge_stats(DIMS, g.unit_gauge(DIMS)), (1.0, 1.0), atol=1e-15)
    U = g.random_gauge(DIMS, 0.5, 14)
    assert np.allclose(g.gauge_stats(DIMS, U), nersc.plaquette_and_trace(U, DIMS), rtol=0, atol=1e-13)
