"""NERSC gauge-file restatement in numpy (TEST INFRASTRUCTURE ONLY: the checker for the
library's reader/writer; the product never imports it).

Follows Grid/parallelIO/NerscIO.h:62-300 and MetaData.h:143-218,320-342:
  * header "BEGIN_HEADER / KEY = value / END_HEADER", then the payload;
  * payload site-lexicographic (x fastest), per site 4 links, per link the first two rows
    (4D_SU3_GAUGE; row 2 = conj(row 0 x row 1)) or all three (4D_SU3_GAUGE_3x3), complex
    (re, im), IEEE32/64, big- or little-endian;
  * CHECKSUM = 32-bit wrapping sum of the payload's 32-bit words in host byte order
    (BinaryIO.h:109-137);
  * PLAQUETTE = avgPlaquette, LINK_TRACE = linkTrace (WilsonLoops.h:88-126,203-218).
"""
from __future__ import annotations

import numpy as np

FORMATS = {"IEEE32BIG": (">f4", 32), "IEEE32": ("<f4", 32), "IEEE64BIG": (">f8", 64), "IEEE64": ("<f8", 64),
           "IEEE64LITTLE": ("<f8", 64)}


def _links(U, dims):
    vol = int(np.prod(dims))
    return np.asarray(U, dtype=np.complex128).reshape(vol, 4, 3, 3)


def plaquette_and_trace(U, dims):
    """(avgPlaquette, linkTrace) with periodic boundaries."""
    Lx, Ly, Lz, Lt = dims
    u = _links(U, dims).reshape(Lt, Lz, Ly, Lx, 4, 3, 3)
    axis = {0: 3, 1: 2, 2: 1, 3: 0}  # mu -> array axis (t, z, y, x order)
    plaq = 0.0
    for mu in range(1, 4):
        for nu in range(mu):
            A = u[..., mu, :, :]
            B = np.roll(u[..., nu, :, :], -1, axis=axis[mu])   # U_nu(x + mu)
            C = u[..., nu, :, :]
            D = np.roll(u[..., mu, :, :], -1, axis=axis[nu])   # U_mu(x + nu)
            M1 = A @ B
            M2 = C @ D
            plaq += np.sum((M1 * np.conj(M2)).real)
    vol = Lx * Ly * Lz * Lt
    tr = np.sum(np.trace(u, axis1=-2, axis2=-1).real)
    return plaq / vol / 6.0 / 3.0, tr / vol / 4.0 / 3.0


def checksum(payload_host_order: np.ndarray) -> int:
    words = np.frombuffer(np.ascontiguousarray(payload_host_order).tobytes(), dtype="<u4")
    return int(np.sum(words, dtype=np.uint64) & 0xFFFFFFFF)


def write(path, U, dims, two_row=False, fmt="IEEE64BIG"):
    dt, bits = FORMATS[fmt]
    u = _links(U, dims)
    rows = u[:, :, :2, :] if two_row else u
    host = np.empty(rows.shape + (2,), dtype="<f4" if bits == 32 else "<f8")
    host[..., 0], host[..., 1] = rows.real, rows.imag
    csum = checksum(host)
    plaq, tr = plaquette_and_trace(u, dims)
    hdr = ["BEGIN_HEADER", "HDR_VERSION = 1.0",
           "DATATYPE = " + ("4D_SU3_GAUGE" if two_row else "4D_SU3_GAUGE_3x3"), "STORAGE_FORMAT = 1.0"]
    hdr += [f"DIMENSION_{d + 1} = {dims[d]}" for d in range(4)]
    hdr += [f"LINK_TRACE = {tr:.10g}", f"PLAQUETTE  = {plaq:.10g}"]
    hdr += [f"BOUNDARY_{d + 1} = PERIODIC" for d in range(4)]
    hdr += [f"CHECKSUM = {csum:10x}", "ENSEMBLE_ID = UKQCD", "ENSEMBLE_LABEL = DWF", "SEQUENCE_NUMBER = 1",
            f"FLOATING_POINT = {fmt}", "END_HEADER"]
    with open(path, "wb") as f:
        f.write(("\n".join(hdr) + "\n").encode())
        f.write(host.astype(dt).tobytes())
    return csum, plaq, tr


def read(path):
    """(U canonical complex128 [vol*4*9], header dict, checksum of the payload)."""
    with open(path, "rb") as f:
        data = f.read()
    end = data.index(b"END_HEADER")
    end = data.index(b"\n", end) + 1
    hdr = {}
    for line in data[:end].decode().splitlines():
        if "=" in line:
            k, v = line.split("=", 1)
            hdr[k.strip()] = v.strip()
    dims = [int(hdr[f"DIMENSION_{d + 1}"]) for d in range(4)]
    dt, bits = FORMATS[hdr["FLOATING_POINT"]]
    two_row = hdr["DATATYPE"] == "4D_SU3_GAUGE"
    rows = 2 if two_row else 3
    vol = int(np.prod(dims))
    raw = np.frombuffer(data[end:], dtype=dt, count=vol * 4 * rows * 3 * 2)
    host = raw.astype("<f4" if bits == 32 else "<f8")
    csum = checksum(host)
    v = host.astype(np.float64).reshape(vol, 4, rows, 3, 2)
    m = v[..., 0] + 1j * v[..., 1]
    if two_row:
        r0, r1 = m[:, :, 0, :], m[:, :, 1, :]
        r2 = np.conj(np.cross(r0, r1))
        m = np.concatenate([m, r2[:, :, None, :]], axis=2)
    return m.reshape(-1), hdr, csum
