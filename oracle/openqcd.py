"""openQCD gauge files restated in numpy (TEST INFRASTRUCTURE ONLY: writes the fixtures
the library's reader is checked against; only tests/ use it).

Follows Grid/parallelIO/OpenQcdIO.h:43-170: a header of int32 Nt, Nx, Ny, Nz and the
double plaquette (Nc times Grid's normalisation), then for every odd site in openQCD's
order (t, x, y, z; index (t Lx Ly Lz + x Ly Lz + y Lz + z) / 2) the links T+, T-, X+,
X-, Y+, Y-, Z+, Z- as little-endian complex doubles: U_mu(x) and U_mu(x - mu).
"""
from __future__ import annotations

import struct

import numpy as np

from oracle import nersc


def write(path, U, dims, plaquette=None):
    """dims in Grid order (Lx, Ly, Lz, Lt); U canonical [site][mu][3][3] (x fastest)."""
    Lx, Ly, Lz, Lt = dims
    u = np.asarray(U, dtype=np.complex128).reshape(Lt, Lz, Ly, Lx, 4, 3, 3)
    if plaquette is None:
        plaquette = nersc.plaquette_and_trace(U, dims)[0]
    vol = Lx * Ly * Lz * Lt
    rec = np.zeros((vol // 2, 8, 3, 3), dtype="<c16")
    grid_axis = {0: 3, 1: 2, 2: 1, 3: 0}  # Grid mu -> array axis of u
    for t in range(Lt):
        for x in range(Lx):
            for y in range(Ly):
                for z in range(Lz):
                    if (x + y + z + t) % 2 == 0:
                        continue
                    io = (t * Lx * Ly * Lz + x * Ly * Lz + y * Lz + z) // 2
                    for mu_o, mu_g in ((0, 3), (1, 0), (2, 1), (3, 2)):
                        c = [t, z, y, x]  # array index order
                        rec[io, 2 * mu_o] = u[c[0], c[1], c[2], c[3], mu_g]
                        ax = grid_axis[mu_g]
                        c[ax] = (c[ax] - 1) % u.shape[ax]
                        rec[io, 2 * mu_o + 1] = u[c[0], c[1], c[2], c[3], mu_g]
    with open(path, "wb") as f:
        f.write(struct.pack("<4id", Lt, Lx, Ly, Lz, 3.0 * plaquette))
        f.write(rec.tobytes())
    return plaquette
