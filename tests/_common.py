"""Shared helpers of the test suite: seeded inputs and an independent numpy restatement
of the free-field (U = 1) operators in momentum space (the known answer of Grid's
tests/core/Test_fft.cc, formula WilsonFermionImplementation.h:177-230)."""
from __future__ import annotations

import numpy as np

import grid_gb300 as g

# Grid's gamma basis (Grid/qcd/spin/TwoSpinor.h:67-140), written out independently of
# the oracle's table
I = 1j
GAMMA = np.array([
    [[0, 0, 0, I], [0, 0, I, 0], [0, -I, 0, 0], [-I, 0, 0, 0]],
    [[0, 0, 0, -1], [0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]],
    [[0, 0, I, 0], [0, 0, 0, -I], [-I, 0, 0, 0], [0, I, 0, 0]],
    [[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]],
], dtype=np.complex128)
GAMMA5 = np.diag([1, 1, -1, -1]).astype(np.complex128)
PPLUS = 0.5 * (np.eye(4) + GAMMA5)
PMINUS = 0.5 * (np.eye(4) - GAMMA5)

# configs of the workloads (sizes reduced where the oracle must finish in seconds)
MOBIUS = dict(M5=1.8, b=1.5, c=0.5)


def fermion(n_sites, L5, seed):
    return g.random_gaussian(n_sites * L5 * 12, seed)


def momenta(dims, antiperiodic_t=True):
    ks = []
    for mu, L in enumerate(dims):
        k = 2 * np.pi * np.arange(L) / L
        if mu == 3 and antiperiodic_t:
            k = k + np.pi / L
        ks.append(k)
    return ks


def _kgrid(dims, antiperiodic_t):
    kx, ky, kz, kt = momenta(dims, antiperiodic_t)
    KT, KZ, KY, KX = np.meshgrid(kt, kz, ky, kx, indexing="ij")
    return [KX, KY, KZ, KT]


def wilson_dirac_k(dims, antiperiodic_t=True):
    """D_W(k) = sum_mu (1 - cos k_mu) + i gamma_mu sin k_mu (no mass), shape (Lt,Lz,Ly,Lx,4,4):
    the plane-wave eigen-operator of Dhop + 4 for psi ~ exp(+i k x)."""
    K = _kgrid(dims, antiperiodic_t)
    D = np.zeros(K[0].shape + (4, 4), dtype=np.complex128)
    for mu in range(4):
        D += (1 - np.cos(K[mu]))[..., None, None] * np.eye(4)
        D += 1j * np.sin(K[mu])[..., None, None] * GAMMA[mu]
    return D


def _to_k(dims, field, nspin_block, antiperiodic_t):
    Lx, Ly, Lz, Lt = dims
    f = field.reshape(Lt, Lz, Ly, Lx, nspin_block, 3)
    if antiperiodic_t:
        t = np.arange(Lt)
        f = f * np.exp(-1j * np.pi * t / Lt)[:, None, None, None, None, None]
    return np.fft.fftn(f, axes=(0, 1, 2, 3))


def _from_k(dims, fk, antiperiodic_t):
    Lx, Ly, Lz, Lt = dims
    f = np.fft.ifftn(fk, axes=(0, 1, 2, 3))
    if antiperiodic_t:
        t = np.arange(Lt)
        f = f * np.exp(1j * np.pi * t / Lt)[:, None, None, None, None, None]
    return f.reshape(-1)


def wilson_free_solve(dims, mass, eta, antiperiodic_t=True):
    """psi = M^{-1} eta for the free Wilson operator M = Dhop + 4 + m."""
    D = wilson_dirac_k(dims, antiperiodic_t) + mass * np.eye(4)
    ek = _to_k(dims, eta, 4, antiperiodic_t)  # (Lt,Lz,Ly,Lx,4,3)
    return _from_k(dims, np.linalg.solve(D, ek), antiperiodic_t)


def mobius_free_matrix(dims, Ls, mf, M5, b, c, antiperiodic_t=True):
    """The Moebius operator at U = 1 as a (4 Ls) x (4 Ls) matrix per momentum, assembled
    from Grid's definition  M = D_W (b + c (P- S+ + P+ S-)) + 1 - (P- S+ + P+ S-)  with the
    mass on the s wrap (CayleyFermion5DImplementation.h:155-306), D_W(k) = D(k) - M5."""
    DW = wilson_dirac_k(dims, antiperiodic_t) - M5 * np.eye(4)
    shape = DW.shape[:-2]
    Sp = np.zeros((Ls, Ls))  # (S+ psi)_s = psi_{s+1} with -mf on the wrap for the c term
    Sm = np.zeros((Ls, Ls))
    for s in range(Ls):
        Sp[s, (s + 1) % Ls] = 1.0 if s < Ls - 1 else -mf
        Sm[s, (s - 1) % Ls] = 1.0 if s > 0 else -mf
    D5 = b * np.kron(np.eye(Ls), np.eye(4)) + c * (np.kron(Sp, PMINUS) + np.kron(Sm, PPLUS))
    # the "1 - P- S+ - P+ S-" part has +mf on the wrap (upper[Ls-1] = lower[0] = mf)
    Tp = np.zeros((Ls, Ls))
    Tm = np.zeros((Ls, Ls))
    for s in range(Ls):
        Tp[s, (s + 1) % Ls] = -1.0 if s < Ls - 1 else mf
        Tm[s, (s - 1) % Ls] = -1.0 if s > 0 else mf
    E = np.eye(4 * Ls) + np.kron(Tp, PMINUS) + np.kron(Tm, PPLUS)
    M = np.einsum("...ij,st->...sitj", DW, np.eye(Ls)).reshape(shape + (4 * Ls, 4 * Ls)) @ D5 + E
    return M


def mobius_free_apply(dims, Ls, mf, M5, b, c, psi, antiperiodic_t=True):
    """M psi for the free Moebius operator through momentum space (canonical 5D layout)."""
    M = mobius_free_matrix(dims, Ls, mf, M5, b, c, antiperiodic_t)
    Lx, Ly, Lz, Lt = dims
    f = psi.reshape(Lt, Lz, Ly, Lx, Ls * 4, 3)
    if antiperiodic_t:
        f = f * np.exp(-1j * np.pi * np.arange(Lt) / Lt)[:, None, None, None, None, None]
    fk = np.fft.fftn(f, axes=(0, 1, 2, 3))
    ok = np.einsum("...ij,...jc->...ic", M, fk)
    o = np.fft.ifftn(ok, axes=(0, 1, 2, 3))
    if antiperiodic_t:
        o = o * np.exp(1j * np.pi * np.arange(Lt) / Lt)[:, None, None, None, None, None]
    return o.reshape(-1)


def mobius_free_solve(dims, Ls, mf, M5, b, c, eta, antiperiodic_t=True):
    M = mobius_free_matrix(dims, Ls, mf, M5, b, c, antiperiodic_t)
    Lx, Ly, Lz, Lt = dims
    f = eta.reshape(Lt, Lz, Ly, Lx, Ls * 4, 3)
    if antiperiodic_t:
        f = f * np.exp(-1j * np.pi * np.arange(Lt) / Lt)[:, None, None, None, None, None]
    fk = np.fft.fftn(f, axes=(0, 1, 2, 3))
    ok = np.linalg.solve(M, fk)
    o = np.fft.ifftn(ok, axes=(0, 1, 2, 3))
    if antiperiodic_t:
        o = o * np.exp(1j * np.pi * np.arange(Lt) / Lt)[:, None, None, None, None, None]
    return o.reshape(-1)


def dminus_free(dims, Ls, c, M5, psi, dag=False, antiperiodic_t=True):
    """Dminus psi = (1 - c D_W) psi on every s at U = 1 (CayleyFermion5DImplementation.h:131-153),
    with D_W(k) = D(k) - M5 in momentum space; dag uses D_W(k)^dagger."""
    DW = wilson_dirac_k(dims, antiperiodic_t) - M5 * np.eye(4)
    if dag:
        DW = np.conj(np.swapaxes(DW, -1, -2))
    A = np.eye(4) - c * DW
    Lx, Ly, Lz, Lt = dims
    f = psi.reshape(Lt, Lz, Ly, Lx, Ls, 4, 3)
    ph = np.exp(-1j * np.pi * np.arange(Lt) / Lt) if antiperiodic_t else np.ones(Lt)
    fk = np.fft.fftn(f * ph[:, None, None, None, None, None, None], axes=(0, 1, 2, 3))
    ok = np.einsum("tzyxij,tzyxsjc->tzyxsic", A, fk)
    o = np.fft.ifftn(ok, axes=(0, 1, 2, 3)) * np.conj(ph)[:, None, None, None, None, None, None]
    return o.reshape(-1)
