"""The Fourier-accelerated Pauli-Villars solve (FourierAcceleratedPV.h) and its pieces on
the GPU: the 5D twisted-mass Wilson operator (WilsonTMFermion5D.h) against the oracle's
Wilson hop plus the chiral diagonal, the fifth-dimension DFT / slot copy / chiral scale
against numpy, the PV inverse against the oracle's mass-1 Moebius operator and against the
red-black PV solver, and MADWF with it."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 4)
VOL = 256


def rhs_major(x, n):
    """[site][s][12] (the oracle's 5D Wilson layout) -> [s][site][12] (a twisted-mass
    field's slices as right-hand sides back to back)."""
    return np.ascontiguousarray(x.reshape(-1, n, 12).transpose(1, 0, 2)).reshape(-1)


def site_major(x, n):
    return np.ascontiguousarray(x.reshape(n, -1, 12).transpose(1, 0, 2)).reshape(-1)


def tm_diag(x, mass, mu, n, dag=False, inverse=False):
    """(4 + m_s) + i mu_s gamma5 (conjugated for dag, inverted for inverse) per slot."""
    xr = x.reshape(-1, n, 12).copy()
    for s in range(n):
        m, u = 4.0 + mass[s], mu[s]
        d_up = complex(m, u)
        if inverse:
            d_up = 1.0 / d_up
        if dag:
            d_up = d_up.conjugate()
        d_dn = d_up.conjugate()
        xr[:, s, :6] *= d_up
        xr[:, s, 6:] *= d_dn
    return xr.reshape(-1)


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_twisted_mass_operator(gpu_available, prec):
    U = g.random_gauge(DIMS, 0.3, 131)
    n = 4
    mass, mu = np.array([0.1, 0.1, -0.3, -0.3]), np.array([0.2, -0.2, 0.05, -0.05])
    tm = g.WilsonTMFermion5D(U, DIMS, mass, mu, precision=prec)
    ref = o.OracleOp(0, 0, DIMS, n, [0.0], U, g.antiperiodic_t())
    tol = 1e-13 if prec == g.F64 else 1e-6
    x = fermion(VOL, n, 132)
    fin, fout = tm.FermionField().import_(rhs_major(x, n)), tm.FermionField()
    tm.M(fin, fout)
    assert o.rel_l2(site_major(fout.export(), n), ref.apply(o.OP_DHOP, x) + tm_diag(x, mass, mu, n)) < tol
    tm.Mdag(fin, fout)
    assert o.rel_l2(site_major(fout.export(), n), ref.apply(o.OP_DHOP_DAG, x) + tm_diag(x, mass, mu, n, dag=True)) < tol
    xh = fermion(VOL // 2, n, 133)
    hin, hout = tm.FermionRedBlackField(g.ODD).import_(rhs_major(xh, n)), tm.FermionRedBlackField(g.ODD)
    for name, dag, inv in (("Mooee", 0, 0), ("MooeeDag", 1, 0), ("MooeeInv", 0, 1), ("MooeeInvDag", 1, 1)):
        getattr(tm, name)(hin, hout)
        want = tm_diag(xh, mass, mu, n, dag=bool(dag), inverse=bool(inv))
        assert o.rel_l2(site_major(hout.export(), n), want) < tol, name
    # update() changes the diagonal
    tm.update(mass + 0.5, -mu)
    tm.Mooee(hin, hout)
    assert o.rel_l2(site_major(hout.export(), n), tm_diag(xh, mass + 0.5, -mu, n)) < tol


def test_fifth_dimension_transforms(gpu_available):
    U = g.random_gauge(DIMS, 0.3, 134)
    Ls = 6
    op = g.MobiusFermion(U, DIMS, Ls, 0.1, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"])
    x = fermion(VOL, Ls, 135)
    fx, fy = op.FermionField().import_(x), op.FermionField()
    rng = np.random.default_rng(1)
    mat = rng.normal(size=(Ls, Ls)) + 1j * rng.normal(size=(Ls, Ls))
    g.dft_s(fx, fy, mat)
    want = np.einsum("ks,nsc->nkc", mat, x.reshape(VOL, Ls, 12)).reshape(-1)
    assert o.rel_l2(fy.export(), want) < 1e-14
    tm = g.WilsonTMFermion5D(U, DIMS, np.zeros(4), np.zeros(4))
    ft = tm.FermionField().zero()
    g.copy_slice5(ft, 3, fx, 1)
    got = ft.export().reshape(4, VOL, 12)  # slices as right-hand sides
    assert np.array_equal(got[3], x.reshape(VOL, Ls, 12)[:, 1]) and not got[:3].any()
    up = rng.normal(size=Ls) + 1j * rng.normal(size=Ls)
    dn = rng.normal(size=Ls) + 1j * rng.normal(size=Ls)
    g.chiral_scale(fx, fy, up, dn)
    want = x.reshape(VOL, Ls, 12).copy()
    want[:, :, :6] *= up[None, :, None]
    want[:, :, 6:] *= dn[None, :, None]
    assert o.rel_l2(fy.export(), want.reshape(-1)) < 1e-15


@pytest.mark.parametrize("Ls,b,c", [(8, 1.5, 0.5), (12, 1.0, 0.0)])
def test_fourier_accelerated_pv_inverse(gpu_available, Ls, b, c):
    U = g.random_gauge(DIMS, 0.3, 136)
    op = g.MobiusFermion(U, DIMS, Ls, 0.05, MOBIUS["M5"], b, c)
    ref = o.OracleOp(1, 0, DIMS, Ls, [1.0, MOBIUS["M5"], b, c], U, g.antiperiodic_t())  # the mass-1 operator
    src = fermion(VOL, Ls, 137)
    fs, fx = op.FermionField().import_(src), op.FermionField()
    g.PauliVillarsSolverFourierAccel(U, g.ConjugateGradient(1e-12, 10000))(op, fs, fx)
    x = fx.export()
    assert o.rel_l2(ref.apply(o.OP_M, x), src) < 1e-9
    fy = op.FermionField().zero()
    g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000)))(op, fs, fy)
    assert o.rel_l2(x, fy.export()) < 1e-9
    assert op.Mass() == 0.05


def test_madwf_with_fourier_accelerated_pv(gpu_available):
    Lo, Li = 8, 4
    U = g.random_gauge(DIMS, 0.3, 5)
    outer = g.MobiusFermion(U, DIMS, Lo, 0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"])
    inner = g.MobiusFermion(U, DIMS, Li, 0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"])
    ref = o.OracleOp(1, 0, DIMS, Lo, [0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    eta = fermion(VOL, 1, 4)
    madwf = g.MADWF(outer, inner, g.PauliVillarsSolverFourierAccel(U, g.ConjugateGradient(1e-12, 10000)),
                    g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000, False)), g.ZeroGuesser(), 1e-9, 20)
    sol = outer.FermionField()
    madwf(eta, sol)
    b = ref.physical(o.IMPORT_PHYSICAL_SOURCE, eta)
    direct, _, _, _ = ref.schur_solve(b, 1e-11, 10000)
    assert madwf.residuals[-1] < 1e-9
    assert o.rel_l2(sol.export(), direct) < 1e-8
