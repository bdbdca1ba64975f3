"""Pins the CPU oracle to the known answers that Grid's own tests hold for this path
(no golden data files ship with Grid, and Grid cannot be built here):

  * Dhop == naive Cshift formula        benchmarks/Benchmark_dwf.cc:145-158,222-232 (dag :235-261)
  * DhopEO (+) DhopOE == Dhop           benchmarks/Benchmark_dwf.cc:329-356
  * even-odd identities                 tests/core/Test_mobius_even_odd.cc, Test_wilson_even_odd.cc
  * free-field propagator               tests/core/Test_fft.cc:159,313 (WilsonFermionImplementation.h:177-230)
  * CG true residual / mixed vs FP64    tests/solver/Test_wilson_cg_unprec.cc, tests/Test_dwf_mixedcg_prec.cc:215
Tolerances: identities at FP64 rounding (1e-12 relative), FP32 restatement 1e-6.
"""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import (GAMMA, GAMMA5, MOBIUS, dminus_free, fermion, mobius_free_apply, mobius_free_solve,
                           wilson_free_solve)

DIMS = (4, 4, 4, 4)
VOL = 256


def _mobius(prec=0, Ls=6, mf=0.1, dims=DIMS, U=None, eps=0.5, seed=11):
    U = g.random_gauge(dims, eps, seed) if U is None else U
    return o.OracleOp(1, prec, dims, Ls, [mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t()), U


# the Ls = 10 omegas of Grid's tests/core/Test_zmobius_even_odd.cc:97-106 (b = 1, c = 0)
ZOMEGA = [1.45806438985048, 1.18231318389348, 0.830951166685955, 0.542352409156791, 0.341985020453729,
          0.21137902619029, 0.126074299502912, 0.0990136651962626, 0.0686324988446592 + 0.0550658530827402j,
          0.0686324988446592 - 0.0550658530827402j]


def zparams(mf, M5, b, c, gamma):
    return [mf, M5, b, c] + [v for z in gamma for v in (complex(z).real, complex(z).imag)]


def _zmobius(prec=0, mf=0.1, dims=DIMS, U=None, eps=0.5, seed=13, gamma=ZOMEGA, b=1.0, c=0.0):
    U = g.random_gauge(dims, eps, seed) if U is None else U
    return o.OracleOp(2, prec, dims, len(gamma), zparams(mf, MOBIUS["M5"], b, c, gamma), U, g.antiperiodic_t()), U


def _wilson(prec=0, L5=1, mass=0.1, dims=DIMS, U=None, eps=0.3, seed=7):
    U = g.random_gauge(dims, eps, seed) if U is None else U
    return o.OracleOp(0, prec, dims, L5, [mass], U, g.antiperiodic_t()), U


def test_gamma_basis_algebra():
    for mu in range(4):
        for nu in range(4):
            ac = GAMMA[mu] @ GAMMA[nu] + GAMMA[nu] @ GAMMA[mu]
            assert np.allclose(ac, 2 * np.eye(4) * (mu == nu))
    assert np.allclose(GAMMA[0] @ GAMMA[1] @ GAMMA[2] @ GAMMA[3], GAMMA5)


def test_gauge_generator_is_su3_and_seeded():
    U = g.random_gauge(DIMS, 0.5, 3).reshape(-1, 3, 3)
    assert np.abs(np.einsum("nij,nkj->nik", U, U.conj()) - np.eye(3)).max() < 1e-14
    assert np.abs(np.linalg.det(U) - 1).max() < 1e-14
    assert np.array_equal(U, g.random_gauge(DIMS, 0.5, 3).reshape(-1, 3, 3))
    assert not np.array_equal(U, g.random_gauge(DIMS, 0.5, 4).reshape(-1, 3, 3))
    # exp(i eps H): distance from 1 grows with eps
    d1 = np.abs(g.random_gauge(DIMS, 0.1, 3).reshape(-1, 3, 3) - np.eye(3)).mean()
    d5 = np.abs(U - np.eye(3)).mean()
    assert d1 < d5
    z = g.random_gaussian(200000, 5)
    assert abs(z.real.std() - 1) < 0.01 and abs(z.imag.mean()) < 0.01


@pytest.mark.parametrize("L5", [1, 3])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("phases", ["antiperiodic", "periodic"])
def test_dhop_equals_naive_cshift(L5, dag, phases):
    ph = g.antiperiodic_t() if phases == "antiperiodic" else g.periodic()
    U = g.random_gauge(DIMS, 0.5, 21)
    op = o.OracleOp(0, 0, DIMS, L5, [0.1], U, ph)
    x = fermion(VOL, L5, 22)
    a = op.apply(o.OP_DHOP_DAG if dag else o.OP_DHOP, x)
    b = o.dhop_naive(DIMS, L5, U, ph, x, dag)
    assert o.rel_l2(a, b) < 1e-14


def test_dhop_eo_oe_equals_dhop():
    op, U = _mobius()
    x = fermion(VOL, 6, 31)
    full = op.apply(o.OP_DHOP, x)
    xe, xo = o.pick(DIMS, 6, x, 0), o.pick(DIMS, 6, x, 1)
    re = op.dhop_cb(xo, 1)  # DhopEO: odd in -> even out
    ro = op.dhop_cb(xe, 0)  # DhopOE
    both = o.setcb(DIMS, 6, ro, 1, o.setcb(DIMS, 6, re, 0))
    assert o.rel_l2(both, full) < 1e-14


@pytest.mark.parametrize("kind", ["mobius", "wilson", "zmobius"])
def test_even_odd_decomposition_identities(kind):
    op, U = {"mobius": _mobius, "wilson": _wilson, "zmobius": _zmobius}[kind]()
    L5 = op.L5
    chi = fermion(VOL, L5, 41)
    phi = fermion(VOL, L5, 42)
    ce, co = o.pick(DIMS, L5, chi, 0), o.pick(DIMS, L5, chi, 1)
    pe, po = o.pick(DIMS, L5, phi, 0), o.pick(DIMS, L5, phi, 1)
    # Meo + Moe + Mee + Moo == M
    for dag in (0, 1):
        oo = op.apply(o.OP_MOOEE_DAG if dag else o.OP_MOOEE, co)
        ee = op.apply(o.OP_MOOEE_DAG if dag else o.OP_MOOEE, ce)
        eo = op.apply(o.OP_MEOOE_DAG if dag else o.OP_MEOOE, co, 1)
        oe = op.apply(o.OP_MEOOE_DAG if dag else o.OP_MEOOE, ce, 0)
        full = o.setcb(DIMS, L5, oo + oe, 1, o.setcb(DIMS, L5, ee + eo, 0))
        ref = op.apply(o.OP_MDAG if dag else o.OP_M, chi)
        assert o.rel_l2(full, ref) < 1e-13
    ip = lambda a, b: np.vdot(a, b)  # noqa: E731
    # <phi|Mooee chi>^* == <chi|MooeeDag phi>
    a = ip(pe, op.apply(o.OP_MOOEE, ce)).conj()
    b = ip(ce, op.apply(o.OP_MOOEE_DAG, pe))
    assert abs(a - b) < 1e-12 * abs(a)
    # <phi|Meooe chi>^* == <chi|MeooeDag phi>   (chi odd -> even)
    a = ip(pe, op.apply(o.OP_MEOOE, co, 1)).conj()
    b = ip(co, op.apply(o.OP_MEOOE_DAG, pe, 0))
    assert abs(a - b) < 1e-12 * abs(a)
    # MooeeInv Mooee == 1 ; MooeeInvDag MooeeDag == 1
    assert o.rel_l2(op.apply(o.OP_MOOEE_INV, op.apply(o.OP_MOOEE, ce)), ce) < 1e-13
    assert o.rel_l2(op.apply(o.OP_MOOEE_INV_DAG, op.apply(o.OP_MOOEE_DAG, ce)), ce) < 1e-13
    # M adjointness and MpcDagMpc Hermitian, Mpc / MpcDag adjoint
    a = ip(phi, op.apply(o.OP_M, chi)).conj()
    b = ip(chi, op.apply(o.OP_MDAG, phi))
    assert abs(a - b) < 1e-12 * abs(a)
    a = ip(po, op.apply(o.OP_MPC, co)).conj()
    b = ip(co, op.apply(o.OP_MPC_DAG, po))
    assert abs(a - b) < 1e-12 * abs(a)
    a = ip(po, op.apply(o.OP_MPCDAGMPC, co)).conj()
    b = ip(co, op.apply(o.OP_MPCDAGMPC, po))
    assert abs(a - b) < 1e-12 * abs(a)
    assert abs(ip(co, op.apply(o.OP_MPCDAGMPC, co)).imag) < 1e-12 * abs(ip(co, co))


def test_cayley_coefficients_config2():
    c = o.cayley_coeffs(16, 0.01, 1.8, 1.5, 0.5)
    assert np.allclose(c["bs"], 1.5) and np.allclose(c["cs"], 0.5)
    assert np.allclose(c["bee"], 4.3) and np.allclose(c["cee"], -0.1)
    # LDU of Mooee: d_{Ls-1} carries the mass correction, the rest equals bee
    assert np.allclose(c["dee"][:-1], 4.3)
    assert c["lee"][-1] == 0 and c["uee"][-1] == 0


def test_free_field_wilson_propagator_momentum_space():
    """Wilson M^{-1} at U = 1 from the oracle's CG equals the momentum-space formula
    [-i gamma sin k + W(k)] / [sin^2 k + W(k)^2] (antiperiodic time)."""
    dims = (4, 4, 4, 6)
    vol = 384
    mass = 0.3
    U = g.unit_gauge(dims)
    op = o.OracleOp(0, 0, dims, 1, [mass], U, g.antiperiodic_t())
    eta = fermion(vol, 1, 51)
    ref = wilson_free_solve(dims, mass, eta)
    # CG on MdagM psi = Mdag eta
    b = op.apply(o.OP_MDAG, eta)
    psi, iters, res = op.cg(0, b, 1e-12, 2000)
    assert res < 1e-11
    assert o.rel_l2(psi, ref) < 1e-10
    # and M applied in momentum space equals the oracle's M
    assert o.rel_l2(op.apply(o.OP_M, ref), eta) < 1e-12


def test_free_field_mobius_momentum_space():
    dims = (4, 4, 4, 4)
    Ls, mf = 6, 0.1
    U = g.unit_gauge(dims)
    op = o.OracleOp(1, 0, dims, Ls, [mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    x = fermion(VOL, Ls, 61)
    ref = mobius_free_apply(dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], x)
    assert o.rel_l2(op.apply(o.OP_M, x), ref) < 1e-12
    eta = fermion(VOL, Ls, 62)
    sol = mobius_free_solve(dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], eta)
    s2, iters, r0, r1 = op.schur_solve(eta, 1e-12, 3000)
    assert r1 < 1e-10
    assert o.rel_l2(s2, sol) < 1e-9


def test_oracle_cg_wilson_unprec_true_residual():
    op, U = _wilson()
    src = fermion(VOL, 1, 71)
    psi, iters, res = op.cg(0, src, 1e-8, 1000)
    assert 0 < iters < 1000
    assert res < 1e-8 * 10
    r = op.apply(o.OP_MDAGM, psi) - src
    assert np.linalg.norm(r) / np.linalg.norm(src) < 1e-7


def test_oracle_schur_solve_mobius():
    op, U = _mobius(mf=0.05)
    src = fermion(VOL, 6, 81)
    sol, iters, r_cg, r_unprec = op.schur_solve(src, 1e-10, 3000)
    assert r_unprec < 1e-9
    assert o.rel_l2(op.apply(o.OP_M, sol), src) < 1e-9


def test_oracle_reliable_update_matches_fp64():
    """tests/Test_dwf_mixedcg_prec.cc:215: mixed and FP64 solutions agree."""
    U = g.random_gauge(DIMS, 0.5, 91)
    od, _ = _mobius(0, U=U, mf=0.05)
    of, _ = _mobius(1, U=U, mf=0.05)
    src = o.pick(DIMS, 6, fermion(VOL, 6, 92), 1)
    x64, it64, r64 = od.cg(1, src, 1e-10, 3000)
    xm, info, rm = o.cg_reliable(od, of, 1, src, 1e-10, 3000, delta=1e-3)
    assert rm < 1e-10 * 2 and r64 < 1e-10 * 2
    assert o.rel_l2(xm, x64) < 1e-8


def test_oracle_fp32_matches_fp64_dhop():
    U = g.random_gauge(DIMS, 0.5, 101)
    od, _ = _mobius(0, U=U)
    of, _ = _mobius(1, U=U)
    x = fermion(VOL, 6, 102)
    xo = o.pick(DIMS, 6, x, 1)
    assert o.rel_l2(of.dhop_cb(xo, 1), od.dhop_cb(xo, 1)) < 1e-6
    assert o.rel_l2(of.apply(o.OP_MPCDAGMPC, xo), od.apply(o.OP_MPCDAGMPC, xo)) < 1e-6


@pytest.mark.parametrize("dag", [0, 1])
def test_physical_surface_fields_free_field(dag):
    """ImportUnphysicalFermion puts P+ eta at s = 0 and P- eta at s = Ls-1; the source export
    undoes it and the solution export annihilates it; Dminus = 1 - c D_W agrees with the
    momentum-space restatement at U = 1; ImportPhysicalFermionSource = Dminus of the
    unphysical import (CayleyFermion5DImplementation.h:57-153)."""
    Ls, mf = 6, 0.1
    ref, _ = _mobius(Ls=Ls, mf=mf, U=g.unit_gauge(DIMS))
    eta = fermion(VOL, 1, 5)
    e5 = ref.physical(o.IMPORT_UNPHYSICAL, eta)
    X = np.zeros((VOL, Ls, 4, 3), dtype=np.complex128)
    E = eta.reshape(VOL, 4, 3)
    X[:, 0, :2], X[:, Ls - 1, 2:] = E[:, :2], E[:, 2:]
    assert np.array_equal(e5, X.reshape(-1))
    assert np.array_equal(ref.physical(o.EXPORT_PHYSICAL_SOURCE, e5), eta)
    assert not np.any(ref.physical(o.EXPORT_PHYSICAL_SOLUTION, e5))
    psi = fermion(VOL, Ls, 6)
    want = dminus_free(DIMS, Ls, MOBIUS["c"], MOBIUS["M5"], psi, dag=bool(dag))
    assert o.rel_l2(ref.apply(o.OP_DMINUS_DAG if dag else o.OP_DMINUS, psi), want) < 1e-12
    if not dag:
        want = dminus_free(DIMS, Ls, MOBIUS["c"], MOBIUS["M5"], e5)
        assert o.rel_l2(ref.physical(o.IMPORT_PHYSICAL_SOURCE, eta), want) < 1e-12


def test_oracle_multishift_free_wilson():
    """The multishift CG restatement (ConjugateGradientMultiShift.h:76-330) solves
    (MdagM + sigma) psi = eta for every shift: checked at U = 1 against the momentum-space
    solve of the free Wilson operator, M(k)^dagger M(k) + sigma."""
    from tests._common import _from_k, _to_k, wilson_dirac_k
    mass, shifts = 0.1, [0.0, 0.05, 0.3, 1.2]
    ref, _ = _wilson(mass=mass, U=g.unit_gauge(DIMS))
    eta = fermion(VOL, 1, 21)
    psi, it, conv, its, res = ref.cg_multishift(0, eta, shifts, [1e-11] * 4, 3000)
    assert conv == 1 and its[0] == it and all(i <= it for i in its)
    Mk = wilson_dirac_k(DIMS) + mass * np.eye(4)
    MdM = np.conj(np.swapaxes(Mk, -1, -2)) @ Mk
    ek = _to_k(DIMS, eta, 4, True)
    for s, x, r in zip(shifts, psi, res):
        want = _from_k(DIMS, np.linalg.solve(MdM + s * np.eye(4), ek), True)
        assert r < 1e-10
        assert o.rel_l2(x, want) < 1e-9, s


@pytest.mark.parametrize("fmt", ["IEEE64BIG", "IEEE64", "IEEE32BIG", "IEEE32"])
@pytest.mark.parametrize("two_row", [False, True])
def test_oracle_nersc_round_trip(tmp_path, fmt, two_row):
    """The NERSC restatement (NerscIO.h): write -> read reproduces the field (exactly for
    64-bit 3x3, within float rounding otherwise; the rebuilt third row of an SU(3) link
    equals the stored one), the header checksum is the payload's, and the unit field has
    plaquette and link trace 1."""
    from oracle import nersc
    dims = (4, 4, 4, 6)
    U = g.random_gauge(dims, 0.7, 3)
    path = tmp_path / "cfg.nersc"
    csum, plaq, tr = nersc.write(path, U, dims, two_row, fmt)
    V, hdr, csum2 = nersc.read(path)
    assert csum2 == csum == int(hdr["CHECKSUM"], 16)
    tol = 0 if (fmt.startswith("IEEE64") and not two_row) else (1e-13 if fmt.startswith("IEEE64") else 1e-6)
    assert np.max(np.abs(V - U)) <= tol
    p2, t2 = nersc.plaquette_and_trace(V, dims)
    assert abs(p2 - plaq) < 1e-6 and abs(t2 - tr) < 1e-6
    one = g.unit_gauge(dims)
    assert np.allclose(nersc.plaquette_and_trace(one, dims), (1.0, 1.0), atol=1e-15)


@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("kind", ["wilson", "mobius"])
def test_oracle_force_is_the_link_derivative(dag, kind):
    """DhopDeriv (WilsonFermion5DImplementation.h:212-246 + InsertForce5D) is the derivative
    of <A|Dhop|B> by the link: with A = 0 at x0 + mu (so only the forward leg at x0 sees
    the link), <A|Dhop(U + D)|B> - <A|Dhop(U)|B> = tr(D U^+ F[x0][mu]) for any 3x3 D, with
    boundary phases +-1; exactly, since Dhop is linear in the link."""
    Ls = 1 if kind == "wilson" else 4
    rng = np.random.default_rng(5 + dag)
    U = g.random_gauge(DIMS, 0.6, 21)
    ph = g.antiperiodic_t()
    mk = (lambda V: o.OracleOp(0, 0, DIMS, 1, [0.1], V, ph)) if kind == "wilson" else \
        (lambda V: o.OracleOp(1, 0, DIMS, Ls, [0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], V, ph))
    ref = mk(U)
    A = fermion(VOL, Ls, 31).reshape(VOL, Ls * 12)
    B = fermion(VOL, Ls, 32)
    for x0, mu in ((5, 0), (VOL - 1, 3), (77, 2)):   # x0 = VOL-1 sits on the time boundary
        x = np.unravel_index(x0, DIMS[::-1])[::-1]
        xp = list(x)
        xp[mu] = (xp[mu] + 1) % DIMS[mu]
        nb = xp[0] + DIMS[0] * (xp[1] + DIMS[1] * (xp[2] + DIMS[2] * xp[3]))
        Az = A.copy()
        Az[nb] = 0
        Az = Az.reshape(-1)
        F = ref.deriv(Az, B, dag).reshape(VOL, 4, 3, 3)
        D = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        U2 = U.reshape(VOL, 4, 3, 3).copy()
        U2[x0, mu] += D
        code = o.OP_DHOP_DAG if dag else o.OP_DHOP
        d_num = np.vdot(Az, mk(U2.reshape(-1)).apply(code, B)) - np.vdot(Az, ref.apply(code, B))
        Ux = U.reshape(VOL, 4, 3, 3)[x0, mu]
        d_ana = np.trace(D @ Ux.conj().T @ F[x0, mu])
        assert abs(d_num - d_ana) < 1e-10 * abs(d_ana), (x0, mu)


def test_zmobius_with_real_unit_omega_is_moebius():
    """ZMobius with omega_s = 1 has the Moebius coefficients: every operator agrees."""
    U = g.random_gauge(DIMS, 0.5, 3)
    Ls, mf = 6, 0.05
    mob, _ = _mobius(Ls=Ls, mf=mf, U=U)
    zmob, _ = _zmobius(mf=mf, U=U, gamma=[1.0] * Ls, b=MOBIUS["b"], c=MOBIUS["c"])
    x = fermion(VOL, Ls, 5)
    xo = o.pick(DIMS, Ls, x, 1)
    for code in (o.OP_M, o.OP_MDAG, o.OP_MDAGM, o.OP_DMINUS, o.OP_DMINUS_DAG):
        assert o.rel_l2(zmob.apply(code, x), mob.apply(code, x)) < 1e-14, code
    for code in (o.OP_MOOEE, o.OP_MOOEE_DAG, o.OP_MOOEE_INV, o.OP_MOOEE_INV_DAG, o.OP_MPC, o.OP_MPC_DAG,
                 o.OP_MPCDAGMPC, o.OP_MEOOE5D, o.OP_MEOOE_DAG5D):
        assert o.rel_l2(zmob.apply(code, xo, 1), mob.apply(code, xo, 1)) < 1e-14, code


def test_zmobius_dminus_adjoint():
    op, _ = _zmobius()
    a, b = fermion(VOL, 10, 7), fermion(VOL, 10, 8)
    lhs = np.vdot(a, op.apply(o.OP_DMINUS, b)).conj()
    rhs = np.vdot(b, op.apply(o.OP_DMINUS_DAG, a))
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


# ---- MADWF pieces (CayleyFermion5DImplementation.h:70-88, MADWF.h) ----------------------
def test_p_is_a_chiral_shift_and_pdag_its_inverse():
    op, _ = _mobius(Ls=6)
    x = fermion(VOL, 6, 21)
    y = op.apply(o.OP_P, x).reshape(VOL, 6, 12)
    xr = x.reshape(VOL, 6, 12)
    assert np.array_equal(y[:, :, 6:], xr[:, :, 6:])                      # P- psi_s
    assert np.array_equal(y[:, :, :6], np.roll(xr[:, :, :6], -1, axis=1))  # P+ psi_{s+1}
    assert np.array_equal(op.apply(o.OP_PDAG, y.reshape(-1)), x)
    # Pdag is the adjoint of P
    z = fermion(VOL, 6, 22)
    assert abs(np.vdot(z, op.apply(o.OP_P, x)) - np.vdot(op.apply(o.OP_PDAG, z), x)) < 1e-12 * VOL


def test_set_mass_equals_a_fresh_operator():
    op, U = _mobius(Ls=6, mf=0.1)
    fresh = o.OracleOp(1, 0, DIMS, 6, [1.0, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    x = fermion(VOL, 6, 23)
    op.set_mass(1.0)
    assert np.array_equal(op.apply(o.OP_M, x), fresh.apply(o.OP_M, x))
    xh = fermion(VOL // 2, 6, 24)
    assert np.array_equal(op.apply(o.OP_MOOEE_INV, xh), fresh.apply(o.OP_MOOEE_INV, xh))


def test_madwf_with_inner_equal_outer_converges_in_one_step():
    """With the inner operator equal to the outer one the defect correction of MADWF.h is
    exact: one step reaches the solver tolerance, and the result is the direct solution."""
    from oracle import madwf as mw
    outer, U = _mobius(Ls=8, mf=0.05, eps=0.3, seed=5)
    inner = o.OracleOp(1, 0, DIMS, 8, [0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    b = outer.physical(o.IMPORT_PHYSICAL_SOURCE, fermion(VOL, 1, 4))
    sol, hist = mw.madwf(outer, 8, 0.05, inner, 8, 0.05, b, 1e-12, 1e-12, 1e-9, 3)
    assert len(hist) == 1 and hist[0] < 1e-10
    ref, _, _, _ = outer.schur_solve(b, 1e-11, 10000)
    assert o.rel_l2(sol, ref) < 1e-9


def test_madwf_with_smaller_ls_inner_converges_to_the_outer_solution():
    """Test_zMADWF_prec.cc's check: the MADWF solution equals the direct outer solve; the
    defect falls geometrically with an Ls = 4 inner operator."""
    from oracle import madwf as mw
    outer, U = _mobius(Ls=8, mf=0.05, eps=0.3, seed=5)
    inner = o.OracleOp(1, 0, DIMS, 4, [0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    b = outer.physical(o.IMPORT_PHYSICAL_SOURCE, fermion(VOL, 1, 4))
    sol, hist = mw.madwf(outer, 8, 0.05, inner, 4, 0.05, b, 1e-12, 1e-12, 1e-7, 20)
    assert hist[-1] < 1e-7 and all(b_ < 0.2 * a for a, b_ in zip(hist, hist[1:]))
    ref, _, _, _ = outer.schur_solve(b, 1e-11, 10000)
    assert o.rel_l2(sol, ref) < 1e-6


def test_reference_arm_generator_and_half_spinor_dhop():
    """The reference arm builds its inputs with the oracle's restatement of the library's
    seeded generator (equal bit for bit) and times the half-spinor CPU Dhop, which must
    equal the oracle's site-loop Dhop (FP32 arithmetic: relative L2 below 1e-6) for both
    checkerboards and both dagger signs."""
    dims, L5 = (4, 4, 4, 8), 8
    U = o.random_gauge(dims, 0.5, 1234)
    assert np.array_equal(U, g.random_gauge(dims, 0.5, 1234))
    assert np.array_equal(o.random_gaussian(999, 7), g.random_gaussian(999, 7))
    nh = int(np.prod(dims)) // 2
    ref = o.OracleOp(1, 0, dims, L5, [0.01, 1.8, 1.5, 0.5], U, g.antiperiodic_t())
    h = o.HalfSpinorDhop(dims, L5, U, g.antiperiodic_t())
    for in_cb in (1, 0):
        for dag in (0, 1):
            x = o.random_gaussian(nh * L5 * 12, 10 + in_cb)
            h.set(in_cb, x)
            h.dhop(1 - in_cb, dag)
            assert o.rel_l2(h.get(1 - in_cb), ref.dhop_cb(x, in_cb, dag)) < 1e-6
